// Inference engine for the MLARM surrogate networks (model_zoo/Net_ves_*.py).
//
// Every network is a chain of blocks with one template (e.g.
// model_zoo/Net_ves_merge_adv.py:6-64), applied independently to each of
// `groups` channel groups (grouped convolutions):
//
//   A = bn1(relu(conv7 s2 p3 circ (x)) ++ relu(conv7 s2 d2 p6 circ (x)))   [2c1][L/2]
//   B = bn2(relu(conv7 s2 p3 circ (A)) ++ relu(conv7 s2 d2 p6 circ (A)))   [2c2][L/4]
//   C = bn3(relu(convT10 s2 p4 (B)))                                    [2c2][L/2]
//   D = bn4(relu(convT10 s2 p4 (C)))                                    [2c2][L]
//   out[0:cmix] = mix3 p1 (D) (+ x[0:cmix] if residual); out[cmix:] = x[cin-npass:cin]
//
// This file holds the CUDA-core path: one CTA runs one whole block for one
// (group, vesicle) pair with every intermediate in shared memory, so a
// block reads its input and writes its output once.  It is templated on the
// arithmetic type: FP64 (parity against the FP64 oracle) and FP32 (the
// reference networks' own precision).
//
// Activations: [nv][groups * channels][L], the reference's (nv, C, L).
// Weights: one contiguous record per (block, group), eval-mode batch norm
// folded into a per-channel scale and shift (y = x * s + t).
#include <algorithm>
#include <cmath>
#include <new>
#include <vector>

#include "ves_internal.h"
#include "ves_nets_tc.h"

namespace {

enum {
  O_W11, O_B11, O_W12, O_B12, O_S1, O_T1,
  O_W21, O_B21, O_W22, O_B22, O_S2, O_T2,
  O_D1, O_BD1, O_S3, O_T3, O_D2, O_BD2, O_S4, O_T4,
  O_M, O_BM, O_END
};

struct BlockGeom {
  int cin, c1, c2, cmix, residual, npass;
  int off[O_END + 1];  // element offsets inside a group record; off[O_END] = record size
};

BlockGeom make_geom(const ves_net_block& b) {
  BlockGeom g;
  g.cin = b.cin;
  g.c1 = b.c1;
  g.c2 = b.c2;
  g.cmix = b.cmix;
  g.residual = b.residual;
  g.npass = b.npass;
  const int d = 2 * b.c2;
  const int sz[O_END] = {
      b.c1 * b.cin * 7, b.c1, b.c1 * b.cin * 7, b.c1, 2 * b.c1, 2 * b.c1,
      b.c2 * 2 * b.c1 * 7, b.c2, b.c2 * 2 * b.c1 * 7, b.c2, d, d,
      d * d * 10, d, d, d, d * d * 10, d, d, d,
      b.cmix * d * 3, b.cmix};
  int o = 0;
  for (int i = 0; i < O_END; ++i) {
    g.off[i] = o;
    o += (sz[i] + 1) & ~1;  // keep every array 16-byte aligned for double2 / float4 reads
  }
  g.off[O_END] = o;
  return g;
}

template <typename Real>
struct BlockArgs {
  const Real* w;  // group-0 record of this block
  int rec;        // elements per group record
  int cin, c1, c2, cmix, residual, npass, L;
  int off[O_END];
};

template <typename Real>
__device__ __forceinline__ Real relu_(Real v) {
  return v < Real(0) ? Real(0) : v;  // NaN propagates as in torch.relu
}

// y[o][p] = bn(relu(conv_branch(o)(x)))   o < 2c, p < Lin/2, circular padding
template <typename Real>
__device__ void conv_pair_s2(const Real* __restrict__ x, int cin, int Lin, const Real* __restrict__ w1,
                             const Real* __restrict__ b1, const Real* __restrict__ w2,
                             const Real* __restrict__ b2, int c, const Real* __restrict__ s,
                             const Real* __restrict__ t, Real* __restrict__ y) {
  const int Lout = Lin >> 1, mask = Lin - 1;
  const int total = 2 * c * Lout;
  for (int idx = threadIdx.x; idx < total; idx += blockDim.x) {
    const int o = idx / Lout, p = idx - o * Lout;
    const bool br = o >= c;
    const int oc = br ? o - c : o;
    const Real* w = (br ? w2 : w1) + oc * cin * 7;
    const int dil = br ? 2 : 1;
    const int base = 2 * p - (br ? 6 : 3);
    Real acc = (br ? b2 : b1)[oc];
    for (int ci = 0; ci < cin; ++ci) {
      const Real* xr = x + ci * Lin;
      const Real* wr = w + ci * 7;
#pragma unroll
      for (int tt = 0; tt < 7; ++tt) acc = fma(wr[tt], xr[(base + dil * tt) & mask], acc);
    }
    y[idx] = fma(relu_(acc), s[o], t[o]);
  }
}

// ConvTranspose1d(C, C, 10, stride 2, padding 4): y[o][j] = b[o] + sum_{c,t} w[c][o][t] x[c][(j+4-t)/2]
template <typename Real>
__device__ void deconv_s2(const Real* __restrict__ x, int C, int Lin, const Real* __restrict__ w,
                          const Real* __restrict__ b, const Real* __restrict__ s, const Real* __restrict__ t,
                          Real* __restrict__ y) {
  const int Lout = 2 * Lin;
  const int total = C * Lout;
  for (int idx = threadIdx.x; idx < total; idx += blockDim.x) {
    const int o = idx / Lout, j = idx - o * Lout;
    const int r = j & 1;
    int ii[5];
#pragma unroll
    for (int u = 0; u < 5; ++u) {
      const int i = (j + 4 - r - 2 * u) >> 1;
      ii[u] = (i >= 0 && i < Lin) ? i : -1;
    }
    Real acc = b[o];
    for (int ci = 0; ci < C; ++ci) {
      const Real* wr = w + (ci * C + o) * 10 + r;
      const Real* xr = x + ci * Lin;
#pragma unroll
      for (int u = 0; u < 5; ++u)
        if (ii[u] >= 0) acc = fma(wr[2 * u], xr[ii[u]], acc);
    }
    y[idx] = fma(relu_(acc), s[o], t[o]);
  }
}

template <typename Real>
__global__ void __launch_bounds__(256) net_block_kernel(BlockArgs<Real> a, const Real* __restrict__ in,
                                                        long long in_vs, Real* __restrict__ out,
                                                        long long out_vs) {
  extern __shared__ __align__(16) unsigned char smraw[];
  Real* sm = reinterpret_cast<Real*>(smraw);
  const int g = blockIdx.x;
  const long long v = blockIdx.y;
  const int L = a.L, L2 = L >> 1, L4 = L >> 2;
  const int d = 2 * a.c2;
  const Real* W = a.w + (long long)g * a.rec;
  Real* x = sm;                                        // [cin][L]
  Real* A = x + a.cin * L;                             // [2c1][L/2], later C [2c2][L/2]
  Real* B = A + max(2 * a.c1, d) * L2;                 // [2c2][L/4], later D [2c2][L]
  const Real* xin = in + v * in_vs + (long long)g * a.cin * L;
  for (int i = threadIdx.x; i < a.cin * L; i += blockDim.x) x[i] = xin[i];
  __syncthreads();
  conv_pair_s2(x, a.cin, L, W + a.off[O_W11], W + a.off[O_B11], W + a.off[O_W12], W + a.off[O_B12], a.c1,
               W + a.off[O_S1], W + a.off[O_T1], A);
  __syncthreads();
  conv_pair_s2(A, 2 * a.c1, L2, W + a.off[O_W21], W + a.off[O_B21], W + a.off[O_W22], W + a.off[O_B22], a.c2,
               W + a.off[O_S2], W + a.off[O_T2], B);
  __syncthreads();
  deconv_s2(B, d, L4, W + a.off[O_D1], W + a.off[O_BD1], W + a.off[O_S3], W + a.off[O_T3], A);
  __syncthreads();
  deconv_s2(A, d, L2, W + a.off[O_D2], W + a.off[O_BD2], W + a.off[O_S4], W + a.off[O_T4], B);
  __syncthreads();
  // mix (kernel 3, zero padding 1), residual, pass-through channels
  const int cout = a.cmix + a.npass;
  Real* o = out + v * out_vs + (long long)g * cout * L;
  const Real* M = W + a.off[O_M];
  const Real* bm = W + a.off[O_BM];
  for (int idx = threadIdx.x; idx < a.cmix * L; idx += blockDim.x) {
    const int oc = idx / L, j = idx - oc * L;
    Real acc = bm[oc];
    for (int ci = 0; ci < d; ++ci) {
      const Real* wr = M + (oc * d + ci) * 3;
      const Real* dr = B + ci * L;
      if (j > 0) acc = fma(wr[0], dr[j - 1], acc);
      acc = fma(wr[1], dr[j], acc);
      if (j + 1 < L) acc = fma(wr[2], dr[j + 1], acc);
    }
    if (a.residual) acc += x[oc * L + j];
    o[idx] = acc;
  }
  for (int idx = threadIdx.x; idx < a.npass * L; idx += blockDim.x)
    o[a.cmix * L + idx] = x[(a.cin - a.npass) * L + idx];
}

template <typename Real>
size_t block_smem(const BlockGeom& b, int L) {
  const int d = 2 * b.c2;
  return (size_t)(b.cin * L + std::max(2 * b.c1, d) * (L / 2) + d * L) * sizeof(Real);
}

}  // namespace

struct ves_net {
  int device = 0;
  int precision = VES_NET_FP32;
  int groups = 0, length = 0;
  std::vector<BlockGeom> blocks;
  std::vector<long long> boff;  // element offset of each block's group-0 record
  int cmax = 0;                 // largest channel count per group of any block output
  void* d_w = nullptr;
  size_t elem = 4;
  // tensor-core path
  std::vector<TcBlock> tcb;
  unsigned char* d_tc = nullptr;
  int mid_max = 0;
  VesDeviceStatus* d_status = nullptr;
  int autotune = 0;             // tensor-core path: time the launch shapes on the first call per nv
};

namespace {

// Fold one block of reference parameters into the per-group records.
void pack_block(const BlockGeom& b, int G, const float* const* p, double* dst) {
  const int d = 2 * b.c2;
  const int rec = b.off[O_END];
  auto bn = [&](const float* w, const float* bias, const float* mean, const float* var, int ch, int n, double* s,
                double* t) {
    for (int i = 0; i < n; ++i) {
      const double inv = 1.0 / std::sqrt((double)var[ch + i] + 1e-5);
      s[i] = (double)w[ch + i] * inv;
      t[i] = (double)bias[ch + i] - (double)mean[ch + i] * s[i];
    }
  };
  for (int g = 0; g < G; ++g) {
    double* r = dst + (size_t)g * rec;
    auto copy = [&](const float* src, size_t start, int n, int slot) {
      for (int i = 0; i < n; ++i) r[b.off[slot] + i] = (double)src[start + i];
    };
    copy(p[0], (size_t)g * b.c1 * b.cin * 7, b.c1 * b.cin * 7, O_W11);
    copy(p[1], (size_t)g * b.c1, b.c1, O_B11);
    copy(p[2], (size_t)g * b.c1 * b.cin * 7, b.c1 * b.cin * 7, O_W12);
    copy(p[3], (size_t)g * b.c1, b.c1, O_B12);
    copy(p[4], (size_t)g * b.c2 * 2 * b.c1 * 7, b.c2 * 2 * b.c1 * 7, O_W21);
    copy(p[5], (size_t)g * b.c2, b.c2, O_B21);
    copy(p[6], (size_t)g * b.c2 * 2 * b.c1 * 7, b.c2 * 2 * b.c1 * 7, O_W22);
    copy(p[7], (size_t)g * b.c2, b.c2, O_B22);
    copy(p[8], (size_t)g * d * d * 10, d * d * 10, O_D1);
    copy(p[9], (size_t)g * d, d, O_BD1);
    copy(p[10], (size_t)g * d * d * 10, d * d * 10, O_D2);
    copy(p[11], (size_t)g * d, d, O_BD2);
    copy(p[12], (size_t)g * b.cmix * d * 3, b.cmix * d * 3, O_M);
    copy(p[13], (size_t)g * b.cmix, b.cmix, O_BM);
    bn(p[14], p[15], p[16], p[17], g * 2 * b.c1, 2 * b.c1, r + b.off[O_S1], r + b.off[O_T1]);
    bn(p[18], p[19], p[20], p[21], g * d, d, r + b.off[O_S2], r + b.off[O_T2]);
    bn(p[22], p[23], p[24], p[25], g * d, d, r + b.off[O_S3], r + b.off[O_T3]);
    bn(p[26], p[27], p[28], p[29], g * d, d, r + b.off[O_S4], r + b.off[O_T4]);
  }
}

template <typename Real>
int run_block(const ves_net* net, int bi, int nv, const Real* in, Real* out, cudaStream_t s) {
  const BlockGeom& b = net->blocks[bi];
  const int L = net->length;
  BlockArgs<Real> a;
  a.w = reinterpret_cast<const Real*>(net->d_w) + net->boff[bi];
  a.rec = b.off[O_END];
  a.cin = b.cin;
  a.c1 = b.c1;
  a.c2 = b.c2;
  a.cmix = b.cmix;
  a.residual = b.residual;
  a.npass = b.npass;
  a.L = L;
  for (int i = 0; i < O_END; ++i) a.off[i] = b.off[i];
  const size_t sh = block_smem<Real>(b, L);
  if (sh > 48 * 1024) {
    int rc = ves_cuda_status(
        cudaFuncSetAttribute(net_block_kernel<Real>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sh),
        "net block smem");
    if (rc) return rc;
  }
  const long long in_vs = (long long)net->groups * b.cin * L;
  const long long out_vs = (long long)net->groups * (b.cmix + b.npass) * L;
  dim3 grid(net->groups, nv);
  ves_count_launch();
  net_block_kernel<Real><<<grid, 256, sh, s>>>(a, in, in_vs, out, out_vs);
  return ves_launch_check("net block");
}

template <typename Real>
int net_forward_t(const ves_net* net, int nv, const Real* in, Real* out, WsCarver& ws, VesDeviceStatus* st,
                  cudaStream_t s) {
  const size_t buf = (size_t)nv * net->groups * net->cmax * net->length;
  const int nb = (int)net->blocks.size();
  Real* p0 = nb > 1 ? ws.take<Real>(buf) : nullptr;
  Real* p1 = nb > 2 ? ws.take<Real>(buf) : nullptr;
  const bool tc = net->precision == VES_NET_BF16;
  // the tensor-core intermediates: nv rounded up to whole tiles of 4 vesicles
  unsigned char* mid = tc ? ws.take<unsigned char>((size_t)((nv + 3) / 4 * 4) * net->groups * net->mid_max) : nullptr;
  if (ws.sizing) return VES_OK;
  if (!ws.ok()) {
    ves_record_error(VES_ERR_WORKSPACE, "net_forward: workspace too small (%zu needed)", ws.off);
    return VES_ERR_WORKSPACE;
  }
  if (nv <= 0) return VES_OK;
  const Real* src = in;
  for (int bi = 0; bi < nb; ++bi) {
    Real* dst = (bi == nb - 1) ? out : ((bi & 1) ? p1 : p0);
    int rc;
    if (tc) {
      const TcBlock& tb = net->tcb[bi];
      rc = tcnet_run_block(tb, net->groups, nv, net->d_tc + tb.down_off, net->d_tc + tb.up1_off, net->d_tc + tb.up2_off,
                           reinterpret_cast<const float*>(src), reinterpret_cast<float*>(dst), mid,
                           st ? st : net->d_status, s, net->autotune != 0);
    } else {
      rc = run_block<Real>(net, bi, nv, src, dst, s);
    }
    if (rc) return rc;
    src = dst;
  }
  return VES_OK;
}

}  // namespace

int net_forward_run(const ves_net* net, int nv, const void* in, void* out, WsCarver& ws, VesDeviceStatus* st,
                    cudaStream_t s) {
  if (net->precision == VES_NET_FP64)
    return net_forward_t<double>(net, nv, (const double*)in, (double*)out, ws, st, s);
  return net_forward_t<float>(net, nv, (const float*)in, (float*)out, ws, st, s);
}

// useful work of one vesicle through the network: 2 x multiply-adds of the
// conv pairs, the two transposed convs (5 taps per output) and the mix
double net_flops_per_vesicle(const ves_net* net) {
  const double L = net->length;
  double f = 0;
  for (const BlockGeom& b : net->blocks) {
    const double d = 2.0 * b.c2;
    f += 2 * (L / 2) * b.c1 * b.cin * 7 + 2 * (L / 4) * b.c2 * 2 * b.c1 * 7;
    f += (L / 2) * d * d * 5 + L * d * d * 5 + L * b.cmix * d * 3;
  }
  return 2.0 * f * net->groups;
}

int net_dims(const ves_net* net, int* groups, int* length, int* cin, int* cout) {
  if (groups) *groups = net->groups;
  if (length) *length = net->length;
  if (cin) *cin = net->blocks.front().cin;
  if (cout) *cout = net->blocks.back().cmix + net->blocks.back().npass;
  return net->precision;
}

extern "C" int ves_net_create(int precision, int groups, int length, int nblocks, const ves_net_block* blocks,
                              const float* const* params, ves_net** out) {
  if (!out || !blocks || !params || nblocks <= 0 || groups <= 0) {
    ves_record_error(VES_ERR_ARG, "net_create: bad arguments");
    return VES_ERR_ARG;
  }
  *out = nullptr;
  if (precision != VES_NET_FP64 && precision != VES_NET_FP32 && precision != VES_NET_BF16) {
    ves_record_error(VES_ERR_ARG, "net_create: precision %d not supported", precision);
    return VES_ERR_ARG;
  }
  if (length < 16 || (length & (length - 1))) {
    ves_record_error(VES_ERR_ARG, "net_create: length %d must be a power of two >= 16", length);
    return VES_ERR_ARG;
  }
  ves_net* net = new (std::nothrow) ves_net;
  if (!net) {
    ves_record_error(VES_ERR_CUDA, "net_create: out of host memory");
    return VES_ERR_CUDA;
  }
  net->precision = precision;
  net->groups = groups;
  net->length = length;
  net->elem = precision == VES_NET_FP64 ? 8 : 4;
  const bool tc = precision == VES_NET_BF16;
  long long total = 0;
  int prev_out = blocks[0].cin;
  for (int i = 0; i < nblocks; ++i) {
    const ves_net_block& b = blocks[i];
    if (b.cin <= 0 || b.c1 <= 0 || b.c2 <= 0 || b.cmix <= 0 || b.npass < 0 || b.npass > b.cin ||
        (b.residual && b.cmix > b.cin) || b.cin != prev_out) {
      ves_record_error(VES_ERR_ARG, "net_create: block %d has inconsistent channel counts", i);
      delete net;
      return VES_ERR_ARG;
    }
    for (int k = 0; k < 30; ++k)
      if (!params[(size_t)i * 30 + k]) {
        ves_record_error(VES_ERR_ARG, "net_create: block %d parameter %d missing", i, k);
        delete net;
        return VES_ERR_ARG;
      }
    BlockGeom g = make_geom(b);
    const size_t sh = precision == VES_NET_FP64 ? block_smem<double>(g, length) : block_smem<float>(g, length);
    if (!tc && sh > 227 * 1024) {
      ves_record_error(VES_ERR_ARG, "net_create: block %d needs %zu bytes of shared memory", i, sh);
      delete net;
      return VES_ERR_ARG;
    }
    net->blocks.push_back(g);
    net->boff.push_back(total);
    total += (long long)g.off[O_END] * groups;
    prev_out = b.cmix + b.npass;
    net->cmax = std::max(net->cmax, prev_out);
  }
  int dev = 0;
  cudaGetDevice(&dev);
  net->device = dev;
  int rc0 = ves_cuda_status(cudaMalloc(&net->d_status, sizeof(VesDeviceStatus)), "net status");
  if (!rc0) rc0 = ves_cuda_status(cudaMemset(net->d_status, 0, sizeof(VesDeviceStatus)), "net status");
  if (rc0) {
    delete net;
    return rc0;
  }
  if (tc) {
    std::vector<unsigned char> img, down, up1, up2;
    for (int i = 0; i < nblocks; ++i) {
      TcBlock tb;
      if (tcnet_pack(blocks[i], groups, length, params + (size_t)i * 30, down, up1, up2, tb)) {
        ves_record_error(VES_ERR_ARG, "net_create: block %d does not fit the tensor-core kernels", i);
        cudaFree(net->d_status);
        delete net;
        return VES_ERR_ARG;
      }
      tb.down_off = img.size();
      img.insert(img.end(), down.begin(), down.end());
      tb.up1_off = img.size();
      img.insert(img.end(), up1.begin(), up1.end());
      tb.up2_off = img.size();
      img.insert(img.end(), up2.begin(), up2.end());
      net->mid_max = std::max(net->mid_max, tb.mid_bytes);
      net->tcb.push_back(tb);
    }
    int rc = ves_cuda_status(cudaMalloc(&net->d_tc, img.size()), "net tc weights");
    if (!rc) rc = ves_cuda_status(cudaMemcpy(net->d_tc, img.data(), img.size(), cudaMemcpyHostToDevice), "net upload");
    if (rc) {
      if (net->d_tc) cudaFree(net->d_tc);
      cudaFree(net->d_status);
      delete net;
      return rc;
    }
    *out = net;
    return VES_OK;
  }
  std::vector<double> host((size_t)total);
  for (int i = 0; i < nblocks; ++i) pack_block(net->blocks[i], groups, params + (size_t)i * 30, host.data() + net->boff[i]);
  int rc = ves_cuda_status(cudaMalloc(&net->d_w, (size_t)total * net->elem), "net weights");
  if (rc) {
    delete net;
    return rc;
  }
  if (precision == VES_NET_FP64) {
    rc = ves_cuda_status(cudaMemcpy(net->d_w, host.data(), (size_t)total * 8, cudaMemcpyHostToDevice), "net upload");
  } else {
    std::vector<float> h32(host.begin(), host.end());
    rc = ves_cuda_status(cudaMemcpy(net->d_w, h32.data(), (size_t)total * 4, cudaMemcpyHostToDevice), "net upload");
  }
  if (rc) {
    cudaFree(net->d_w);
    delete net;
    return rc;
  }
  *out = net;
  return VES_OK;
}

extern "C" int ves_net_destroy(ves_net* net) {
  if (!net) return VES_OK;
  if (net->d_w) cudaFree(net->d_w);
  if (net->d_tc) cudaFree(net->d_tc);
  if (net->d_status) cudaFree(net->d_status);
  delete net;
  return VES_OK;
}

extern "C" int ves_net_set_autotune(ves_net* net, int on) {
  if (!net) return VES_ERR_ARG;
  net->autotune = on ? 1 : 0;
  return VES_OK;
}

extern "C" int ves_net_info(const ves_net* net, int* precision, int* groups, int* length, int* cin, int* cout) {
  if (!net) return VES_ERR_ARG;
  const int p = net_dims(net, groups, length, cin, cout);
  if (precision) *precision = p;
  return VES_OK;
}

extern "C" size_t ves_net_forward_workspace(const ves_net* net, int nv) {
  if (!net) return 0;
  WsCarver w(nullptr, 0);
  net_forward_run(net, nv, nullptr, nullptr, w, nullptr, 0);
  return w.off + 256;
}

extern "C" int ves_net_forward(const ves_net* net, int nv, const void* in, void* out, void* ws, size_t ws_bytes,
                               void* stream) {
  if (!net || (nv > 0 && (!in || !out))) {
    ves_record_error(VES_ERR_ARG, "net_forward: bad arguments");
    return VES_ERR_ARG;
  }
  if (!ws && net->blocks.size() > 1 && nv > 0) {
    ves_record_error(VES_ERR_WORKSPACE, "net_forward: workspace required");
    return VES_ERR_WORKSPACE;
  }
  char none = 0;  // a non-null base so that a one-block network (no workspace) runs
  WsCarver w(ws ? ws : (void*)&none, ws ? ws_bytes : 0);
  cudaStream_t s = (cudaStream_t)stream;
  int rc = net_forward_run(net, nv, in, out, w, nullptr, s);
  if (rc || net->precision != VES_NET_BF16) return rc;
  // the tensor-core kernels report bounded-wait timeouts in the status word
  VesDeviceStatus h;
  rc = ves_cuda_status(cudaMemcpyAsync(&h, net->d_status, sizeof(h), cudaMemcpyDeviceToHost, s), "net status");
  if (!rc) rc = ves_cuda_status(cudaStreamSynchronize(s), "net status sync");
  if (rc) return rc;
  if (h.code != VES_OK) {
    ves_record_error(h.code, "net_forward: tensor-core kernel reported status %d (site %d)", h.code, h.where);
    return h.code;
  }
  return VES_OK;
}
