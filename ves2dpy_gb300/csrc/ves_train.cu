// Training engine for the MLARM networks (the block template of
// model_zoo/Net_ves_merge_adv.py:6-191, Net_ves_factor.py:6-61 and siblings)
// with one channel group: forward with stored activations, backward through
// every layer type, Adam.  The reference ships no training code on the hot
// path; its networks were trained per Fourier mode and merged into grouped
// convolutions (get_network_torch.py:99-128).  Here one group is trained on a
// batch of samples; a merged network carries the trained weights in each of
// its groups.
//
// Layers of a block (x: cin channels of length L):
//   a = bn1(relu(conv7_s2(x)) ++ relu(conv7_s2_dil2(x)))    circular padding 3 / 6
//   b = bn2(relu(conv7_s2(a)) ++ relu(conv7_s2_dil2(a)))
//   c = bn3(relu(deconv10_s2(b)))   d = bn4(relu(deconv10_s2(c)))   padding 4, zero fill
//   m = mix3(d)   out = [m + x[:cmix] if residual] ++ x[cin-npass:]
// Batch norm is the evaluation-mode affine map with frozen running statistics
// (its weight and bias are trained).
//
// Every kernel stages one sample's activations in shared memory and walks a
// tile of output channels (forward and data gradients) or of weight
// coefficients (weight gradients) over a chunk of samples; the weight
// gradients of the chunks meet in global memory by atomic addition.
#include <math.h>
#include <string.h>

#include <algorithm>
#include <new>
#include <vector>

#include "ves_internal.h"

namespace {

constexpr int kOT = 16;      // output channels per CTA (forward / data gradients)
constexpr int kThreads = 256;
constexpr double kBnEps = 1e-5;

template <typename Real>
__device__ __forceinline__ Real relu(Real v) {
  return v > Real(0) ? v : Real(0);
}

// ---- forward -----------------------------------------------------------------

// stride-2 circular convolution (kernel 7, dilation dil, padding pad), ReLU;
// out[b][coff + o][p] of a ctot-channel tensor of length L/2
template <typename Real>
__global__ void __launch_bounds__(kThreads) conv_fwd_kernel(int B, int spg, int cin, int L, int cout, int dil, int pad,
                                                            const Real* __restrict__ W, const Real* __restrict__ bias,
                                                            const Real* __restrict__ x, int ctot, int coff,
                                                            Real* __restrict__ out) {
  extern __shared__ unsigned char smraw[];
  Real* sw = (Real*)smraw;            // [kOT][cin][7]
  Real* sx = sw + kOT * cin * 7;      // [cin][L]
  const int o0 = blockIdx.x * kOT, no = min(kOT, cout - o0);
  const int Lo = L / 2;
  for (int i = threadIdx.x; i < no * cin * 7; i += blockDim.x) sw[i] = W[(long long)o0 * cin * 7 + i];
  const int b0 = blockIdx.y * spg, b1 = min(B, b0 + spg);
  for (int b = b0; b < b1; ++b) {
    __syncthreads();
    for (int i = threadIdx.x; i < cin * L; i += blockDim.x) sx[i] = x[(long long)b * cin * L + i];
    __syncthreads();
    for (int idx = threadIdx.x; idx < no * Lo; idx += blockDim.x) {
      const int o = idx / Lo, p = idx % Lo;
      Real s = bias[o0 + o];
      const Real* w = sw + o * cin * 7;
      for (int c = 0; c < cin; ++c) {
        const Real* xc = sx + c * L;
#pragma unroll
        for (int k = 0; k < 7; ++k) {
          int q = 2 * p + dil * k - pad;
          q = q < 0 ? q + L : (q >= L ? q - L : q);
          s += w[c * 7 + k] * xc[q];
        }
      }
      out[((long long)b * ctot + coff + o0 + o) * Lo + p] = relu(s);
    }
  }
}

// transposed convolution, kernel 10, stride 2, padding 4 (output 2 Lin), ReLU;
// W[ci][co][10].  Output j = 2m + par takes taps k = par + 2u (u = 0..4) of
// input i = m + 2 - u: a 5-tap convolution per output parity.  A thread
// computes kR consecutive m of one (channel, parity) from kR + 4 inputs held
// in registers (zero halo of 2 in shared memory).
constexpr int kR = 4;

template <typename Real>
__global__ void __launch_bounds__(kThreads) deconv_fwd_kernel(int B, int spg, int d, int Lin, const Real* __restrict__ W,
                                                              const Real* __restrict__ bias, const Real* __restrict__ x,
                                                              Real* __restrict__ out) {
  extern __shared__ unsigned char smraw[];
  Real* sw = (Real*)smraw;          // [d][kOT][10]
  Real* sx = sw + d * kOT * 10;     // [d][Lin + 4], input i at i + 2
  const int o0 = blockIdx.x * kOT, no = min(kOT, d - o0);
  const int Lp = Lin + 4, Lo = 2 * Lin;
  const int nmb = (Lin + kR - 1) / kR;
  for (int i = threadIdx.x; i < d * no * 10; i += blockDim.x) {
    const int c = i / (no * 10), r = i % (no * 10);
    sw[c * kOT * 10 + r] = W[((long long)c * d + o0) * 10 + r];
  }
  const int b0 = blockIdx.y * spg, b1 = min(B, b0 + spg);
  for (int b = b0; b < b1; ++b) {
    __syncthreads();
    for (int i = threadIdx.x; i < d * Lp; i += blockDim.x) {
      const int c = i / Lp, q = i % Lp - 2;
      sx[i] = (q >= 0 && q < Lin) ? x[((long long)b * d + c) * Lin + q] : Real(0);
    }
    __syncthreads();
    for (int item = threadIdx.x; item < no * 2 * nmb; item += blockDim.x) {
      const int o = item / (2 * nmb), rem = item % (2 * nmb), par = rem / nmb, m0 = (rem % nmb) * kR;
      Real acc[kR];
#pragma unroll
      for (int r = 0; r < kR; ++r) acc[r] = bias[o0 + o];
      for (int c = 0; c < d; ++c) {
        const Real* xc = sx + c * Lp + m0;  // xc[t] = input m0 - 2 + t
        const Real* w = sw + (c * kOT + o) * 10 + par;
        Real xi[kR + 4];
#pragma unroll
        for (int t = 0; t < kR + 4; ++t) xi[t] = (m0 + t < Lp) ? xc[t] : Real(0);
#pragma unroll
        for (int u = 0; u < 5; ++u) {
          const Real wv = w[2 * u];
#pragma unroll
          for (int r = 0; r < kR; ++r) acc[r] += wv * xi[r + 4 - u];
        }
      }
#pragma unroll
      for (int r = 0; r < kR; ++r) {
        const int m = m0 + r;
        if (m < Lin) out[((long long)b * d + o0 + o) * Lo + 2 * m + par] = relu(acc[r]);
      }
    }
  }
}

// mixing convolution (kernel 3, padding 1, zero fill) + residual and
// pass-through channels: out[b][cout][L]
template <typename Real>
__global__ void __launch_bounds__(kThreads) mix_fwd_kernel(int B, int spg, int d, int L, int cmix, int cin, int npass,
                                                           int residual, const Real* __restrict__ W,
                                                           const Real* __restrict__ bias, const Real* __restrict__ D,
                                                           const Real* __restrict__ x0, Real* __restrict__ out) {
  extern __shared__ unsigned char smraw[];
  Real* sw = (Real*)smraw;        // [kOT][d][3]
  Real* sd = sw + kOT * d * 3;    // [d][L]
  const int o0 = blockIdx.x * kOT, no = min(kOT, cmix - o0);
  const int cout = cmix + npass;
  for (int i = threadIdx.x; i < no * d * 3; i += blockDim.x) sw[i] = W[(long long)o0 * d * 3 + i];
  const int b0 = blockIdx.y * spg, b1 = min(B, b0 + spg);
  for (int b = b0; b < b1; ++b) {
    __syncthreads();
    for (int i = threadIdx.x; i < d * L; i += blockDim.x) sd[i] = D[(long long)b * d * L + i];
    __syncthreads();
    for (int idx = threadIdx.x; idx < no * L; idx += blockDim.x) {
      const int o = idx / L, p = idx % L;
      Real s = bias[o0 + o];
      const Real* w = sw + o * d * 3;
      for (int c = 0; c < d; ++c) {
        const Real* dc = sd + c * L;
        if (p > 0) s += w[c * 3] * dc[p - 1];
        s += w[c * 3 + 1] * dc[p];
        if (p + 1 < L) s += w[c * 3 + 2] * dc[p + 1];
      }
      if (residual) s += x0[((long long)b * cin + o0 + o) * L + p];
      out[((long long)b * cout + o0 + o) * L + p] = s;
    }
    if (blockIdx.x == 0)
      for (int idx = threadIdx.x; idx < npass * L; idx += blockDim.x) {
        const int q = idx / L, p = idx % L;
        out[((long long)b * cout + cmix + q) * L + p] = x0[((long long)b * cin + cin - npass + q) * L + p];
      }
  }
}

// evaluation-mode batch norm: out = (R - rm) / sqrt(rv + eps) * w + bb
template <typename Real>
__global__ void bn_fwd_kernel(long long n, int C, int len, const Real* __restrict__ R, const Real* __restrict__ w,
                              const Real* __restrict__ bb, const Real* __restrict__ rm, const Real* __restrict__ rv,
                              Real* __restrict__ out) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int c = (int)((i / len) % C);
  const Real rs = Real(1) / sqrt(rv[c] + Real(kBnEps));
  out[i] = (R[i] - rm[c]) * rs * w[c] + bb[c];
}

// ---- backward ----------------------------------------------------------------

// batch norm + ReLU: dZ = dY * w / sqrt(rv + eps) where R > 0 (R = relu output),
// dw += sum dY (R - rm)/sqrt(rv + eps), db += sum dY.  dZ may alias dY.
template <typename Real>
__global__ void __launch_bounds__(kThreads) bn_bwd_kernel(int B, int spg, int C, int len, const Real* dY,
                                                          const Real* __restrict__ R, const Real* __restrict__ w,
                                                          const Real* __restrict__ rm, const Real* __restrict__ rv,
                                                          Real* dZ, Real* __restrict__ dw, Real* __restrict__ db) {
  __shared__ Real red[2][kThreads];
  const int c = blockIdx.x;
  const Real rs = Real(1) / sqrt(rv[c] + Real(kBnEps));
  const Real sc = w[c] * rs, m = rm[c];
  Real aw = 0, ab = 0;
  const int b0 = blockIdx.y * spg, b1 = min(B, b0 + spg);
  for (int b = b0; b < b1; ++b) {
    const long long base = ((long long)b * C + c) * len;
    for (int p = threadIdx.x; p < len; p += blockDim.x) {
      const Real g = dY[base + p], r = R[base + p];
      aw += g * (r - m) * rs;
      ab += g;
      dZ[base + p] = r > Real(0) ? g * sc : Real(0);
    }
  }
  red[0][threadIdx.x] = aw;
  red[1][threadIdx.x] = ab;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) {
      red[0][threadIdx.x] += red[0][threadIdx.x + s];
      red[1][threadIdx.x] += red[1][threadIdx.x + s];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    atomicAdd(&dw[c], red[0][0]);
    atomicAdd(&db[c], red[1][0]);
  }
}

// bias gradient: db[o] += sum over samples and positions of dZ[b][coff+o][p]
template <typename Real>
__global__ void __launch_bounds__(kThreads) bias_grad_kernel(int B, int spg, int ctot, int coff, int len,
                                                             const Real* __restrict__ dZ, Real* __restrict__ db) {
  __shared__ Real red[kThreads];
  const int o = blockIdx.x;
  Real a = 0;
  const int b0 = blockIdx.y * spg, b1 = min(B, b0 + spg);
  for (int b = b0; b < b1; ++b) {
    const long long base = ((long long)b * ctot + coff + o) * len;
    for (int p = threadIdx.x; p < len; p += blockDim.x) a += dZ[base + p];
  }
  red[threadIdx.x] = a;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0) atomicAdd(&db[o], red[0]);
}

// mix data gradient: dD[b][c][q] = sum_o sum_k W[o][c][k] dOut[b][o][q - k + 1]
template <typename Real>
__global__ void __launch_bounds__(kThreads) mix_bwd_data_kernel(int B, int spg, int d, int L, int cmix, int cout,
                                                                const Real* __restrict__ W,
                                                                const Real* __restrict__ dout, Real* __restrict__ dD) {
  extern __shared__ unsigned char smraw[];
  Real* sw = (Real*)smraw;        // [cmix][kOT][3]
  Real* sg = sw + cmix * kOT * 3; // [cmix][L]
  const int c0 = blockIdx.x * kOT, nc = min(kOT, d - c0);
  for (int i = threadIdx.x; i < cmix * nc * 3; i += blockDim.x) {
    const int o = i / (nc * 3), r = i % (nc * 3);
    sw[o * kOT * 3 + r] = W[((long long)o * d + c0) * 3 + r];
  }
  const int b0 = blockIdx.y * spg, b1 = min(B, b0 + spg);
  for (int b = b0; b < b1; ++b) {
    __syncthreads();
    for (int i = threadIdx.x; i < cmix * L; i += blockDim.x) sg[i] = dout[(long long)b * cout * L + i];
    __syncthreads();
    for (int idx = threadIdx.x; idx < nc * L; idx += blockDim.x) {
      const int c = idx / L, q = idx % L;
      Real s = 0;
      for (int o = 0; o < cmix; ++o) {
        const Real* w = sw + (o * kOT + c) * 3;
        const Real* g = sg + o * L;
        if (q + 1 < L) s += w[0] * g[q + 1];
        s += w[1] * g[q];
        if (q > 0) s += w[2] * g[q - 1];
      }
      dD[((long long)b * d + c0 + c) * L + q] = s;
    }
  }
}

// transposed-conv data gradient: dIn[b][c][i] = sum_o sum_k W[c][o][k] dZ[b][o][2i + k - 4]
// = sum_o sum_par sum_u W[c][o][par + 2u] dZ_par[o][i + u - 2] with dZ_par[o][m] =
// dZ[o][2m + par]; a thread computes kR consecutive i of one channel
template <typename Real>
__global__ void __launch_bounds__(kThreads) deconv_bwd_data_kernel(int B, int spg, int d, int Lin,
                                                                   const Real* __restrict__ W,
                                                                   const Real* __restrict__ dZ,
                                                                   Real* __restrict__ dIn) {
  extern __shared__ unsigned char smraw[];
  Real* sw = (Real*)smraw;          // [kOT][d][10]
  Real* sg = sw + kOT * d * 10;     // [2][d][Lin + 4]: parity, channel, m + 2
  const int c0 = blockIdx.x * kOT, nc = min(kOT, d - c0);
  const int Lp = Lin + 4, Lo = 2 * Lin;
  const int nib = (Lin + kR - 1) / kR;
  for (int i = threadIdx.x; i < nc * d * 10; i += blockDim.x) sw[i] = W[(long long)c0 * d * 10 + i];
  const int b0 = blockIdx.y * spg, b1 = min(B, b0 + spg);
  for (int b = b0; b < b1; ++b) {
    __syncthreads();
    for (int i = threadIdx.x; i < 2 * d * Lp; i += blockDim.x) {
      const int par = i / (d * Lp), rem = i % (d * Lp), o = rem / Lp, m = rem % Lp - 2;
      sg[i] = (m >= 0 && m < Lin) ? dZ[((long long)b * d + o) * Lo + 2 * m + par] : Real(0);
    }
    __syncthreads();
    for (int item = threadIdx.x; item < nc * nib; item += blockDim.x) {
      const int c = item / nib, i0 = (item % nib) * kR;
      Real acc[kR];
#pragma unroll
      for (int r = 0; r < kR; ++r) acc[r] = 0;
      const Real* w = sw + c * d * 10;
      for (int par = 0; par < 2; ++par)
        for (int o = 0; o < d; ++o) {
          const Real* g = sg + (par * d + o) * Lp + i0;  // g[t] = dZ_par[o][i0 - 2 + t]
          Real gi[kR + 4];
#pragma unroll
          for (int t = 0; t < kR + 4; ++t) gi[t] = (i0 + t < Lp) ? g[t] : Real(0);
#pragma unroll
          for (int u = 0; u < 5; ++u) {
            const Real wv = w[o * 10 + par + 2 * u];
#pragma unroll
            for (int r = 0; r < kR; ++r) acc[r] += wv * gi[r + u];
          }
        }
#pragma unroll
      for (int r = 0; r < kR; ++r)
        if (i0 + r < Lin) dIn[((long long)b * d + c0 + c) * Lin + i0 + r] = acc[r];
    }
  }
}

// stride-2 conv data gradient (accumulate): dIn[b][c][q] += sum_o sum_k
// W[o][c][k] dZ[b][zoff + o][p] with 2p = (q + pad - dil k) mod L
template <typename Real>
__global__ void __launch_bounds__(kThreads) conv_bwd_data_kernel(int B, int spg, int cin, int L, int cout, int dil,
                                                                 int pad, const Real* __restrict__ W, int ztot, int zoff,
                                                                 const Real* __restrict__ dZ, int accumulate,
                                                                 Real* __restrict__ dIn) {
  extern __shared__ unsigned char smraw[];
  Real* sw = (Real*)smraw;          // [cout][kOT][7]
  Real* sg = sw + cout * kOT * 7;   // [cout][L/2]
  const int c0 = blockIdx.x * kOT, nc = min(kOT, cin - c0);
  const int Lo = L / 2;
  for (int i = threadIdx.x; i < cout * nc * 7; i += blockDim.x) {
    const int o = i / (nc * 7), r = i % (nc * 7);
    sw[o * kOT * 7 + r] = W[((long long)o * cin + c0) * 7 + r];
  }
  const int b0 = blockIdx.y * spg, b1 = min(B, b0 + spg);
  for (int b = b0; b < b1; ++b) {
    __syncthreads();
    for (int i = threadIdx.x; i < cout * Lo; i += blockDim.x) sg[i] = dZ[((long long)b * ztot + zoff) * Lo + i];
    __syncthreads();
    for (int idx = threadIdx.x; idx < nc * L; idx += blockDim.x) {
      const int c = idx / L, q = idx % L;
      Real s = 0;
#pragma unroll
      for (int k = 0; k < 7; ++k) {
        int t = q + pad - dil * k;
        t = t < 0 ? t + L : (t >= L ? t - L : t);
        if (t & 1) continue;
        const int p = t >> 1;
        for (int o = 0; o < cout; ++o) s += sw[(o * kOT + c) * 7 + k] * sg[o * Lo + p];
      }
      const long long oi = ((long long)b * cin + c0 + c) * L + q;
      dIn[oi] = accumulate ? dIn[oi] + s : s;
    }
  }
}

// ---- weight gradients: a tile of coefficients per CTA over a chunk of samples
constexpr int kCPT = 4;  // coefficients per thread

// conv: dW[o][c][k] += sum_b sum_p dZ[b][zoff+o][p] x[b][c][(2p + dil k - pad) mod L]
template <typename Real>
__global__ void __launch_bounds__(kThreads) conv_wgrad_kernel(int B, int spc, int cin, int L, int cout, int dil, int pad,
                                                              const Real* __restrict__ x, int ztot, int zoff,
                                                              const Real* __restrict__ dZ, Real* __restrict__ dW) {
  extern __shared__ unsigned char smraw[];
  Real* sx = (Real*)smraw;  // [cin][L]
  Real* sg = sx + cin * L;  // [cout][L/2]
  const int Lo = L / 2;
  const int ncoef = cout * cin * 7;
  const int base = blockIdx.x * kThreads * kCPT;
  Real acc[kCPT];
  int oo[kCPT], cc[kCPT], kk[kCPT];
#pragma unroll
  for (int r = 0; r < kCPT; ++r) {
    acc[r] = 0;
    const int e = base + r * kThreads + threadIdx.x;
    const int ee = e < ncoef ? e : 0;
    oo[r] = ee / (cin * 7);
    cc[r] = (ee / 7) % cin;
    kk[r] = ee % 7;
  }
  const int b0 = blockIdx.y * spc, b1 = min(B, b0 + spc);
  for (int b = b0; b < b1; ++b) {
    __syncthreads();
    for (int i = threadIdx.x; i < cin * L; i += blockDim.x) sx[i] = x[(long long)b * cin * L + i];
    for (int i = threadIdx.x; i < cout * Lo; i += blockDim.x) sg[i] = dZ[((long long)b * ztot + zoff) * Lo + i];
    __syncthreads();
#pragma unroll
    for (int r = 0; r < kCPT; ++r) {
      if (base + r * kThreads + threadIdx.x >= ncoef) continue;
      const Real* g = sg + oo[r] * Lo;
      const Real* xc = sx + cc[r] * L;
      int q = dil * kk[r] - pad;
      q = q < 0 ? q + L : q;
      Real s = 0;
      for (int p = 0; p < Lo; ++p) {
        s += g[p] * xc[q];
        q += 2;
        if (q >= L) q -= L;
      }
      acc[r] += s;
    }
  }
#pragma unroll
  for (int r = 0; r < kCPT; ++r) {
    const int e = base + r * kThreads + threadIdx.x;
    if (e < ncoef) atomicAdd(&dW[e], acc[r]);
  }
}

// transposed conv: dW[c][o][k] += sum_b sum_i x[b][c][i] dZ[b][o][2i + k - 4].
// A CTA takes a 16 x 16 tile of (c, o) pairs, one pair per thread with its 10
// coefficients in registers; dZ[o][2i - 4 .. 2i + 5] slides through
// registers two entries per i (zero halo of 4 in shared memory).
constexpr int kWT = 16;

template <typename Real>
__global__ void __launch_bounds__(kWT * kWT) deconv_wgrad_kernel(int B, int spc, int d, int Lin,
                                                                 const Real* __restrict__ x,
                                                                 const Real* __restrict__ dZ, Real* __restrict__ dW) {
  extern __shared__ unsigned char smraw[];
  const int Lo = 2 * Lin, Lg = Lo + 10;
  Real* sx = (Real*)smraw;          // [kWT][Lin]
  Real* sg = sx + kWT * Lin;        // [kWT][Lo + 10], dZ j at j + 4
  const int tiles = (d + kWT - 1) / kWT;
  const int c0 = (blockIdx.x / tiles) * kWT, o0 = (blockIdx.x % tiles) * kWT;
  const int cl = threadIdx.x / kWT, ol = threadIdx.x % kWT;
  const bool live = c0 + cl < d && o0 + ol < d;
  Real acc[10];
#pragma unroll
  for (int k = 0; k < 10; ++k) acc[k] = 0;
  const int b0 = blockIdx.y * spc, b1 = min(B, b0 + spc);
  for (int b = b0; b < b1; ++b) {
    __syncthreads();
    for (int i = threadIdx.x; i < kWT * Lin; i += blockDim.x) {
      const int c = c0 + i / Lin;
      sx[i] = c < d ? x[((long long)b * d + c) * Lin + i % Lin] : Real(0);
    }
    for (int i = threadIdx.x; i < kWT * Lg; i += blockDim.x) {
      const int o = o0 + i / Lg, j = i % Lg - 4;
      sg[i] = (o < d && j >= 0 && j < Lo) ? dZ[((long long)b * d + o) * Lo + j] : Real(0);
    }
    __syncthreads();
    if (live) {
      const Real* xc = sx + cl * Lin;
      const Real* g = sg + ol * Lg;  // g[t] = dZ[o][t - 4]
      Real win[10];
#pragma unroll
      for (int k = 0; k < 10; ++k) win[k] = g[k];
      for (int i = 0; i < Lin; ++i) {
        const Real xv = xc[i];
#pragma unroll
        for (int k = 0; k < 10; ++k) acc[k] += xv * win[k];
        // advance the window by two: win[k] = g[2 (i + 1) + k]
#pragma unroll
        for (int k = 0; k < 8; ++k) win[k] = win[k + 2];
        win[8] = g[2 * i + 10];
        win[9] = g[2 * i + 11];
      }
    }
  }
  if (live)
#pragma unroll
    for (int k = 0; k < 10; ++k) atomicAdd(&dW[((long long)(c0 + cl) * d + o0 + ol) * 10 + k], acc[k]);
}

// mix: dW[o][c][k] += sum_b sum_p dOut[b][o][p] D[b][c][p + k - 1]
template <typename Real>
__global__ void __launch_bounds__(kThreads) mix_wgrad_kernel(int B, int spc, int d, int L, int cmix, int cout,
                                                             const Real* __restrict__ D, const Real* __restrict__ dout,
                                                             Real* __restrict__ dW) {
  extern __shared__ unsigned char smraw[];
  Real* sx = (Real*)smraw;  // [d][L]
  Real* sg = sx + d * L;    // [cmix][L]
  const int ncoef = cmix * d * 3;
  const int base = blockIdx.x * kThreads * kCPT;
  Real acc[kCPT];
  int oo[kCPT], cc[kCPT], kk[kCPT];
#pragma unroll
  for (int r = 0; r < kCPT; ++r) {
    acc[r] = 0;
    const int e = base + r * kThreads + threadIdx.x;
    const int ee = e < ncoef ? e : 0;
    oo[r] = ee / (d * 3);
    cc[r] = (ee / 3) % d;
    kk[r] = ee % 3;
  }
  const int b0 = blockIdx.y * spc, b1 = min(B, b0 + spc);
  for (int b = b0; b < b1; ++b) {
    __syncthreads();
    for (int i = threadIdx.x; i < d * L; i += blockDim.x) sx[i] = D[(long long)b * d * L + i];
    for (int i = threadIdx.x; i < cmix * L; i += blockDim.x) sg[i] = dout[(long long)b * cout * L + i];
    __syncthreads();
#pragma unroll
    for (int r = 0; r < kCPT; ++r) {
      if (base + r * kThreads + threadIdx.x >= ncoef) continue;
      const Real* g = sg + oo[r] * L;
      const Real* xc = sx + cc[r] * L;
      const int sh = kk[r] - 1;
      const int p0 = sh < 0 ? 1 : 0, p1 = sh > 0 ? L - 1 : L;
      Real s = 0;
      for (int p = p0; p < p1; ++p) s += g[p] * xc[p + sh];
      acc[r] += s;
    }
  }
#pragma unroll
  for (int r = 0; r < kCPT; ++r) {
    const int e = base + r * kThreads + threadIdx.x;
    if (e < ncoef) atomicAdd(&dW[e], acc[r]);
  }
}

// residual and pass-through channels of the block input: dX0[:cmix] += dOut[:cmix]
// (residual), dX0[cin - npass:] += dOut[cmix:]
template <typename Real>
__global__ void block_input_grad_kernel(long long n, int cin, int cout, int cmix, int npass, int residual, int L,
                                        const Real* __restrict__ dout, Real* __restrict__ dx0) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;  // n = B * cin * L
  const int p = (int)(i % L);
  const int c = (int)((i / L) % cin);
  const long long b = i / ((long long)cin * L);
  Real g = dx0[i];
  if (residual && c < cmix) g += dout[(b * cout + c) * L + p];
  if (c >= cin - npass) g += dout[(b * cout + cmix + c - (cin - npass)) * L + p];
  dx0[i] = g;
}

// weighted mean squared error: loss += sum w_b w_c (y - t)^2 / count;
// dy = 2 w_b w_c (y - t) / count (sample weights w_b, channel weights w_c)
template <typename Real>
__global__ void mse_kernel(long long n, int C, int L, double inv_count, const Real* __restrict__ y,
                           const Real* __restrict__ t, const Real* __restrict__ wch, const Real* __restrict__ wsm,
                           Real* __restrict__ dy, double* __restrict__ loss) {
  __shared__ double red[kThreads];
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  double l = 0.0;
  if (i < n) {
    const int c = (int)((i / L) % C);
    const long long b = i / ((long long)C * L);
    const Real w = (wch ? wch[c] : Real(1)) * (wsm ? wsm[b] : Real(1));
    const Real e = y[i] - t[i];
    l = (double)(w * e * e) * inv_count;
    dy[i] = Real(2.0 * inv_count) * w * e;
  }
  red[threadIdx.x] = l;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0) atomicAdd(loss, red[0]);
}

template <typename Real>
__global__ void adam_kernel(long long n, Real* __restrict__ p, const Real* __restrict__ g, Real* __restrict__ m,
                            Real* __restrict__ v, const unsigned char* __restrict__ trainable, double lr, double b1,
                            double b2, double eps, double c1, double c2) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n || !trainable[i]) return;
  const double gi = (double)g[i];
  const double mi = b1 * (double)m[i] + (1.0 - b1) * gi;
  const double vi = b2 * (double)v[i] + (1.0 - b2) * gi * gi;
  m[i] = (Real)mi;
  v[i] = (Real)vi;
  p[i] = (Real)((double)p[i] - lr * (mi / c1) / (sqrt(vi / c2) + eps));
}

template <typename Real>
__global__ void convert_kernel(long long n, const float* __restrict__ a, Real* __restrict__ b) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) b[i] = (Real)a[i];
}

template <typename Real>
__global__ void convert_back_kernel(long long n, const Real* __restrict__ a, float* __restrict__ b) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) b[i] = (float)a[i];
}

}  // namespace

// ---------------------------------------------------------------------------
// host side

namespace {

constexpr int kSegs = 30;  // parameter arrays per block, in the reference's order (see mlarm.py)
enum Seg {
  S_C11W, S_C11B, S_C12W, S_C12B, S_C21W, S_C21B, S_C22W, S_C22B, S_D1W, S_D1B, S_D2W, S_D2B, S_MXW, S_MXB,
  S_BN1W, S_BN1B, S_BN1M, S_BN1V, S_BN2W, S_BN2B, S_BN2M, S_BN2V, S_BN3W, S_BN3B, S_BN3M, S_BN3V,
  S_BN4W, S_BN4B, S_BN4M, S_BN4V
};

struct TBlock {
  ves_net_block b;
  size_t seg[kSegs];     // offsets into the parameter buffer (elements)
  size_t seglen[kSegs];
  // activations (elements, per sample): R1, A, R2, Bt, R3, C, R4, D and the output
  size_t act[9];
};

}  // namespace

struct ves_trainer {
  int precision;  // VES_NET_FP32 or VES_NET_FP64
  int L, nblocks, max_batch;
  std::vector<TBlock> blk;
  size_t nparam;
  size_t esize;
  void* d_param;
  void* d_grad;
  void* d_m;
  void* d_v;
  unsigned char* d_train;   // 1 for trainable entries (convolutions, batch-norm affine maps)
  void* d_act;              // per block: input copy, R1, A, R2, Bt, R3, C, R4, D; plus the final output
  std::vector<size_t> act_off;  // element offsets per block of [x0, R1, A, R2, Bt, R3, C, R4, D], then output
  size_t act_total;
  void* d_gbuf;             // gradient scratch: two block-output buffers + dD, dC, dBt, dA
  size_t g_io, g_d;
  double* d_loss;
  double* h_loss;
  int cin0, cout_last;
};

namespace {

size_t seg_sizes(const ves_net_block& b, size_t* len) {
  const int d = 2 * b.c2;
  const size_t L[kSegs] = {
      (size_t)b.c1 * b.cin * 7, (size_t)b.c1, (size_t)b.c1 * b.cin * 7, (size_t)b.c1,
      (size_t)b.c2 * 2 * b.c1 * 7, (size_t)b.c2, (size_t)b.c2 * 2 * b.c1 * 7, (size_t)b.c2,
      (size_t)d * d * 10, (size_t)d, (size_t)d * d * 10, (size_t)d, (size_t)b.cmix * d * 3, (size_t)b.cmix,
      (size_t)2 * b.c1, (size_t)2 * b.c1, (size_t)2 * b.c1, (size_t)2 * b.c1,
      (size_t)d, (size_t)d, (size_t)d, (size_t)d, (size_t)d, (size_t)d, (size_t)d, (size_t)d,
      (size_t)d, (size_t)d, (size_t)d, (size_t)d};
  size_t t = 0;
  for (int i = 0; i < kSegs; ++i) {
    len[i] = L[i];
    t += L[i];
  }
  return t;
}

int grid_groups(int B, int ctas_x, int* per) {
  // about two waves of CTAs over 152 SMs
  const int want = std::max(1, 304 / std::max(ctas_x, 1));
  const int groups = std::min(B, want);
  *per = (B + groups - 1) / groups;
  return (B + *per - 1) / *per;
}

template <typename Real>
int set_smem(const void* fn, size_t bytes) {
  if (bytes > 48 * 1024)
    return ves_cuda_status(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes),
                           "trainer smem");
  return VES_OK;
}

template <typename Real>
struct Tr {
  ves_trainer* t;
  cudaStream_t s;
  Real* P() const { return (Real*)t->d_param; }
  Real* Gr() const { return (Real*)t->d_grad; }
  Real* A(int i, int which) const { return (Real*)t->d_act + t->act_off[(size_t)i * 9 + which]; }
  Real* out() const { return (Real*)t->d_act + t->act_off[(size_t)t->nblocks * 9]; }
  const Real* p(int i, int sg) const { return P() + t->blk[i].seg[sg]; }
  Real* g(int i, int sg) const { return Gr() + t->blk[i].seg[sg]; }
  // the input of block i is the output of block i-1 (block 0: its own copy)
  Real* in(int i) const { return i == 0 ? A(0, 0) : (i < t->nblocks ? A(i, 0) : out()); }

  int conv_fwd(int B, int cin, int L, int cout, int dil, int pad, const Real* W, const Real* bias, const Real* x,
               int ctot, int coff, Real* out) {
    const int tx = (cout + kOT - 1) / kOT;
    int spg;
    const int ty = grid_groups(B, tx, &spg);
    const size_t sh = ((size_t)kOT * cin * 7 + (size_t)cin * L) * sizeof(Real);
    int rc = set_smem<Real>((const void*)conv_fwd_kernel<Real>, sh);
    if (rc) return rc;
    ves_count_launch();
    conv_fwd_kernel<Real><<<dim3(tx, ty), kThreads, sh, s>>>(B, spg, cin, L, cout, dil, pad, W, bias, x, ctot, coff,
                                                             out);
    return VES_OK;
  }
  void bn_fwd(int B, int C, int len, const Real* R, int i, int sw, Real* out) {
    const long long n = (long long)B * C * len;
    ves_count_launch();
    bn_fwd_kernel<Real><<<ceil_div(n, 256), 256, 0, s>>>(n, C, len, R, p(i, sw), p(i, sw + 1), p(i, sw + 2),
                                                         p(i, sw + 3), out);
  }
  int forward(int B) {
    for (int i = 0; i < t->nblocks; ++i) {
      const ves_net_block& b = t->blk[i].b;
      const int L = t->L, d = 2 * b.c2;
      const Real* x = in(i);
      int rc;
      if ((rc = conv_fwd(B, b.cin, L, b.c1, 1, 3, p(i, S_C11W), p(i, S_C11B), x, 2 * b.c1, 0, A(i, 1)))) return rc;
      if ((rc = conv_fwd(B, b.cin, L, b.c1, 2, 6, p(i, S_C12W), p(i, S_C12B), x, 2 * b.c1, b.c1, A(i, 1)))) return rc;
      bn_fwd(B, 2 * b.c1, L / 2, A(i, 1), i, S_BN1W, A(i, 2));
      if ((rc = conv_fwd(B, 2 * b.c1, L / 2, b.c2, 1, 3, p(i, S_C21W), p(i, S_C21B), A(i, 2), d, 0, A(i, 3)))) return rc;
      if ((rc = conv_fwd(B, 2 * b.c1, L / 2, b.c2, 2, 6, p(i, S_C22W), p(i, S_C22B), A(i, 2), d, b.c2, A(i, 3))))
        return rc;
      bn_fwd(B, d, L / 4, A(i, 3), i, S_BN2W, A(i, 4));
      {
        const int tx = (d + kOT - 1) / kOT;
        int spg;
        const int ty = grid_groups(B, tx, &spg);
        size_t sh = ((size_t)d * kOT * 10 + (size_t)d * (L / 4 + 4)) * sizeof(Real);
        if ((rc = set_smem<Real>((const void*)deconv_fwd_kernel<Real>,
                                 ((size_t)d * kOT * 10 + (size_t)d * (L / 2 + 4)) * sizeof(Real))))
          return rc;
        ves_count_launch(2);
        deconv_fwd_kernel<Real><<<dim3(tx, ty), kThreads, sh, s>>>(B, spg, d, L / 4, p(i, S_D1W), p(i, S_D1B), A(i, 4),
                                                                   A(i, 5));
        bn_fwd(B, d, L / 2, A(i, 5), i, S_BN3W, A(i, 6));
        sh = ((size_t)d * kOT * 10 + (size_t)d * (L / 2 + 4)) * sizeof(Real);
        deconv_fwd_kernel<Real><<<dim3(tx, ty), kThreads, sh, s>>>(B, spg, d, L / 2, p(i, S_D2W), p(i, S_D2B), A(i, 6),
                                                                   A(i, 7));
        bn_fwd(B, d, L, A(i, 7), i, S_BN4W, A(i, 8));
      }
      {
        const int tx = (b.cmix + kOT - 1) / kOT;
        int spg;
        const int ty = grid_groups(B, tx, &spg);
        const size_t sh = ((size_t)kOT * d * 3 + (size_t)d * L) * sizeof(Real);
        if ((rc = set_smem<Real>((const void*)mix_fwd_kernel<Real>, sh))) return rc;
        ves_count_launch();
        mix_fwd_kernel<Real><<<dim3(tx, ty), kThreads, sh, s>>>(B, spg, d, L, b.cmix, b.cin, b.npass, b.residual,
                                                                p(i, S_MXW), p(i, S_MXB), A(i, 8), x, in(i + 1));
      }
    }
    return ves_launch_check("trainer forward");
  }

  int bn_bwd(int B, int C, int len, Real* dY, const Real* R, int i, int sw) {
    int spg;
    const int ty = grid_groups(B, C, &spg);
    ves_count_launch();
    bn_bwd_kernel<Real><<<dim3(C, ty), kThreads, 0, s>>>(B, spg, C, len, dY, R, p(i, sw), p(i, sw + 2), p(i, sw + 3),
                                                         dY, g(i, sw), g(i, sw + 1));
    return VES_OK;
  }
  void bias_grad(int B, int ctot, int coff, int cout, int len, const Real* dZ, Real* db) {
    int spg;
    const int ty = grid_groups(B, cout, &spg);
    ves_count_launch();
    bias_grad_kernel<Real><<<dim3(cout, ty), kThreads, 0, s>>>(B, spg, ctot, coff, len, dZ, db);
  }
  int conv_bwd(int B, int cin, int L, int cout, int dil, int pad, int i, int sw, const Real* x, int ztot, int zoff,
               const Real* dZ, int accumulate, Real* dIn) {
    int rc;
    if (dIn) {
      const int tx = (cin + kOT - 1) / kOT;
      int spg;
      const int ty = grid_groups(B, tx, &spg);
      const size_t sh = ((size_t)cout * kOT * 7 + (size_t)cout * (L / 2)) * sizeof(Real);
      if ((rc = set_smem<Real>((const void*)conv_bwd_data_kernel<Real>, sh))) return rc;
      ves_count_launch();
      conv_bwd_data_kernel<Real><<<dim3(tx, ty), kThreads, sh, s>>>(B, spg, cin, L, cout, dil, pad, p(i, sw), ztot,
                                                                    zoff, dZ, accumulate, dIn);
    }
    const int ncoef = cout * cin * 7;
    const int tx = (ncoef + kThreads * kCPT - 1) / (kThreads * kCPT);
    int spc;
    const int ty = grid_groups(B, tx, &spc);
    const size_t sh = ((size_t)cin * L + (size_t)cout * (L / 2)) * sizeof(Real);
    if ((rc = set_smem<Real>((const void*)conv_wgrad_kernel<Real>, sh))) return rc;
    ves_count_launch();
    conv_wgrad_kernel<Real><<<dim3(tx, ty), kThreads, sh, s>>>(B, spc, cin, L, cout, dil, pad, x, ztot, zoff, dZ,
                                                               g(i, sw));
    bias_grad(B, ztot, zoff, cout, L / 2, dZ, g(i, sw + 1));
    return VES_OK;
  }
  int deconv_bwd(int B, int d, int Lin, int i, int sw, const Real* x, const Real* dZ, Real* dIn) {
    int rc;
    {
      const int tx = (d + kOT - 1) / kOT;
      int spg;
      const int ty = grid_groups(B, tx, &spg);
      const size_t sh = ((size_t)kOT * d * 10 + (size_t)2 * d * (Lin + 4)) * sizeof(Real);
      if ((rc = set_smem<Real>((const void*)deconv_bwd_data_kernel<Real>, sh))) return rc;
      ves_count_launch();
      deconv_bwd_data_kernel<Real><<<dim3(tx, ty), kThreads, sh, s>>>(B, spg, d, Lin, p(i, sw), dZ, dIn);
    }
    const int tiles = (d + kWT - 1) / kWT;
    const int tx = tiles * tiles;
    int spc;
    const int ty = grid_groups(B, tx, &spc);
    const size_t sh = ((size_t)kWT * Lin + (size_t)kWT * (2 * Lin + 10)) * sizeof(Real);
    if ((rc = set_smem<Real>((const void*)deconv_wgrad_kernel<Real>, sh))) return rc;
    ves_count_launch();
    deconv_wgrad_kernel<Real><<<dim3(tx, ty), kWT * kWT, sh, s>>>(B, spc, d, Lin, x, dZ, g(i, sw));
    bias_grad(B, d, 0, d, 2 * Lin, dZ, g(i, sw + 1));
    return VES_OK;
  }

  // dout: gradient w.r.t. the output of block i (B x cout x L); dx0: gradient
  // w.r.t. its input (written)
  int block_backward(int B, int i, const Real* dout, Real* dx0) {
    const ves_net_block& b = t->blk[i].b;
    const int L = t->L, d = 2 * b.c2, cout = b.cmix + b.npass;
    Real* gb = (Real*)t->d_gbuf;
    Real* dD = gb + 2 * t->g_io;            // [B][d][L]
    Real* dC = dD + t->g_d;                 // [B][d][L/2]
    Real* dBt = dC + t->g_d;                // [B][d][L/4]
    Real* dA = dBt + t->g_d;                // [B][2c1][L/2]
    const Real* x = in(i);
    int rc;
    // mix
    {
      const int tx = (d + kOT - 1) / kOT;
      int spg;
      const int ty = grid_groups(B, tx, &spg);
      const size_t sh = ((size_t)b.cmix * kOT * 3 + (size_t)b.cmix * L) * sizeof(Real);
      if ((rc = set_smem<Real>((const void*)mix_bwd_data_kernel<Real>, sh))) return rc;
      ves_count_launch();
      mix_bwd_data_kernel<Real><<<dim3(tx, ty), kThreads, sh, s>>>(B, spg, d, L, b.cmix, cout, p(i, S_MXW), dout, dD);
      const int ncoef = b.cmix * d * 3;
      const int tw = (ncoef + kThreads * kCPT - 1) / (kThreads * kCPT);
      int spc;
      const int tyw = grid_groups(B, tw, &spc);
      const size_t shw = ((size_t)d * L + (size_t)b.cmix * L) * sizeof(Real);
      if ((rc = set_smem<Real>((const void*)mix_wgrad_kernel<Real>, shw))) return rc;
      ves_count_launch();
      mix_wgrad_kernel<Real><<<dim3(tw, tyw), kThreads, shw, s>>>(B, spc, d, L, b.cmix, cout, A(i, 8), dout,
                                                                  g(i, S_MXW));
      bias_grad(B, cout, 0, b.cmix, L, dout, g(i, S_MXB));
    }
    // bn4 + relu, deconv2
    bn_bwd(B, d, L, dD, A(i, 7), i, S_BN4W);
    if ((rc = deconv_bwd(B, d, L / 2, i, S_D2W, A(i, 6), dD, dC))) return rc;
    // bn3 + relu, deconv1
    bn_bwd(B, d, L / 2, dC, A(i, 5), i, S_BN3W);
    if ((rc = deconv_bwd(B, d, L / 4, i, S_D1W, A(i, 4), dC, dBt))) return rc;
    // bn2 + relu, the second conv pair
    bn_bwd(B, d, L / 4, dBt, A(i, 3), i, S_BN2W);
    if ((rc = conv_bwd(B, 2 * b.c1, L / 2, b.c2, 1, 3, i, S_C21W, A(i, 2), d, 0, dBt, 0, dA))) return rc;
    if ((rc = conv_bwd(B, 2 * b.c1, L / 2, b.c2, 2, 6, i, S_C22W, A(i, 2), d, b.c2, dBt, 1, dA))) return rc;
    // bn1 + relu, the first conv pair (the first block's input needs no gradient)
    bn_bwd(B, 2 * b.c1, L / 2, dA, A(i, 1), i, S_BN1W);
    Real* dxin = (i > 0) ? dx0 : nullptr;
    if ((rc = conv_bwd(B, b.cin, L, b.c1, 1, 3, i, S_C11W, x, 2 * b.c1, 0, dA, 0, dxin))) return rc;
    if ((rc = conv_bwd(B, b.cin, L, b.c1, 2, 6, i, S_C12W, x, 2 * b.c1, b.c1, dA, 1, dxin))) return rc;
    if (dxin) {
      const long long n = (long long)B * b.cin * L;
      ves_count_launch();
      block_input_grad_kernel<Real><<<ceil_div(n, 256), 256, 0, s>>>(n, b.cin, cout, b.cmix, b.npass, b.residual, L,
                                                                     dout, dxin);
    }
    return VES_OK;
  }

  int backward_mse(int B, const Real* target, const Real* wch, const Real* wsm) {
    const int C = t->cout_last, L = t->L;
    const long long n = (long long)B * C * L;
    Real* gb = (Real*)t->d_gbuf;
    Real* g0 = gb;
    Real* g1 = gb + t->g_io;
    int rc = ves_cuda_status(cudaMemsetAsync(t->d_grad, 0, t->nparam * sizeof(Real), s), "zero grads");
    if (!rc) rc = ves_cuda_status(cudaMemsetAsync(t->d_loss, 0, sizeof(double), s), "zero loss");
    if (rc) return rc;
    ves_count_launch();
    mse_kernel<Real><<<ceil_div(n, kThreads), kThreads, 0, s>>>(n, C, L, 1.0 / (double)n, out(), target, wch, wsm,
                                                                g0, t->d_loss);
    for (int i = t->nblocks - 1; i >= 0; --i) {
      if ((rc = block_backward(B, i, g0, g1))) return rc;
      std::swap(g0, g1);
    }
    return ves_launch_check("trainer backward");
  }
};

}  // namespace

extern "C" int ves_trainer_create(int precision, int L, int nblocks, const ves_net_block* blocks,
                                  const float* const* params, int max_batch, ves_trainer** out) {
  if (!out || !blocks || !params || nblocks <= 0 || max_batch <= 0 || L <= 0 || L % 4 != 0 ||
      (precision != VES_NET_FP32 && precision != VES_NET_FP64)) {
    ves_record_error(VES_ERR_ARG, "trainer_create: bad arguments");
    return VES_ERR_ARG;
  }
  *out = nullptr;
  for (int i = 0; i < nblocks; ++i) {
    const ves_net_block& b = blocks[i];
    if (b.cin <= 0 || b.c1 <= 0 || b.c2 <= 0 || b.cmix <= 0 || b.npass < 0 || b.npass > b.cin ||
        (b.residual && b.cmix > b.cin) || (i > 0 && b.cin != blocks[i - 1].cmix + blocks[i - 1].npass)) {
      ves_record_error(VES_ERR_SHAPE, "trainer_create: block %d has inconsistent channel counts", i);
      return VES_ERR_SHAPE;
    }
  }
  ves_trainer* t = new (std::nothrow) ves_trainer();
  if (!t) {
    ves_record_error(VES_ERR_CUDA, "trainer_create: out of host memory");
    return VES_ERR_CUDA;
  }
  t->precision = precision;
  t->L = L;
  t->nblocks = nblocks;
  t->max_batch = max_batch;
  t->esize = precision == VES_NET_FP64 ? 8 : 4;
  t->cin0 = blocks[0].cin;
  t->cout_last = blocks[nblocks - 1].cmix + blocks[nblocks - 1].npass;
  size_t off = 0, act = 0, gio = 0, gd = 0;
  std::vector<unsigned char> train;
  for (int i = 0; i < nblocks; ++i) {
    TBlock tb;
    tb.b = blocks[i];
    size_t len[kSegs];
    seg_sizes(blocks[i], len);
    for (int sg = 0; sg < kSegs; ++sg) {
      tb.seg[sg] = off;
      tb.seglen[sg] = len[sg];
      off += len[sg];
      const bool stat = (sg >= S_BN1W) && ((sg - S_BN1W) % 4 >= 2);
      train.insert(train.end(), len[sg], stat ? 0 : 1);
    }
    const ves_net_block& b = blocks[i];
    const int d = 2 * b.c2;
    const size_t per[9] = {(size_t)b.cin * L, (size_t)2 * b.c1 * (L / 2), (size_t)2 * b.c1 * (L / 2),
                           (size_t)d * (L / 4), (size_t)d * (L / 4), (size_t)d * (L / 2), (size_t)d * (L / 2),
                           (size_t)d * L, (size_t)d * L};
    for (int w = 0; w < 9; ++w) {
      t->act_off.push_back(act);
      act += per[w] * (size_t)max_batch;
    }
    gio = std::max(gio, std::max((size_t)b.cin, (size_t)(b.cmix + b.npass)) * L);
    gd = std::max(gd, std::max((size_t)d * L, (size_t)2 * b.c1 * (L / 2)));
    t->blk.push_back(tb);
  }
  t->act_off.push_back(act);
  act += (size_t)t->cout_last * L * max_batch;
  t->act_total = act;
  t->nparam = off;
  t->g_io = gio * (size_t)max_batch;
  t->g_d = gd * (size_t)max_batch;
  const size_t es = t->esize;
  int rc = ves_cuda_status(cudaMalloc(&t->d_param, off * es), "trainer params");
  if (!rc) rc = ves_cuda_status(cudaMalloc(&t->d_grad, off * es), "trainer grads");
  if (!rc) rc = ves_cuda_status(cudaMalloc(&t->d_m, off * es), "trainer adam m");
  if (!rc) rc = ves_cuda_status(cudaMalloc(&t->d_v, off * es), "trainer adam v");
  if (!rc) rc = ves_cuda_status(cudaMalloc(&t->d_train, off), "trainer mask");
  if (!rc) rc = ves_cuda_status(cudaMalloc(&t->d_act, act * es), "trainer activations");
  if (!rc) rc = ves_cuda_status(cudaMalloc(&t->d_gbuf, (2 * t->g_io + 4 * t->g_d) * es), "trainer gradients");
  if (!rc) rc = ves_cuda_status(cudaMalloc(&t->d_loss, sizeof(double)), "trainer loss");
  if (!rc) rc = ves_cuda_status(cudaMallocHost(&t->h_loss, sizeof(double)), "trainer loss host");
  if (!rc) rc = ves_cuda_status(cudaMemset(t->d_m, 0, off * es), "trainer zero m");
  if (!rc) rc = ves_cuda_status(cudaMemset(t->d_v, 0, off * es), "trainer zero v");
  if (!rc) rc = ves_cuda_status(cudaMemcpy(t->d_train, train.data(), off, cudaMemcpyHostToDevice), "trainer mask");
  if (!rc) {
    // parameters: float32 host arrays, 30 per block in the reference's order
    float* tmp = nullptr;
    size_t maxlen = 0;
    for (const TBlock& tb : t->blk)
      for (int sg = 0; sg < kSegs; ++sg) maxlen = std::max(maxlen, tb.seglen[sg]);
    rc = ves_cuda_status(cudaMalloc(&tmp, maxlen * sizeof(float)), "trainer upload");
    for (int i = 0; i < nblocks && !rc; ++i)
      for (int sg = 0; sg < kSegs && !rc; ++sg) {
        const float* src = params[(size_t)i * kSegs + sg];
        const size_t n = t->blk[i].seglen[sg];
        if (!src) {
          ves_record_error(VES_ERR_ARG, "trainer_create: parameter %d of block %d missing", sg, i);
          rc = VES_ERR_ARG;
          break;
        }
        rc = ves_cuda_status(cudaMemcpy(tmp, src, n * sizeof(float), cudaMemcpyHostToDevice), "trainer upload");
        if (rc) break;
        if (precision == VES_NET_FP64)
          convert_kernel<double><<<ceil_div((long long)n, 256), 256>>>(n, tmp, (double*)t->d_param + t->blk[i].seg[sg]);
        else
          convert_kernel<float><<<ceil_div((long long)n, 256), 256>>>(n, tmp, (float*)t->d_param + t->blk[i].seg[sg]);
        rc = ves_cuda_status(cudaDeviceSynchronize(), "trainer upload");
      }
    if (tmp) cudaFree(tmp);
  }
  if (rc) {
    ves_trainer_destroy(t);
    return rc;
  }
  *out = t;
  return VES_OK;
}

extern "C" int ves_trainer_destroy(ves_trainer* t) {
  if (!t) return VES_OK;
  void* bufs[] = {t->d_param, t->d_grad, t->d_m, t->d_v, t->d_train, t->d_act, t->d_gbuf, t->d_loss};
  for (void* b : bufs)
    if (b) cudaFree(b);
  if (t->h_loss) cudaFreeHost(t->h_loss);
  delete t;
  return VES_OK;
}

extern "C" long long ves_trainer_num_params(const ves_trainer* t) { return t ? (long long)t->nparam : -1; }

extern "C" int ves_trainer_forward(ves_trainer* t, int B, const void* x, void* y, void* stream) {
  if (!t || !x || B <= 0 || B > t->max_batch) {
    ves_record_error(VES_ERR_ARG, "trainer_forward: bad arguments (batch %d, max %d)", B, t ? t->max_batch : 0);
    return VES_ERR_ARG;
  }
  cudaStream_t s = (cudaStream_t)stream;
  const size_t es = t->esize;
  int rc = ves_cuda_status(
      cudaMemcpyAsync((char*)t->d_act, x, (size_t)B * t->cin0 * t->L * es, cudaMemcpyDeviceToDevice, s), "input");
  if (rc) return rc;
  if (t->precision == VES_NET_FP64) {
    Tr<double> tr{t, s};
    rc = tr.forward(B);
    if (!rc && y) rc = ves_cuda_status(cudaMemcpyAsync(y, tr.out(), (size_t)B * t->cout_last * t->L * es,
                                                       cudaMemcpyDeviceToDevice, s), "output");
  } else {
    Tr<float> tr{t, s};
    rc = tr.forward(B);
    if (!rc && y) rc = ves_cuda_status(cudaMemcpyAsync(y, tr.out(), (size_t)B * t->cout_last * t->L * es,
                                                       cudaMemcpyDeviceToDevice, s), "output");
  }
  return rc;
}

extern "C" int ves_trainer_backward_mse(ves_trainer* t, int B, const void* target, const void* channel_weights,
                                        const void* sample_weights, double* loss, void* stream) {
  if (!t || !target || B <= 0 || B > t->max_batch) {
    ves_record_error(VES_ERR_ARG, "trainer_backward: bad arguments");
    return VES_ERR_ARG;
  }
  cudaStream_t s = (cudaStream_t)stream;
  int rc = (t->precision == VES_NET_FP64)
               ? Tr<double>{t, s}.backward_mse(B, (const double*)target, (const double*)channel_weights,
                                               (const double*)sample_weights)
               : Tr<float>{t, s}.backward_mse(B, (const float*)target, (const float*)channel_weights,
                                              (const float*)sample_weights);
  if (rc) return rc;
  if (loss) {
    rc = ves_cuda_status(cudaMemcpyAsync(t->h_loss, t->d_loss, sizeof(double), cudaMemcpyDeviceToHost, s), "loss");
    if (!rc) rc = ves_cuda_status(cudaStreamSynchronize(s), "loss sync");
    if (!rc) *loss = *t->h_loss;
  }
  return rc;
}

extern "C" int ves_trainer_adam(ves_trainer* t, double lr, double beta1, double beta2, double eps, int step,
                                void* stream) {
  if (!t || step <= 0) {
    ves_record_error(VES_ERR_ARG, "trainer_adam: bad arguments");
    return VES_ERR_ARG;
  }
  cudaStream_t s = (cudaStream_t)stream;
  const double c1 = 1.0 - pow(beta1, step), c2 = 1.0 - pow(beta2, step);
  const long long n = (long long)t->nparam;
  ves_count_launch();
  if (t->precision == VES_NET_FP64)
    adam_kernel<double><<<ceil_div(n, 256), 256, 0, s>>>(n, (double*)t->d_param, (const double*)t->d_grad,
                                                         (double*)t->d_m, (double*)t->d_v, t->d_train, lr, beta1,
                                                         beta2, eps, c1, c2);
  else
    adam_kernel<float><<<ceil_div(n, 256), 256, 0, s>>>(n, (float*)t->d_param, (const float*)t->d_grad,
                                                        (float*)t->d_m, (float*)t->d_v, t->d_train, lr, beta1, beta2,
                                                        eps, c1, c2);
  return ves_launch_check("trainer adam");
}

static int trainer_copy_out(const ves_trainer* t, const void* src, float* const* arrays, void* stream) {
  if (!t || !arrays) {
    ves_record_error(VES_ERR_ARG, "trainer params: bad arguments");
    return VES_ERR_ARG;
  }
  cudaStream_t s = (cudaStream_t)stream;
  float* tmp = nullptr;
  int rc = ves_cuda_status(cudaMalloc(&tmp, t->nparam * sizeof(float)), "trainer params");
  if (rc) return rc;
  const long long n = (long long)t->nparam;
  if (t->precision == VES_NET_FP64)
    convert_back_kernel<double><<<ceil_div(n, 256), 256, 0, s>>>(n, (const double*)src, tmp);
  else
    convert_back_kernel<float><<<ceil_div(n, 256), 256, 0, s>>>(n, (const float*)src, tmp);
  std::vector<float> h(t->nparam);
  rc = ves_cuda_status(cudaMemcpyAsync(h.data(), tmp, t->nparam * sizeof(float), cudaMemcpyDeviceToHost, s),
                       "trainer params");
  if (!rc) rc = ves_cuda_status(cudaStreamSynchronize(s), "trainer params");
  cudaFree(tmp);
  if (rc) return rc;
  for (int i = 0; i < t->nblocks; ++i)
    for (int sg = 0; sg < kSegs; ++sg) {
      float* dst = arrays[(size_t)i * kSegs + sg];
      if (dst) memcpy(dst, h.data() + t->blk[i].seg[sg], t->blk[i].seglen[sg] * sizeof(float));
    }
  return VES_OK;
}

extern "C" int ves_trainer_get_params(const ves_trainer* t, float* const* arrays, void* stream) {
  return trainer_copy_out(t, t ? t->d_param : nullptr, arrays, stream);
}

extern "C" int ves_trainer_get_grads(const ves_trainer* t, float* const* arrays, void* stream) {
  return trainer_copy_out(t, t ? t->d_grad : nullptr, arrays, stream);
}

extern "C" int ves_trainer_get_grads_f64(const ves_trainer* t, double* out, void* stream) {
  if (!t || !out || t->precision != VES_NET_FP64) {
    ves_record_error(VES_ERR_ARG, "trainer_get_grads_f64: FP64 trainer and an output array required");
    return VES_ERR_ARG;
  }
  cudaStream_t s = (cudaStream_t)stream;
  int rc = ves_cuda_status(cudaMemcpyAsync(out, t->d_grad, t->nparam * sizeof(double), cudaMemcpyDeviceToHost, s),
                           "grads");
  if (!rc) rc = ves_cuda_status(cudaStreamSynchronize(s), "grads sync");
  return rc;
}
