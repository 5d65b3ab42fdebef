// Tensor-core (tcgen05, BF16 operands, FP32 accumulation) path of the MLARM
// network engine.  Same block template as ves_nets.cu; every convolution is a
// sum of shifted GEMMs
//     D[o][p] += sum_c W_s[o][c] * X[p + s][c]
// with D (positions x output channels) in tensor memory, X (positions x
// channels, the MMA's A operand) and W_s (output channels x channels, one
// matrix per input shift s, the B operand) K-major in shared memory.  A shift
// is a start-address offset of X's descriptor (ves_tc.cuh), so no im2col copy
// is made:
//   * stride-2 convolutions read the input split by position parity, with
//     circular halos of 3 rows: input position 2p + s is row p + (s >> 1) of
//     parity s & 1; the two branches (dilation 1 and 2) share the shifts
//     -6..6 (except +-5) and fill the output rows [0, c1) and [c1, 2c1);
//   * transposed convolutions (kernel 10, stride 2, padding 4) are split by
//     output parity r: out[2q + r] = sum_{u<5} W[r + 2u] in[q + 2 - u], zero
//     halos of 2 rows;
//   * the mixing convolution (kernel 3) reads shifts -1, 0, 1 of a zero-halo
//     array.
// Positions are the MMA's M = 128 rows (one TMEM lane each, so every thread of
// an epilogue owns one position and writes 16-byte rows of 8 channels);
// layers with fewer positions leave the remaining rows to read whatever
// follows in shared memory, and those rows are never read back.  Output
// channels are N, rounded up to 16.
//
// Two kernels per block: "down" (conv pair 1, conv pair 2) and "up"
// (transposed convs, mix, residual and pass-through).  The block input and
// output stay FP32 in global memory ([nv][groups*channels][L]); the down ->
// up intermediate is BF16 in the K-major layout.  Kernels are persistent:
// each CTA walks a contiguous range of (group, vesicle) items, loading a
// group's weight image into shared memory once per group it meets.
#include <math.h>
#include <string.h>

#include <algorithm>
#include <vector>

#include "ves_internal.h"
#include "ves_tc.cuh"
#include <cuda_bf16.h>

namespace tcnet {

constexpr int kThreads = 256;
constexpr int kOffsets = 11;  // input shifts of a conv pair: -6..6 without +-5
__host__ __device__ constexpr int shift_of(int oi) { return oi < 2 ? -6 + 2 * oi : (oi < 9 ? oi - 5 : 2 * oi - 14); }

__host__ __device__ constexpr int rup(int a, int b) { return (a + b - 1) / b * b; }

// Geometry of one block, shared by host packing and kernels (bytes unless noted).
struct Geo {
  int cin, c1, c2, cmix, residual, npass, L;
  int n1, d;             // conv-pair output channels
  int kcin, kc1, kcd;    // 8-channel K chunks of the three GEMM inputs (even)
  // down image: W1 [11][kcin][n1][16B], W2 [11][kc1][d][16B], consts [6][128] f32
  int dw1, dw2, dcst, dsize;
  // down smem: image, xs [2][kcin][L/2+6][16B], as [2][kc1][L/4+6][16B], stage [kcd][L/4][16B], tail
  int dxs, das, dstage, dsmem;
  // up image: D1 [2][5][kcd][d][16B], D2 same, M [3][kcd][cmix][16B], consts [7][128] f32
  int uw1, uw2, uwm, ucst, usize;
  // up smem: image, bs [kcd][L/4+4][16B], cs [kcd][L/2+4][16B], ds [kcd][L+2][16B], tail
  int ubs, ucs, uds, uxr, usmem;  // uxr: FP32 residual x[0:cmix][L] of the current item
  int mid_bytes;         // down -> up intermediate per (vesicle, group): [kcd][L/4][16B]
};

inline Geo make_geo(const ves_net_block& b, int L) {
  Geo g;
  g.cin = b.cin;
  g.c1 = b.c1;
  g.c2 = b.c2;
  g.cmix = b.cmix;
  g.residual = b.residual;
  g.npass = b.npass;
  g.L = L;
  g.n1 = 2 * b.c1;
  g.d = 2 * b.c2;
  g.kcin = rup(b.cin, 16) / 8;
  g.kc1 = rup(g.n1, 16) / 8;
  g.kcd = rup(g.d, 16) / 8;
  int o = 0;
  g.dw1 = o;
  o += kOffsets * g.kcin * g.n1 * 16;
  g.dw2 = o;
  o += kOffsets * g.kc1 * g.d * 16;
  g.dcst = o;
  o += 6 * 128 * 4;
  g.dsize = o;
  g.dxs = o;
  o += 2 * g.kcin * (L / 2 + 6) * 16;
  g.das = o;
  o += 2 * g.kc1 * (L / 4 + 6) * 16;
  g.dstage = o;
  o += g.kcd * (L / 4) * 16;
  g.dsmem = o + 128 * 16;
  o = 0;
  g.uw1 = o;
  o += 10 * g.kcd * g.d * 16;
  g.uw2 = o;
  o += 10 * g.kcd * g.d * 16;
  g.uwm = o;
  o += 3 * g.kcd * g.cmix * 16;
  g.ucst = o;
  o += 7 * 128 * 4;
  g.usize = o;
  g.ubs = o;
  o += g.kcd * (L / 4 + 4) * 16;
  g.ucs = o;
  o += g.kcd * (L / 2 + 4) * 16;
  g.uds = o;
  o += g.kcd * (L + 2) * 16;
  g.uxr = o + 128 * 16;  // after the tail that A-operand reads may run into
  o = g.uxr + rup(b.cmix * L * 4, 16);
  g.usmem = o;
  g.mid_bytes = g.kcd * (L / 4) * 16;
  return g;
}

struct KArgs {
  Geo g;
  int G, nv;
  long long items;
  const unsigned char* img;  // group 0 image of this block; group stride = image size
  const float* x;            // block input [nv][G*cin][L]
  float* out;                // block output [nv][G*cout][L]
  unsigned char* mid;        // [nv][G][mid_bytes]
  VesDeviceStatus* st;
};

__device__ __forceinline__ uint16_t f2bf(float f) {
  return __bfloat16_as_ushort(__float2bfloat16_rn(f));
}

__device__ __forceinline__ void copy16(unsigned char* dst, const unsigned char* src, int bytes) {
  const uint4* s = reinterpret_cast<const uint4*>(src);
  uint4* d = reinterpret_cast<uint4*>(dst);
  for (int i = threadIdx.x; i < bytes / 16; i += blockDim.x) d[i] = s[i];
}
__device__ __forceinline__ void zero16(unsigned char* dst, int bytes) {
  uint4* d = reinterpret_cast<uint4*>(dst);
  const uint4 z = make_uint4(0, 0, 0, 0);
  for (int i = threadIdx.x; i < bytes / 16; i += blockDim.x) d[i] = z;
}

// all writes to shared memory so far -> visible to the tensor core; CTA barrier
__device__ __forceinline__ void sync_for_mma() {
  tc_fence_async_smem();
  tc_fence_before_sync();
  __syncthreads();
  tc_fence_after_sync();
}

struct Range {
  long long lo, hi;
};
__device__ __forceinline__ Range my_items(long long items) {
  const long long per = items / gridDim.x, rem = items % gridDim.x;
  const long long b = blockIdx.x;
  const long long lo = b * per + (b < rem ? b : rem);
  return {lo, lo + per + (b < rem ? 1 : 0)};
}

// ---------------------------------------------------------------------------
// Epilogue helpers.  D[p][c] sits in TMEM with the position p on lane p and
// the channel c in column c; each thread owns one position and reads 8
// channels at a time, which is one 16-byte row of the next layer's K-major
// operand.

// 8 channels [8kc, 8kc+8) of this thread's position: relu(v + b) * s + t, 0 beyond nreal
__device__ __forceinline__ uint4 act8(const float* v, const float* cst, int kc, int nreal, int ob, int os, int ot) {
  float b[8], sc[8], sh[8];
  *reinterpret_cast<float4*>(b) = *reinterpret_cast<const float4*>(cst + ob + 8 * kc);
  *reinterpret_cast<float4*>(b + 4) = *reinterpret_cast<const float4*>(cst + ob + 8 * kc + 4);
  *reinterpret_cast<float4*>(sc) = *reinterpret_cast<const float4*>(cst + os + 8 * kc);
  *reinterpret_cast<float4*>(sc + 4) = *reinterpret_cast<const float4*>(cst + os + 8 * kc + 4);
  *reinterpret_cast<float4*>(sh) = *reinterpret_cast<const float4*>(cst + ot + 8 * kc);
  *reinterpret_cast<float4*>(sh + 4) = *reinterpret_cast<const float4*>(cst + ot + 8 * kc + 4);
  uint32_t w[4];
#pragma unroll
  for (int e = 0; e < 8; e += 2) {
    const int c0 = 8 * kc + e;
    const float y0 = c0 < nreal ? fmaf(fmaxf(v[e] + b[e], 0.f), sc[e], sh[e]) : 0.f;
    const float y1 = c0 + 1 < nreal ? fmaf(fmaxf(v[e + 1] + b[e + 1], 0.f), sc[e + 1], sh[e + 1]) : 0.f;
    w[e >> 1] = (uint32_t)f2bf(y0) | ((uint32_t)f2bf(y1) << 16);
  }
  return make_uint4(w[0], w[1], w[2], w[3]);
}

// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(kThreads, 1) down_kernel(KArgs a) {
  extern __shared__ __align__(128) unsigned char sm[];
  __shared__ uint64_t bar;
  __shared__ uint32_t tbase;
  const Geo& g = a.g;
  const int L = g.L, L2 = L / 2, L4 = L / 4;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int qd = warp & 3, hf = warp >> 2;  // lane quarter (positions), column half
  const Range rg = my_items(a.items);
  if (rg.lo >= rg.hi) return;
  const uint32_t ncols = 128;
  if (tid == 0) {
    tc_mbar_init(&bar, 1);
    tc_mbar_fence_init();
  }
  if (warp == 0) tc_tmem_alloc(&tbase, ncols);
  zero16(sm + g.dxs, g.dsmem - g.dxs);  // K padding of the activation arrays stays zero
  tc_fence_before_sync();
  __syncthreads();
  tc_fence_after_sync();
  const uint32_t t0 = tbase;
  const int N1 = g.kc1 * 8, N2 = g.kcd * 8;
  const uint32_t d1 = t0, d2 = t0 + N1;
  const uint32_t sbase = tc_smem_u32(sm);
  const float* cst = reinterpret_cast<const float*>(sm + g.dcst);
  unsigned phase = 0;
  bool failed = false;
  int cur_g = -1;
  const int P1 = L2 + 6, P2 = L4 + 6;
  uint4* xs = reinterpret_cast<uint4*>(sm + g.dxs);
  uint4* as = reinterpret_cast<uint4*>(sm + g.das);
  uint4* stage = reinterpret_cast<uint4*>(sm + g.dstage);
  // input x[v][grp*cin + c][pos] -> parity-split BF16 rows with circular halos;
  // one thread per (position, 8-channel chunk)
  auto load_x = [&](long long item) {
    const int grp = (int)(item / a.nv);
    const long long v = item % a.nv;
    const float* __restrict__ xin = a.x + ((long long)v * a.G + grp) * (long long)g.cin * L;
    for (int i = tid; i < g.kcin * L; i += blockDim.x) {
      const int kc = i / L, pos = i - kc * L;
      float y[8];
#pragma unroll
      for (int e = 0; e < 8; ++e) y[e] = (8 * kc + e < g.cin) ? __ldg(xin + (size_t)(8 * kc + e) * L + pos) : 0.f;
      uint32_t w[4];
#pragma unroll
      for (int e = 0; e < 8; e += 2) w[e >> 1] = (uint32_t)f2bf(y[e]) | ((uint32_t)f2bf(y[e + 1]) << 16);
      const uint4 val = make_uint4(w[0], w[1], w[2], w[3]);
      const int par = pos & 1, q = pos >> 1;
      uint4* base = xs + (size_t)(par * g.kcin + kc) * P1;
      base[q + 3] = val;
      if (q >= L2 - 3) base[q + 3 - L2] = val;
      if (q < 3) base[q + 3 + L2] = val;
    }
  };
  load_x(rg.lo);
  for (long long it = rg.lo; it < rg.hi && !failed; ++it) {
    const int grp = (int)(it / a.nv);
    const long long v = it % a.nv;
    if (grp != cur_g) {  // weights and constants of this group
      __syncthreads();
      copy16(sm, a.img + (size_t)grp * g.dsize, g.dsize);
      cur_g = grp;
    }
    sync_for_mma();
    // conv pair 1: D1[p][o], p < L/2 on the lanes, o < n1 in the columns
    if (tid == 0) {
      const uint32_t idesc = tc_idesc_bf16(128, N1);
      const uint32_t lboA = P1 * 16, lboB = g.n1 * 16;
      for (int oi = 0; oi < kOffsets; ++oi) {
        const int s = shift_of(oi);
        const int par = s & 1, row = 3 + (s >> 1);
        for (int j = 0; j < g.kcin / 2; ++j) {
          const uint64_t ad = tc_desc(sbase + g.dxs + (par * g.kcin + 2 * j) * lboA + row * 16, lboA, 128);
          const uint64_t bd = tc_desc(sbase + g.dw1 + (oi * g.kcin + 2 * j) * lboB, lboB, 128);
          tc_mma_bf16(d1, ad, bd, idesc, (oi | j) ? 1u : 0u);
        }
      }
      tc_commit(&bar);
    }
    if (__syncthreads_or(!tc_mbar_wait(&bar, phase, a.st, 21))) {
      failed = true;
      break;
    }
    phase ^= 1;
    tc_fence_after_sync();
    if (32 * qd < L2 && 4 * hf < g.kc1) {  // half hf: channel chunks [4hf, 4hf+4)
      const int p = 32 * qd + lane;
      const int par = p & 1, q = p >> 1;
      float vv[32];
      tc_ld32(d1 + ((uint32_t)(32 * qd) << 16) + 32 * hf, vv);
      for (int k = 0; k < 4 && 4 * hf + k < g.kc1; ++k) {
        const int kc = 4 * hf + k;
        const uint4 val = act8(vv + 8 * k, cst, kc, g.n1, 0, 128, 256);
        uint4* base = as + (size_t)(par * g.kc1 + kc) * P2;
        base[q + 3] = val;
        if (q >= L4 - 3) base[q + 3 - L4] = val;
        if (q < 3) base[q + 3 + L4] = val;
      }
    }
    sync_for_mma();
    // conv pair 2: D2[p][o], p < L/4, o < d
    if (tid == 0) {
      const uint32_t idesc = tc_idesc_bf16(128, N2);
      const uint32_t lboA = P2 * 16, lboB = g.d * 16;
      for (int oi = 0; oi < kOffsets; ++oi) {
        const int s = shift_of(oi);
        const int par = s & 1, row = 3 + (s >> 1);
        for (int j = 0; j < g.kc1 / 2; ++j) {
          const uint64_t ad = tc_desc(sbase + g.das + (par * g.kc1 + 2 * j) * lboA + row * 16, lboA, 128);
          const uint64_t bd = tc_desc(sbase + g.dw2 + (oi * g.kc1 + 2 * j) * lboB, lboB, 128);
          tc_mma_bf16(d2, ad, bd, idesc, (oi | j) ? 1u : 0u);
        }
      }
      tc_commit(&bar);
    }
    // xs is free once conv pair 1 has completed: stage the next item's input
    if (it + 1 < rg.hi) load_x(it + 1);
    if (__syncthreads_or(!tc_mbar_wait(&bar, phase, a.st, 22))) {
      failed = true;
      break;
    }
    phase ^= 1;
    tc_fence_after_sync();
    if (32 * qd < L4 && 4 * hf < g.kcd) {
      const int p = 32 * qd + lane;
      float vv[32];
      tc_ld32(d2 + ((uint32_t)(32 * qd) << 16) + 32 * hf, vv);
      for (int k = 0; k < 4 && 4 * hf + k < g.kcd; ++k) {
        const int kc = 4 * hf + k;
        stage[(size_t)kc * L4 + p] = act8(vv + 8 * k, cst, kc, g.d, 384, 512, 640);
      }
    }
    __syncthreads();
    copy16(a.mid + ((size_t)v * a.G + grp) * g.mid_bytes, sm + g.dstage, g.mid_bytes);
  }
  if (failed) tc_mbar_wait(&bar, phase, nullptr, 0);  // bounded: let outstanding MMAs drain
  tc_fence_before_sync();
  __syncthreads();
  if (warp == 0) tc_tmem_dealloc(t0, ncols);
}

// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(kThreads, 1) up_kernel(KArgs a) {
  extern __shared__ __align__(128) unsigned char sm[];
  __shared__ uint64_t bar;
  __shared__ uint32_t tbase;
  const Geo& g = a.g;
  const int L = g.L, L2 = L / 2, L4 = L / 4;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int qd = warp & 3, hf = warp >> 2;
  const Range rg = my_items(a.items);
  if (rg.lo >= rg.hi) return;
  const uint32_t ncols = 128;
  if (tid == 0) {
    tc_mbar_init(&bar, 1);
    tc_mbar_fence_init();
  }
  if (warp == 0) tc_tmem_alloc(&tbase, ncols);
  zero16(sm + g.ubs, g.usmem - g.ubs);  // halos and K padding stay zero
  tc_fence_before_sync();
  __syncthreads();
  tc_fence_after_sync();
  const uint32_t dt = tbase;
  const uint32_t sbase = tc_smem_u32(sm);
  const float* cst = reinterpret_cast<const float*>(sm + g.ucst);
  const int PB = L4 + 4, PC = L2 + 4, PD = L + 2;
  const int Nd = g.kcd * 8, Nm = rup(g.cmix, 16);
  const int cout = g.cmix + g.npass;
  uint4* bs = reinterpret_cast<uint4*>(sm + g.ubs);
  uint4* cs = reinterpret_cast<uint4*>(sm + g.ucs);
  uint4* ds = reinterpret_cast<uint4*>(sm + g.uds);
  float* xres = reinterpret_cast<float*>(sm + g.uxr);
  // intermediate [kcd][L/4][16B] of an item -> bs rows 2 .. L/4+1
  auto load_mid = [&](long long item) {
    const int grp = (int)(item / a.nv);
    const long long v = item % a.nv;
    const uint4* __restrict__ src = reinterpret_cast<const uint4*>(a.mid + ((size_t)v * a.G + grp) * g.mid_bytes);
    for (int i = tid; i < g.kcd * L4; i += blockDim.x) {
      const int kc = i / L4, q = i - kc * L4;
      bs[kc * PB + q + 2] = __ldg(src + i);
    }
  };
  unsigned phase = 0;
  bool failed = false;
  int cur_g = -1;
  load_mid(rg.lo);
  for (long long it = rg.lo; it < rg.hi && !failed; ++it) {
    const int grp = (int)(it / a.nv);
    const long long v = it % a.nv;
    if (grp != cur_g) {
      __syncthreads();
      copy16(sm, a.img + (size_t)grp * g.usize, g.usize);
      cur_g = grp;
    }
    const float* __restrict__ xin = a.x + ((long long)v * a.G + grp) * (long long)g.cin * L;
    float* __restrict__ op = a.out + ((long long)v * a.G + grp) * (long long)cout * L;
    sync_for_mma();
    // transposed conv 1: parity r in TMEM columns [r*Nd, (r+1)*Nd), rows q < L/4
    if (tid == 0) {
      const uint32_t idesc = tc_idesc_bf16(128, Nd);
      const uint32_t lboA = PB * 16, lboB = g.d * 16;
      for (int r = 0; r < 2; ++r)
        for (int u = 0; u < 5; ++u)
          for (int j = 0; j < g.kcd / 2; ++j) {
            const uint64_t ad = tc_desc(sbase + g.ubs + 2 * j * lboA + (4 - u) * 16, lboA, 128);
            const uint64_t bd = tc_desc(sbase + g.uw1 + ((r * 5 + u) * g.kcd + 2 * j) * lboB, lboB, 128);
            tc_mma_bf16(dt + r * Nd, ad, bd, idesc, (u | j) ? 1u : 0u);
          }
      tc_commit(&bar);
    }
    // while the tensor core runs: residual channels to shared memory, pass-through channels
    if (g.residual) {
      const float4* __restrict__ src = reinterpret_cast<const float4*>(xin);
      float4* dst = reinterpret_cast<float4*>(xres);
      for (int i = tid; i < g.cmix * L / 4; i += blockDim.x) dst[i] = __ldg(src + i);
    }
    {
      const float4* __restrict__ src = reinterpret_cast<const float4*>(xin + (size_t)(g.cin - g.npass) * L);
      float4* dst = reinterpret_cast<float4*>(op + (size_t)g.cmix * L);
      for (int i = tid; i < g.npass * L / 4; i += blockDim.x) dst[i] = __ldg(src + i);
    }
    if (__syncthreads_or(!tc_mbar_wait(&bar, phase, a.st, 23))) {
      failed = true;
      break;
    }
    phase ^= 1;
    tc_fence_after_sync();
    if (32 * qd < L4) {  // half hf = output parity r
      const int q = 32 * qd + lane, r = hf;
      for (int k0 = 0; k0 < g.kcd; k0 += 4) {
        float vv[32];
        tc_ld32(dt + ((uint32_t)(32 * qd) << 16) + r * Nd + 8 * k0, vv);
        for (int k = 0; k < 4 && k0 + k < g.kcd; ++k)
          cs[(size_t)(k0 + k) * PC + 2 * q + r + 2] = act8(vv + 8 * k, cst, k0 + k, g.d, 0, 128, 256);
      }
    }
    sync_for_mma();
    // transposed conv 2: parity r in columns [r*Nd, (r+1)*Nd), rows q < L/2
    if (tid == 0) {
      const uint32_t idesc = tc_idesc_bf16(128, Nd);
      const uint32_t lboA = PC * 16, lboB = g.d * 16;
      for (int r = 0; r < 2; ++r)
        for (int u = 0; u < 5; ++u)
          for (int j = 0; j < g.kcd / 2; ++j) {
            const uint64_t ad = tc_desc(sbase + g.ucs + 2 * j * lboA + (4 - u) * 16, lboA, 128);
            const uint64_t bd = tc_desc(sbase + g.uw2 + ((r * 5 + u) * g.kcd + 2 * j) * lboB, lboB, 128);
            tc_mma_bf16(dt + r * Nd, ad, bd, idesc, (u | j) ? 1u : 0u);
          }
      tc_commit(&bar);
    }
    if (__syncthreads_or(!tc_mbar_wait(&bar, phase, a.st, 24))) {
      failed = true;
      break;
    }
    phase ^= 1;
    tc_fence_after_sync();
    if (32 * qd < L2) {
      for (int qq = 32 * qd; qq < L2; qq += 128) {  // L/2 = 128 positions fill all four lane quarters
        const int q = qq + lane, r = hf;
        for (int k0 = 0; k0 < g.kcd; k0 += 4) {
          float vv[32];
          tc_ld32(dt + ((uint32_t)(32 * qd) << 16) + r * Nd + 8 * k0, vv);
          for (int k = 0; k < 4 && k0 + k < g.kcd; ++k)
            ds[(size_t)(k0 + k) * PD + 2 * q + r + 1] = act8(vv + 8 * k, cst, k0 + k, g.d, 384, 512, 640);
        }
      }
    }
    sync_for_mma();
    // mix: D[p][o] = sum_t d[p + t - 1] M_t; positions in halves of 128 rows
    if (tid == 0) {
      const uint32_t idesc = tc_idesc_bf16(128, Nm);
      const uint32_t lboA = PD * 16, lboB = g.cmix * 16;
      for (int h = 0; h < L / 128; ++h)
        for (int t = 0; t < 3; ++t)
          for (int j = 0; j < g.kcd / 2; ++j) {
            const uint64_t ad = tc_desc(sbase + g.uds + 2 * j * lboA + (t + 128 * h) * 16, lboA, 128);
            const uint64_t bd = tc_desc(sbase + g.uwm + (t * g.kcd + 2 * j) * lboB, lboB, 128);
            tc_mma_bf16(dt + h * Nm, ad, bd, idesc, (t | j) ? 1u : 0u);
          }
      tc_commit(&bar);
    }
    // bs is free once the first transposed conv has completed: next item's input
    if (it + 1 < rg.hi) load_mid(it + 1);
    if (__syncthreads_or(!tc_mbar_wait(&bar, phase, a.st, 25))) {
      failed = true;
      break;
    }
    phase ^= 1;
    tc_fence_after_sync();
    for (int h = 0; h < L / 128; ++h) {
      // L = 256: half hf takes position half h; L = 128: half hf takes channels [16hf, 16hf+16)
      if (L == 256 && h != hf) continue;
      const int p = 128 * h + 32 * qd + lane;
      float vv[32];
      tc_ld32(dt + ((uint32_t)(32 * qd) << 16) + h * Nm, vv);
      const int o0 = (L == 256) ? 0 : 16 * hf, o1 = (L == 256) ? Nm : 16 * hf + 16;
      for (int o = o0; o < o1 && o < g.cmix; ++o) {
        float y = vv[o] + cst[768 + o];
        if (g.residual) y += xres[(size_t)o * L + p];
        op[(size_t)o * L + p] = y;
      }
    }
    tc_fence_before_sync();
    __syncthreads();
  }
  if (failed) tc_mbar_wait(&bar, phase, nullptr, 0);  // bounded: let outstanding MMAs drain
  tc_fence_before_sync();
  __syncthreads();
  if (warp == 0) tc_tmem_dealloc(dt, ncols);
}

}  // namespace tcnet

// ---------------------------------------------------------------------------
// host side
#include "ves_nets_tc.h"

namespace {

uint16_t bf16_rn(float f) {
  uint32_t u;
  memcpy(&u, &f, 4);
  if ((u & 0x7f800000u) == 0x7f800000u) return (uint16_t)(u >> 16);  // inf / nan
  const uint32_t lsb = (u >> 16) & 1u;
  u += 0x7fffu + lsb;
  return (uint16_t)(u >> 16);
}

void put_row(unsigned char* img, size_t off, const float* vals8) {
  uint16_t* p = reinterpret_cast<uint16_t*>(img + off);
  for (int e = 0; e < 8; ++e) p[e] = bf16_rn(vals8[e]);
}

}  // namespace

int tcnet_pack(const ves_net_block& b, int G, int L, const float* const* p, std::vector<unsigned char>& down,
               std::vector<unsigned char>& up, TcBlock& out) {
  using namespace tcnet;
  const Geo g = make_geo(b, L);
  out.geo_bytes = sizeof(Geo);
  memcpy(out.geo, &g, sizeof(Geo));
  out.dsize = g.dsize;
  out.usize = g.usize;
  out.dsmem = g.dsmem;
  out.usmem = g.usmem;
  out.mid_bytes = g.mid_bytes;
  if (g.n1 > 128 || g.d > 128 || g.cmix > 128 || g.dsmem > 227 * 1024 || g.usmem > 227 * 1024 || L > 256 ||
      (L / 4) % 16 != 0)
    return VES_ERR_ARG;
  const int c1 = b.c1, c2 = b.c2, d = g.d, cin = b.cin, cmix = b.cmix;
  down.assign((size_t)g.dsize * G, 0);
  up.assign((size_t)g.usize * G, 0);
  auto bn = [&](int idx, int ch, float* s, float* t) {
    const float* w = p[14 + 4 * idx];
    const float* bb = p[15 + 4 * idx];
    const float* mean = p[16 + 4 * idx];
    const float* var = p[17 + 4 * idx];
    const double inv = 1.0 / std::sqrt((double)var[ch] + 1e-5);
    *s = (float)((double)w[ch] * inv);
    *t = (float)((double)bb[ch] - (double)mean[ch] * (double)w[ch] * inv);
  };
  for (int grp = 0; grp < G; ++grp) {
    unsigned char* D = down.data() + (size_t)grp * g.dsize;
    unsigned char* U = up.data() + (size_t)grp * g.usize;
    float v8[8];
    // conv pair 1
    for (int oi = 0; oi < kOffsets; ++oi) {
      const int s = shift_of(oi);
      for (int kc = 0; kc < g.kcin; ++kc)
        for (int o = 0; o < g.n1; ++o) {
          for (int e = 0; e < 8; ++e) {
            const int c = kc * 8 + e;
            float w = 0.f;
            if (c < cin) {
              if (o < c1) {
                const int t = s + 3;
                if (t >= 0 && t < 7) w = p[0][((size_t)(grp * c1 + o) * cin + c) * 7 + t];
              } else if ((s & 1) == 0) {
                const int t = (s + 6) / 2;
                w = p[2][((size_t)(grp * c1 + o - c1) * cin + c) * 7 + t];
              }
            }
            v8[e] = w;
          }
          put_row(D, g.dw1 + ((size_t)(oi * g.kcin + kc) * g.n1 + o) * 16, v8);
        }
      for (int kc = 0; kc < g.kc1; ++kc)
        for (int o = 0; o < d; ++o) {
          for (int e = 0; e < 8; ++e) {
            const int c = kc * 8 + e;
            float w = 0.f;
            if (c < g.n1) {
              if (o < c2) {
                const int t = s + 3;
                if (t >= 0 && t < 7) w = p[4][((size_t)(grp * c2 + o) * g.n1 + c) * 7 + t];
              } else if ((s & 1) == 0) {
                const int t = (s + 6) / 2;
                w = p[6][((size_t)(grp * c2 + o - c2) * g.n1 + c) * 7 + t];
              }
            }
            v8[e] = w;
          }
          put_row(D, g.dw2 + ((size_t)(oi * g.kc1 + kc) * d + o) * 16, v8);
        }
    }
    float* dc = reinterpret_cast<float*>(D + g.dcst);
    for (int o = 0; o < g.n1; ++o) {
      dc[o] = o < c1 ? p[1][grp * c1 + o] : p[3][grp * c1 + o - c1];
      bn(0, grp * g.n1 + o, &dc[128 + o], &dc[256 + o]);
    }
    for (int o = 0; o < d; ++o) {
      dc[384 + o] = o < c2 ? p[5][grp * c2 + o] : p[7][grp * c2 + o - c2];
      bn(1, grp * d + o, &dc[512 + o], &dc[640 + o]);
    }
    // transposed convs: A[o][c] = W[grp*d + c][o][r + 2u]
    for (int layer = 0; layer < 2; ++layer) {
      const float* W = p[8 + 2 * layer];
      const int base = layer ? g.uw2 : g.uw1;
      for (int r = 0; r < 2; ++r)
        for (int u = 0; u < 5; ++u)
          for (int kc = 0; kc < g.kcd; ++kc)
            for (int o = 0; o < d; ++o) {
              for (int e = 0; e < 8; ++e) {
                const int c = kc * 8 + e;
                v8[e] = c < d ? W[((size_t)(grp * d + c) * d + o) * 10 + r + 2 * u] : 0.f;
              }
              put_row(U, base + ((size_t)((r * 5 + u) * g.kcd + kc) * d + o) * 16, v8);
            }
    }
    for (int t = 0; t < 3; ++t)
      for (int kc = 0; kc < g.kcd; ++kc)
        for (int o = 0; o < cmix; ++o) {
          for (int e = 0; e < 8; ++e) {
            const int c = kc * 8 + e;
            v8[e] = c < d ? p[12][((size_t)(grp * cmix + o) * d + c) * 3 + t] : 0.f;
          }
          put_row(U, g.uwm + ((size_t)(t * g.kcd + kc) * cmix + o) * 16, v8);
        }
    float* uc = reinterpret_cast<float*>(U + g.ucst);
    for (int o = 0; o < d; ++o) {
      uc[o] = p[9][grp * d + o];
      bn(2, grp * d + o, &uc[128 + o], &uc[256 + o]);
      uc[384 + o] = p[11][grp * d + o];
      bn(3, grp * d + o, &uc[512 + o], &uc[640 + o]);
    }
    for (int o = 0; o < cmix; ++o) uc[768 + o] = p[13][grp * cmix + o];
  }
  return VES_OK;
}

int tcnet_run_block(const TcBlock& tb, int G, int nv, const unsigned char* d_down, const unsigned char* d_up,
                    const float* x, float* out, unsigned char* mid, VesDeviceStatus* st, cudaStream_t s) {
  using namespace tcnet;
  KArgs a;
  memcpy(&a.g, tb.geo, sizeof(Geo));
  a.G = G;
  a.nv = nv;
  a.items = (long long)G * nv;
  a.x = x;
  a.out = out;
  a.mid = mid;
  a.st = st;
  int dev = 0, nsm = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  int rc = ves_cuda_status(cudaFuncSetAttribute(down_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, tb.dsmem),
                           "tc down smem");
  if (rc) return rc;
  rc = ves_cuda_status(cudaFuncSetAttribute(up_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, tb.usmem),
                       "tc up smem");
  if (rc) return rc;
  auto grid_for = [&](int smem) {
    const int per_sm = std::max(1, std::min(2, (227 * 1024) / (smem + 1024)));
    return (int)std::min<long long>(a.items, (long long)nsm * per_sm);
  };
  a.img = d_down;
  ves_count_launch(2);
  down_kernel<<<grid_for(tb.dsmem), kThreads, tb.dsmem, s>>>(a);
  a.img = d_up;
  up_kernel<<<grid_for(tb.usmem), kThreads, tb.usmem, s>>>(a);
  return ves_launch_check("tc net block");
}
