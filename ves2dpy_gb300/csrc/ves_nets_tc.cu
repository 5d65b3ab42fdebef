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
// Three kernels per block: "down" (conv pair 1, conv pair 2), "up1"
// (transposed conv 1) and "up2" (transposed conv 2, mix, residual and
// pass-through).  up1 works on tiles of V1 = 128 / (L/4) vesicles of one
// group whose rows are interleaved (row q*V1 + j holds position q of the
// tile's vesicle j), so that its MMAs use all 128 rows: a shift of the input
// by u positions is a shift by u*V1 rows, and every row still only meets
// rows of its own vesicle.  down writes the intermediate in that layout.
// down itself works on tiles of vd = 2 vesicles at L = 128 (conv pair 1
// then fills 128 rows, conv pair 2 64), one vesicle at L = 256.  The block input and output stay FP32 in global memory
// ([nv][groups*channels][L]); the intermediates between the kernels are BF16
// in the K-major layout.  Kernels are persistent: each CTA walks a contiguous
// range of (group, vesicle) items, loading a group's weight image into shared
// memory once per group it meets, and runs several warp groups, each on its
// own items (3, 4 and 3 when TMEM and shared memory allow): while one waits
// for its MMAs the others run their epilogues.  Splitting the transposed
// convs over two kernels keeps each weight image small enough for that.
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <vector>

#include "ves_internal.h"
#include "ves_tc.cuh"
#include <cuda_bf16.h>

namespace tcnet {

constexpr int kGroupThreads = 128;
constexpr int kMinSmem = 117 * 1024;
constexpr int kOffsets = 11;  // input shifts of a conv pair: -6..6 without +-5
__host__ __device__ constexpr int shift_of(int oi) { return oi < 2 ? -6 + 2 * oi : (oi < 9 ? oi - 5 : 2 * oi - 14); }

__host__ __device__ constexpr int rup(int a, int b) { return (a + b - 1) / b * b; }

// Geometry of one block, shared by host packing and kernels (bytes unless noted).
// Shared memory holds one weight image and, per warp group, its own
// activation arrays (each warp group runs its own (group, vesicle) items).
struct Geo {
  int cin, c1, c2, cmix, residual, npass, L, lgL;
  int n1, d;             // conv-pair output channels
  int kcin, kc1, kcd;    // 8-channel K chunks of the three GEMM inputs (even)
  // down image: W1 [11][kcin][n1][16B], W2 [11][kc1][d][16B], consts [6][128] f32
  int dw1, dw2, dcst, dsize;
  // down arrays of warp group 0 (group k at + k*dgrp): xs [2][kcin][L/2+6][16B],
  // as [2][kc1][L/4+6][16B], xf [cin][L] f32 (the
  // block input as it arrives by bulk copy); a tail of 2 KB follows the groups
  int dxs, das, dxf, dgrp;
  // up1 image (transposed conv 1): W (u1merge = 0: [2][5][kcd][d][16B], output
  // parity r, tap u, the parities M-split over the lanes; u1merge = 1: the
  // merged layout of up2, both parities in one operand of N = 2*kcd*8),
  // consts [7][128] f32; arrays of warp group 0: bs [kcd][L/4+4][16B]
  int u1merge, u1w, u1cst, u1size, u1bs, u1grp;
  // up2 image (transposed conv 2 and mix): W (u2merge = 1: [5][kcd][2*kcd*8][16B],
  // both output parities in one operand of N = 2*kcd*8 rows, parity r at row
  // r*kcd*8; u2merge = 0: as up1), M [3][kcd][cmix][16B], consts [7][128] f32;
  // arrays of warp group 0: cs [kcd][L/2+4][16B], ds [kcd][L+2][16B] (at least
  // cin*L*4 bytes: it first receives the block input)
  int u2merge, u2w, u2wm, u2cst, u2size, u2cs, u2ds, u2grp;
  // down -> up1 per tile of v1 vesicles: [kcd][L/4][v1][16B] (mid_bytes per
  // vesicle); up1 -> up2 per (vesicle, group) item: [kcd][L/2][16B]
  int mid_bytes, mid2_bytes, mid_stride;
  int v1;  // vesicles per up1 tile (v1 * L/4 = 128 rows)
  int vd;  // vesicles per down tile (2 at L = 128: the block input is read
           // from global memory (L2-prefetched) with no FP32 staging copy)
};

constexpr int kMaxSmem = 227 * 1024 - 256;  // dynamic shared memory available next to the static part
constexpr int kTail = 128 * 16;             // after the groups' arrays: rows an MMA reads past the last one

// byte offset of row o of K chunk kc of tap u, output parity r, in the
// unmerged layout [2][5][kcd][d][16B] (base = start of the weights)
__host__ __device__ inline int dec_w_off(const Geo& g, int base, int r, int u, int kc, int o) {
  return base + (((r * 5 + u) * g.kcd + kc) * g.d + o) * 16;
}
// same in the merged layout [5][kcd][2*kcd*8][16B]
__host__ __device__ inline int dec_w_off_merged(const Geo& g, int base, int r, int u, int kc, int o) {
  return base + ((u * g.kcd + kc) * 2 * g.kcd * 8 + r * g.kcd * 8 + o) * 16;
}

// transposed conv 1 with both output parities in one MMA (VES_TC_UP1_MERGE=0/1
// overrides the default; read once)
inline int tcnet_up1_merge(int L) {
  static int v = -2;
  if (v == -2) {
    const char* e = getenv("VES_TC_UP1_MERGE");
    v = e ? (atoi(e) ? 1 : 0) : -1;
  }
  if (v >= 0) return v;
  (void)L;
  return 1;  // measured 1-2% faster networks than the M-split at L = 128 and 256
}

inline Geo make_geo(const ves_net_block& b, int L) {
  Geo g;
  g.cin = b.cin;
  g.c1 = b.c1;
  g.c2 = b.c2;
  g.cmix = b.cmix;
  g.residual = b.residual;
  g.npass = b.npass;
  g.L = L;
  g.lgL = 0;
  while ((1 << g.lgL) < L) ++g.lgL;
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
  g.vd = (L / 2 <= 64) ? 2 : 1;
  g.dxs = o;
  o += 2 * g.kcin * (L / 2 + 6) * g.vd * 16;
  g.das = o;
  o += 2 * g.kc1 * (L / 4 + 6) * g.vd * 16;
  g.dxf = o;
  o += g.vd == 1 ? rup(g.cin * L * 4, 16) : 0;
  g.dgrp = o - g.dxs;
  const int dec_unmerged = 10 * g.kcd * g.d * 16;
  // up1: both parities in one MMA of N = 2*Nd (u1merge, fewer and larger MMAs,
  // half the lanes busy) or M-split over the lanes (unmerged layout)
  g.u1merge = tcnet_up1_merge(L);
  g.u1w = 0;
  g.u1cst = g.u1merge ? 5 * g.kcd * 2 * g.kcd * 8 * 16 : dec_unmerged;
  g.u1size = g.u1cst + 7 * 128 * 4;
  g.u1bs = g.u1size;
  g.v1 = 128 / (L / 4);
  g.u1grp = g.kcd * (L / 4 + 4) * g.v1 * 16;
  // up2: merged image (both parities in one operand of N = 2*Nd rows) when it
  // still leaves room for three warp groups
  g.u2grp = g.kcd * (L / 2 + 4) * 16 + std::max(g.kcd * (L + 2) * 16, rup(g.cin * L * 4, 16));
  for (g.u2merge = 1; g.u2merge >= 0; --g.u2merge) {
    const int dbytes = g.u2merge ? 5 * g.kcd * 2 * g.kcd * 8 * 16 : dec_unmerged;
    g.u2w = 0;
    g.u2wm = dbytes;
    g.u2cst = g.u2wm + 3 * g.kcd * g.cmix * 16;
    g.u2size = g.u2cst + 7 * 128 * 4;
    if (g.u2size + 3 * g.u2grp + kTail <= kMaxSmem) break;
  }
  if (g.u2merge < 0) g.u2merge = 0;
  g.u2cs = g.u2size;
  g.u2ds = g.u2cs + g.kcd * (L / 2 + 4) * 16;
  g.mid_bytes = g.kcd * (L / 4) * 16;
  g.mid2_bytes = g.kcd * (L / 2) * 16;
  g.mid_stride = g.mid_bytes + g.mid2_bytes;
  return g;
}

struct KArgs {
  Geo g;
  int G, nv;
  int m64;                   // layers of at most 64 positions use M = 64 MMAs
  long long items;
  const unsigned char* img;  // group 0 image of this block; group stride = image size
  const float* x;            // block input [nv][G*cin][L]
  float* out;                // block output [nv][G*cout][L]
  unsigned char* mid;        // down -> up1: [ntiles][G][v1 * mid_bytes]
  unsigned char* mid2;       // up1 -> up2: [nv][G][mid2_bytes]
  int per_grp;               // items per channel group (nv, or up1 tiles)
  VesDeviceStatus* st;
};

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

// barrier of one warp group (named barrier 1 + group, 128 threads)
__device__ __forceinline__ void group_sync(int wg) {
  asm volatile("bar.sync %0, %1;" ::"r"(1 + wg), "r"(kGroupThreads) : "memory");
}
// all of the group's writes to shared memory so far -> visible to the tensor core
__device__ __forceinline__ void group_sync_for_mma(int wg) {
  tc_fence_async_smem();
  tc_fence_before_sync();
  group_sync(wg);
  tc_fence_after_sync();
}
// Bounded wait of one warp group on an mbarrier; true when the phase
// completed (the answer is uniform across the group).  Thread 0 of the group
// polls (sleeping between polls) and the others wait in the group barrier, so
// a wait that is not yet satisfied takes no issue slots from the other groups.
__device__ __forceinline__ bool group_wait_one(uint64_t* bar, unsigned phase, VesDeviceStatus* st, int site, int wg,
                                               int gt, int* flag) {
  if (gt == 0 && !tc_mbar_wait_sleep(bar, phase, st, site)) atomicExch(flag, 1);
  group_sync(wg);
  return *(volatile int*)flag == 0;
}

// MMA issue sequences.  The issuing lane runs them as straight-line code:
// each is a template on the number of 16-channel K steps (NK), picked by one
// switch, so that no loop branch sits between two tcgen05.mma (a branching
// loop in the single issuing lane costs more than the tensor core's time per
// MMA).  Descriptors advance by adds: the start address is the low 14 bits of
// a descriptor, in 16-byte units.

// conv pair: 11 input shifts x NK K steps.  A at a0 + par*aPar + row*rowMul
// (rowMul: vesicles per tile, rows interleaved), B at b0 + oi*bOi; K steps at
// stepA / stepB.
template <int NK>
__device__ __forceinline__ void issue_conv(uint32_t d, uint64_t a0, uint64_t b0, uint32_t aPar, uint32_t bOi,
                                           uint32_t stepA, uint32_t stepB, uint32_t idesc, uint32_t rowMul = 1) {
#pragma unroll
  for (int oi = 0; oi < kOffsets; ++oi) {
    const int s = shift_of(oi);
    const uint64_t ad = a0 + (uint32_t)((s & 1) * aPar + (3 + (s >> 1)) * rowMul);
    const uint64_t bd = b0 + (uint32_t)oi * bOi;
#pragma unroll
    for (int j = 0; j < NK; ++j) tc_mma_bf16(d, ad + j * stepA, bd + j * stepB, idesc, (oi | j) ? 1u : 0u);
  }
}
// transposed conv, one output parity: 5 taps u (A rows (4 - u) * tapRows) x NK K steps.
template <int NK>
__device__ __forceinline__ void issue_deconv(uint32_t d, uint64_t a0, uint64_t b0, uint32_t bTap, uint32_t stepA,
                                             uint32_t stepB, uint32_t idesc, uint32_t tapRows = 1) {
#pragma unroll
  for (int u = 0; u < 5; ++u) {
    const uint64_t ad = a0 + (uint32_t)(4 - u) * tapRows, bd = b0 + (uint32_t)u * bTap;
#pragma unroll
    for (int j = 0; j < NK; ++j) tc_mma_bf16(d, ad + j * stepA, bd + j * stepB, idesc, (u | j) ? 1u : 0u);
  }
}
// mix of one 128-position half: 3 taps t (A rows t) x NK K steps, onto the
// preset accumulator
template <int NK>
__device__ __forceinline__ void issue_mix(uint32_t d, uint64_t a0, uint64_t b0, uint32_t bTap, uint32_t stepA,
                                          uint32_t stepB, uint32_t idesc) {
#pragma unroll
  for (int t = 0; t < 3; ++t) {
    const uint64_t ad = a0 + (uint32_t)t, bd = b0 + (uint32_t)t * bTap;
#pragma unroll
    for (int j = 0; j < NK; ++j) tc_mma_bf16(d, ad + j * stepA, bd + j * stepB, idesc, 1u);
  }
}
#define VES_TC_NK_SWITCH(nk, call)                                                                            \
  switch (nk) {                                                                                               \
    case 1: call(1); break;                                                                                   \
    case 2: call(2); break;                                                                                   \
    case 3: call(3); break;                                                                                   \
    case 4: call(4); break;                                                                                   \
    case 5: call(5); break;                                                                                   \
    case 6: call(6); break;                                                                                   \
    case 7: call(7); break;                                                                                   \
    default: call(8); break;                                                                                  \
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

// two FP32 values -> one 32-bit word of two BF16 (round to nearest even), low half first
__device__ __forceinline__ uint32_t pack_bf2(float lo, float hi) {
  const __nv_bfloat162 h = __floats2bfloat162_rn(lo, hi);
  return *reinterpret_cast<const uint32_t*>(&h);
}

// 8 channels [8kc, 8kc+8) of this thread's position: relu(v + b) * s + t, 0 beyond nreal
__device__ __forceinline__ uint4 act8(const float* v, const float* cst, int kc, int nreal, int ob, int os, int ot) {
  float b[8], sc[8], sh[8];
  *reinterpret_cast<float4*>(b) = *reinterpret_cast<const float4*>(cst + ob + 8 * kc);
  *reinterpret_cast<float4*>(b + 4) = *reinterpret_cast<const float4*>(cst + ob + 8 * kc + 4);
  *reinterpret_cast<float4*>(sc) = *reinterpret_cast<const float4*>(cst + os + 8 * kc);
  *reinterpret_cast<float4*>(sc + 4) = *reinterpret_cast<const float4*>(cst + os + 8 * kc + 4);
  *reinterpret_cast<float4*>(sh) = *reinterpret_cast<const float4*>(cst + ot + 8 * kc);
  *reinterpret_cast<float4*>(sh + 4) = *reinterpret_cast<const float4*>(cst + ot + 8 * kc + 4);
  float y[8];
  // packed FP32x2 add and fma: per lane the same rounding as fadd / fmaf
#pragma unroll
  for (int e = 0; e < 8; e += 2) {
    float2 z = __fadd2_rn(make_float2(v[e], v[e + 1]), make_float2(b[e], b[e + 1]));
    z.x = fmaxf(z.x, 0.f);
    z.y = fmaxf(z.y, 0.f);
    z = __ffma2_rn(z, make_float2(sc[e], sc[e + 1]), make_float2(sh[e], sh[e + 1]));
    y[e] = z.x;
    y[e + 1] = z.y;
  }
  if (8 * kc + 8 > nreal) {  // the chunk that holds the padding channels (TMEM columns past nreal are not defined)
#pragma unroll
    for (int e = 0; e < 8; ++e)
      if (8 * kc + e >= nreal) y[e] = 0.f;
  }
  return make_uint4(pack_bf2(y[0], y[1]), pack_bf2(y[2], y[3]), pack_bf2(y[4], y[5]), pack_bf2(y[6], y[7]));
}

// Rows of an accumulator of M rows in TMEM: M = 128 puts row r on lane r;
// M = 64 (half the A tile per MMA, for layers of at most 64 positions) puts
// rows 16 q .. 16 q + 15 on lanes 32 q .. 32 q + 15 (measured on a GB300).
// The row this thread's lane holds, or -1.
__device__ __forceinline__ int acc_row(int M, int qd, int lane) {
  return M == 128 ? 32 * qd + lane : (lane < 16 ? 16 * qd + lane : -1);
}
// first row held by warp quarter qd (uniform across the warp)
__device__ __forceinline__ int acc_row0(int M, int qd) { return M == 128 ? 32 * qd : 16 * qd; }

// accumulators of at most 64 rows use M = 64 MMAs (VES_TC_M64=0 turns this off; read once)
inline bool tcnet_m64() {
  static int v = -1;
  if (v < 0) {
    const char* e = getenv("VES_TC_M64");
    v = (e && atoi(e) == 0) ? 0 : 1;
  }
  return v != 0;
}

// ---------------------------------------------------------------------------
// Segments: the CTA's contiguous item range split where the channel group
// changes; the weight image is reloaded (whole CTA) at each segment start and
// the warp groups take the segment's items in turn.
struct Seg {
  long long lo, hi;
  int grp;
};
__device__ __forceinline__ Seg next_seg(long long lo, long long hi, int nv) {
  const int grp = (int)(lo / nv);
  const long long end = (long long)(grp + 1) * nv;
  return {lo, end < hi ? end : hi, grp};
}

// KC1 / KCD: compile-time K chunk counts of the two conv pairs' outputs (0:
// read them from the geometry); fixed counts let every epilogue and issue
// loop unroll.  NG: warp groups per CTA, each running its own items (2: 256
// TMEM columns each; 3 or 4: 128 columns each, when N1 + N2 <= 128 and the
// groups' arrays fit in shared memory).
template <int KC1, int KCD, int NG>
__global__ void __launch_bounds__(NG * kGroupThreads, 1) down_kernel(KArgs a) {
  extern __shared__ __align__(128) unsigned char sm[];
  __shared__ uint64_t bar[NG], xbar[NG];  // per warp group: MMA completion, input arrival
  __shared__ uint32_t tbase;
  __shared__ int fail[NG];
  const Geo& g = a.g;
  const int kc1 = KC1 ? KC1 : g.kc1, kcd = KCD ? KCD : g.kcd;
  const int L = g.L, L2 = L / 2, L4 = L / 4;
  const int VD = g.vd;          // vesicles per item (tile), rows interleaved
  const int ntl = a.per_grp;    // tiles per channel group
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int wg = tid / kGroupThreads, gt = tid % kGroupThreads;  // warp group, thread within it
  const int qd = warp & 3;                                       // TMEM lane quarter = position block
  const Range rg = my_items(a.items);
  if (rg.lo >= rg.hi) return;
  const uint32_t ncols = 512;  // all of TMEM (one CTA per SM)
  if (tid == 0) {
    for (int k = 0; k < NG; ++k) {
      tc_mbar_init(&bar[k], 1);
      tc_mbar_init(&xbar[k], 1);
      fail[k] = 0;
    }
    tc_mbar_fence_init();
  }
  if (warp == 0) tc_tmem_alloc(&tbase, ncols);
  zero16(sm + g.dxs, NG * g.dgrp + 128 * 16);  // K padding of the activation arrays stays zero
  tc_fence_async_smem();
  tc_fence_before_sync();
  __syncthreads();
  tc_fence_after_sync();
  const int N1 = kc1 * 8, N2 = kcd * 8;
  const uint32_t tcol = tbase + (NG == 2 ? 256 : 128) * wg;
  const uint32_t d1 = tcol, d2 = tcol + N1;
  const uint32_t sbase = tc_smem_u32(sm);
  const int goff = wg * g.dgrp;
  const float* cst = reinterpret_cast<const float*>(sm + g.dcst);
  const int P1 = (L2 + 6) * VD, P2 = (L4 + 6) * VD;  // rows per K chunk (circular halos of 3 positions)
  uint4* xs = reinterpret_cast<uint4*>(sm + g.dxs + goff);
  uint4* as = reinterpret_cast<uint4*>(sm + g.das + goff);
  float* xf = reinterpret_cast<float*>(sm + g.dxf + goff);
  const uint32_t xbytes = (uint32_t)(g.cin * L * 4);
  unsigned phase = 0, xphase = 0;
  bool xpend = false;  // a bulk copy into xf is in flight
  // block input x[v][grp*cin + c][pos] (cin*L contiguous floats) of the
  // item's vesicles: one vesicle -> xf by bulk copy; a tile of two -> L2
  // (read by convert_x straight from global memory)
  auto fetch_x = [&](long long item) {
    const int grp = (int)(item / ntl);
    const long long t = item % ntl;
    if (VD == 1) {
      if (gt == 0) {
        tc_expect_tx(&xbar[wg], xbytes);
        tc_bulk_g2s(xf, a.x + ((long long)t * a.G + grp) * (long long)g.cin * L, xbytes, &xbar[wg]);
      }
      xpend = true;
    } else if (gt < VD && t * VD + gt < a.nv) {
      tc_prefetch_l2(a.x + ((t * VD + gt) * a.G + grp) * (long long)g.cin * L, xbytes);
    }
  };
  // block input -> parity-split BF16 rows with circular halos of 3
  // positions, position m of vesicle j at row (m + 3)*VD + j; one thread per
  // (8-channel chunk, vesicle, position pair 2m, 2m+1)
  auto convert_x = [&](long long t, int grp) {
    const int lg2 = g.lgL - 1;
    for (int i = gt; i < g.kcin * VD * L2; i += kGroupThreads) {
      const int m = i & (L2 - 1), kj = i >> lg2, kc = kj / VD, j = kj - kc * VD;
      const long long v = t * VD + j;
      float2 y[8];
      if (VD == 1) {
#pragma unroll
        for (int e = 0; e < 8; ++e)
          y[e] = (8 * kc + e < g.cin) ? *reinterpret_cast<const float2*>(xf + (8 * kc + e) * L + 2 * m)
                                      : make_float2(0.f, 0.f);
      } else {
        const float* src = a.x + ((v < a.nv ? v : 0) * a.G + grp) * (long long)g.cin * L;
#pragma unroll
        for (int e = 0; e < 8; ++e)
          y[e] = (8 * kc + e < g.cin && v < a.nv) ? __ldg(reinterpret_cast<const float2*>(src + (8 * kc + e) * L + 2 * m))
                                                  : make_float2(0.f, 0.f);
      }
      const uint4 v0 = make_uint4(pack_bf2(y[0].x, y[1].x), pack_bf2(y[2].x, y[3].x), pack_bf2(y[4].x, y[5].x),
                                  pack_bf2(y[6].x, y[7].x));
      const uint4 v1 = make_uint4(pack_bf2(y[0].y, y[1].y), pack_bf2(y[2].y, y[3].y), pack_bf2(y[4].y, y[5].y),
                                  pack_bf2(y[6].y, y[7].y));
      uint4* b0 = xs + (size_t)kc * P1 + j;
      uint4* b1 = xs + (size_t)(g.kcin + kc) * P1 + j;
      b0[(m + 3) * VD] = v0;
      b1[(m + 3) * VD] = v1;
      if (m >= L2 - 3) {
        b0[(m + 3 - L2) * VD] = v0;
        b1[(m + 3 - L2) * VD] = v1;
      }
      if (m < 3) {
        b0[(m + 3 + L2) * VD] = v0;
        b1[(m + 3 + L2) * VD] = v1;
      }
    }
  };
  bool failed = false, stuck = false;  // stuck: this warp group's own MMA wait timed out
  for (long long lo = rg.lo; lo < rg.hi && !failed;) {
    const Seg sg = next_seg(lo, rg.hi, ntl);
    __syncthreads();
    copy16(sm, a.img + (size_t)sg.grp * g.dsize, g.dsize);  // whole CTA
    tc_fence_async_smem();  // weights (and the zeroed padding) -> tensor core, for both groups
    __syncthreads();
    if (sg.lo + wg < sg.hi) fetch_x(sg.lo + wg);
    for (long long it = sg.lo + wg; it < sg.hi; it += NG) {
      const long long t = it % ntl;
      if (VD == 1) {
        if (!group_wait_one(&xbar[wg], xphase, a.st, 20, wg, gt, &fail[wg])) {
          failed = true;
          break;
        }
        xphase ^= 1;
        xpend = false;
      }
      convert_x(t, sg.grp);
      group_sync_for_mma(wg);  // xs complete; xf fully read
      if (it + NG < sg.hi) fetch_x(it + NG);
      // conv pair 1: D1[r][o], rows r = p*VD + j (p < L/2) on the lanes, o < n1 in the columns
      const int M1 = (a.m64 && L2 * VD <= 64) ? 64 : 128, M2 = (a.m64 && L4 * VD <= 64) ? 64 : 128;
      if (gt == 0) {
        const uint32_t idesc = tc_idesc_bf16(M1, N1);
        const uint32_t lboA = P1 * 16, lboB = g.n1 * 16;
        const uint64_t a0 = tc_desc(sbase + g.dxs + goff, lboA, 128), b0 = tc_desc(sbase + g.dw1, lboB, 128);
#define VES_CONV1(NK) issue_conv<NK>(d1, a0, b0, (g.kcin * lboA) >> 4, (g.kcin * lboB) >> 4, (2 * lboA) >> 4, (2 * lboB) >> 4, idesc, (uint32_t)VD)
        VES_TC_NK_SWITCH(g.kcin / 2, VES_CONV1)
#undef VES_CONV1
        tc_commit(&bar[wg]);
      }
      if (!group_wait_one(&bar[wg], phase, a.st, 21, wg, gt, &fail[wg])) {
        failed = stuck = true;
        break;
      }
      phase ^= 1;
      tc_fence_after_sync();
      // the epilogue's row r holds position p = r / VD of the tile's vesicle j = r % VD;
      // conv pair 2 reads position q of parity par at row (q + 3)*VD + j
      if (KC1 != 0 && M1 == 64) {
        // M = 64: threads 0-15 and 16-31 of a warp take the two halves of the
        // channel chunks of the same 16 rows (16x32bx2 loads)
        const int r = 16 * qd + (lane & 15), p = r / VD, j = r - p * VD, par = p & 1, q = p >> 1;
        const int kb = (lane >> 4) * (KC1 / 2);
        float vv[32];
        tc_ld16x2_32<4 * KC1>(d1 + ((uint32_t)(32 * qd) << 16), vv);
        if (p < L2) {
#pragma unroll
          for (int k = 0; k < KC1 / 2; ++k) {
            const int kc = kb + k;
            const uint4 val = act8(vv + 8 * k, cst, kc, g.n1, 0, 128, 256);
            uint4* base = as + (size_t)(par * kc1 + kc) * P2 + j;
            base[(q + 3) * VD] = val;
            if (q >= L4 - 3) base[(q + 3 - L4) * VD] = val;
            if (q < 3) base[(q + 3 + L4) * VD] = val;
          }
        }
      } else if (acc_row0(M1, qd) < L2 * VD) {  // uniform per warp: the TMEM loads are warp-wide
        const int r = acc_row(M1, qd, lane), p = r / VD, j = r - p * VD;
        const bool own = r >= 0 && p < L2;
        const int par = p & 1, q = p >> 1;
#pragma unroll
        for (int k0 = 0; k0 < kc1; k0 += 4) {
          float vv[32];
          tc_ld32(d1 + ((uint32_t)(32 * qd) << 16) + 8 * k0, vv);
          if (own) {
#pragma unroll
            for (int k = 0; k < 4; ++k) {
              const int kc = k0 + k;
              if (kc >= kc1) break;
              const uint4 val = act8(vv + 8 * k, cst, kc, g.n1, 0, 128, 256);
              uint4* base = as + (size_t)(par * kc1 + kc) * P2 + j;
              base[(q + 3) * VD] = val;
              if (q >= L4 - 3) base[(q + 3 - L4) * VD] = val;
              if (q < 3) base[(q + 3 + L4) * VD] = val;
            }
          }
        }
      }
      group_sync_for_mma(wg);
      // conv pair 2: D2[p][o], p < L/4, o < d
      if (gt == 0) {
        const uint32_t idesc = tc_idesc_bf16(M2, N2);
        const uint32_t lboA = P2 * 16, lboB = g.d * 16;
        const uint64_t a0 = tc_desc(sbase + g.das + goff, lboA, 128), b0 = tc_desc(sbase + g.dw2, lboB, 128);
#define VES_CONV2(NK) issue_conv<NK>(d2, a0, b0, (kc1 * lboA) >> 4, (kc1 * lboB) >> 4, (2 * lboA) >> 4, (2 * lboB) >> 4, idesc, (uint32_t)VD)
        VES_TC_NK_SWITCH(kc1 / 2, VES_CONV2)
#undef VES_CONV2
        tc_commit(&bar[wg]);
      }
      if (!group_wait_one(&bar[wg], phase, a.st, 22, wg, gt, &fail[wg])) {
        failed = stuck = true;
        break;
      }
      phase ^= 1;
      tc_fence_after_sync();
      // the intermediate goes straight to global memory: row (kc, p) of
      // vesicle v = t*VD + j sits in its up1 tile (v / v1) at ((kc * L/4 + p) * v1 + v % v1)
      if (KCD != 0 && M2 == 64) {
        // M = 64, the two halves of the chunks on the two half-warps, as above
        if (16 * qd < L4 * VD) {  // uniform per warp
          const int r = 16 * qd + (lane & 15), p = r / VD, j = r - p * VD;
          const long long v = t * VD + j;
          const int V1 = g.v1, kb = (lane >> 4) * (KCD / 2);
          const long long vs = v < a.nv ? v : 0;
          uint4* gmid = reinterpret_cast<uint4*>(a.mid + ((size_t)(vs / V1) * a.G + sg.grp) * (size_t)V1 * g.mid_bytes) +
                        (vs % V1);
          float vv[32];
          tc_ld16x2_32<4 * KCD>(d2 + ((uint32_t)(32 * qd) << 16), vv);
          if (p < L4 && v < a.nv) {
#pragma unroll
            for (int k = 0; k < KCD / 2; ++k)
              gmid[((size_t)(kb + k) * L4 + p) * V1] = act8(vv + 8 * k, cst, kb + k, g.d, 384, 512, 640);
          }
        }
      } else if (acc_row0(M2, qd) < L4 * VD) {
        const int r = acc_row(M2, qd, lane), p = r / VD, j = r - p * VD;
        const long long v = t * VD + j;
        const bool own = r >= 0 && p < L4 && v < a.nv;
        const int V1 = g.v1;
        const long long vs = own ? v : 0;
        uint4* gmid = reinterpret_cast<uint4*>(a.mid + ((size_t)(vs / V1) * a.G + sg.grp) * (size_t)V1 * g.mid_bytes) +
                      (vs % V1);
#pragma unroll
        for (int k0 = 0; k0 < kcd; k0 += 4) {
          float vv[32];
          tc_ld32(d2 + ((uint32_t)(32 * qd) << 16) + 8 * k0, vv);
          if (own) {
#pragma unroll
            for (int k = 0; k < 4; ++k)
              if (k0 + k < kcd)
                gmid[((size_t)(k0 + k) * L4 + p) * V1] = act8(vv + 8 * k, cst, k0 + k, g.d, 384, 512, 640);
          }
        }
      }
      tc_fence_before_sync();
      group_sync(wg);  // every TMEM read done before the next item's MMAs
    }
    lo = sg.hi;
    failed = __syncthreads_or(failed ? 1 : 0) != 0;  // every thread takes part
  }
  // bounded drains: this group's MMAs and bulk copies still in flight after a failure
  if (stuck) tc_mbar_wait(&bar[wg], phase, nullptr, 0);
  if (xpend) tc_mbar_wait(&xbar[wg], xphase, nullptr, 0);
  tc_fence_before_sync();
  __syncthreads();
  if (warp == 0) tc_tmem_dealloc(tbase, ncols);
}

// ---------------------------------------------------------------------------
// ---------------------------------------------------------------------------
// The transposed convolutions, split in two kernels so that their weight
// images and per-group arrays are small enough for more warp groups per SM:
//   up1: transposed conv 1 (intermediate [kcd][L/4] -> [kcd][L/2], BF16 rows
//        to global memory);
//   up2: transposed conv 2, mix, residual and pass-through channels.
// Both M-split a transposed conv when its two output parities fit in 128
// lanes (2*npos <= 128): parity r's operand starts r*npos rows early, so its
// valid rows land on lanes [r*npos, (r+1)*npos) and every warp has epilogue
// work; otherwise both parities share one MMA of N = 2*Nd (merged image) or
// run as two MMAs on the same lanes.  Parity r accumulates in TMEM columns
// [r*Nd, (r+1)*Nd) either way.

// Issue one transposed conv (thread 0 of the group).  w0/w1: byte offsets of
// parity 0/1 weights (tap 0, chunk 0, row 0), bTap: tap stride (16-byte
// units), lboB: K-chunk stride of B in bytes, merged: both parities in one
// operand of N = 2*Nd rows at w0.
template <int KCD>
__device__ __forceinline__ void deconv_issue(uint32_t dt, uint32_t sbase, uint32_t a_off, uint32_t lboA, int npos,
                                             int Nd, int kcd, bool merged, uint32_t w0, uint32_t w1, uint32_t bTap,
                                             uint32_t lboB, bool allow_split = true, int Mrows = 128,
                                             uint32_t tapRows = 1) {
  const bool msplit = allow_split && 2 * npos <= 128;
  const uint32_t stepA = (2 * lboA) >> 4;
  if (merged && !msplit) {
    const uint32_t idesc = tc_idesc_bf16(Mrows, 2 * Nd);
    const uint64_t a0 = tc_desc(sbase + a_off, lboA, 128), b0 = tc_desc(sbase + w0, lboB, 128);
#define VES_DEC(NK) issue_deconv<NK>(dt, a0, b0, bTap, stepA, (2 * lboB) >> 4, idesc, tapRows)
    VES_TC_NK_SWITCH(kcd / 2, VES_DEC)
#undef VES_DEC
  } else {
    const uint32_t idesc = tc_idesc_bf16(128, Nd);
    for (int r = 0; r < 2; ++r) {
      const int lift = msplit ? r * npos * 16 : 0;
      const uint64_t a0 = tc_desc(sbase + a_off - lift, lboA, 128);
      const uint64_t b0 = tc_desc(sbase + (r ? w1 : w0), lboB, 128);
#define VES_DEC(NK) issue_deconv<NK>(dt + r * Nd, a0, b0, bTap, stepA, (2 * lboB) >> 4, idesc, tapRows)
      VES_TC_NK_SWITCH(kcd / 2, VES_DEC)
#undef VES_DEC
    }
  }
}

// Epilogue of a transposed conv over npos input rows: 8 channels of output
// position 2q + r for this thread's lane go to dst[kc * pitch + 2q + r + row0].
template <int KCD>
__device__ __forceinline__ void deconv_epilogue(uint32_t dt, int qd, int lane, int npos, int Nd, int kcd, int nreal,
                                                const float* cst, int ob, int os, int ot, uint4* dst, int pitch,
                                                int row0, bool allow_split = true, int Mrows = 128) {
  const bool msplit = allow_split && 2 * npos <= 128;
  const int lane0 = 32 * qd;
  if (!msplit) {
    // both parities on this lane: one wait for the two parities' columns
    if (acc_row0(Mrows, qd) >= npos) return;  // uniform per warp
    const int q = acc_row(Mrows, qd, lane);
    const bool own = q >= 0 && q < npos;
#pragma unroll
    for (int k0 = 0; k0 < (KCD ? KCD : 8); k0 += 4) {
      if (k0 >= kcd) break;
      float vv[64];
      tc_ld32x2(dt + ((uint32_t)lane0 << 16) + 8 * k0, dt + ((uint32_t)lane0 << 16) + Nd + 8 * k0, vv);
      if (own) {
#pragma unroll
        for (int r = 0; r < 2; ++r)
#pragma unroll
          for (int k = 0; k < 4; ++k)
            if (k0 + k < kcd)
              dst[(size_t)(k0 + k) * pitch + 2 * q + r + row0] = act8(vv + 32 * r + 8 * k, cst, k0 + k, nreal, ob, os, ot);
      }
    }
    return;
  }
#pragma unroll
  for (int r = 0; r < 2; ++r) {
    int q;
    bool own = true;
    if (msplit) {
      if (lane0 < r * npos || lane0 >= (r + 1) * npos) continue;  // uniform per warp
      q = lane0 + lane - r * npos;
    } else {
      if (acc_row0(Mrows, qd) >= npos) continue;  // uniform per warp
      q = acc_row(Mrows, qd, lane);
      own = q >= 0 && q < npos;
    }
#pragma unroll
    for (int k0 = 0; k0 < (KCD ? KCD : 8); k0 += 4) {
      if (k0 >= kcd) break;
      float vv[32];
      tc_ld32(dt + ((uint32_t)lane0 << 16) + r * Nd + 8 * k0, vv);
      if (own) {
#pragma unroll
        for (int k = 0; k < 4; ++k)
          if (k0 + k < kcd)
            dst[(size_t)(k0 + k) * pitch + 2 * q + r + row0] = act8(vv + 8 * k, cst, k0 + k, nreal, ob, os, ot);
      }
    }
  }
}

// up1: transposed conv 1 on tiles of v1 vesicles with interleaved rows
// (M = v1 * L/4 = 128), both output parities in one MMA of N = 2*Nd (merged
// image) or two MMAs on the same lanes.  KCD compile-time K chunk count (0:
// from the geometry); NG warp groups (TMEM columns [128*wg, 128*wg + 2*Nd)
// each).  Items are (group, tile) pairs, a.per_grp tiles per group.
template <int KCD, int NG>
__global__ void __launch_bounds__(NG * kGroupThreads, 1) up1_kernel(KArgs a) {
  extern __shared__ __align__(128) unsigned char sm[];
  __shared__ uint64_t bar[NG], mbar[NG];  // per warp group: MMA completion, intermediate arrival
  __shared__ uint32_t tbase;
  __shared__ int fail[NG];
  const Geo& g = a.g;
  const int kcd = KCD ? KCD : g.kcd;
  const int L = g.L, L2 = L / 2, L4 = L / 4, V1 = g.v1;
  const int ntiles = a.per_grp;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int wg = tid / kGroupThreads, gt = tid % kGroupThreads;
  const int qd = warp & 3;
  const Range rg = my_items(a.items);
  if (rg.lo >= rg.hi) return;
  const uint32_t ncols = 512;
  if (tid == 0) {
    for (int k = 0; k < NG; ++k) {
      tc_mbar_init(&bar[k], 1);
      tc_mbar_init(&mbar[k], 1);
      fail[k] = 0;
    }
    tc_mbar_fence_init();
  }
  if (warp == 0) tc_tmem_alloc(&tbase, ncols);
  zero16(sm + g.u1bs, NG * g.u1grp + 128 * 16);  // halos and K padding stay zero
  tc_fence_async_smem();
  tc_fence_before_sync();
  __syncthreads();
  tc_fence_after_sync();
  const uint32_t dt = tbase + 128 * wg;
  const uint32_t sbase = tc_smem_u32(sm);
  const float* cst = reinterpret_cast<const float*>(sm + g.u1cst);
  const int PB = (L4 + 4) * V1;  // rows per K chunk: 2*v1 zero rows, the tile's L4*v1 rows, 2*v1 zero rows
  const int Nd = kcd * 8;
  const uint32_t chunk = (uint32_t)(L4 * V1 * 16);  // bytes of one K chunk of a tile
  uint4* bs = reinterpret_cast<uint4*>(sm + g.u1bs + wg * g.u1grp);
  const uint32_t bTap = (uint32_t)((g.u1merge ? 2 * Nd : g.d) * kcd * 16) >> 4;
  const uint32_t lboB1 = (uint32_t)((g.u1merge ? 2 * Nd : g.d) * 16);
  const uint32_t w1 = g.u1merge ? (uint32_t)(g.u1w + Nd * 16) : (uint32_t)(g.u1w + 5 * kcd * g.d * 16);
  // this thread's accumulator row: position q of the tile's vesicle j
  const int row = 32 * qd + lane, q = row / V1, j = row % V1;
  unsigned phase = 0, mphase = 0;
  bool mpend = false;  // a bulk copy into bs is in flight
  // intermediate of a tile [kcd][L/4 * v1][16B] -> bs rows 2*v1 .. (L/4 + 2)*v1 - 1 of each chunk
  auto fetch_mid = [&](long long item) {
    if (gt == 0) {
      const int grp = (int)(item / ntiles);
      const long long t = item % ntiles;
      const unsigned char* src = a.mid + ((size_t)t * a.G + grp) * (size_t)V1 * g.mid_bytes;
      tc_expect_tx(&mbar[wg], chunk * (uint32_t)kcd);
      for (int kc = 0; kc < kcd; ++kc) tc_bulk_g2s(bs + kc * PB + 2 * V1, src + (size_t)kc * chunk, chunk, &mbar[wg]);
    }
    mpend = true;
  };
  bool failed = false, stuck = false;
  for (long long lo = rg.lo; lo < rg.hi && !failed;) {
    const Seg sg = next_seg(lo, rg.hi, ntiles);
    __syncthreads();
    copy16(sm, a.img + (size_t)sg.grp * g.u1size, g.u1size);
    tc_fence_async_smem();
    __syncthreads();
    if (sg.lo + wg < sg.hi) fetch_mid(sg.lo + wg);
    for (long long it = sg.lo + wg; it < sg.hi; it += NG) {
      const long long t = it % ntiles;
      if (!group_wait_one(&mbar[wg], mphase, a.st, 26, wg, gt, &fail[wg])) {
        failed = true;
        break;
      }
      mphase ^= 1;
      mpend = false;
      tc_fence_after_sync();
      if (gt == 0) {
        deconv_issue<KCD>(dt, sbase, g.u1bs + wg * g.u1grp, PB * 16, 128, Nd, kcd, g.u1merge != 0, g.u1w, w1, bTap,
                          lboB1, false, 128, (uint32_t)V1);
        tc_commit(&bar[wg]);
      }
      if (!group_wait_one(&bar[wg], phase, a.st, 23, wg, gt, &fail[wg])) {
        failed = stuck = true;
        break;
      }
      phase ^= 1;
      tc_fence_after_sync();
      // bs is free once the MMAs have completed: this group's next item
      if (it + NG < sg.hi) fetch_mid(it + NG);
      // output positions 2q + r of vesicle t*v1 + j -> its up1 -> up2 record
      const long long v = t * V1 + j;
      const bool own = v < a.nv;
      uint4* dst = reinterpret_cast<uint4*>(a.mid2 + ((size_t)(own ? v : 0) * a.G + sg.grp) * g.mid2_bytes);
#pragma unroll
      for (int r = 0; r < 2; ++r) {
#pragma unroll
        for (int k0 = 0; k0 < (KCD ? KCD : 8); k0 += 4) {
          if (k0 >= kcd) break;
          float vv[32];
          tc_ld32(dt + ((uint32_t)(32 * qd) << 16) + r * Nd + 8 * k0, vv);
          if (own) {
#pragma unroll
            for (int k = 0; k < 4; ++k)
              if (k0 + k < kcd)
                dst[(size_t)(k0 + k) * L2 + 2 * q + r] = act8(vv + 8 * k, cst, k0 + k, g.d, 0, 128, 256);
          }
        }
      }
      tc_fence_before_sync();
      group_sync(wg);  // every TMEM read done before the next item's MMAs
    }
    lo = sg.hi;
    failed = __syncthreads_or(failed ? 1 : 0) != 0;  // every thread takes part
  }
  if (stuck) tc_mbar_wait(&bar[wg], phase, nullptr, 0);
  if (mpend) tc_mbar_wait(&mbar[wg], mphase, nullptr, 0);
  tc_fence_before_sync();
  __syncthreads();
  if (warp == 0) tc_tmem_dealloc(tbase, ncols);
}

// up2: transposed conv 2, mix, residual and pass-through.  NG warp groups,
// TMEM columns [cstride*wg, cstride*wg + 2*Nd + nh*Nm) each.
template <int KCD, int NG>
__global__ void __launch_bounds__(NG * kGroupThreads, 1) up2_kernel(KArgs a) {
  extern __shared__ __align__(128) unsigned char sm[];
  __shared__ uint64_t bar[NG], mbar[NG], rbar[NG];  // per warp group: MMA completion, intermediate, block input
  __shared__ uint32_t tbase;
  __shared__ int fail[NG];
  const Geo& g = a.g;
  const int kcd = KCD ? KCD : g.kcd;
  const int L = g.L, L2 = L / 2;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int wg = tid / kGroupThreads, gt = tid % kGroupThreads;
  const int qd = warp & 3;
  const Range rg = my_items(a.items);
  if (rg.lo >= rg.hi) return;
  const uint32_t ncols = 512;
  if (tid == 0) {
    for (int k = 0; k < NG; ++k) {
      tc_mbar_init(&bar[k], 1);
      tc_mbar_init(&mbar[k], 1);
      tc_mbar_init(&rbar[k], 1);
      fail[k] = 0;
    }
    tc_mbar_fence_init();
  }
  if (warp == 0) tc_tmem_alloc(&tbase, ncols);
  zero16(sm + g.u2cs, NG * g.u2grp + 128 * 16);  // halos and K padding stay zero
  tc_fence_async_smem();
  tc_fence_before_sync();
  __syncthreads();
  tc_fence_after_sync();
  const uint32_t dt = tbase + (NG == 2 ? 256 : 160) * wg;
  const uint32_t sbase = tc_smem_u32(sm);
  const int goff = wg * g.u2grp;
  const float* cst = reinterpret_cast<const float*>(sm + g.u2cst);
  const int PC = L2 + 4, PD = L + 2;
  const int Nd = kcd * 8, Nm = rup(g.cmix, 16);
  const int cout = g.cmix + g.npass;
  const int nh = L / 128;   // 128-position halves of the mix
  const int mcol = 2 * Nd;  // first TMEM column of the mix accumulators (after the transposed conv's)
  uint4* cs = reinterpret_cast<uint4*>(sm + g.u2cs + goff);
  uint4* ds = reinterpret_cast<uint4*>(sm + g.u2ds + goff);
  const float* xf = reinterpret_cast<const float*>(ds);  // block input while it sits in ds
  const bool need_x = g.residual || g.npass > 0;
  // transposed conv of at most 64 input positions on the merged image: one
  // M = 64 MMA per (tap, K step) with both parities on N
  const bool m64dec = KCD != 0 && g.u2merge && L2 <= 64;
  const uint32_t xbytes = (uint32_t)(g.cin * L * 4);
  const uint32_t bTap = (uint32_t)((g.u2merge ? 2 * Nd : g.d) * kcd * 16) >> 4;
  const uint32_t lboB = (uint32_t)((g.u2merge ? 2 * Nd : g.d) * 16);
  const uint32_t w1 = g.u2merge ? (uint32_t)(g.u2w + Nd * 16) : (uint32_t)(g.u2w + 5 * kcd * g.d * 16);
  unsigned phase = 0, mphase = 0, rphase = 0;
  bool mpend = false, rpend = false;  // bulk copies into cs / ds in flight
  // up1 output [kcd][L/2][16B] of an item -> cs rows 2 .. L/2+1 of each chunk
  auto fetch_mid = [&](long long item) {
    if (gt == 0) {
      const int grp = (int)(item / a.nv);
      const long long v = item % a.nv;
      const unsigned char* src = a.mid2 + ((size_t)v * a.G + grp) * g.mid2_bytes;
      tc_expect_tx(&mbar[wg], (uint32_t)g.mid2_bytes);
      for (int kc = 0; kc < kcd; ++kc) tc_bulk_g2s(cs + kc * PC + 2, src + kc * L2 * 16, L2 * 16, &mbar[wg]);
    }
    mpend = true;
  };
  // block input x[v][grp*cin + c][pos] of an item -> ds (free once the
  // group's previous mix has completed)
  auto fetch_x = [&](long long item) {
    if (gt == 0) {
      const int grp = (int)(item / a.nv);
      const long long v = item % a.nv;
      tc_expect_tx(&rbar[wg], xbytes);
      tc_bulk_g2s(ds, a.x + ((long long)v * a.G + grp) * (long long)g.cin * L, xbytes, &rbar[wg]);
    }
    rpend = true;
  };
  bool failed = false, stuck = false;
  for (long long lo = rg.lo; lo < rg.hi && !failed;) {
    const Seg sg = next_seg(lo, rg.hi, a.nv);
    __syncthreads();
    copy16(sm, a.img + (size_t)sg.grp * g.u2size, g.u2size);
    tc_fence_async_smem();
    __syncthreads();
    if (sg.lo + wg < sg.hi) {
      fetch_mid(sg.lo + wg);
      if (need_x) fetch_x(sg.lo + wg);
    }
    for (long long it = sg.lo + wg; it < sg.hi; it += NG) {
      const long long v = it % a.nv;
      float* __restrict__ op = a.out + ((long long)v * a.G + sg.grp) * (long long)cout * L;
      if (need_x) {
        if (!group_wait_one(&rbar[wg], rphase, a.st, 27, wg, gt, &fail[wg])) {
          failed = true;
          break;
        }
        rphase ^= 1;
        rpend = false;
        // pass-through channels
        const float4* src = reinterpret_cast<const float4*>(xf + (size_t)(g.cin - g.npass) * L);
        float4* dst = reinterpret_cast<float4*>(op + (size_t)g.cmix * L);
        for (int i = gt; i < g.npass * L / 4; i += kGroupThreads) dst[i] = src[i];
      }
      {
        // mix accumulators preset to residual + bias (columns [mcol, mcol + nh*Nm))
        const int p0 = 32 * qd + lane;
        for (int h = 0; h < nh; ++h) {
          float r0[32];
#pragma unroll
          for (int o = 0; o < 32; ++o) {
            const bool on = o < g.cmix;
            r0[o] = (on && g.residual ? xf[o * L + 128 * h + p0] : 0.f) + (on ? cst[768 + o] : 0.f);
          }
          tc_st32(dt + ((uint32_t)(32 * qd) << 16) + mcol + h * Nm, r0);
        }
        tc_wait_st();
      }
      if (!group_wait_one(&mbar[wg], mphase, a.st, 26, wg, gt, &fail[wg])) {
        failed = true;
        break;
      }
      mphase ^= 1;
      mpend = false;
      group_sync_for_mma(wg);  // also: every read of the block input in ds is done
      if (gt == 0) {
        deconv_issue<KCD>(dt, sbase, g.u2cs + goff, PC * 16, L2, Nd, kcd, g.u2merge != 0, g.u2w, w1, bTap, lboB,
                          !m64dec, m64dec ? 64 : 128);
        tc_commit(&bar[wg]);
      }
      if (!group_wait_one(&bar[wg], phase, a.st, 24, wg, gt, &fail[wg])) {
        failed = stuck = true;
        break;
      }
      phase ^= 1;
      tc_fence_after_sync();
      // cs is free once the transposed conv has completed: this group's next item
      if (it + NG < sg.hi) fetch_mid(it + NG);
      if (m64dec) {
        // M = 64 rows (input positions q), parity r = lane / 16 at TMEM columns r*Nd (16x32bx2 loads)
        const int q = 16 * qd + (lane & 15), r = lane >> 4;
#pragma unroll
        for (int k0 = 0; k0 < (KCD ? KCD : 8); k0 += 4) {
          float vv[32];
          tc_ld16x2_32<(KCD ? KCD : 8) * 8>(dt + ((uint32_t)(32 * qd) << 16) + 8 * k0, vv);
#pragma unroll
          for (int k = 0; k < 4; ++k)
            if (k0 + k < kcd) ds[(size_t)(k0 + k) * PD + 2 * q + r + 1] = act8(vv + 8 * k, cst, k0 + k, g.d, 384, 512, 640);
        }
      } else {
        deconv_epilogue<KCD>(dt, qd, lane, L2, Nd, kcd, g.d, cst, 384, 512, 640, ds, PD, 1);
      }
      // the halo rows of ds (zero padding of the mix) held block input
      if (gt < 2 * kcd) ds[(gt >> 1) * PD + ((gt & 1) ? L + 1 : 0)] = make_uint4(0, 0, 0, 0);
      group_sync_for_mma(wg);
      // mix: D[p][o] = sum_t d[p + t - 1] M_t; positions in halves of 128 rows
      if (gt == 0) {
        const uint32_t idesc = tc_idesc_bf16(128, Nm);
        const uint32_t lboA = PD * 16, lboM = g.cmix * 16;
        const uint64_t a0 = tc_desc(sbase + g.u2ds + goff, lboA, 128), b0 = tc_desc(sbase + g.u2wm, lboM, 128);
        for (int h = 0; h < nh; ++h) {  // onto residual + bias
#define VES_MIX(NK) issue_mix<NK>(dt + mcol + h * Nm, a0 + (uint32_t)(128 * h), b0, (kcd * lboM) >> 4, (2 * lboA) >> 4, (2 * lboM) >> 4, idesc)
          VES_TC_NK_SWITCH(kcd / 2, VES_MIX)
#undef VES_MIX
        }
        tc_commit(&bar[wg]);
      }
      if (!group_wait_one(&bar[wg], phase, a.st, 25, wg, gt, &fail[wg])) {
        failed = stuck = true;
        break;
      }
      phase ^= 1;
      tc_fence_after_sync();
      // ds is free once the mix has completed: the block input of this group's next item
      if (need_x && it + NG < sg.hi) fetch_x(it + NG);
      if (nh == 2) {  // both 128-position halves, one wait
        const int p = 32 * qd + lane;
        float vv[64];
        tc_ld32x2(dt + ((uint32_t)(32 * qd) << 16) + mcol, dt + ((uint32_t)(32 * qd) << 16) + mcol + Nm, vv);
#pragma unroll
        for (int o = 0; o < 32; ++o)
          if (o < g.cmix) {
            op[(size_t)o * L + p] = vv[o];
            op[(size_t)o * L + 128 + p] = vv[32 + o];
          }
      } else {
        for (int h = 0; h < nh; ++h) {
          const int p = 128 * h + 32 * qd + lane;
          float vv[32];
          tc_ld32(dt + ((uint32_t)(32 * qd) << 16) + mcol + h * Nm, vv);
#pragma unroll
          for (int o = 0; o < 32; ++o)
            if (o < g.cmix) op[(size_t)o * L + p] = vv[o];
        }
      }
      tc_fence_before_sync();
      group_sync(wg);
    }
    lo = sg.hi;
    failed = __syncthreads_or(failed ? 1 : 0) != 0;  // every thread takes part
  }
  // bounded drains: this group's MMAs and bulk copies still in flight after a failure
  if (stuck) tc_mbar_wait(&bar[wg], phase, nullptr, 0);
  if (mpend) tc_mbar_wait(&mbar[wg], mphase, nullptr, 0);
  if (rpend) tc_mbar_wait(&rbar[wg], rphase, nullptr, 0);
  tc_fence_before_sync();
  __syncthreads();
  if (warp == 0) tc_tmem_dealloc(tbase, ncols);
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
               std::vector<unsigned char>& up1, std::vector<unsigned char>& up2, TcBlock& out) {
  using namespace tcnet;
  const Geo g = make_geo(b, L);
  static_assert(sizeof(Geo) <= sizeof(out.geo), "geometry record too large");
  out.geo_bytes = sizeof(Geo);
  memcpy(out.geo, &g, sizeof(Geo));
  out.dsize = g.dsize;
  out.u1size = g.u1size;
  out.u2size = g.u2size;
  out.mid_bytes = g.mid_stride;
  // TMEM per warp group with two groups (256 columns each): N1 + N2 (down),
  // 2 * Nd (up1) and 2 * Nd + the mix halves (up2); the mix epilogue reads 32
  // columns; each lane quarter holds 32 whole positions; every kernel fits
  // two warp groups in shared memory
  if (g.n1 > 128 || g.d > 128 || g.cmix > 32 || 2 * g.kcd * 8 + (L / 128) * rup(g.cmix, 16) > 256 ||
      g.dxs + 2 * g.dgrp + kTail > kMaxSmem || g.u1size + 2 * g.u1grp + kTail > kMaxSmem ||
      g.u2size + 2 * g.u2grp + kTail > kMaxSmem || L > 256 || (L / 4) % 32 != 0)
    return VES_ERR_ARG;
  const int c1 = b.c1, c2 = b.c2, d = g.d, cin = b.cin, cmix = b.cmix;
  down.assign((size_t)g.dsize * G, 0);
  up1.assign((size_t)g.u1size * G, 0);
  up2.assign((size_t)g.u2size * G, 0);
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
    unsigned char* U1 = up1.data() + (size_t)grp * g.u1size;
    unsigned char* U2 = up2.data() + (size_t)grp * g.u2size;
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
      for (int r = 0; r < 2; ++r)
        for (int u = 0; u < 5; ++u)
          for (int kc = 0; kc < g.kcd; ++kc)
            for (int o = 0; o < d; ++o) {
              for (int e = 0; e < 8; ++e) {
                const int c = kc * 8 + e;
                v8[e] = c < d ? W[((size_t)(grp * d + c) * d + o) * 10 + r + 2 * u] : 0.f;
              }
              if (layer == 0)
                put_row(U1, g.u1merge ? dec_w_off_merged(g, g.u1w, r, u, kc, o) : dec_w_off(g, g.u1w, r, u, kc, o),
                        v8);
              else if (g.u2merge)
                put_row(U2, dec_w_off_merged(g, g.u2w, r, u, kc, o), v8);
              else
                put_row(U2, dec_w_off(g, g.u2w, r, u, kc, o), v8);
            }
    }
    for (int t = 0; t < 3; ++t)
      for (int kc = 0; kc < g.kcd; ++kc)
        for (int o = 0; o < cmix; ++o) {
          for (int e = 0; e < 8; ++e) {
            const int c = kc * 8 + e;
            v8[e] = c < d ? p[12][((size_t)(grp * cmix + o) * d + c) * 3 + t] : 0.f;
          }
          put_row(U2, g.u2wm + ((size_t)(t * g.kcd + kc) * cmix + o) * 16, v8);
        }
    float* uc = reinterpret_cast<float*>(U1 + g.u1cst);
    for (int o = 0; o < d; ++o) {
      uc[o] = p[9][grp * d + o];
      bn(2, grp * d + o, &uc[128 + o], &uc[256 + o]);
      uc[384 + o] = p[11][grp * d + o];
      bn(3, grp * d + o, &uc[512 + o], &uc[640 + o]);
    }
    for (int o = 0; o < cmix; ++o) uc[768 + o] = p[13][grp * cmix + o];
    memcpy(U2 + g.u2cst, U1 + g.u1cst, 7 * 128 * 4);  // both up kernels carry the full constants block
  }
  return VES_OK;
}

// Warp groups allowed in the down kernel (VES_TC_DOWN_GROUPS=2 or 3 caps
// them; read once).
static int tcnet_down_groups_max() {
  static int v = -1;
  if (v < 0) {
    const char* e = getenv("VES_TC_DOWN_GROUPS");
    const int k = e ? atoi(e) : 4;
    v = (k == 2 || k == 3) ? k : 4;
  }
  return v;
}

namespace {

// compiled chunk-count variants; others run the generic kernels
void (*pick_down(int kc1, int kcd, int ng))(tcnet::KArgs) {
  using namespace tcnet;
#define VES_DK(A, B) return ng == 4 ? down_kernel<A, B, 4> : (ng == 3 ? down_kernel<A, B, 3> : down_kernel<A, B, 2>)
  if (kc1 == 4 && kcd == 6) VES_DK(4, 6);
  if (kc1 == 6 && kcd == 6) VES_DK(6, 6);
  if (kc1 == 6 && kcd == 8) VES_DK(6, 8);
  if (kc1 == 8 && kcd == 8) VES_DK(8, 8);
  VES_DK(0, 0);
#undef VES_DK
}

void (*pick_up1(int kcd, int ng))(tcnet::KArgs) {
  using namespace tcnet;
  if (kcd == 6) return ng == 4 ? up1_kernel<6, 4> : up1_kernel<6, 2>;
  if (kcd == 8) return ng == 4 ? up1_kernel<8, 4> : up1_kernel<8, 2>;
  return ng == 4 ? up1_kernel<0, 4> : up1_kernel<0, 2>;
}

void (*pick_up2(int kcd, int ng))(tcnet::KArgs) {
  using namespace tcnet;
  if (kcd == 6) return ng == 3 ? up2_kernel<6, 3> : up2_kernel<6, 2>;
  if (kcd == 8) return ng == 3 ? up2_kernel<8, 3> : up2_kernel<8, 2>;
  return ng == 3 ? up2_kernel<0, 3> : up2_kernel<0, 2>;
}

bool autotune_log() {
  static int v = -1;
  if (v < 0) {
    const char* e = getenv("VES_TC_AUTOTUNE_LOG");
    v = (e && atoi(e)) ? 1 : 0;
  }
  return v != 0;
}

}  // namespace

int tcnet_run_block(const TcBlock& tb, int G, int nv, const unsigned char* d_down, const unsigned char* d_up1,
                    const unsigned char* d_up2, const float* x, float* out, unsigned char* mid, VesDeviceStatus* st,
                    cudaStream_t s, bool autotune) {
  using namespace tcnet;
  // the block input and the intermediates are fetched by 16-byte bulk copies
  if ((reinterpret_cast<uintptr_t>(x) | reinterpret_cast<uintptr_t>(mid)) & 15u) {
    ves_record_error(VES_ERR_ARG, "net_forward: input and workspace must be 16-byte aligned");
    return VES_ERR_ARG;
  }
  KArgs a;
  memcpy(&a.g, tb.geo, sizeof(Geo));
  const Geo& g = a.g;
  a.G = G;
  a.nv = nv;
  a.m64 = 0;
  a.items = (long long)G * nv;
  a.x = x;
  a.out = out;
  a.per_grp = nv;
  const int ntiles = (nv + g.v1 - 1) / g.v1;
  a.mid = mid;
  a.mid2 = mid + (size_t)ntiles * G * g.v1 * g.mid_bytes;
  a.st = st;
  int dev = 0, nsm = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  const int kc1 = g.kc1, kcd = g.kcd, Nd = kcd * 8;
  // warp groups per CTA that fit: TMEM (512 columns) and shared memory
  const int down3 = g.dxs + 3 * g.dgrp + kTail, down4 = g.dxs + 4 * g.dgrp + kTail,
            up1_4 = g.u1size + 4 * g.u1grp + kTail, up2_3 = g.u2size + 3 * g.u2grp + kTail;
  const bool dn3 = (kc1 + kcd) * 8 <= 128 && down3 <= kMaxSmem;
  const bool dn4 = dn3 && down4 <= kMaxSmem;
  const bool u14 = 2 * Nd <= 128 && up1_4 <= kMaxSmem;
  const bool u23 = 2 * Nd + (g.L / 128) * rup(g.cmix, 16) <= 160 && up2_3 <= kMaxSmem;
  const int grid = (int)std::min<long long>(a.items, (long long)nsm);
  // one CTA per SM (it allocates all 512 TMEM columns): at least 117 KB of
  // shared memory per CTA keeps a second one off the SM
  auto launch = [&](int which, int ng, int m64) -> int {
    KArgs b = a;
    b.m64 = m64;
    void (*fn)(KArgs);
    int smem;
    int nblk = grid;
    if (which == 0) {
      fn = pick_down(kc1, kcd, ng);
      smem = std::max(g.dxs + ng * g.dgrp + kTail, kMinSmem);
      b.img = d_down;
      b.per_grp = (nv + g.vd - 1) / g.vd;  // items: (group, tile of vd vesicles)
      b.items = (long long)G * b.per_grp;
      nblk = (int)std::min<long long>(b.items, (long long)nsm);
    } else if (which == 1) {
      fn = pick_up1(kcd, ng);
      smem = std::max(g.u1size + ng * g.u1grp + kTail, kMinSmem);
      b.img = d_up1;
      b.per_grp = ntiles;  // items: (group, tile)
      b.items = (long long)G * ntiles;
      nblk = (int)std::min<long long>(b.items, (long long)nsm);
    } else {
      fn = pick_up2(kcd, ng);
      smem = std::max(g.u2size + ng * g.u2grp + kTail, kMinSmem);
      b.img = d_up2;
    }
    int rc = ves_cuda_status(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, smem),
                             "tc smem attribute");
    if (rc) return rc;
    ves_count_launch();
    fn<<<nblk, ng * kGroupThreads, smem, s>>>(b);
    return ves_launch_check("tc net block");
  };
  // the fixed rule: the most warp groups that fit, M = 64 MMAs where allowed
  const int m64_default = tcnet_m64() ? 1 : 0;
  const int dmax = tcnet_down_groups_max();
  TcPlan plan{nv, (dn4 && dmax >= 4) ? 4 : ((dn3 && dmax >= 3) ? 3 : 2), m64_default, u14 ? 4 : 2, m64_default,
              u23 ? 3 : 2};
  const TcPlan* found = nullptr;
  for (const TcPlan& p : tb.plans)
    if (p.nv == nv) found = &p;
  if (found) {
    plan = *found;
  } else if (autotune) {
    cudaEvent_t e0, e1;
    int rc = ves_cuda_status(cudaEventCreate(&e0), "tune event");
    if (!rc) rc = ves_cuda_status(cudaEventCreate(&e1), "tune event");
    if (rc) return rc;
    auto timed = [&](int which, int ng, int m64, float& ms) -> int {
      ms = 1e30f;
      for (int rep = 0; rep < 2; ++rep) {
        int r = ves_cuda_status(cudaEventRecord(e0, s), "tune record");
        if (!r) r = launch(which, ng, m64);
        if (!r) r = ves_cuda_status(cudaEventRecord(e1, s), "tune record");
        if (!r) r = ves_cuda_status(cudaEventSynchronize(e1), "tune sync");
        float t = 0.f;
        if (!r) r = ves_cuda_status(cudaEventElapsedTime(&t, e0, e1), "tune elapsed");
        if (r) return r;
        ms = std::min(ms, t);
      }
      return VES_OK;
    };
    float best = 1e30f, t = 0.f;
    // each kernel in the order the block runs them, so that the next one reads a valid input
    const int ngd[3] = {2, 3, 4};
    for (int i = 0; i < 3 && !rc; ++i) {
      const int ng = ngd[i];
      if ((ng == 3 && !dn3) || (ng == 4 && !dn4)) continue;
      for (int m = 0; m < 2 && !rc; ++m) {
        if ((rc = timed(0, ng, m, t))) break;
        if (t < best) best = t, plan.ng_down = ng, plan.m64_down = m;
      }
    }
    if (!rc) rc = launch(0, plan.ng_down, plan.m64_down);
    best = 1e30f;
    for (int ng = 2; ng <= 4 && !rc; ng += 2) {
      if (ng == 4 && !u14) continue;
      for (int m = 0; m < 1 && !rc; ++m) {
        if ((rc = timed(1, ng, m, t))) break;
        if (t < best) best = t, plan.ng_up1 = ng, plan.m64_up1 = m;
      }
    }
    if (!rc) rc = launch(1, plan.ng_up1, plan.m64_up1);
    best = 1e30f;
    for (int ng = 2; ng <= 3 && !rc; ++ng) {
      if (ng == 3 && !u23) continue;
      if ((rc = timed(2, ng, 0, t))) break;
      if (t < best) best = t, plan.ng_up2 = ng;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (rc) return rc;
    tb.plans.push_back(plan);
    if (autotune_log())
      fprintf(stderr, "tcnet autotune: L=%d kc1=%d kcd=%d nv=%d -> down %d groups m64 %d, up1 %d groups m64 %d, up2 %d groups\n",
              g.L, kc1, kcd, nv, plan.ng_down, plan.m64_down, plan.ng_up1, plan.m64_up1, plan.ng_up2);
  }
  int rc = launch(0, plan.ng_down, plan.m64_down);
  if (!rc) rc = launch(1, plan.ng_up1, plan.m64_up1);
  if (!rc) rc = launch(2, plan.ng_up2, 0);
  return rc;
}
