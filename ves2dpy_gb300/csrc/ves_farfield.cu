// All-pairs Stokeslet sum between vesicles (allExactStokesSLTarget_compare1/2,
// mytorch/biem_support.py:7-272; Poten.exactStokesSL, mytorch/poten.py:280-336):
//
//   u(x_t) = 1/(4 pi) sum_{s != self(t), (t, s) not near} sum_j
//            [ -1/2 log|r|^2 den_j + (r . den_j) r / |r|^2 ],  r = x_t - y_j.
//
// Design (one GB300 SM = 4 SMSPs, FP32 pipe + MUFU):
// * A CTA owns 8 warps x 128 consecutive target points (4 per lane, held in
//   registers for the whole launch) and a contiguous range of source vesicles.
// * Source vesicles are staged into shared memory, whole vesicles at a time,
//   by one elected thread with cp.async.bulk (TMA bulk copy) completing on an
//   mbarrier; two stages are in flight.  Every warp reads each staged source
//   record as a broadcast.
// * FP32C path: coordinates are stored relative to the centre of their own
//   vesicle; for every (target vesicle, source vesicle) pair the centre offset
//   is formed from hi/lo FP32 centres, so r carries no cancellation error from
//   large absolute coordinates.  The log is taken relative to the source
//   centre, log|r|^2 = log(|r|^2/|r_c|^2) + log|r_c|^2, with the second term
//   applied once per pair through the source vesicle's density sum; this
//   removes the cancellation between the log terms of a force-free vesicle.
//   1/|r|^2 and log2 run on the MUFU unit (rcp.approx, lg2.approx).  The
//   partial over one source vesicle is added to a Kahan-compensated total.
// * The whole contribution of a (target point, source vesicle) pair is dropped
//   when the pair is in the near list (biem_support.py:218-219), and the
//   target's own vesicle is skipped.
// * Each CTA writes an FP64 partial for its source range; a fixed-order
//   reduction over the ranges produces the result (deterministic).
#include "ves_internal.h"

namespace {

#ifndef VES_FF_PAIRED_RCP
#define VES_FF_PAIRED_RCP 0
#endif
#ifndef VES_FF_MINB
#define VES_FF_MINB 2  // resident CTAs per SM requested from the register allocator
#endif
constexpr int FF_WARPS = 8;
constexpr int FF_TPL = 4;  // target slots per lane
constexpr int FF_PTS_PER_WARP = 32 * FF_TPL;
constexpr int FF_PTS_PER_CTA = FF_WARPS * FF_PTS_PER_WARP;
constexpr double FF_HALF_LN2 = 0.34657359027997264;  // 0.5*ln(2)

struct __align__(32) Rec64 {
  double x, y, z, w;  // local x, local y, den x, den y (float4 field names)
};

template <typename Real>
struct FFT;
template <>
struct FFT<float> {
  typedef float4 Rec;  // x, y (local), denx, deny
  typedef float2 Pair;
  static __device__ __forceinline__ float rcp(float x) { return mufu_rcp(x); }
  static __device__ __forceinline__ float lg2(float x) { return mufu_lg2(x); }
  static __device__ __forceinline__ Rec rec(float x, float y, float a, float b) { return make_float4(x, y, a, b); }
  static __device__ __forceinline__ Pair pair(float a, float b) { return make_float2(a, b); }
};
template <>
struct FFT<double> {
  typedef Rec64 Rec;
  typedef double2 Pair;
  static __device__ __forceinline__ double rcp(double x) { return 1.0 / x; }
  static __device__ __forceinline__ double lg2(double x) { return log2(x); }
  static __device__ __forceinline__ Rec rec(double x, double y, double a, double b) { return Rec64{x, y, a, b}; }
  static __device__ __forceinline__ Pair pair(double a, double b) { return make_double2(a, b); }
};

// --------------------------------------------------------------------------
// mbarrier / bulk-copy helpers (PTX ISA: mbarrier, cp.async.bulk)
__device__ __forceinline__ unsigned smem_addr(const void* p) { return (unsigned)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t* bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_fence_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
               : "memory");
}
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, unsigned bytes, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
          smem_addr(dst)),
      "l"(src), "r"(bytes), "r"(smem_addr(bar))
      : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, unsigned phase) {
  unsigned ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(smem_addr(bar)), "r"(phase)
      : "memory");
  return ok != 0;
}
// Bounded wait: gives up after a fixed number of polls (each try_wait blocks
// for a hardware-defined interval) and reports VES_ERR_TIMEOUT.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, unsigned phase, VesDeviceStatus* st, int site) {
  for (int it = 0; it < (1 << 22); ++it)
    if (mbar_try_wait(bar, phase)) return true;
  ves_set_error(st, VES_ERR_TIMEOUT, site, (long long)blockIdx.x);
  return false;
}

template <typename Real>
struct FFArgs {
  int nsrc, ns, nt, ntp;
  long long total_pts;
  const typename FFT<Real>::Rec* src;
  const typename FFT<Real>::Pair* src_hi;   // centre, high part
  const typename FFT<Real>::Pair* src_lo;   // centre, low part (0 in FP64)
  const typename FFT<Real>::Pair* src_dsum; // sum of den over the vesicle
  const typename FFT<Real>::Pair* tgt_local;
  const typename FFT<Real>::Pair* tgt_hi;
  const typename FFT<Real>::Pair* tgt_lo;
  const int* self_idx;
  const int* cand_count;
  const int* cand_src;
  const uint32_t* excl_mask;
  int maxc, nwords;
  int sv_per_stage, src_per_split, nsplit;
  double* partial;  // [nsplit][total_pts][2]
  VesDeviceStatus* st;
};

// --------------------------------------------------------------------------
// deterministic block sum of two values (blockDim.x == 256)
__device__ __forceinline__ void block_sum2(double& a, double& b, double (*red)[256]) {
  red[0][threadIdx.x] = a;
  red[1][threadIdx.x] = b;
  __syncthreads();
  for (int w = 128; w > 0; w >>= 1) {
    if (threadIdx.x < w) {
      red[0][threadIdx.x] += red[0][threadIdx.x + w];
      red[1][threadIdx.x] += red[1][threadIdx.x + w];
    }
    __syncthreads();
  }
  a = red[0][0];
  b = red[1][0];
  __syncthreads();
}

// prep of one point set per block: centre = mean of the points, local
// coordinates, and (sources) the density records and density sums.
template <typename Real>
__global__ void __launch_bounds__(256) ff_prep_kernel(int n, const double* __restrict__ X,
                                                      const double* __restrict__ den,
                                                      typename FFT<Real>::Rec* __restrict__ rec,
                                                      typename FFT<Real>::Pair* __restrict__ local,
                                                      typename FFT<Real>::Pair* __restrict__ chi,
                                                      typename FFT<Real>::Pair* __restrict__ clo,
                                                      typename FFT<Real>::Pair* __restrict__ dsum) {
  __shared__ double red[2][256];
  const int k = blockIdx.x;
  const double* x = X + (long long)k * 2 * n;
  double sx = 0, sy = 0;
  for (int j = threadIdx.x; j < n; j += blockDim.x) {
    sx += x[j];
    sy += x[n + j];
  }
  block_sum2(sx, sy, red);
  const double cx = sx / n, cy = sy / n;
  double ax = 0, ay = 0;
  for (int j = threadIdx.x; j < n; j += blockDim.x) {
    const Real lx = (Real)(x[j] - cx), ly = (Real)(x[n + j] - cy);
    if (rec) {
      const Real dx = (Real)den[(long long)k * 2 * n + j], dy = (Real)den[(long long)k * 2 * n + n + j];
      rec[(long long)k * n + j] = FFT<Real>::rec(lx, ly, dx, dy);
      ax += (double)dx;
      ay += (double)dy;
    }
    if (local) local[(long long)k * n + j] = FFT<Real>::pair(lx, ly);
  }
  if (dsum) block_sum2(ax, ay, red);
  if (threadIdx.x == 0) {
    const Real hx = (Real)cx, hy = (Real)cy;
    chi[k] = FFT<Real>::pair(hx, hy);
    clo[k] = FFT<Real>::pair((Real)(cx - (double)hx), (Real)(cy - (double)hy));
    if (dsum) dsum[k] = FFT<Real>::pair((Real)ax, (Real)ay);
  }
}

// --------------------------------------------------------------------------
template <typename Real>
__global__ void __launch_bounds__(FF_WARPS * 32, VES_FF_MINB) ff_main_kernel(FFArgs<Real> p) {
  typedef typename FFT<Real>::Rec Rec;
  typedef typename FFT<Real>::Pair Pair;
  extern __shared__ __align__(128) unsigned char ff_smem[];
  __shared__ __align__(8) uint64_t bars[2];
  const int stage_elems = p.sv_per_stage * p.ns;
  Rec* buf0 = reinterpret_cast<Rec*>(ff_smem);
  Rec* buf1 = buf0 + stage_elems;

  const int warp = threadIdx.x / 32, lane = threadIdx.x % 32;
  const int split = blockIdx.y;
  const int s_begin = split * p.src_per_split;
  const int s_end = min(p.nsrc, s_begin + p.src_per_split);

  // target slots
  long long pt[FF_TPL];
  int col[FF_TPL], pidx[FF_TPL], self[FF_TPL], cur[FF_TPL], cend[FF_TPL];
  bool valid[FF_TPL];
  Pair tl[FF_TPL], thi[FF_TPL], tlo[FF_TPL];
  Real tot_x[FF_TPL], tot_y[FF_TPL], cmp_x[FF_TPL], cmp_y[FF_TPL];
#pragma unroll
  for (int q = 0; q < FF_TPL; ++q) {
    pt[q] = ((long long)blockIdx.x * FF_WARPS + warp) * FF_PTS_PER_WARP + q * 32 + lane;
    valid[q] = pt[q] < p.total_pts;
    const long long pq = valid[q] ? pt[q] : 0;
    col[q] = (int)(pq / p.ntp);
    pidx[q] = (int)(pq % p.ntp);
    self[q] = p.self_idx ? p.self_idx[col[q]] : -1;
    tl[q] = p.tgt_local[pq];
    thi[q] = p.tgt_hi[col[q]];
    tlo[q] = p.tgt_lo[col[q]];
    cur[q] = 0;
    cend[q] = p.cand_count ? min(p.cand_count[col[q]], p.maxc) : 0;
    tot_x[q] = tot_y[q] = cmp_x[q] = cmp_y[q] = Real(0);
  }

  const int nstages = (s_end > s_begin) ? (s_end - s_begin + p.sv_per_stage - 1) / p.sv_per_stage : 0;
  if (threadIdx.x == 0) {
    mbar_init(&bars[0], 1);
    mbar_init(&bars[1], 1);
    mbar_fence_init();
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int st = 0; st < 2 && st < nstages; ++st) {
      const int v0 = s_begin + st * p.sv_per_stage;
      const int nvs = min(p.sv_per_stage, s_end - v0);
      const unsigned bytes = (unsigned)((size_t)nvs * p.ns * sizeof(Rec));
      mbar_arrive_expect_tx(&bars[st], bytes);
      bulk_g2s(st ? buf1 : buf0, p.src + (long long)v0 * p.ns, bytes, &bars[st]);
    }
  }

  int issued = nstages < 2 ? nstages : 2;
  for (int st = 0; st < nstages; ++st) {
    const unsigned phase = (st >> 1) & 1;
    if (!mbar_wait_bounded(&bars[st & 1], phase, p.st, 10)) break;
    const Rec* S = (st & 1) ? buf1 : buf0;
    const int v0 = s_begin + st * p.sv_per_stage;
    const int nvs = min(p.sv_per_stage, s_end - v0);
    for (int v = 0; v < nvs; ++v) {
      const int s = v0 + v;
      const Pair shi = p.src_hi[s], slo = p.src_lo[s], dsum = p.src_dsum[s];
      Real tx[FF_TPL], ty[FF_TPL], irc2[FF_TPL];
      Real acx[FF_TPL], acy[FF_TPL], alx[FF_TPL], aly[FF_TPL];
#pragma unroll
      for (int q = 0; q < FF_TPL; ++q) {
        const Real ox = (thi[q].x - shi.x) + (tlo[q].x - slo.x);
        const Real oy = (thi[q].y - shi.y) + (tlo[q].y - slo.y);
        tx[q] = tl[q].x + ox;
        ty[q] = tl[q].y + oy;
        irc2[q] = FFT<Real>::rcp(tx[q] * tx[q] + ty[q] * ty[q]);
        acx[q] = acy[q] = alx[q] = aly[q] = Real(0);
      }
      const Rec* Sv = S + v * p.ns;
      if (sizeof(Real) == 4 && VES_FF_PAIRED_RCP) {
        // One MUFU reciprocal per two target slots: 1/a = b * rcp(a*b).  The
        // 1e-20 inside the FMA keeps a*b normal when a slot coincides with a
        // source (its own vesicle, whose result is discarded) and is below one
        // ulp of every separated pair's |r|^2.
#pragma unroll 2
        for (int j = 0; j < p.ns; ++j) {
          const Rec r = Sv[j];
#pragma unroll
          for (int q = 0; q < FF_TPL; q += 2) {
            const Real dx0 = tx[q] - r.x, dy0 = ty[q] - r.y;
            const Real dx1 = tx[q + 1] - r.x, dy1 = ty[q + 1] - r.y;
            const Real r20 = fma(dx0, dx0, fma(dy0, dy0, Real(1e-20)));
            const Real r21 = fma(dx1, dx1, fma(dy1, dy1, Real(1e-20)));
            const Real ip = FFT<Real>::rcp(r20 * r21);
            const Real inv0 = r21 * ip, inv1 = r20 * ip;
            const Real lg0 = FFT<Real>::lg2(r20 * irc2[q]);
            const Real lg1 = FFT<Real>::lg2(r21 * irc2[q + 1]);
            const Real cc0 = fma(dx0, r.z, dy0 * r.w) * inv0;
            const Real cc1 = fma(dx1, r.z, dy1 * r.w) * inv1;
            acx[q] = fma(cc0, dx0, acx[q]);
            acy[q] = fma(cc0, dy0, acy[q]);
            alx[q] = fma(lg0, r.z, alx[q]);
            aly[q] = fma(lg0, r.w, aly[q]);
            acx[q + 1] = fma(cc1, dx1, acx[q + 1]);
            acy[q + 1] = fma(cc1, dy1, acy[q + 1]);
            alx[q + 1] = fma(lg1, r.z, alx[q + 1]);
            aly[q + 1] = fma(lg1, r.w, aly[q + 1]);
          }
        }
      } else {
#pragma unroll 2
        for (int j = 0; j < p.ns; ++j) {
          const Rec r = Sv[j];
#pragma unroll
          for (int q = 0; q < FF_TPL; ++q) {
            const Real dx = tx[q] - r.x, dy = ty[q] - r.y;
            const Real r2 = fma(dx, dx, dy * dy);
            const Real inv = FFT<Real>::rcp(r2);
            const Real lg = FFT<Real>::lg2(r2 * irc2[q]);
            const Real cc = fma(dx, r.z, dy * r.w) * inv;
            acx[q] = fma(cc, dx, acx[q]);
            acy[q] = fma(cc, dy, acy[q]);
            alx[q] = fma(lg, r.z, alx[q]);
            aly[q] = fma(lg, r.w, aly[q]);
          }
        }
      }
#pragma unroll
      for (int q = 0; q < FF_TPL; ++q) {
        // near-pair exclusion list: ascending source vesicles per target column
        bool excl = false;
        if (cend[q] > 0) {
          const int* cs = p.cand_src + (long long)col[q] * p.maxc;
          while (cur[q] < cend[q] && cs[cur[q]] < s) ++cur[q];
          if (cur[q] < cend[q] && cs[cur[q]] == s) {
            const uint32_t w = p.excl_mask[((long long)col[q] * p.maxc + cur[q]) * p.nwords + (pidx[q] >> 5)];
            excl = (w >> (pidx[q] & 31)) & 1u;
          }
        }
        if (valid[q] && s != self[q] && !excl) {
          const Real lgc = FFT<Real>::lg2(tx[q] * tx[q] + ty[q] * ty[q]);
          const Real px = acx[q] - Real(FF_HALF_LN2) * fma(lgc, dsum.x, alx[q]);
          const Real py = acy[q] - Real(FF_HALF_LN2) * fma(lgc, dsum.y, aly[q]);
          // Kahan-Babuska (Neumaier) compensated accumulation
          Real t = tot_x[q] + px;
          cmp_x[q] += (fabs(tot_x[q]) >= fabs(px)) ? (tot_x[q] - t) + px : (px - t) + tot_x[q];
          tot_x[q] = t;
          t = tot_y[q] + py;
          cmp_y[q] += (fabs(tot_y[q]) >= fabs(py)) ? (tot_y[q] - t) + py : (py - t) + tot_y[q];
          tot_y[q] = t;
        }
      }
    }
    __syncthreads();
    if (threadIdx.x == 0 && issued < nstages) {
      const int sn = issued;
      const int v0n = s_begin + sn * p.sv_per_stage;
      const int nvn = min(p.sv_per_stage, s_end - v0n);
      const unsigned bytes = (unsigned)((size_t)nvn * p.ns * sizeof(Rec));
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      mbar_arrive_expect_tx(&bars[sn & 1], bytes);
      bulk_g2s((sn & 1) ? buf1 : buf0, p.src + (long long)v0n * p.ns, bytes, &bars[sn & 1]);
    }
    ++issued;
  }
#pragma unroll
  for (int q = 0; q < FF_TPL; ++q) {
    if (!valid[q]) continue;
    double* o = p.partial + ((long long)split * p.total_pts + pt[q]) * 2;
    o[0] = (double)tot_x[q] + (double)cmp_x[q];
    o[1] = (double)tot_y[q] + (double)cmp_y[q];
  }
}

// out[col][c][pidx] = sum over splits (fixed order) / (4 pi)
__global__ void ff_reduce_kernel(long long total_pts, int ntp, int nsplit, const double* __restrict__ partial,
                                 double* __restrict__ out) {
  const long long pt = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (pt >= total_pts) return;
  double sx = 0, sy = 0;
  for (int s = 0; s < nsplit; ++s) {
    sx += partial[((long long)s * total_pts + pt) * 2];
    sy += partial[((long long)s * total_pts + pt) * 2 + 1];
  }
  const long long col = pt / ntp, j = pt % ntp;
  const double scale = 1.0 / (4.0 * VES_PI);
  out[col * 2 * ntp + j] = sx * scale;
  out[col * 2 * ntp + ntp + j] = sy * scale;
}

struct FFPlan {
  int sv_per_stage, nsplit, src_per_split, tgt_blocks;
  size_t smem;
};

template <typename Real>
FFPlan ff_plan(int nsrc, int ns, long long total_pts) {
  FFPlan pl;
  const size_t rec = sizeof(typename FFT<Real>::Rec);
  const size_t stage_budget = sizeof(Real) == 4 ? 24 * 1024 : 48 * 1024;
  pl.sv_per_stage = (int)(stage_budget / (rec * (size_t)ns));
  if (pl.sv_per_stage < 1) pl.sv_per_stage = 1;
  if (pl.sv_per_stage > nsrc) pl.sv_per_stage = nsrc > 0 ? nsrc : 1;
  pl.tgt_blocks = (int)((total_pts + FF_PTS_PER_CTA - 1) / FF_PTS_PER_CTA);
  // aim for >= 8 waves of 152 SMs x 2 CTAs, but keep >= 2 stages per split
  const long long want = 152LL * 2 * 8;
  int nsplit = (int)((want + pl.tgt_blocks - 1) / pl.tgt_blocks);
  const int max_split = (nsrc + 2 * pl.sv_per_stage - 1) / (2 * pl.sv_per_stage);
  if (nsplit > max_split) nsplit = max_split;
  if (nsplit < 1) nsplit = 1;
  int per = (nsrc + nsplit - 1) / nsplit;
  per = ((per + pl.sv_per_stage - 1) / pl.sv_per_stage) * pl.sv_per_stage;
  pl.src_per_split = per > 0 ? per : 1;
  pl.nsplit = (nsrc + pl.src_per_split - 1) / pl.src_per_split;
  if (pl.nsplit < 1) pl.nsplit = 1;
  pl.smem = 2 * (size_t)pl.sv_per_stage * ns * rec;
  return pl;
}

template <typename Real>
int ff_run(const FFEnv& env, int nsrc, int ns, const double* Xsrc, const double* den, int nt, int ntp,
           const double* Xtar, const int* self_idx, const ves_near_lists* nl, double* out, WsCarver& ws,
           cudaStream_t s) {
  typedef typename FFT<Real>::Rec Rec;
  typedef typename FFT<Real>::Pair Pair;
  const long long total_pts = (long long)nt * ntp;
  const FFPlan pl = ff_plan<Real>(nsrc, ns, total_pts);
  Rec* rec = ws.take<Rec>((size_t)nsrc * ns);
  Pair* shi = ws.take<Pair>(nsrc);
  Pair* slo = ws.take<Pair>(nsrc);
  Pair* dsum = ws.take<Pair>(nsrc);
  Pair* tloc = ws.take<Pair>((size_t)total_pts);
  Pair* thi = ws.take<Pair>(nt);
  Pair* tlo = ws.take<Pair>(nt);
  double* partial = ws.take<double>((size_t)pl.nsplit * total_pts * 2);
  if (ws.sizing) return VES_OK;
  if (!ws.ok()) {
    ves_record_error(VES_ERR_WORKSPACE, "farfield: workspace too small");
    return VES_ERR_WORKSPACE;
  }
  if (total_pts == 0) return VES_OK;
  if (nsrc == 0) return ves_cuda_status(cudaMemsetAsync(out, 0, (size_t)total_pts * 2 * sizeof(double), s), "ff zero");
  if (nl && ntp != env.N) {
    ves_record_error(VES_ERR_SHAPE, "farfield: near lists need N target points per column");
    return VES_ERR_SHAPE;
  }
  ves_count_launch();
  ff_prep_kernel<Real><<<nsrc, 256, 0, s>>>(ns, Xsrc, den, rec, nullptr, shi, slo, dsum);
  ves_count_launch();
  ff_prep_kernel<Real><<<nt, 256, 0, s>>>(ntp, Xtar, nullptr, nullptr, tloc, thi, tlo, nullptr);
  FFArgs<Real> a;
  a.nsrc = nsrc;
  a.ns = ns;
  a.nt = nt;
  a.ntp = ntp;
  a.total_pts = total_pts;
  a.src = rec;
  a.src_hi = shi;
  a.src_lo = slo;
  a.src_dsum = dsum;
  a.tgt_local = tloc;
  a.tgt_hi = thi;
  a.tgt_lo = tlo;
  a.self_idx = self_idx;
  a.cand_count = nl ? nl->cand_count : nullptr;
  a.cand_src = nl ? nl->cand_src : nullptr;
  a.excl_mask = nl ? nl->excl_mask : nullptr;
  a.maxc = nl ? nl->maxc : 0;
  a.nwords = (env.N + 31) / 32;
  a.sv_per_stage = pl.sv_per_stage;
  a.src_per_split = pl.src_per_split;
  a.nsplit = pl.nsplit;
  a.partial = partial;
  a.st = env.status;
  if (pl.smem > 32 * 1024) {  // dynamic + static shared memory must fit the opt-in limit
    cudaError_t e = cudaFuncSetAttribute(ff_main_kernel<Real>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)pl.smem);
    if (e != cudaSuccess) return ves_cuda_status(e, "farfield smem attribute");
  }
  dim3 grid(pl.tgt_blocks, pl.nsplit);
  ves_count_launch();
  if (env.timing) ves_ff_timing_begin(env.timing, s);
  ff_main_kernel<Real><<<grid, FF_WARPS * 32, pl.smem, s>>>(a);
  if (env.timing) ves_ff_timing_end(env.timing, s, (double)total_pts * ns * (double)nsrc);
  ves_count_launch();
  ff_reduce_kernel<<<ceil_div(total_pts, 256), 256, 0, s>>>(total_pts, ntp, pl.nsplit, partial, out);
  return ves_launch_check("farfield");
}

}  // namespace

int farfield_run_env(const FFEnv& env, int precision, int nsrc, int ns, const double* Xsrc, const double* den,
                     int nt, int ntp, const double* Xtar, const int* self_idx, const ves_near_lists* nl,
                     double* out, WsCarver& ws, cudaStream_t s) {
  if (precision == VES_PREC_FP64)
    return ff_run<double>(env, nsrc, ns, Xsrc, den, nt, ntp, Xtar, self_idx, nl, out, ws, s);
  if (precision == VES_PREC_FP32C)
    return ff_run<float>(env, nsrc, ns, Xsrc, den, nt, ntp, Xtar, self_idx, nl, out, ws, s);
  if (precision == VES_PREC_FP32M)
    return farfield_mp_run(env, nsrc, ns, Xsrc, den, nt, ntp, Xtar, self_idx, nl, out, ws, s);
  ves_record_error(VES_ERR_ARG, "farfield: bad precision %d", precision);
  return VES_ERR_ARG;
}

int farfield_run(ves_ctx* c, int precision, int nsrc, int ns, const double* Xsrc, const double* den, int nt,
                 int ntp, const double* Xtar, const int* self_idx, const ves_near_lists* nl, double* out,
                 WsCarver& ws, cudaStream_t s) {
  FFEnv env;
  env.status = c ? c->status : nullptr;
  env.N = c ? c->N : ntp;
  env.timing = c;
  if (precision == VES_PREC_FP64 || precision == VES_PREC_FP32C || precision == VES_PREC_FP32M)
    return farfield_run_env(env, precision, nsrc, ns, Xsrc, den, nt, ntp, Xtar, self_idx, nl, out, ws, s);
  ves_record_error(VES_ERR_ARG, "farfield: bad precision %d", precision);
  return VES_ERR_ARG;
}
