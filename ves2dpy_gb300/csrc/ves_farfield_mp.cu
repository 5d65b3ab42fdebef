// All-pairs Stokeslet sum (allExactStokesSLTarget_compare1/2,
// mytorch/biem_support.py:7-272; Poten.exactStokesSL, mytorch/poten.py:280-336)
// evaluated with a multipole expansion of each source vesicle for the
// vesicle pairs that are well separated, and by the direct FP32 sum for the
// others (precision VES_PREC_FP32M).
//
// The sum is the reference's: for a target x and a source vesicle with
// upsampled points w_j and quadrature-weighted densities f_j (complex
// notation, f = fx + i fy),
//
//   u(x) = sum_j [ -1/2 log|r_j|^2 f_j + (r_j . f_j) r_j / |r_j|^2 ],  r_j = x - w_j
//        = sum_j [ -1/2 log|r_j|^2 f_j + 1/2 f_j + 1/2 conj(f_j) r_j / conj(r_j) ].
//
// With the source centre c, v_j = w_j - c, omega = x - c, R >= max |v_j|,
// normalised vt_j = v_j / R and tau = R / omega (|tau| = rho < 1):
//
//   u = -log|omega| F0 + F0/2 + sum_{k>=1} [tau^k A_k + conj(tau)^k B_k] / (2k)
//       + 1/2 (omega / conj(omega)) conj(sum_{k>=0} tau^k A_k)
//       - 1/2 conj(tau sum_{k>=0} tau^k E_k)
//
//   F0 = sum f_j,  A_k = sum f_j vt_j^k,  B_k = sum f_j conj(vt_j)^k,
//   E_k = sum f_j conj(vt_j) vt_j^k
//
// (series of log(1 - v/omega) and 1/(1 - conj(v/omega))).  Truncating at
// order P leaves at most sum_j |f_j| rho^(P+1) / (1 - rho) per series.  A
// (target vesicle, source vesicle) pair uses the expansion when
// rho_pair = R_s / (|c_t - c_s| - R_t) <= kRhoMax, with P the smallest order
// whose bound is below kEps (relative to sum |f_j|); every other pair, every
// pair on the target's near-candidate list (where single target points are
// excluded, biem_support.py:218-219), is summed directly over the
// upsampled points in FP32 with the source-centred logarithm of the FP32C
// path.  The moments are sums over exactly the upsampled points of the direct
// rule (centre, radius and F0 in FP64, the others in FP32, stored in FP32);
// the series are evaluated in FP32 (Horner) and the per-source contributions
// are added with Neumaier compensation.
#include "ves_internal.h"

namespace {

constexpr int kPMax = 24;                 // highest expansion order
constexpr float kRhoMax = 0.35f;          // 0.35^25 / 0.65 < 1e-11
constexpr float kEps = 1e-10f;            // truncation bound relative to sum |f_j|
constexpr int kStage = 16;                // source vesicles per shared-memory stage
constexpr int kDrecChunk = 512;           // direct-rule points per shared-memory stage (8 KB)
constexpr double kHalfLn2 = 0.34657359027997264;

struct __align__(16) MPSrc {
  float2 chi, clo;  // centre, high and low FP32 parts
  float2 f0;        // sum of the density
  float R;          // bound on |w_j - c| over the upsampled points
  float pad;
};

// one order k of one source: Al = A_k/(2k) (0 at k=0), Bc = conj(B_k/(2k)) (0 at k=0), A_k, E_k
struct __align__(16) MPMom {
  float2 al, bc, ac, ec;
};

__device__ __forceinline__ float2 cmulf(float2 a, float2 b) {
  return make_float2(fmaf(a.x, b.x, -a.y * b.y), fmaf(a.x, b.y, a.y * b.x));
}

// ---------------------------------------------------------------------------
// One CTA (256 threads) per source vesicle: centre, FP32 records for the
// direct rule, density sum, radius bound and the normalised moments.
__global__ void __launch_bounds__(256) mp_prep_kernel(int ns, const double* __restrict__ X,
                                                      const double* __restrict__ den, float4* __restrict__ rec,
                                                      MPSrc* __restrict__ src, MPMom* __restrict__ mom) {
  __shared__ double red[3][256];
  const int s = blockIdx.x, t = threadIdx.x;
  const double* x = X + (long long)s * 2 * ns;
  const double* f = den + (long long)s * 2 * ns;
  double sx = 0, sy = 0;
  for (int j = t; j < ns; j += 256) {
    sx += x[j];
    sy += x[ns + j];
  }
  red[0][t] = sx;
  red[1][t] = sy;
  __syncthreads();
  for (int w = 128; w > 0; w >>= 1) {
    if (t < w) {
      red[0][t] += red[0][t + w];
      red[1][t] += red[1][t + w];
    }
    __syncthreads();
  }
  const double cx = red[0][0] / ns, cy = red[1][0] / ns;
  __syncthreads();
  double r2 = 0, fx = 0, fy = 0;
  for (int j = t; j < ns; j += 256) {
    const double lx = x[j] - cx, ly = x[ns + j] - cy;
    rec[(long long)s * ns + j] = make_float4((float)lx, (float)ly, (float)f[j], (float)f[ns + j]);
    r2 = fmax(r2, lx * lx + ly * ly);
    fx += f[j];
    fy += f[ns + j];
  }
  red[0][t] = r2;
  red[1][t] = fx;
  red[2][t] = fy;
  __syncthreads();
  for (int w = 128; w > 0; w >>= 1) {
    if (t < w) {
      red[0][t] = fmax(red[0][t], red[0][t + w]);
      red[1][t] += red[1][t + w];
      red[2][t] += red[2][t + w];
    }
    __syncthreads();
  }
  double R = sqrt(red[0][0]) * (1.0 + 1e-6);
  if (!(R > 0)) R = 1.0;
  if (t == 0) {
    MPSrc o;
    o.chi = make_float2((float)cx, (float)cy);
    o.clo = make_float2((float)(cx - (double)o.chi.x), (float)(cy - (double)o.chi.y));
    o.f0 = make_float2((float)red[1][0], (float)red[2][0]);
    o.R = (float)R;
    o.pad = 0.f;
    src[s] = o;
  }
  // moments: warp w takes orders k = w, w + 8, w + 16, ... (<= kPMax); lanes
  // split the points.  FP32 sums: a moment of order k enters the series
  // multiplied by rho^k and is stored in FP32, so FP32 accumulation (errors
  // of a few 1e-8 of sum |f| |v|^k) matches the storage; the monopole F0 is
  // the FP64 density sum above.
  const int warp = t >> 5, lane = t & 31;
  constexpr int kPer = (kPMax + 8) / 8;  // orders per warp
  float2 A[kPer], B[kPer], E[kPer];
#pragma unroll
  for (int q = 0; q < kPer; ++q) A[q] = B[q] = E[q] = make_float2(0.f, 0.f);
  const double iR = 1.0 / R;
  for (int j = lane; j < ns; j += 32) {
    const float2 v = make_float2((float)((x[j] - cx) * iR), (float)((x[ns + j] - cy) * iR));
    const float2 fj = make_float2((float)f[j], (float)f[ns + j]);
    float2 pw = make_float2(1.f, 0.f), v8 = v;  // pw = v^warp, v8 = v^8
    for (int e = 0; e < warp; ++e) pw = cmulf(pw, v);
    v8 = cmulf(v8, v8);
    v8 = cmulf(v8, v8);
    v8 = cmulf(v8, v8);
    const float2 fvb = cmulf(fj, make_float2(v.x, -v.y));  // f conj(v)
#pragma unroll
    for (int q = 0; q < kPer; ++q) {
      const float2 a = cmulf(fj, pw);
      const float2 b = cmulf(fj, make_float2(pw.x, -pw.y));
      const float2 e = cmulf(fvb, pw);
      A[q].x += a.x;
      A[q].y += a.y;
      B[q].x += b.x;
      B[q].y += b.y;
      E[q].x += e.x;
      E[q].y += e.y;
      pw = cmulf(pw, v8);
    }
  }
#pragma unroll
  for (int q = 0; q < kPer; ++q) {
    for (int o = 16; o > 0; o >>= 1) {
      A[q].x += __shfl_xor_sync(0xffffffffu, A[q].x, o);
      A[q].y += __shfl_xor_sync(0xffffffffu, A[q].y, o);
      B[q].x += __shfl_xor_sync(0xffffffffu, B[q].x, o);
      B[q].y += __shfl_xor_sync(0xffffffffu, B[q].y, o);
      E[q].x += __shfl_xor_sync(0xffffffffu, E[q].x, o);
      E[q].y += __shfl_xor_sync(0xffffffffu, E[q].y, o);
    }
    const int k = warp + 8 * q;
    if (lane == 0 && k <= kPMax) {
      MPMom m;
      const float h = k > 0 ? 0.5f / k : 0.f;
      m.al = make_float2(A[q].x * h, A[q].y * h);
      m.bc = make_float2(B[q].x * h, -B[q].y * h);
      m.ac = k > 0 ? A[q] : make_float2((float)red[1][0], (float)red[2][0]);  // A_0 = F0 (FP64 sum)
      m.ec = E[q];
      mom[(long long)s * (kPMax + 1) + k] = m;
    }
  }
}

// target vesicles: centre (hi/lo) and FP32 local coordinates
__global__ void __launch_bounds__(256) mp_prep_targets_kernel(int ntp, const double* __restrict__ X,
                                                              float2* __restrict__ local, float2* __restrict__ chi,
                                                              float2* __restrict__ clo) {
  __shared__ double red[2][256];
  const int k = blockIdx.x, t = threadIdx.x;
  const double* x = X + (long long)k * 2 * ntp;
  double sx = 0, sy = 0;
  for (int j = t; j < ntp; j += 256) {
    sx += x[j];
    sy += x[ntp + j];
  }
  red[0][t] = sx;
  red[1][t] = sy;
  __syncthreads();
  for (int w = 128; w > 0; w >>= 1) {
    if (t < w) {
      red[0][t] += red[0][t + w];
      red[1][t] += red[1][t + w];
    }
    __syncthreads();
  }
  const double cx = red[0][0] / ntp, cy = red[1][0] / ntp;
  for (int j = t; j < ntp; j += 256) local[(long long)k * ntp + j] = make_float2((float)(x[j] - cx), (float)(x[ntp + j] - cy));
  if (t == 0) {
    const float hx = (float)cx, hy = (float)cy;
    chi[k] = make_float2(hx, hy);
    clo[k] = make_float2((float)(cx - (double)hx), (float)(cy - (double)hy));
  }
}

__device__ __forceinline__ void neumaier(float& tot, float& cmp, float v) {
  const float t = tot + v;
  cmp += (fabsf(tot) >= fabsf(v)) ? (tot - t) + v : (v - t) + tot;
  tot = t;
}

// One source set (the upsampled points of one group of vesicles).
struct MPSet {
  int nsrc, ns;
  const float4* rec;  // [nsrc][ns] direct-rule records
  const MPSrc* src;   // [nsrc]
  const MPMom* mom;   // [nsrc][kPMax + 1]
};

// The near-candidate list of one target column against one source set.
struct MPNearCol {
  int self;              // source index of the target's own vesicle, or -1
  int cend;              // candidates on the list
  const int* cands;      // ascending source indices
  const uint32_t* excl;  // [maxc][nwords] excluded target points per candidate
  int nwords;
};

// Per-CTA staging of the source records and moments.
struct MPStage {
  MPSrc* src;                 // [kStage]
  MPMom (*mom)[kPMax + 1];    // [kStage][kPMax + 1]
  float4* drec;               // [ns] direct-rule records of one source
};

// Sum over every source of one set onto this thread's target point (tl
// relative to the target centre thi + tlo, RT the target radius): the
// expansion for well-separated pairs, the direct rule for the others and for
// every pair on the near list (excluded points dropped); the target's own
// vesicle is skipped.  Uniform control flow across the CTA.
__device__ __forceinline__ void mp_sum_set(const MPSet& S, const MPNearCol& nr, const MPStage& st, int i, bool valid,
                                           float2 tl, float2 thi, float2 tlo, float RT, float& tot_x, float& tot_y,
                                           float& cmp_x, float& cmp_y, unsigned long long& terms,
                                           unsigned long long& ndirect) {
  int cur = 0;
  for (int s0 = 0; s0 < S.nsrc; s0 += kStage) {
    const int nst = min(kStage, S.nsrc - s0);
    __syncthreads();
    for (int q = i; q < nst; q += blockDim.x) st.src[q] = S.src[s0 + q];
    for (int q = i; q < nst * (kPMax + 1); q += blockDim.x)
      (&st.mom[0][0])[q] = S.mom[(long long)s0 * (kPMax + 1) + q];
    __syncthreads();
    for (int q = 0; q < nst; ++q) {
      const int s = s0 + q;
      if (s == nr.self) continue;
      const MPSrc Sq = st.src[q];
      // target relative to the source centre (hi/lo: no cancellation from absolute positions)
      const float ox = (thi.x - Sq.chi.x) + (tlo.x - Sq.clo.x);
      const float oy = (thi.y - Sq.chi.y) + (tlo.y - Sq.clo.y);
      // near-candidate list of this column: ascending source indices
      bool cand = false;
      int cidx = 0;
      if (nr.cend > 0) {
        while (cur < nr.cend && nr.cands[cur] < s) ++cur;
        cand = cur < nr.cend && nr.cands[cur] == s;
        cidx = cur;
      }
      const float dc = sqrtf(ox * ox + oy * oy) - RT;
      const float rp = dc > 0.f ? Sq.R / dc : 2.f;
      if (!cand && rp <= kRhoMax) {
        // expansion of order P: rp^(P+1) / (1 - rp) <= kEps
        int P = rp > 0.f ? (int)ceilf(__logf(kEps * (1.f - rp)) / __logf(rp)) - 1 : 1;
        P = max(1, min(P, kPMax));
        terms += (unsigned long long)(P + 1);
        const float tx = tl.x + ox, ty = tl.y + oy;  // omega
        const float om2 = fmaf(tx, tx, ty * ty);
        const float iom2 = mufu_rcp(om2);
        const float ur = Sq.R * tx * iom2, ui = -Sq.R * ty * iom2;  // tau = R / omega
        float2 hA = st.mom[q][P].al, hB = st.mom[q][P].bc, hC = st.mom[q][P].ac, hE = st.mom[q][P].ec;
        for (int k = P - 1; k >= 0; --k) {
          const MPMom m = st.mom[q][k];
          float2 n;
          n.x = fmaf(hA.x, ur, fmaf(-hA.y, ui, m.al.x));
          n.y = fmaf(hA.x, ui, fmaf(hA.y, ur, m.al.y));
          hA = n;
          n.x = fmaf(hB.x, ur, fmaf(-hB.y, ui, m.bc.x));
          n.y = fmaf(hB.x, ui, fmaf(hB.y, ur, m.bc.y));
          hB = n;
          n.x = fmaf(hC.x, ur, fmaf(-hC.y, ui, m.ac.x));
          n.y = fmaf(hC.x, ui, fmaf(hC.y, ur, m.ac.y));
          hC = n;
          n.x = fmaf(hE.x, ur, fmaf(-hE.y, ui, m.ec.x));
          n.y = fmaf(hE.x, ui, fmaf(hE.y, ur, m.ec.y));
          hE = n;
        }
        const float lnom = (float)kHalfLn2 * mufu_lg2(om2);  // log|omega|
        // (omega / conj(omega)) conj(hC) and conj(tau hE)
        const float qr = (tx * tx - ty * ty) * iom2, qi = 2.f * tx * ty * iom2;
        const float wcr = qr * hC.x + qi * hC.y, wci = qi * hC.x - qr * hC.y;
        const float ter = ur * hE.x - ui * hE.y, tei = -(ur * hE.y + ui * hE.x);
        const float px = fmaf(-lnom, Sq.f0.x, 0.5f * Sq.f0.x) + hA.x + hB.x + 0.5f * (wcr - ter);
        const float py = fmaf(-lnom, Sq.f0.y, 0.5f * Sq.f0.y) + hA.y - hB.y + 0.5f * (wci - tei);
        if (valid) {
          neumaier(tot_x, cmp_x, px);
          neumaier(tot_y, cmp_y, py);
        }
      } else {
        // direct rule over the upsampled points (FP32, log relative to the
        // source centre), staged kDrecChunk points at a time (the same order
        // of summation as one stage)
        ++ndirect;
        const float4* R4 = S.rec + (long long)s * S.ns;
        bool excl = false;
        if (cand && valid) {
          const uint32_t w = nr.excl[(long long)cidx * nr.nwords + (i >> 5)];
          excl = (w >> (i & 31)) & 1u;
        }
        const float tx = tl.x + ox, ty = tl.y + oy;
        const float rc2 = fmaf(tx, tx, ty * ty);
        const float irc2 = mufu_rcp(rc2);
        float acx = 0.f, acy = 0.f, alx = 0.f, aly = 0.f;
        for (int j0 = 0; j0 < S.ns; j0 += kDrecChunk) {
          const int nj = min(kDrecChunk, S.ns - j0);
          __syncthreads();
          for (int j = i; j < nj; j += blockDim.x) st.drec[j] = R4[j0 + j];
          __syncthreads();
#pragma unroll 4
          for (int j = 0; j < nj; ++j) {
            const float4 r = st.drec[j];
            const float dx = tx - r.x, dy = ty - r.y;
            const float r2 = fmaf(dx, dx, dy * dy);
            const float inv = mufu_rcp(r2);
            const float lg = mufu_lg2(r2 * irc2);
            const float cc = fmaf(dx, r.z, dy * r.w) * inv;
            acx = fmaf(cc, dx, acx);
            acy = fmaf(cc, dy, acy);
            alx = fmaf(lg, r.z, alx);
            aly = fmaf(lg, r.w, aly);
          }
        }
        if (valid && !excl) {
          const float lgc = mufu_lg2(rc2);
          const float px = acx - (float)kHalfLn2 * fmaf(lgc, Sq.f0.x, alx);
          const float py = acy - (float)kHalfLn2 * fmaf(lgc, Sq.f0.y, aly);
          neumaier(tot_x, cmp_x, px);
          neumaier(tot_y, cmp_y, py);
        }
      }
    }
  }
}

// radius of the target vesicle about its centre (max over the CTA's valid points)
__device__ __forceinline__ float mp_target_radius(float2 tl, int i, float* rmax_w) {
  float rt = sqrtf(tl.x * tl.x + tl.y * tl.y);
  for (int o = 16; o > 0; o >>= 1) rt = fmaxf(rt, __shfl_xor_sync(0xffffffffu, rt, o));
  if ((i & 31) == 0) rmax_w[i >> 5] = rt;
  __syncthreads();
  float RT = 0.f;
  for (int w = 0; w < (int)(blockDim.x >> 5); ++w) RT = fmaxf(RT, rmax_w[w]);
  return RT * (1.0f + 1e-6f);
}

struct MPArgs {
  int nsrc, ns, ntp;
  const float4* rec;
  const MPSrc* src;
  const MPMom* mom;
  const float2* tloc;
  const float2* thi;
  const float2* tlo;
  const int* self_idx;
  const int* cand_count;
  const int* cand_src;
  const uint32_t* excl_mask;
  int maxc, nwords;
  double* out;               // [nt][2][ntp], scaled by 1/(4 pi)
  unsigned long long* work;  // optional: series terms, direct pairs (per target point)
};

// One CTA per target column (blockDim = ntp rounded up to a warp multiple).
// Dynamic shared memory: direct-rule records of one source, min(ns,
// kDrecChunk) float4.
__global__ void __launch_bounds__(128) mp_eval_kernel(MPArgs p) {
  extern __shared__ __align__(16) float4 drec[];
  __shared__ MPSrc ssrc[kStage];
  __shared__ MPMom smom[kStage][kPMax + 1];
  __shared__ float rmax_w[32];
  const int col = blockIdx.x, i = threadIdx.x;
  const bool valid = i < p.ntp;
  const float2 tl = valid ? p.tloc[(long long)col * p.ntp + i] : make_float2(0.f, 0.f);
  const float2 thi = p.thi[col], tlo = p.tlo[col];
  const float RT = mp_target_radius(tl, i, rmax_w);
  MPSet S{p.nsrc, p.ns, p.rec, p.src, p.mom};
  MPNearCol nr;
  nr.self = p.self_idx ? p.self_idx[col] : -1;
  nr.cend = p.cand_count ? min(p.cand_count[col], p.maxc) : 0;
  nr.cands = p.cand_src ? p.cand_src + (long long)col * p.maxc : nullptr;
  nr.excl = p.excl_mask ? p.excl_mask + (long long)col * p.maxc * p.nwords : nullptr;
  nr.nwords = p.nwords;
  MPStage st{ssrc, smom, drec};
  float tot_x = 0.f, tot_y = 0.f, cmp_x = 0.f, cmp_y = 0.f;
  unsigned long long terms = 0, ndirect = 0;  // work of this column (uniform across the CTA)
  mp_sum_set(S, nr, st, i, valid, tl, thi, tlo, RT, tot_x, tot_y, cmp_x, cmp_y, terms, ndirect);
  if (p.work && i == 0) {
    atomicAdd(&p.work[0], terms * (unsigned long long)p.ntp);
    atomicAdd(&p.work[1], ndirect * (unsigned long long)p.ntp * (unsigned long long)p.ns);
  }
  if (valid) {
    const double scale = 1.0 / (4.0 * VES_PI);
    p.out[(long long)col * 2 * p.ntp + i] = ((double)tot_x + (double)cmp_x) * scale;
    p.out[(long long)col * 2 * p.ntp + p.ntp + i] = ((double)tot_y + (double)cmp_y) * scale;
  }
}

// ---------------------------------------------------------------------------
// Several point sets (a suspension of vesicles with different point counts)
// in one launch: every target column of every set against every source set.
constexpr int kMPSets = 4;

struct MPGroupArgs {
  int ng;
  MPSet set[kMPSets];            // source sets
  int col0[kMPSets + 1];         // first target column of each target set
  int ntp[kMPSets];
  const float2* tloc[kMPSets];   // [nt][ntp] per target set
  const float2* thi;             // [total columns]
  const float2* tlo;
  double* out[kMPSets];          // [nt][2][ntp] per target set
  // near lists of target set g against source set q, [g][q]
  const int* cand_count[kMPSets][kMPSets];
  const int* cand_src[kMPSets][kMPSets];
  const uint32_t* excl_mask[kMPSets][kMPSets];
  int maxc[kMPSets][kMPSets];
  int nwords[kMPSets];
};

__global__ void __launch_bounds__(128) mp_eval_groups_kernel(MPGroupArgs p) {
  extern __shared__ __align__(16) float4 drec[];
  __shared__ MPSrc ssrc[kStage];
  __shared__ MPMom smom[kStage][kPMax + 1];
  __shared__ float rmax_w[32];
  const int col = blockIdx.x, i = threadIdx.x;
  int g = 0;
  while (g + 1 < p.ng && col >= p.col0[g + 1]) ++g;
  const int lc = col - p.col0[g], ntp = p.ntp[g];
  const bool valid = i < ntp;
  const float2 tl = valid ? p.tloc[g][(long long)lc * ntp + i] : make_float2(0.f, 0.f);
  const float2 thi = p.thi[col], tlo = p.tlo[col];
  const float RT = mp_target_radius(tl, i, rmax_w);
  MPStage st{ssrc, smom, drec};
  float tot_x = 0.f, tot_y = 0.f, cmp_x = 0.f, cmp_y = 0.f;
  unsigned long long terms = 0, ndirect = 0;
  for (int q = 0; q < p.ng; ++q) {
    MPNearCol nr;
    nr.self = q == g ? lc : -1;
    const int mc = p.maxc[g][q];
    nr.cend = p.cand_count[g][q] ? min(p.cand_count[g][q][lc], mc) : 0;
    nr.cands = p.cand_src[g][q] ? p.cand_src[g][q] + (long long)lc * mc : nullptr;
    nr.excl = p.excl_mask[g][q] ? p.excl_mask[g][q] + (long long)lc * mc * p.nwords[g] : nullptr;
    nr.nwords = p.nwords[g];
    mp_sum_set(p.set[q], nr, st, i, valid, tl, thi, tlo, RT, tot_x, tot_y, cmp_x, cmp_y, terms, ndirect);
  }
  if (valid) {
    const double scale = 1.0 / (4.0 * VES_PI);
    double* o = p.out[g] + (long long)lc * 2 * ntp;
    o[i] = ((double)tot_x + (double)cmp_x) * scale;
    o[ntp + i] = ((double)tot_y + (double)cmp_y) * scale;
  }
}

}  // namespace

int farfield_mp_run(const FFEnv& env, int nsrc, int ns, const double* Xsrc, const double* den, int nt, int ntp,
                    const double* Xtar, const int* self_idx, const ves_near_lists* nl, double* out, WsCarver& ws,
                    cudaStream_t s) {
  const long long total_pts = (long long)nt * ntp;
  float4* rec = ws.take<float4>((size_t)nsrc * ns);
  MPSrc* src = ws.take<MPSrc>(nsrc);
  MPMom* mom = ws.take<MPMom>((size_t)nsrc * (kPMax + 1));
  float2* tloc = ws.take<float2>((size_t)total_pts);
  float2* thi = ws.take<float2>(nt);
  float2* tlo = ws.take<float2>(nt);
  if (ws.sizing) return VES_OK;
  if (!ws.ok()) {
    ves_record_error(VES_ERR_WORKSPACE, "farfield: workspace too small");
    return VES_ERR_WORKSPACE;
  }
  if (total_pts == 0) return VES_OK;
  if (nsrc == 0) return ves_cuda_status(cudaMemsetAsync(out, 0, (size_t)total_pts * 2 * sizeof(double), s), "ff zero");
  if (ntp > 128) {
    ves_record_error(VES_ERR_SHAPE, "farfield: the multipole path takes at most 128 points per target column");
    return VES_ERR_SHAPE;
  }
  if (nl && ntp != env.N) {
    ves_record_error(VES_ERR_SHAPE, "farfield: near lists need N target points per column");
    return VES_ERR_SHAPE;
  }
  const size_t dsmem = (size_t)std::min(ns, kDrecChunk) * sizeof(float4);
  ves_count_launch(2);
  mp_prep_kernel<<<nsrc, 256, 0, s>>>(ns, Xsrc, den, rec, src, mom);
  mp_prep_targets_kernel<<<nt, 256, 0, s>>>(ntp, Xtar, tloc, thi, tlo);
  MPArgs a;
  a.nsrc = nsrc;
  a.ns = ns;
  a.ntp = ntp;
  a.rec = rec;
  a.src = src;
  a.mom = mom;
  a.tloc = tloc;
  a.thi = thi;
  a.tlo = tlo;
  a.self_idx = self_idx;
  a.cand_count = nl ? nl->cand_count : nullptr;
  a.cand_src = nl ? nl->cand_src : nullptr;
  a.excl_mask = nl ? nl->excl_mask : nullptr;
  a.maxc = nl ? nl->maxc : 0;
  a.nwords = (env.N + 31) / 32;
  a.out = out;
  a.work = (env.timing && env.timing->timing) ? env.timing->d_mp : nullptr;
  if (dsmem > 32 * 1024) {
    cudaError_t e = cudaFuncSetAttribute(mp_eval_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)dsmem);
    if (e != cudaSuccess) return ves_cuda_status(e, "farfield multipole smem attribute");
  }
  const int threads = ((ntp + 31) / 32) * 32;
  ves_count_launch();
  if (env.timing) ves_ff_timing_begin(env.timing, s);
  mp_eval_kernel<<<nt, threads, dsmem, s>>>(a);
  if (env.timing) ves_ff_timing_end(env.timing, s, (double)total_pts * ns * (double)nsrc);
  return ves_launch_check("farfield multipole");
}

int farfield_mp_groups_run(const FFEnv& env, int ng, const int* nsrc, const int* ns, const double* const* Xsrc,
                           const double* const* den, const int* nt, const int* ntp, const double* const* Xtar,
                           const ves_near_lists* const* nl, double* const* out, WsCarver& ws, cudaStream_t s) {
  (void)env;
  if (ng < 1 || ng > kMPSets) {
    if (!ws.sizing) ves_record_error(VES_ERR_ARG, "farfield groups: 1 to %d point sets", kMPSets);
    return VES_ERR_ARG;
  }
  float4* rec[kMPSets];
  MPSrc* src[kMPSets];
  MPMom* mom[kMPSets];
  float2* tloc[kMPSets];
  long long cols = 0;
  int nsmax = 0, ntpmax = 0;
  for (int g = 0; g < ng; ++g) {
    rec[g] = ws.take<float4>((size_t)nsrc[g] * ns[g]);
    src[g] = ws.take<MPSrc>(nsrc[g]);
    mom[g] = ws.take<MPMom>((size_t)nsrc[g] * (kPMax + 1));
    tloc[g] = ws.take<float2>((size_t)nt[g] * ntp[g]);
    cols += nt[g];
    nsmax = std::max(nsmax, ns[g]);
    ntpmax = std::max(ntpmax, ntp[g]);
  }
  float2* thi = ws.take<float2>((size_t)cols);
  float2* tlo = ws.take<float2>((size_t)cols);
  if (ws.sizing) return VES_OK;
  if (!ws.ok()) {
    ves_record_error(VES_ERR_WORKSPACE, "farfield groups: workspace too small");
    return VES_ERR_WORKSPACE;
  }
  if (cols == 0) return VES_OK;
  if (ntpmax > 128) {
    ves_record_error(VES_ERR_SHAPE, "farfield groups: at most 128 target points per vesicle");
    return VES_ERR_SHAPE;
  }
  MPGroupArgs a;
  memset(&a, 0, sizeof(a));
  a.ng = ng;
  a.thi = thi;
  a.tlo = tlo;
  a.col0[0] = 0;
  for (int g = 0; g < ng; ++g) {
    if (nsrc[g] > 0) {
      ves_count_launch();
      mp_prep_kernel<<<nsrc[g], 256, 0, s>>>(ns[g], Xsrc[g], den[g], rec[g], src[g], mom[g]);
    }
    if (nt[g] > 0) {
      ves_count_launch();
      mp_prep_targets_kernel<<<nt[g], 256, 0, s>>>(ntp[g], Xtar[g], tloc[g], thi + a.col0[g], tlo + a.col0[g]);
    }
    a.set[g] = MPSet{nsrc[g], ns[g], rec[g], src[g], mom[g]};
    a.col0[g + 1] = a.col0[g] + nt[g];
    a.ntp[g] = ntp[g];
    a.tloc[g] = tloc[g];
    a.out[g] = out[g];
    a.nwords[g] = (ntp[g] + 31) / 32;
    for (int q = 0; q < ng; ++q) {
      const ves_near_lists* L = nl ? nl[g * ng + q] : nullptr;
      a.cand_count[g][q] = L ? L->cand_count : nullptr;
      a.cand_src[g][q] = L ? L->cand_src : nullptr;
      a.excl_mask[g][q] = L ? L->excl_mask : nullptr;
      a.maxc[g][q] = L ? L->maxc : 0;
    }
  }
  const size_t dsmem = (size_t)std::min(nsmax, kDrecChunk) * sizeof(float4);
  if (dsmem > 32 * 1024) {
    cudaError_t e = cudaFuncSetAttribute(mp_eval_groups_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)dsmem);
    if (e != cudaSuccess) return ves_cuda_status(e, "farfield groups smem attribute");
  }
  ves_count_launch();
  mp_eval_groups_kernel<<<(unsigned)cols, ((ntpmax + 31) / 32) * 32, dsmem, s>>>(a);
  return ves_launch_check("farfield groups");
}
