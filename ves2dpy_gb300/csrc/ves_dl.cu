// Double-layer potential of vesicles with a viscosity contrast.
//
// * stokesDLmatrix (mytorch/poten.py:102-175).  On the Nup-upsampled curve
//   (the geometry of capsules(Xup): xt, sa, cur by diffProp), for target a and
//   source b != a with d = x_b - x_a and c = -(1 - visc),
//     K(a, b) = c ((d_x ty_b - d_y tx_b) / |d|^4) sa_b,
//     Dup11 = K d_x^2,  Dup12 = K d_x d_y,  Dup22 = K d_y^2,
//   and on the diagonal the limit c/2 cur_a sa_a {tx_a^2, tx_a ty_a, ty_a^2};
//   then D = (1/pi)(2 pi/Nup) [R Dup11 P, R Dup12 P; R Dup12 P, R Dup22 P]
//   with the restriction R and prolongation P of the Alpert build.  A vesicle
//   without a contrast (visc == 1) has D = 0.
// * exactStokesDL (poten.py:399-441, matlab/poten_py.m:419-470): the direct
//   sum over the source points of the given vesicles
//     u(x) = 1/pi sum_j ((r.n_j)(r.den_j) / |r|^4) r,   r = x - y_j,
//     n = (ty, -tx),   den = f sa (2 pi / ns) (1 - visc).
//   One CTA per target column walks every source vesicle (sorted near lists
//   remove (target point, source vesicle) pairs as in the single-layer sum);
//   FP64 throughout, deterministic (no atomics).
// * The same sum with a multipole expansion of each source vesicle for the
//   well-separated vesicle pairs (precision FP32M).  In complex notation
//   (r = x - y as rho, n, d complex) the pair term is
//     (r.n)(r.d) r / |r|^4 = [conj(c) rho / conj(rho)^2 + e / conj(rho) + c / rho] / 4
//   with c = n d and e = 2 Re(conj(n) d) (real).  About the source centre (v = y - c0,
//   omega = x - c0, R >= max |v|, tau = R / omega, vt = v / R):
//     4 pi u = h1 / omega + conj(h2 / omega) + (omega / conj(omega)^2) conj(h3)
//              - R conj(h4 / omega^2),
//     h1 = sum_k C_k tau^k, h2 = sum_k E_k tau^k, h3 = sum_k (k+1) C_k tau^k,
//     h4 = sum_k (k+1) G_k tau^k,
//     C_k = sum_j c_j vt_j^k, E_k = sum_j e_j vt_j^k, G_k = sum_j c_j conj(vt_j) vt_j^k
//   (series of 1/(1 - v/omega) and its square).  The moments are taken of the
//   density minus its weighted mean (f - fbar on the quadrature weights): the
//   double layer of a constant density vanishes outside the curve, and the
//   trapezoid rule keeps that to rounding for separated targets, while the
//   mean of a position-like density (the step applies the operator to X) would
//   otherwise dominate the FP32 moments.  Close pairs and pairs on the near
//   candidate list are summed directly in FP32 over the upsampled points with
//   the same mean-free density: a target more than 12 upsampled spacings from
//   every source point sees the trapezoid rule of the constant density's
//   double layer exact to rounding (its error decays like
//   exp(-2 pi distance / spacing)), so dropping the mean changes the sum by
//   rounding only; a target closer than that is summed again in FP64 with the
//   full density (only without near lists: the near zone of the step, 1/N for
//   unit length, is those 12 spacings, and its points are excluded).
//   Sources without a contrast (visc == 1) have zero density and are skipped.
#include "ves_internal.h"

namespace {

constexpr int kDLTile = 256;  // source points staged per shared-memory tile

// Rows of Dup (three fields) for ROWS targets per CTA; kernel values in FP64,
// stored as T for the R Dup P products.
template <typename T, int ROWS>
__global__ void __launch_bounds__(256) dl_rows_kernel(int Nup, const double* __restrict__ Xup,
                                                      const double* __restrict__ tang, const double* __restrict__ sa,
                                                      const double* __restrict__ cur, const double* __restrict__ visc,
                                                      T* __restrict__ Dup, int k0) {
  __shared__ double xa[ROWS], ya[ROWS];
  const int kl = blockIdx.y;
  const int k = k0 + kl;
  const int a0 = blockIdx.x * ROWS;
  const double* xk = Xup + (long long)k * 2 * Nup;
  const double* tk = tang + (long long)k * 2 * Nup;
  const double* sk = sa + (long long)k * Nup;
  const double* ck = cur + (long long)k * Nup;
  if (threadIdx.x < ROWS) {
    const int a = min(a0 + (int)threadIdx.x, Nup - 1);
    xa[threadIdx.x] = xk[a];
    ya[threadIdx.x] = xk[Nup + a];
  }
  __syncthreads();
  const double coef = -(1.0 - visc[k]);
  const long long NN = (long long)Nup * Nup;
  T* D11 = Dup + (long long)kl * 3 * NN;
  T* D12 = D11 + NN;
  T* D22 = D12 + NN;
  for (int b = threadIdx.x; b < Nup; b += blockDim.x) {
    const double xb = xk[b], yb = xk[Nup + b], txb = tk[b], tyb = tk[Nup + b], sab = sk[b];
#pragma unroll
    for (int r = 0; r < ROWS; ++r) {
      const int a = a0 + r;
      if (a >= Nup) break;
      double v11, v12, v22;
      if (a == b) {
        const double fac = 0.5 * coef * ck[b] * sab;
        v11 = fac * (txb * txb);
        v12 = fac * (txb * tyb);
        v22 = fac * (tyb * tyb);
      } else {
        const double dx = xb - xa[r], dy = yb - ya[r];
        const double r2 = dx * dx + dy * dy;
        const double rho4 = 1.0 / (r2 * r2);
        const double K = coef * ((dx * tyb - dy * txb) * rho4 * sab);
        v11 = K * (dx * dx);
        v12 = K * (dx * dy);
        v22 = K * (dy * dy);
      }
      const long long o = (long long)a * Nup + b;
      D11[o] = (T)v11;
      D12[o] = (T)v12;
      D22[o] = (T)v22;
    }
  }
}

// D[k] = (1/pi)(2 pi/Nup) [[F11, F12], [F12, F22]] from the restricted fields
template <typename T>
__global__ void dl_assemble_kernel(int N, int Nup, const T* __restrict__ Df, double* __restrict__ D, int k0) {
  const int kl = blockIdx.y;
  const long long NN = (long long)N * N;
  const T* f11 = Df + (long long)kl * 3 * NN;
  const T* f12 = f11 + NN;
  const T* f22 = f12 + NN;
  double* Dk = D + (long long)(k0 + kl) * 4 * NN;
  const double w = 2.0 * VES_PI / Nup;
  for (long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x; idx < 4 * NN;
       idx += (long long)gridDim.x * blockDim.x) {
    const int r = (int)(idx / (2 * N)), c = (int)(idx % (2 * N));
    const int i = r % N, j = c % N;
    const T* src = (r < N) ? ((c < N) ? f11 : f12) : ((c < N) ? f12 : f22);
    Dk[idx] = ((1.0 / VES_PI) * (double)src[(long long)i * N + j]) * w;
  }
}

// den[k][c][j] = f sa (2 pi / ns) (1 - visc[k])
__global__ void dl_density_kernel(int nv, int ns, const double* __restrict__ f, const double* __restrict__ sa,
                                  const double* __restrict__ visc, double* __restrict__ den) {
  const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= (long long)nv * 2 * ns) return;
  const long long k = idx / (2 * ns);
  const int j = (int)(idx % ns);
  den[idx] = ((f[idx] * sa[k * ns + j]) * (2.0 * VES_PI / ns)) * (1.0 - (visc ? visc[k] : 1.0));
}

// One CTA per target column; PT target points per thread (ntp <= 256 * PT).
template <int PT>
__global__ void __launch_bounds__(256) dl_direct_kernel(int nsrc, int ns, const double* __restrict__ Xsrc,
                                                        const double* __restrict__ tang,
                                                        const double* __restrict__ den, int ntp,
                                                        const double* __restrict__ Xtar,
                                                        const int* __restrict__ self_idx,
                                                        const int* __restrict__ cand_count,
                                                        const int* __restrict__ cand_src,
                                                        const uint32_t* __restrict__ excl_mask, int maxc,
                                                        int nwords, double* __restrict__ out) {
  __shared__ double sx[kDLTile], sy[kDLTile], snx[kDLTile], sny[kDLTile], sdx[kDLTile], sdy[kDLTile];
  const int t = blockIdx.x;
  const double* xt = Xtar + (long long)t * 2 * ntp;
  double px[PT], py[PT], ax[PT], ay[PT];
#pragma unroll
  for (int q = 0; q < PT; ++q) {
    const int i = threadIdx.x + q * blockDim.x;
    px[q] = i < ntp ? xt[i] : 0.0;
    py[q] = i < ntp ? xt[ntp + i] : 0.0;
    ax[q] = ay[q] = 0.0;
  }
  const int skip = self_idx ? self_idx[t] : -1;
  const int nc = cand_count ? cand_count[t] : 0;
  int cur = 0;
  for (int s = 0; s < nsrc; ++s) {
    if (s == skip) continue;
    bool ex[PT];
#pragma unroll
    for (int q = 0; q < PT; ++q) ex[q] = (threadIdx.x + q * blockDim.x) >= ntp;
    if (cand_src) {
      const int* cs = cand_src + (long long)t * maxc;
      while (cur < nc && cs[cur] < s) ++cur;
      if (cur < nc && cs[cur] == s) {
        const uint32_t* m = excl_mask + ((long long)t * maxc + cur) * nwords;
#pragma unroll
        for (int q = 0; q < PT; ++q) {
          const int i = threadIdx.x + q * blockDim.x;
          if (i < ntp && ((m[i >> 5] >> (i & 31)) & 1u)) ex[q] = true;
        }
      }
    }
    const double* xs = Xsrc + (long long)s * 2 * ns;
    const double* ts = tang + (long long)s * 2 * ns;
    const double* ds = den + (long long)s * 2 * ns;
    for (int j0 = 0; j0 < ns; j0 += kDLTile) {
      const int nj = min(kDLTile, ns - j0);
      __syncthreads();
      for (int j = threadIdx.x; j < nj; j += blockDim.x) {
        sx[j] = xs[j0 + j];
        sy[j] = xs[ns + j0 + j];
        snx[j] = ts[ns + j0 + j];   // n = (ty, -tx)
        sny[j] = -ts[j0 + j];
        sdx[j] = ds[j0 + j];
        sdy[j] = ds[ns + j0 + j];
      }
      __syncthreads();
#pragma unroll
      for (int q = 0; q < PT; ++q) {
        if (ex[q]) continue;
        double bx = 0.0, by = 0.0;
        for (int j = 0; j < nj; ++j) {
          const double dx = px[q] - sx[j], dy = py[q] - sy[j];
          const double d2 = dx * dx + dy * dy;
          const double c = ((dx * snx[j] + dy * sny[j]) / (d2 * d2)) * (dx * sdx[j] + dy * sdy[j]);
          bx = fma(c, dx, bx);
          by = fma(c, dy, by);
        }
        ax[q] += bx;
        ay[q] += by;
      }
    }
  }
  double* o = out + (long long)t * 2 * ntp;
#pragma unroll
  for (int q = 0; q < PT; ++q) {
    const int i = threadIdx.x + q * blockDim.x;
    if (i < ntp) {
      o[i] = ax[q] / VES_PI;
      o[ntp + i] = ay[q] / VES_PI;
    }
  }
}

int dl_chunk(const ves_ctx* c, int nv, size_t es) {
  const size_t per = (size_t)3 * c->Nup * c->Nup * es;
  const size_t budget = (size_t)2 << 30;  // ~2 GiB of Dup per chunk
  int ch = (int)(budget / per);
  if (ch < 1) ch = 1;
  if (ch > nv) ch = nv;
  return ch;
}

template <typename T>
int dl_matrix_impl(ves_ctx* c, int nv, const double* X, const double* visc, double* D, WsCarver& ws,
                   cudaStream_t s) {
  const int N = c->N, Nup = c->Nup;
  const int chunk = nv > 0 ? dl_chunk(c, nv, sizeof(T)) : 1;
  double* Xup = ws.take<double>((size_t)nv * 2 * Nup);
  double* sa = ws.take<double>((size_t)nv * Nup);
  double* tang = ws.take<double>((size_t)nv * 2 * Nup);
  double* cur = ws.take<double>((size_t)nv * Nup);
  T* Dup = ws.take<T>((size_t)chunk * 3 * Nup * Nup);
  T* Tm = ws.take<T>((size_t)chunk * 3 * Nup * N);
  T* Df = ws.take<T>((size_t)chunk * 3 * N * N);
  if (ws.sizing) return VES_OK;
  if (!ws.ok()) {
    ves_record_error(VES_ERR_WORKSPACE, "stokes_dl_matrix: workspace too small");
    return VES_ERR_WORKSPACE;
  }
  if (nv <= 0) return VES_OK;
  // capsules(Xup): the upsampled curve's own jacobian, tangent and curvature
  launch_upsample_geom(c, nv, X, Xup, sa, tang, cur, s);
  const T* Pm = (const T*)(sizeof(T) == 8 ? (const void*)c->Pm : (const void*)c->Pm32);
  const T* Rm = (const T*)(sizeof(T) == 8 ? (const void*)c->Rm : (const void*)c->Rm32);
  constexpr int ROWS = 8;
  for (int k0 = 0; k0 < nv; k0 += chunk) {
    const int nk = min(chunk, nv - k0);
    dim3 grid(ceil_div(Nup, ROWS), nk);
    ves_count_launch();
    dl_rows_kernel<T, ROWS><<<grid, 256, 0, s>>>(Nup, Xup, tang, sa, cur, visc, Dup, k0);
    const long long NN = (long long)Nup * Nup;
    if (sizeof(T) == 8) {
      launch_bgemm_f64(3 * nk, Nup, N, Nup, 1.0, (const double*)Dup, Nup, NN, (const double*)Pm, N, 0, 0.0,
                       (double*)Tm, N, (long long)Nup * N, s);
      launch_bgemm_f64(3 * nk, N, N, Nup, 1.0, (const double*)Rm, Nup, 0, (const double*)Tm, N,
                       (long long)Nup * N, 0.0, (double*)Df, N, (long long)N * N, s);
    } else {
      launch_bgemm_f32(3 * nk, Nup, N, Nup, 1.0f, (const float*)Dup, Nup, NN, (const float*)Pm, N, 0, 0.0f,
                       (float*)Tm, N, (long long)Nup * N, s);
      launch_bgemm_f32(3 * nk, N, N, Nup, 1.0f, (const float*)Rm, Nup, 0, (const float*)Tm, N,
                       (long long)Nup * N, 0.0f, (float*)Df, N, (long long)N * N, s);
    }
    dim3 ga(ceil_div(4LL * N * N, 256), nk);
    ves_count_launch();
    dl_assemble_kernel<T><<<ga, 256, 0, s>>>(N, Nup, Df, D, k0);
  }
  return ves_launch_check("stokes_dl_matrix");
}

}  // namespace

int stokes_dl_matrix(ves_ctx* c, int nv, const double* X, const double* visc, int precision, double* D, WsCarver& ws,
                     cudaStream_t s) {
  if (precision == VES_PREC_FP64) return dl_matrix_impl<double>(c, nv, X, visc, D, ws, s);
  if (precision == VES_PREC_FP32C) return dl_matrix_impl<float>(c, nv, X, visc, D, ws, s);
  ves_record_error(VES_ERR_ARG, "stokes_dl_matrix: bad precision %d", precision);
  return VES_ERR_ARG;
}

void launch_dl_density(int nv, int ns, const double* f, const double* sa, const double* visc, double* den,
                       cudaStream_t s) {
  const long long n = (long long)nv * 2 * ns;
  if (n <= 0) return;
  ves_count_launch();
  dl_density_kernel<<<ceil_div(n, 256), 256, 0, s>>>(nv, ns, f, sa, visc, den);
}

int farfield_dl_direct_run(ves_ctx* c, int nsrc, int ns, const double* Xsrc, const double* tang, const double* den,
                           int nt, int ntp, const double* Xtar, const int* self_idx, const ves_near_lists* nl,
                           double* out, cudaStream_t s) {
  if (nsrc < 0 || ns <= 0 || nt < 0 || ntp <= 0 || ntp > 1024) {
    ves_record_error(VES_ERR_SHAPE, "farfield_dl: bad sizes (ns %d, ntp %d; at most 1024 target points)", ns, ntp);
    return VES_ERR_SHAPE;
  }
  if (nl && (!nl->cand_count || !nl->cand_src || !nl->excl_mask || nl->maxc <= 0 || nt != nsrc ||
             (c && ntp != c->N))) {
    ves_record_error(VES_ERR_ARG, "farfield_dl: near lists need nt == nsrc and ntp == N");
    return VES_ERR_ARG;
  }
  if (nt == 0) return VES_OK;
  const int* cc = nl ? nl->cand_count : nullptr;
  const int* cs = nl ? nl->cand_src : nullptr;
  const uint32_t* em = nl ? nl->excl_mask : nullptr;
  const int maxc = nl ? nl->maxc : 0;
  const int nwords = (ntp + 31) / 32;
  ves_count_launch();
  if (ntp <= 256)
    dl_direct_kernel<1><<<nt, 256, 0, s>>>(nsrc, ns, Xsrc, tang, den, ntp, Xtar, self_idx, cc, cs, em, maxc, nwords, out);
  else if (ntp <= 512)
    dl_direct_kernel<2><<<nt, 256, 0, s>>>(nsrc, ns, Xsrc, tang, den, ntp, Xtar, self_idx, cc, cs, em, maxc, nwords, out);
  else
    dl_direct_kernel<4><<<nt, 256, 0, s>>>(nsrc, ns, Xsrc, tang, den, ntp, Xtar, self_idx, cc, cs, em, maxc, nwords, out);
  return ves_launch_check("farfield_dl");
}

// ---------------------------------------------------------------------------
// Double-layer multipole path (FP32M)
namespace {

constexpr int kDLPMax = 24;          // highest expansion order
constexpr float kDLRhoMax = 0.35f;   // expansion used for rho_pair <= this
constexpr float kDLEps = 1e-10f;     // truncation bound relative to sum |c|, sum |e|
constexpr int kDLStage = 16;         // source vesicles per shared-memory stage

struct __align__(16) DLSrc {
  float2 chi, clo;  // centre, high and low FP32 parts
  float R;          // bound on |y_j - c0|
  int skip;         // no contrast: zero density
  float thr2;       // (12 upsampled spacings)^2: closer targets are summed in FP64
  float pad1;
};
// one order k: C_k, E_k, (k+1) C_k, (k+1) G_k of the normalised moments
struct __align__(16) DLMom {
  float2 c, e, c1, g1;
};

__device__ __forceinline__ double2 zmul(double2 a, double2 b) {
  return make_double2(fma(a.x, b.x, -a.y * b.y), fma(a.x, b.y, a.y * b.x));
}

// One CTA (256 threads) per source vesicle: centre, radius, weighted mean of
// the density, FP64 moments of the mean-free density, stored in FP32.
__global__ void __launch_bounds__(256) dl_mp_prep_kernel(int ns, const double* __restrict__ X,
                                                         const double* __restrict__ tang,
                                                         const double* __restrict__ den,
                                                         const double* __restrict__ sa,
                                                         const double* __restrict__ visc, DLSrc* __restrict__ src,
                                                         DLMom* __restrict__ mom, float4* __restrict__ recA,
                                                         float2* __restrict__ recB) {
  __shared__ double red[4][256];
  const int s = blockIdx.x, t = threadIdx.x;
  const double* x = X + (long long)s * 2 * ns;
  const double* tg = tang + (long long)s * 2 * ns;
  const double* d = den + (long long)s * 2 * ns;
  const double* js = sa + (long long)s * ns;
  const double wscale = (2.0 * VES_PI / ns) * (1.0 - (visc ? visc[s] : 1.0));
  auto block_sum4 = [&](double a, double b, double c, double e, bool use_max_a) {
    red[0][t] = a;
    red[1][t] = b;
    red[2][t] = c;
    red[3][t] = e;
    __syncthreads();
    for (int w = 128; w > 0; w >>= 1) {
      if (t < w) {
        red[0][t] = use_max_a ? fmax(red[0][t], red[0][t + w]) : red[0][t] + red[0][t + w];
        red[1][t] += red[1][t + w];
        red[2][t] += red[2][t + w];
        red[3][t] += red[3][t + w];
      }
      __syncthreads();
    }
  };
  double sx = 0, sy = 0, sw = 0, sdx = 0, sdy = 0, sl = 0;
  for (int j = t; j < ns; j += 256) {
    sx += x[j];
    sy += x[ns + j];
    sw += js[j] * wscale;
    sdx += d[j];
    sdy += d[ns + j];
    sl += js[j];
  }
  block_sum4(sx, sy, sw, sl, false);
  const double ccx = red[0][0] / ns, ccy = red[1][0] / ns, W = red[2][0];
  const double hsp = red[3][0] * (2.0 * VES_PI / ns) / ns;  // mean spacing = length / ns
  __syncthreads();
  block_sum4(0.0, sdx, sdy, 0.0, false);
  const double fbx = (W != 0.0) ? red[1][0] / W : 0.0, fby = (W != 0.0) ? red[2][0] / W : 0.0;
  __syncthreads();
  double r2 = 0;
  for (int j = t; j < ns; j += 256) {
    const double lx = x[j] - ccx, ly = x[ns + j] - ccy;
    r2 = fmax(r2, lx * lx + ly * ly);
    // FP32 records of the direct rule: local position, normal, mean-free density
    const double w = js[j] * wscale;
    recA[(long long)s * ns + j] = make_float4((float)lx, (float)ly, (float)tg[ns + j], (float)(-tg[j]));
    recB[(long long)s * ns + j] = make_float2((float)(d[j] - fbx * w), (float)(d[ns + j] - fby * w));
  }
  block_sum4(r2, 0.0, 0.0, 0.0, true);
  double R = sqrt(red[0][0]) * (1.0 + 1e-6);
  if (!(R > 0)) R = 1.0;
  if (t == 0) {
    DLSrc o;
    o.chi = make_float2((float)ccx, (float)ccy);
    o.clo = make_float2((float)(ccx - (double)o.chi.x), (float)(ccy - (double)o.chi.y));
    o.R = (float)R;
    o.skip = (wscale == 0.0) ? 1 : 0;
    o.thr2 = (float)(144.0 * hsp * hsp);
    o.pad1 = 0.f;
    src[s] = o;
  }
  // moments: warp w takes orders k = w, w + 8, ... (<= kDLPMax); lanes split the points
  const int warp = t >> 5, lane = t & 31;
  constexpr int kPer = (kDLPMax + 8) / 8;
  double2 C[kPer], E[kPer], G[kPer];
#pragma unroll
  for (int q = 0; q < kPer; ++q) C[q] = E[q] = G[q] = make_double2(0.0, 0.0);
  const double iR = 1.0 / R;
  for (int j = lane; j < ns; j += 32) {
    const double2 v = make_double2((x[j] - ccx) * iR, (x[ns + j] - ccy) * iR);
    const double w = js[j] * wscale;
    const double2 dj = make_double2(d[j] - fbx * w, d[ns + j] - fby * w);  // mean-free density
    const double2 nj = make_double2(tg[ns + j], -tg[j]);                     // n = (ty, -tx)
    const double2 cj = zmul(nj, dj);
    const double ej = 2.0 * (nj.x * dj.x + nj.y * dj.y);                     // 2 Re(conj(n) d)
    const double2 cvb = zmul(cj, make_double2(v.x, -v.y));                   // c conj(v)
    double2 pw = make_double2(1.0, 0.0), v8 = v;
    for (int e = 0; e < warp; ++e) pw = zmul(pw, v);
    v8 = zmul(v8, v8);
    v8 = zmul(v8, v8);
    v8 = zmul(v8, v8);
#pragma unroll
    for (int q = 0; q < kPer; ++q) {
      const double2 a = zmul(cj, pw);
      const double2 g = zmul(cvb, pw);
      C[q].x += a.x;
      C[q].y += a.y;
      E[q].x += ej * pw.x;
      E[q].y += ej * pw.y;
      G[q].x += g.x;
      G[q].y += g.y;
      pw = zmul(pw, v8);
    }
  }
#pragma unroll
  for (int q = 0; q < kPer; ++q) {
    for (int o = 16; o > 0; o >>= 1) {
      C[q].x += __shfl_xor_sync(0xffffffffu, C[q].x, o);
      C[q].y += __shfl_xor_sync(0xffffffffu, C[q].y, o);
      E[q].x += __shfl_xor_sync(0xffffffffu, E[q].x, o);
      E[q].y += __shfl_xor_sync(0xffffffffu, E[q].y, o);
      G[q].x += __shfl_xor_sync(0xffffffffu, G[q].x, o);
      G[q].y += __shfl_xor_sync(0xffffffffu, G[q].y, o);
    }
    const int k = warp + 8 * q;
    if (lane == 0 && k <= kDLPMax) {
      DLMom m;
      m.c = make_float2((float)C[q].x, (float)C[q].y);
      m.e = make_float2((float)E[q].x, (float)E[q].y);
      m.c1 = make_float2((float)((k + 1) * C[q].x), (float)((k + 1) * C[q].y));
      m.g1 = make_float2((float)((k + 1) * G[q].x), (float)((k + 1) * G[q].y));
      mom[(long long)s * (kDLPMax + 1) + k] = m;
    }
  }
}

// target columns: centre (hi/lo) and FP32 local coordinates
__global__ void __launch_bounds__(256) dl_mp_targets_kernel(int ntp, const double* __restrict__ X,
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
  for (int j = t; j < ntp; j += 256)
    local[(long long)k * ntp + j] = make_float2((float)(x[j] - cx), (float)(x[ntp + j] - cy));
  if (t == 0) {
    const float hx = (float)cx, hy = (float)cy;
    chi[k] = make_float2(hx, hy);
    clo[k] = make_float2((float)(cx - (double)hx), (float)(cy - (double)hy));
  }
}

struct DLMPArgs {
  int nsrc, ns, ntp;
  const float4* recA;  // [nsrc][ns] local x, y, normal x, y
  const float2* recB;  // [nsrc][ns] mean-free density
  const double* Xsrc;  // the FP64 sources (targets within 6 spacings)
  const double* tang;
  const double* den;
  const double* Xtar;
  const DLSrc* src;
  const DLMom* mom;
  const float2* tloc;
  const float2* thi;
  const float2* tlo;
  const int* self_idx;
  const int* cand_count;
  const int* cand_src;
  const uint32_t* excl_mask;
  int maxc, nwords;
  double* out;
};

// smallest P with rho^(P+1) ((P+2)(1-rho) + rho) / (1-rho)^2 <= eps (the
// (k+1)-weighted tail; it also bounds the plain one)
__device__ __forceinline__ int dl_order(float rp) {
  float pw = rp;  // rho^(P+1)
  const float om = 1.f - rp;
  for (int P = 1; P <= kDLPMax; ++P) {
    pw *= rp;
    if (pw * ((P + 2) * om + rp) <= kDLEps * om * om) return P;
  }
  return kDLPMax;
}

// One CTA per target column (blockDim = ntp rounded up to a warp multiple, <= 128).
// Dynamic shared memory: the direct-rule records of one source (ns float4 + ns float2).
__global__ void __launch_bounds__(128) dl_mp_eval_kernel(DLMPArgs p) {
  extern __shared__ __align__(16) float4 dA[];
  float2* dB = reinterpret_cast<float2*>(dA + p.ns);
  __shared__ DLSrc ssrc[kDLStage];
  __shared__ DLMom smom[kDLStage][kDLPMax + 1];
  __shared__ float rmax_w[4];
  const int col = blockIdx.x, i = threadIdx.x;
  const bool valid = i < p.ntp;
  const float2 tl = valid ? p.tloc[(long long)col * p.ntp + i] : make_float2(0.f, 0.f);
  const float2 thi = p.thi[col], tlo = p.tlo[col];
  const double txa = valid ? p.Xtar[(long long)col * 2 * p.ntp + i] : 0.0;
  const double tya = valid ? p.Xtar[(long long)col * 2 * p.ntp + p.ntp + i] : 0.0;
  float rt = sqrtf(tl.x * tl.x + tl.y * tl.y);
  for (int o = 16; o > 0; o >>= 1) rt = fmaxf(rt, __shfl_xor_sync(0xffffffffu, rt, o));
  if ((i & 31) == 0) rmax_w[i >> 5] = rt;
  __syncthreads();
  float RT = 0.f;
  for (int w = 0; w < (int)(blockDim.x >> 5); ++w) RT = fmaxf(RT, rmax_w[w]);
  RT *= 1.0f + 1e-6f;
  const int self = p.self_idx ? p.self_idx[col] : -1;
  const int cend = p.cand_count ? min(p.cand_count[col], p.maxc) : 0;
  const int* cands = p.cand_src ? p.cand_src + (long long)col * p.maxc : nullptr;
  int cur = 0;
  double ax = 0.0, ay = 0.0;  // pi * u
  for (int s0 = 0; s0 < p.nsrc; s0 += kDLStage) {
    const int nst = min(kDLStage, p.nsrc - s0);
    __syncthreads();
    for (int q = i; q < nst; q += blockDim.x) ssrc[q] = p.src[s0 + q];
    for (int q = i; q < nst * (kDLPMax + 1); q += blockDim.x)
      (&smom[0][0])[q] = p.mom[(long long)s0 * (kDLPMax + 1) + q];
    __syncthreads();
    for (int q = 0; q < nst; ++q) {
      const int s = s0 + q;
      if (s == self) continue;
      const DLSrc S = ssrc[q];
      bool cand = false;
      int cidx = 0;
      if (cend > 0) {
        while (cur < cend && cands[cur] < s) ++cur;
        cand = cur < cend && cands[cur] == s;
        cidx = cur;
      }
      if (S.skip) continue;
      const float ox = (thi.x - S.chi.x) + (tlo.x - S.clo.x);
      const float oy = (thi.y - S.chi.y) + (tlo.y - S.clo.y);
      const float dc = sqrtf(ox * ox + oy * oy) - RT;
      const float rp = dc > 0.f ? S.R / dc : 2.f;
      if (!cand && rp <= kDLRhoMax) {
        const int P = dl_order(rp);
        const float wx = tl.x + ox, wy = tl.y + oy;  // omega
        const float om2 = fmaf(wx, wx, wy * wy);
        const float iom2 = 1.0f / om2;
        const float iwr = wx * iom2, iwi = -wy * iom2;       // 1 / omega
        const float ur = S.R * iwr, ui = S.R * iwi;          // tau = R / omega
        float2 h1 = smom[q][P].c, h2 = smom[q][P].e, h3 = smom[q][P].c1, h4 = smom[q][P].g1;
        for (int k = P - 1; k >= 0; --k) {
          const DLMom m = smom[q][k];
          float2 n;
          n.x = fmaf(h1.x, ur, fmaf(-h1.y, ui, m.c.x));
          n.y = fmaf(h1.x, ui, fmaf(h1.y, ur, m.c.y));
          h1 = n;
          n.x = fmaf(h2.x, ur, fmaf(-h2.y, ui, m.e.x));
          n.y = fmaf(h2.x, ui, fmaf(h2.y, ur, m.e.y));
          h2 = n;
          n.x = fmaf(h3.x, ur, fmaf(-h3.y, ui, m.c1.x));
          n.y = fmaf(h3.x, ui, fmaf(h3.y, ur, m.c1.y));
          h3 = n;
          n.x = fmaf(h4.x, ur, fmaf(-h4.y, ui, m.g1.x));
          n.y = fmaf(h4.x, ui, fmaf(h4.y, ur, m.g1.y));
          h4 = n;
        }
        // t1 = h1 / omega, t2 = conj(h2 / omega)
        const float t1r = h1.x * iwr - h1.y * iwi, t1i = h1.x * iwi + h1.y * iwr;
        const float t2r = h2.x * iwr - h2.y * iwi, t2i = -(h2.x * iwi + h2.y * iwr);
        // t3 = (omega / conj(omega)^2) conj(h3) = omega conj(1/omega)^2 conj(h3)
        const float qbr = iwr * iwr - iwi * iwi, qbi = -2.f * iwr * iwi;  // conj(1/omega)^2
        const float qr = wx * qbr - wy * qbi, qi = wx * qbi + wy * qbr;
        const float t3r = qr * h3.x + qi * h3.y, t3i = qi * h3.x - qr * h3.y;
        // t4 = R conj(h4 / omega^2)
        const float i2r = iwr * iwr - iwi * iwi, i2i = 2.f * iwr * iwi;   // 1/omega^2
        const float t4r = S.R * (h4.x * i2r - h4.y * i2i), t4i = -S.R * (h4.x * i2i + h4.y * i2r);
        if (valid) {
          ax += 0.25 * (double)(t1r + t2r + t3r - t4r);
          ay += 0.25 * (double)(t1i + t2i + t3i - t4i);
        }
      } else {
        // direct rule over the upsampled points, FP32, coordinates relative to the source centre
        __syncthreads();
        const float4* A4 = p.recA + (long long)s * p.ns;
        const float2* B2 = p.recB + (long long)s * p.ns;
        for (int j = i; j < p.ns; j += blockDim.x) {
          dA[j] = A4[j];
          dB[j] = B2[j];
        }
        __syncthreads();
        bool excl = !valid;
        if (cand && valid) {
          const uint32_t w = p.excl_mask[((long long)col * p.maxc + cidx) * p.nwords + (i >> 5)];
          excl = (w >> (i & 31)) & 1u;
        }
        if (!excl) {
          const float tx = tl.x + ox, ty = tl.y + oy;
          float bx = 0.f, by = 0.f, dmin = 3.0e38f;
#pragma unroll 4
          for (int j = 0; j < p.ns; ++j) {
            const float4 a = dA[j];
            const float2 b = dB[j];
            const float dx = tx - a.x, dy = ty - a.y;
            const float d2 = fmaf(dx, dx, dy * dy);
            dmin = fminf(dmin, d2);
            const float inv = 1.0f / d2;
            const float c = fmaf(dx, a.z, dy * a.w) * fmaf(dx, b.x, dy * b.y) * (inv * inv);
            bx = fmaf(c, dx, bx);
            by = fmaf(c, dy, by);
          }
          if (dmin >= S.thr2) {
            ax += (double)bx;
            ay += (double)by;
          } else {  // within 12 spacings: the full density in FP64
            const double* xs = p.Xsrc + (long long)s * 2 * p.ns;
            const double* ts = p.tang + (long long)s * 2 * p.ns;
            const double* ds = p.den + (long long)s * 2 * p.ns;
            double cx = 0.0, cy = 0.0;
            for (int j = 0; j < p.ns; ++j) {
              const double dx = txa - xs[j], dy = tya - xs[p.ns + j];
              const double d2 = dx * dx + dy * dy;
              const double c = ((dx * ts[p.ns + j] - dy * ts[j]) / (d2 * d2)) * (dx * ds[j] + dy * ds[p.ns + j]);
              cx = fma(c, dx, cx);
              cy = fma(c, dy, cy);
            }
            ax += cx;
            ay += cy;
          }
        }
      }
    }
  }
  if (valid) {
    p.out[(long long)col * 2 * p.ntp + i] = ax / VES_PI;
    p.out[(long long)col * 2 * p.ntp + p.ntp + i] = ay / VES_PI;
  }
}

}  // namespace

int farfield_dl_mp_run(ves_ctx* c, int nsrc, int ns, const double* Xsrc, const double* tang, const double* den,
                       const double* sa, const double* visc, int nt, int ntp, const double* Xtar,
                       const int* self_idx, const ves_near_lists* nl, double* out, WsCarver& ws, cudaStream_t s) {
  DLSrc* src = ws.take<DLSrc>(nsrc > 0 ? nsrc : 1);
  DLMom* mom = ws.take<DLMom>((size_t)(nsrc > 0 ? nsrc : 1) * (kDLPMax + 1));
  float4* recA = ws.take<float4>((size_t)(nsrc > 0 ? nsrc : 1) * ns);
  float2* recB = ws.take<float2>((size_t)(nsrc > 0 ? nsrc : 1) * ns);
  float2* tloc = ws.take<float2>((size_t)(nt > 0 ? nt : 1) * (ntp > 0 ? ntp : 1));
  float2* thi = ws.take<float2>(nt > 0 ? nt : 1);
  float2* tlo = ws.take<float2>(nt > 0 ? nt : 1);
  if (ws.sizing) return VES_OK;
  if (!ws.ok()) {
    ves_record_error(VES_ERR_WORKSPACE, "farfield_dl: workspace too small");
    return VES_ERR_WORKSPACE;
  }
  if (ntp <= 0 || ntp > 128) {
    ves_record_error(VES_ERR_SHAPE, "farfield_dl: the multipole path takes 1..128 points per target column");
    return VES_ERR_SHAPE;
  }
  if (nl && (!nl->cand_count || !nl->cand_src || !nl->excl_mask || nl->maxc <= 0 || nt != nsrc ||
             (c && ntp != c->N))) {
    ves_record_error(VES_ERR_ARG, "farfield_dl: near lists need nt == nsrc and ntp == N");
    return VES_ERR_ARG;
  }
  if (nt == 0) return VES_OK;
  if (nsrc == 0) return ves_cuda_status(cudaMemsetAsync(out, 0, (size_t)nt * 2 * ntp * sizeof(double), s), "dl zero");
  if (!sa) {
    ves_record_error(VES_ERR_ARG, "farfield_dl: the multipole path needs the source jacobian sa");
    return VES_ERR_ARG;
  }
  const size_t dsmem = (size_t)ns * (sizeof(float4) + sizeof(float2));
  if (dsmem > 200 * 1024) {
    ves_record_error(VES_ERR_SHAPE, "farfield_dl: %d source points per vesicle exceed the multipole path", ns);
    return VES_ERR_SHAPE;
  }
  if (dsmem > 32 * 1024) {  // with the ~13 KB of static shared memory, past the 48 KB default
    const int rc = ves_cuda_status(
        cudaFuncSetAttribute(dl_mp_eval_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)dsmem), "dl smem");
    if (rc) return rc;
  }
  ves_count_launch(3);
  dl_mp_prep_kernel<<<nsrc, 256, 0, s>>>(ns, Xsrc, tang, den, sa, visc, src, mom, recA, recB);
  dl_mp_targets_kernel<<<nt, 256, 0, s>>>(ntp, Xtar, tloc, thi, tlo);
  DLMPArgs a;
  a.nsrc = nsrc;
  a.ns = ns;
  a.ntp = ntp;
  a.recA = recA;
  a.recB = recB;
  a.Xsrc = Xsrc;
  a.tang = tang;
  a.den = den;
  a.Xtar = Xtar;
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
  a.nwords = (ntp + 31) / 32;
  a.out = out;
  dl_mp_eval_kernel<<<nt, ((ntp + 31) / 32) * 32, dsmem, s>>>(a);
  return ves_launch_check("farfield_dl multipole");
}

int farfield_dl_mp_run(ves_ctx* c, int nsrc, int ns, const double* Xsrc, const double* tang, const double* den,
                       const double* sa, const double* visc, int nt, int ntp, const double* Xtar,
                       const int* self_idx, const ves_near_lists* nl, double* out, WsCarver& ws, cudaStream_t s);

int farfield_dl_run(ves_ctx* c, int precision, int nsrc, int ns, const double* Xsrc, const double* tang,
                    const double* den, const double* sa, const double* visc, int nt, int ntp, const double* Xtar,
                    const int* self_idx, const ves_near_lists* nl, double* out, WsCarver& ws, cudaStream_t s) {
  if (precision == VES_PREC_FP64) {
    if (ws.sizing) return VES_OK;
    return farfield_dl_direct_run(c, nsrc, ns, Xsrc, tang, den, nt, ntp, Xtar, self_idx, nl, out, s);
  }
  if (precision == VES_PREC_FP32C || precision == VES_PREC_FP32M)
    return farfield_dl_mp_run(c, nsrc, ns, Xsrc, tang, den, sa, visc, nt, ntp, Xtar, self_idx, nl, out, ws, s);
  ves_record_error(VES_ERR_ARG, "farfield_dl: bad precision %d", precision);
  return VES_ERR_ARG;
}

// ---------------------------------------------------------------------------
extern "C" int ves_upsample_geometry(ves_ctx* c, int nv, const double* X, double* Xup, double* sa, double* tang,
                                     double* cur, void* stream) {
  if (!c || nv < 0 || (nv > 0 && !X)) {
    ves_record_error(VES_ERR_ARG, "upsample_geometry: bad arguments");
    return VES_ERR_ARG;
  }
  launch_upsample_geom(c, nv, X, Xup, sa, tang, cur, (cudaStream_t)stream);
  return ves_launch_check("upsample_geometry");
}

extern "C" size_t ves_stokes_dl_matrix_workspace(ves_ctx* c, int nv, int precision) {
  if (!c) return 0;
  WsCarver w(nullptr, 0);
  stokes_dl_matrix(c, nv, nullptr, nullptr, precision, nullptr, w, 0);
  return w.off + 256;
}

extern "C" int ves_stokes_dl_matrix(ves_ctx* c, int nv, const double* X, const double* visc, int precision,
                                    double* D, void* ws, size_t ws_bytes, void* stream) {
  if (!c || nv < 0 || (nv > 0 && (!X || !visc || !D || !ws))) {
    ves_record_error(VES_ERR_ARG, "stokes_dl_matrix: bad arguments");
    return VES_ERR_ARG;
  }
  if (precision != VES_PREC_FP64 && precision != VES_PREC_FP32C) {
    ves_record_error(VES_ERR_ARG, "stokes_dl_matrix: precision must be fp64 or fp32c");
    return VES_ERR_ARG;
  }
  WsCarver w(ws, ws_bytes);
  return stokes_dl_matrix(c, nv, X, visc, precision, D, w, (cudaStream_t)stream);
}

extern "C" int ves_dl_density(int nv, int ns, const double* f, const double* sa, const double* visc, double* den,
                              void* stream) {
  if (nv < 0 || ns <= 0 || (nv > 0 && (!f || !sa || !den))) {
    ves_record_error(VES_ERR_ARG, "dl_density: bad arguments");
    return VES_ERR_ARG;
  }
  launch_dl_density(nv, ns, f, sa, visc, den, (cudaStream_t)stream);
  return ves_launch_check("dl_density");
}

extern "C" size_t ves_farfield_dl_workspace(int precision, int nsrc, int nt, int ntp) {
  WsCarver w(nullptr, 0);
  farfield_dl_run(nullptr, precision, nsrc, 1, nullptr, nullptr, nullptr, nullptr, nullptr, nt, ntp, nullptr, nullptr,
                  nullptr, nullptr, w, 0);
  return w.off + 256;
}

extern "C" int ves_farfield_dl(ves_ctx* c, int precision, int nsrc, int ns, const double* Xsrc, const double* tang,
                               const double* den, const double* sa, const double* visc, int nt, int ntp,
                               const double* Xtar, const int* self_idx, const ves_near_lists* nl, double* out,
                               void* ws, size_t ws_bytes, void* stream) {
  if (nt > 0 && (!Xtar || !out || (nsrc > 0 && (!Xsrc || !tang || !den)))) {
    ves_record_error(VES_ERR_ARG, "farfield_dl: bad arguments");
    return VES_ERR_ARG;
  }
  WsCarver w(ws, ws_bytes);
  return farfield_dl_run(c, precision, nsrc, ns, Xsrc, tang, den, sa, visc, nt, ntp, Xtar, self_idx, nl, out, w,
                         (cudaStream_t)stream);
}
