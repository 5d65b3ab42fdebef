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

int farfield_dl_run(ves_ctx* c, int nsrc, int ns, const double* Xsrc, const double* tang, const double* den, int nt,
                    int ntp, const double* Xtar, const int* self_idx, const ves_near_lists* nl, double* out,
                    cudaStream_t s) {
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

extern "C" int ves_farfield_dl(ves_ctx* c, int nsrc, int ns, const double* Xsrc, const double* tang, const double* den,
                               int nt, int ntp, const double* Xtar, const int* self_idx, const ves_near_lists* nl,
                               double* out, void* stream) {
  if (nt > 0 && (!Xtar || !out || (nsrc > 0 && (!Xsrc || !tang || !den)))) {
    ves_record_error(VES_ERR_ARG, "farfield_dl: bad arguments");
    return VES_ERR_ARG;
  }
  return farfield_dl_run(c, nsrc, ns, Xsrc, tang, den, nt, ntp, Xtar, self_idx, nl, out, (cudaStream_t)stream);
}
