// Alpert log-singular single-layer matrix (Poten.stokesSLmatrix,
// mytorch/poten.py:40-99, weights poten.py:899-974).
//
// For target s of the Nup-upsampled curve the quadrature has 14 off-grid
// nodes (7 on each side, at offsets +-v_q*h) whose positions come from the
// trig interpolant, and Nup-9 on-grid nodes s+i, i = 5..Nup-5.  With
// F_q(s) = w_q * {1/2 log rho, dx^2 rho, dx dy rho, dy^2 rho},
// rho = 1/(|x_s - node|^2 + 1e-7), the row of the Nup x Nup matrix is
//   W(s, i) = [5 <= i <= Nup-5] F_{i+2}(s) + sum_{dense q} A_q(i) F_q(s),
//   Gup[s][(s+i) mod Nup] = sa_up[(s+i) mod Nup] * W(s, i),
// and G = R * Gup * P restricts it to the N-point grid.
#include "ves_internal.h"

template <typename T>
__device__ __forceinline__ T tlog(T x);
template <>
__device__ __forceinline__ float tlog<float>(float x) { return logf(x); }
template <>
__device__ __forceinline__ double tlog<double>(double x) { return log(x); }

// Kernel A: per (vesicle, target s) the 14 off-grid node field values.
template <typename T>
__global__ void alpert_dense_nodes_kernel(int N, int Nup, int m, int nquad, const double* __restrict__ X,
                                          const double* __restrict__ Xup, const double* __restrict__ cq,
                                          const double* __restrict__ qw, T* __restrict__ Fd) {
  extern __shared__ double sh[];
  double* x = sh;
  double* y = x + N;
  const int k = blockIdx.y;
  for (int i = threadIdx.x; i < N; i += blockDim.x) {
    x[i] = X[(long long)k * 2 * N + i];
    y[i] = X[(long long)k * 2 * N + N + i];
  }
  __syncthreads();
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= Nup) return;
  const double xs = Xup[(long long)k * 2 * Nup + s], ys = Xup[(long long)k * 2 * Nup + Nup + s];
  T* out = Fd + ((long long)k * Nup + s) * 56;
  for (int q = 0; q < 14; ++q) {
    const double* cr = cq + (long long)q * Nup;
    double nx = 0, ny = 0;
    int r = s;
    for (int i = 0; i < N; ++i) {
      nx = fma(cr[r], x[i], nx);
      ny = fma(cr[r], y[i], ny);
      r -= m;
      if (r < 0) r += Nup;
    }
    const T dx = (T)(xs - nx), dy = (T)(ys - ny);
    const T rho = T(1) / (dx * dx + dy * dy + T(1e-7));
    const T w = (T)(q < 7 ? qw[q] : qw[nquad - 14 + q]);
    out[q * 4 + 0] = T(0.5) * w * tlog<T>(rho);
    out[q * 4 + 1] = w * dx * dx * rho;
    out[q * 4 + 2] = w * dx * dy * rho;
    out[q * 4 + 3] = w * dy * dy * rho;
  }
}

// Kernel B: rows of Gup (three fields G11, G12, G22) for ROWS targets per CTA.
template <typename T, int ROWS>
__global__ void __launch_bounds__(256) alpert_rows_kernel(int Nup, int nquad, const double* __restrict__ Xup,
                                                          const double* __restrict__ sa_up,
                                                          const T* __restrict__ adense,
                                                          const double* __restrict__ qw,
                                                          const T* __restrict__ Fd, T* __restrict__ Gup,
                                                          int k0) {
  __shared__ T fd[ROWS][56];
  __shared__ double txs[ROWS], tys[ROWS];
  const int kl = blockIdx.y;        // vesicle within chunk
  const int k = k0 + kl;            // global vesicle
  const int s0 = blockIdx.x * ROWS;
  for (int idx = threadIdx.x; idx < ROWS * 56; idx += blockDim.x) {
    const int r = idx / 56, e = idx % 56;
    fd[r][e] = (s0 + r < Nup) ? Fd[((long long)k * Nup + s0 + r) * 56 + e] : T(0);
  }
  if (threadIdx.x < ROWS) {
    const int s = min(s0 + threadIdx.x, Nup - 1);
    txs[threadIdx.x] = Xup[(long long)k * 2 * Nup + s];
    tys[threadIdx.x] = Xup[(long long)k * 2 * Nup + Nup + s];
  }
  __syncthreads();
  const T wg = (T)qw[7];  // on-grid weight h/(4 pi)
  const double* xk = Xup + (long long)k * 2 * Nup;
  const double* sak = sa_up + (long long)k * Nup;
  const long long NN = (long long)Nup * Nup;
  T* G11 = Gup + (long long)kl * 3 * NN;
  T* G12 = G11 + NN;
  T* G22 = G12 + NN;
  for (int i = threadIdx.x; i < Nup; i += blockDim.x) {
    T a[14];
#pragma unroll
    for (int q = 0; q < 14; ++q) a[q] = adense[(long long)q * Nup + i];
    const bool grid = (i >= 5 && i <= Nup - 5);
#pragma unroll
    for (int r = 0; r < ROWS; ++r) {
      const int s = s0 + r;
      if (s >= Nup) break;
      T wl = 0, wxx = 0, wxy = 0, wyy = 0;
#pragma unroll
      for (int q = 0; q < 14; ++q) {
        wl += a[q] * fd[r][q * 4 + 0];
        wxx += a[q] * fd[r][q * 4 + 1];
        wxy += a[q] * fd[r][q * 4 + 2];
        wyy += a[q] * fd[r][q * 4 + 3];
      }
      int col = s + i;
      if (col >= Nup) col -= Nup;
      if (grid) {
        const T dx = (T)(txs[r] - xk[col]), dy = (T)(tys[r] - xk[Nup + col]);
        const T rho = T(1) / (dx * dx + dy * dy + T(1e-7));
        wl += T(0.5) * wg * tlog<T>(rho);
        wxx += wg * dx * dx * rho;
        wxy += wg * dx * dy * rho;
        wyy += wg * dy * dy * rho;
      }
      const T sa = (T)sak[col];
      const long long o = (long long)s * Nup + col;
      G11[o] = (wl + wxx) * sa;
      G12[o] = wxy * sa;
      G22[o] = (wl + wyy) * sa;
    }
  }
}

template <typename T>
__global__ void alpert_assemble_kernel(int N, const T* __restrict__ Gf, double* __restrict__ G, int k0) {
  const int kl = blockIdx.y;
  const long long NN = (long long)N * N;
  const T* g11 = Gf + (long long)kl * 3 * NN;
  const T* g12 = g11 + NN;
  const T* g22 = g12 + NN;
  double* Gk = G + (long long)(k0 + kl) * 4 * NN;
  for (int idx = blockIdx.x * blockDim.x + threadIdx.x; idx < 4 * NN; idx += gridDim.x * blockDim.x) {
    const int r = idx / (2 * N), c = idx % (2 * N);
    const int i = r % N, j = c % N;
    const T* src = (r < N) ? ((c < N) ? g11 : g12) : ((c < N) ? g12 : g22);
    Gk[idx] = (double)src[(long long)i * N + j];
  }
}

__global__ void nonfinite_check_kernel(long long n, const double* __restrict__ a, VesDeviceStatus* st) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    if (!isfinite(a[i])) {
      ves_set_error(st, VES_ERR_NONFINITE, 2, i);
      return;
    }
}

static int alpert_chunk(const ves_ctx* c, int nv, int precision) {
  const size_t es = precision == VES_PREC_FP64 ? 8 : 4;
  const size_t per = (size_t)3 * c->Nup * c->Nup * es;
  size_t budget = (size_t)2 << 30;  // ~2 GiB of Gup per chunk
  int ch = (int)(budget / per);
  if (ch < 1) ch = 1;
  if (ch > nv) ch = nv;
  return ch;
}

template <typename T>
static int alpert_impl(ves_ctx* c, int nv, const double* X, double* G, WsCarver& ws, cudaStream_t s) {
  const int N = c->N, Nup = c->Nup;
  const int chunk = alpert_chunk(c, nv, sizeof(T) == 8 ? VES_PREC_FP64 : VES_PREC_FP32C);
  double* Xup = ws.take<double>((size_t)nv * 2 * Nup);
  double* sa_up = ws.take<double>((size_t)nv * Nup);
  T* Fd = ws.take<T>((size_t)nv * Nup * 56);
  T* Gup = ws.take<T>((size_t)chunk * 3 * Nup * Nup);
  T* Tm = ws.take<T>((size_t)chunk * 3 * Nup * N);
  T* Gf = ws.take<T>((size_t)chunk * 3 * N * N);
  if (ws.sizing) return VES_OK;
  if (!ws.ok()) {
    ves_record_error(VES_ERR_WORKSPACE, "stokes_sl_matrix: workspace too small");
    return VES_ERR_WORKSPACE;
  }
  if (nv <= 0) return VES_OK;
  launch_upsample_deriv(c, nv, X, Xup, nullptr, sa_up, s);
  {
    dim3 grid(ceil_div(Nup, 128), nv);
    ves_count_launch();
    alpert_dense_nodes_kernel<T><<<grid, 128, (size_t)2 * N * sizeof(double), s>>>(N, Nup, c->m, c->nquad, X,
                                                                                   Xup, c->cq, c->qw, Fd);
  }
  const T* adense = (const T*)(sizeof(T) == 8 ? (const void*)c->adense : (const void*)c->adense32);
  const T* Pm = (const T*)(sizeof(T) == 8 ? (const void*)c->Pm : (const void*)c->Pm32);
  const T* Rm = (const T*)(sizeof(T) == 8 ? (const void*)c->Rm : (const void*)c->Rm32);
  constexpr int ROWS = 8;
  for (int k0 = 0; k0 < nv; k0 += chunk) {
    const int nk = min(chunk, nv - k0);
    dim3 grid(ceil_div(Nup, ROWS), nk);
    ves_count_launch();
    alpert_rows_kernel<T, ROWS><<<grid, 256, 0, s>>>(Nup, c->nquad, Xup, sa_up, adense, c->qw, Fd, Gup, k0);
    const long long NN = (long long)Nup * Nup;
    // T = Gup * P for the 3*nk fields; Gf = R * T
    if (sizeof(T) == 8) {
      launch_bgemm_f64(3 * nk, Nup, N, Nup, 1.0, (const double*)Gup, Nup, NN, (const double*)Pm, N, 0, 0.0,
                       (double*)Tm, N, (long long)Nup * N, s);
      launch_bgemm_f64(3 * nk, N, N, Nup, 1.0, (const double*)Rm, Nup, 0, (const double*)Tm, N,
                       (long long)Nup * N, 0.0, (double*)Gf, N, (long long)N * N, s);
    } else {
      launch_bgemm_f32(3 * nk, Nup, N, Nup, 1.0f, (const float*)Gup, Nup, NN, (const float*)Pm, N, 0, 0.0f,
                       (float*)Tm, N, (long long)Nup * N, s);
      launch_bgemm_f32(3 * nk, N, N, Nup, 1.0f, (const float*)Rm, Nup, 0, (const float*)Tm, N,
                       (long long)Nup * N, 0.0f, (float*)Gf, N, (long long)N * N, s);
    }
    dim3 ga(ceil_div(4LL * N * N, 256), nk);
    ves_count_launch();
    alpert_assemble_kernel<T><<<ga, 256, 0, s>>>(N, Gf, G, k0);
  }
  ves_count_launch();
  nonfinite_check_kernel<<<256, 256, 0, s>>>((long long)nv * 4 * N * N, G, c->status);
  return ves_launch_check("stokes_sl_matrix");
}

int alpert_sl_matrix(ves_ctx* c, int nv, const double* X, int precision, double* G, WsCarver& ws,
                     cudaStream_t s) {
  if (precision == VES_PREC_FP64) return alpert_impl<double>(c, nv, X, G, ws, s);
  if (precision == VES_PREC_FP32C) return alpert_impl<float>(c, nv, X, G, ws, s);
  ves_record_error(VES_ERR_ARG, "stokes_sl_matrix: bad precision %d", precision);
  return VES_ERR_ARG;
}
