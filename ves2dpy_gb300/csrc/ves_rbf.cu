// Near-field correction by Gaussian RBF fits (nearSingInt_rbf,
// mytorch/poten.py:643-785; nearFieldCorrectionUP_SOLVE :788-894;
// exactStokesSL_onlyself biem_support.py:468-516), the near-singular scheme of
// the newtorch BIEM step (newtorch/tstep_biem.py:431).
//
// The far field arrives with the near (target point, source vesicle) pairs
// excluded (the compare2 exclusions of naiveNearZoneInfo).  For a source
// vesicle v the reference fits its own single-layer velocity on three layers
// of N points -- the boundary (velocity vself = G f) and two copies shifted by
// 1/(2N) and 1/N along the outward normal (ty, -tx) of the coarse curve, where
// the self single layer is summed over the curve and density upsampled to
// M = N*2*ceil(sqrt(2N)) points -- with Gaussians exp(-|p - q|^2 / w^2)
// centred at those 3N points (w = 0.672 for N = 32, 0.0132 otherwise;
// diagonal 1e-6), and adds the fit, evaluated at the target point, for each
// near pair.  Only the fits of source vesicles that have near pairs are
// computed (the others are never evaluated).
//
// Kernels: rbf_flag / rbf_compact pick the vesicles to fit; rbf_layers (one
// CTA per fitted vesicle) upsamples by FP64 FFTs in shared memory and sums the
// layer velocities; rbf_matrix builds the Gaussian matrices, which the
// batched FP64 LU of ves_blas.cu factors and solves (the reference uses a
// Cholesky factorisation of the same symmetric matrices); rbf_correct (one
// warp per target vesicle, candidates in list order, no atomics) adds the
// fits at the near target points.
#include "ves_internal.h"
#include "ves_fft.cuh"

namespace {

constexpr int kLayers = 3;
constexpr int kChunk = 256;  // fits per pass (bounds the workspace: kChunk (3N)^2 doubles)

__host__ __device__ inline int rbf_fine(int N) {
  int c = 1;
  while (c * c < (kLayers - 1) * N) ++c;
  return N * (kLayers - 1) * c;
}
__host__ __device__ inline double rbf_width(int N) { return N == 32 ? 0.672 : 0.0132; }

__global__ void rbf_twiddle_kernel(int M, double* __restrict__ cs, double* __restrict__ sn) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j < M) sincospi(2.0 * j / M, &sn[j], &cs[j]);
}

// need[v] = 1 when some target point has source vesicle v as a near pair
__global__ void rbf_flag_kernel(int nv, int maxc, int nwords, const int* __restrict__ cand_count,
                                const int* __restrict__ cand_src, const uint32_t* __restrict__ excl,
                                int* __restrict__ need) {
  const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= (long long)nv * maxc) return;
  const int k = (int)(e / maxc), c = (int)(e % maxc);
  if (c >= min(cand_count[k], maxc)) return;
  uint32_t any = 0;
  for (int w = 0; w < nwords; ++w) any |= excl[e * nwords + w];
  if (any) need[cand_src[e]] = 1;
}

// list of flagged vesicles (ascending) and slot[v] = position in it or -1;
// count[0] = number of fits.  One CTA of 1024 threads.
__global__ void __launch_bounds__(1024) rbf_compact_kernel(int nv, const int* __restrict__ need,
                                                           int* __restrict__ list, int* __restrict__ slot,
                                                           int* __restrict__ count) {
  __shared__ int base;
  __shared__ int wsum[32];
  if (threadIdx.x == 0) base = 0;
  __syncthreads();
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int v0 = 0; v0 < nv; v0 += blockDim.x) {
    const int v = v0 + threadIdx.x;
    const int fl = v < nv ? need[v] : 0;
    const unsigned m = __ballot_sync(0xffffffffu, fl);
    if (lane == 0) wsum[warp] = __popc(m);
    __syncthreads();
    int off = base;
    for (int w = 0; w < warp; ++w) off += wsum[w];
    off += __popc(m & ((1u << lane) - 1u));
    if (v < nv) {
      slot[v] = fl ? off : -1;
      if (fl) list[off] = v;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      int t = 0;
      for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += wsum[w];
      base += t;
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) count[0] = base;
}

// fine spectrum (unnormalised) of the trigonometric interpolant of a coarse
// spectrum (zr, zi) of length N on M points; derivative when deriv != 0.  The
// coarse Nyquist coefficient is split over +-N/2 (interpft's real interpolant).
__device__ __forceinline__ void fine_spectrum(int N, int M, const double* zr, const double* zi, int deriv, double* re,
                                              double* im) {
  for (int j = threadIdx.x; j < M; j += blockDim.x) {
    const int k = j < M / 2 ? j : j - M;
    double r = 0, i = 0;
    if (k > -N / 2 && k < N / 2) {
      const int c = k >= 0 ? k : k + N;
      r = zr[c];
      i = zi[c];
    } else if (k == N / 2 || k == -N / 2) {
      r = 0.5 * zr[N / 2];
      i = 0.5 * zi[N / 2];
    }
    if (deriv) {
      const double t = r;
      r = -k * i;
      i = k * t;
    }
    re[j] = r;
    im[j] = i;
  }
}

// One CTA (256 threads) per fitted vesicle: layer points and velocities in the
// reference's (N, 3) flattening (row i*3 + l), x and y rows in separate arrays.
__global__ void __launch_bounds__(256) rbf_layers_kernel(int N, int M, const int* __restrict__ list, int first,
                                                         const double* __restrict__ X, const double* __restrict__ f,
                                                         const double* __restrict__ tang,
                                                         const double* __restrict__ vself,
                                                         const double* __restrict__ cs, const double* __restrict__ sn,
                                                         double* __restrict__ px, double* __restrict__ py,
                                                         double* __restrict__ velx, double* __restrict__ vely) {
  extern __shared__ double sm[];
  double* zr = sm;  // coarse spectra and scratch [N each]
  double* zi = zr + N;
  double* gr = zi + N;
  double* gi = gr + N;
  double* tr = gi + N;
  double* ti = tr + N;
  double* a0 = ti + N;  // fine arrays [M each]
  double* a1 = a0 + M;
  double* a2 = a1 + M;
  double* a3 = a2 + M;
  double* a4 = a3 + M;
  double* a5 = a4 + M;
  const int s = first + blockIdx.x;
  const int v = list[s];
  const int n = kLayers * N;
  const double* x = X + (long long)v * 2 * N;
  const double* fv = f + (long long)v * 2 * N;
  for (int j = threadIdx.x; j < N; j += blockDim.x) {
    zr[j] = x[j];
    zi[j] = x[N + j];
    gr[j] = fv[j];
    gi[j] = fv[N + j];
  }
  // coarse spectra of z = x + iy and g = fx + i fy (the fine table at stride M/N)
  ves_fft(zr, zi, tr, ti, N, cs, sn, -1, M / N);
  ves_fft(gr, gi, tr, ti, N, cs, sn, -1, M / N);
  // density on the fine grid -> a0, a1 (N times the values)
  fine_spectrum(N, M, gr, gi, 0, a0, a1);
  ves_fft(a0, a1, a2, a3, M, cs, sn, 1);
  // derivative of the curve -> a2, a3; jacobian -> density weights in a0, a1
  fine_spectrum(N, M, zr, zi, 1, a2, a3);
  ves_fft(a2, a3, a4, a5, M, cs, sn, 1);
  const double wq = 2.0 * VES_PI / M / ((double)N * N);  // quadrature weight, two factors 1/N
  for (int j = threadIdx.x; j < M; j += blockDim.x) {
    const double sa = sqrt(a2[j] * a2[j] + a3[j] * a3[j]);
    a0[j] *= sa * wq;
    a1[j] *= sa * wq;
  }
  // the curve itself -> a2, a3
  fine_spectrum(N, M, zr, zi, 0, a2, a3);
  ves_fft(a2, a3, a4, a5, M, cs, sn, 1);
  const double iN = 1.0 / N;
  for (int j = threadIdx.x; j < M; j += blockDim.x) {
    a2[j] *= iN;
    a3[j] *= iN;
  }
  __syncthreads();
  // layer 0: the boundary and vself
  for (int i = threadIdx.x; i < N; i += blockDim.x) {
    const long long o = (long long)s * n + i * kLayers;
    px[o] = x[i];
    py[o] = x[N + i];
    velx[o] = vself[(long long)v * 2 * N + i];
    vely[o] = vself[(long long)v * 2 * N + N + i];
  }
  // layers 1, 2: distances 1/(2N), 1/N along (ty, -tx); self single layer from the fine curve
  const double* tg = tang + (long long)v * 2 * N;
  for (int t = threadIdx.x; t < 2 * N; t += blockDim.x) {
    const int l = 1 + t / N, i = t % N;
    const double d = l == 1 ? 0.5 / N : 1.0 / N;
    const double qx = x[i] + tg[N + i] * d, qy = x[N + i] - tg[i] * d;
    double sx = 0, sy = 0, cxs = 0, cys = 0;
    for (int j = 0; j < M; ++j) {
      const double rx = qx - a2[j], ry = qy - a3[j];
      const double r2 = rx * rx + ry * ry;
      const double lg = 0.5 * log(r2);
      sx += lg * a0[j];
      sy += lg * a1[j];
      const double c = (rx * a0[j] + ry * a1[j]) / r2;
      cxs += c * rx;
      cys += c * ry;
    }
    const long long o = (long long)s * n + i * kLayers + l;
    px[o] = qx;
    py[o] = qy;
    velx[o] = (-sx + cxs) / (4.0 * VES_PI);
    vely[o] = (-sy + cys) / (4.0 * VES_PI);
  }
}

// Gaussian matrices of the fits in [first, first + cnt): A[s][a][b]
__global__ void rbf_matrix_kernel(int n, int first, int cnt, double w, const double* __restrict__ px,
                                  const double* __restrict__ py, double* __restrict__ A) {
  const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= (long long)cnt * n * n) return;
  const int s = (int)(e / ((long long)n * n));
  const int a = (int)((e / n) % n), b = (int)(e % n);
  const long long o = (long long)(first + s) * n;
  const double dx = px[o + a] / w - px[o + b] / w, dy = py[o + a] / w - py[o + b] / w;
  A[e] = exp(-(dx * dx + dy * dy)) + (a == b ? 1e-6 : 0.0);
}

// one warp per target vesicle: add the fits of its near pairs (fits in [first, first + cnt))
__global__ void rbf_correct_kernel(int N, int nv, int maxc, int nwords, int first, int cnt, double w,
                                   const int* __restrict__ cand_count, const int* __restrict__ cand_src,
                                   const uint32_t* __restrict__ excl, const int* __restrict__ slot,
                                   const double* __restrict__ X, const double* __restrict__ px,
                                   const double* __restrict__ py, const double* __restrict__ cx,
                                   const double* __restrict__ cy, double* __restrict__ LP) {
  const int k = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (k >= nv) return;
  const int n = kLayers * N;
  const int nc = min(cand_count[k], maxc);
  for (int c = 0; c < nc; ++c) {
    const long long e = (long long)k * maxc + c;
    const int sl = slot[cand_src[e]];
    if (sl < first || sl >= first + cnt) continue;
    const long long o = (long long)sl * n;
    for (int wd = 0; wd < nwords; ++wd) {
      uint32_t bits = excl[e * nwords + wd];
      while (bits) {
        const int i = wd * 32 + __ffs(bits) - 1;
        bits &= bits - 1;
        const double qx = X[(long long)k * 2 * N + i] / w, qy = X[(long long)k * 2 * N + N + i] / w;
        double sx = 0, sy = 0;
        for (int a = lane; a < n; a += 32) {
          const double dx = qx - px[o + a] / w, dy = qy - py[o + a] / w;
          const double g = exp(-(dx * dx + dy * dy));
          sx += g * cx[o + a];
          sy += g * cy[o + a];
        }
        for (int m = 16; m > 0; m >>= 1) {
          sx += __shfl_xor_sync(0xffffffffu, sx, m);
          sy += __shfl_xor_sync(0xffffffffu, sy, m);
        }
        if (lane == 0) {
          LP[(long long)k * 2 * N + i] += sx;
          LP[(long long)k * 2 * N + N + i] += sy;
        }
      }
    }
  }
}

}  // namespace

// Add the RBF near-field fits to LP ([nv][2][N], the far field without the
// near pairs).  X, f, vself: [nv][2][N]; nl: the py_hh near lists.
int rbf_near_correct(ves_ctx* c, int nv, const double* X, const double* f, const double* vself,
                     const ves_near_lists* nl, double* LP, WsCarver& ws, cudaStream_t s) {
  const int N = c->N, M = rbf_fine(N), n = kLayers * N;
  const int chunk = nv < kChunk ? (nv > 0 ? nv : 1) : kChunk;
  int* need = ws.take<int>((size_t)nv + 1);
  int* list = ws.take<int>((size_t)nv + 1);
  int* slot = ws.take<int>((size_t)nv + 1);
  int* count = ws.take<int>(1);
  double* cs = ws.take<double>(M);
  double* sn = ws.take<double>(M);
  double* tang = ws.take<double>((size_t)nv * 2 * N);
  double* px = ws.take<double>((size_t)nv * n);
  double* py = ws.take<double>((size_t)nv * n);
  double* vx = ws.take<double>((size_t)nv * n);
  double* vy = ws.take<double>((size_t)nv * n);
  double* cx = ws.take<double>((size_t)nv * n);
  double* cy = ws.take<double>((size_t)nv * n);
  double* A = ws.take<double>((size_t)chunk * n * n);
  int* piv = ws.take<int>((size_t)chunk * n);
  if (ws.sizing) return VES_OK;
  if (!ws.ok()) {
    ves_record_error(VES_ERR_WORKSPACE, "near_sing_int (rbf): workspace too small");
    return VES_ERR_WORKSPACE;
  }
  if (nv <= 1) return VES_OK;
  if (!ves_fft_size_ok(N) || !ves_fft_size_ok(M) || M % N != 0) {
    ves_record_error(VES_ERR_SHAPE, "near_sing_int (rbf): N=%d not supported", N);
    return VES_ERR_SHAPE;
  }
  const size_t sh = (size_t)(6 * N + 6 * M) * sizeof(double);
  if (sh > 227 * 1024) {
    ves_record_error(VES_ERR_SHAPE, "near_sing_int (rbf): N=%d needs %zu bytes of shared memory", N, sh);
    return VES_ERR_SHAPE;
  }
  const int nwords = (N + 31) / 32;
  int rc = ves_cuda_status(cudaMemsetAsync(need, 0, (size_t)nv * sizeof(int), s), "rbf need");
  if (rc) return rc;
  ves_count_launch(3);
  rbf_twiddle_kernel<<<ceil_div(M, 256), 256, 0, s>>>(M, cs, sn);
  rbf_flag_kernel<<<ceil_div((long long)nv * nl->maxc, 256), 256, 0, s>>>(nv, nl->maxc, nwords, nl->cand_count,
                                                                          nl->cand_src, nl->excl_mask, need);
  rbf_compact_kernel<<<1, 1024, 0, s>>>(nv, need, list, slot, count);
  int nfit = 0;
  rc = ves_cuda_status(cudaMemcpyAsync(&nfit, count, sizeof(int), cudaMemcpyDeviceToHost, s), "rbf count");
  if (!rc) rc = ves_cuda_status(cudaStreamSynchronize(s), "rbf count sync");
  if (rc || nfit == 0) return rc;
  launch_diff_prop(c, 0, nv, X, nullptr, nullptr, tang, nullptr, s);
  if (sh > 48 * 1024) {
    rc = ves_cuda_status(cudaFuncSetAttribute(rbf_layers_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sh),
                         "rbf smem attribute");
    if (rc) return rc;
  }
  const double w = rbf_width(N);
  ves_count_launch();
  rbf_layers_kernel<<<nfit, 256, sh, s>>>(N, M, list, 0, X, f, tang, vself, cs, sn, px, py, vx, vy);
  for (int first = 0; first < nfit; first += chunk) {
    const int cnt = nfit - first < chunk ? nfit - first : chunk;
    ves_count_launch();
    rbf_matrix_kernel<<<ceil_div((long long)cnt * n * n, 256), 256, 0, s>>>(n, first, cnt, w, px, py, A);
    if ((rc = launch_lu_factor(c, cnt, n, A, piv, s))) return rc;
    launch_lu_solve(cnt, n, A, piv, vx + (long long)first * n, cx + (long long)first * n, s);
    launch_lu_solve(cnt, n, A, piv, vy + (long long)first * n, cy + (long long)first * n, s);
    ves_count_launch();
    rbf_correct_kernel<<<ceil_div(nv * 32, 256), 256, 0, s>>>(N, nv, nl->maxc, nwords, first, cnt, w, nl->cand_count,
                                                             nl->cand_src, nl->excl_mask, slot, X, px, py, cx, cy,
                                                             LP);
  }
  return ves_launch_check("near_sing_int (rbf)");
}
