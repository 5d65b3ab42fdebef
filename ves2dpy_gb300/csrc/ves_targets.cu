// Training targets of the MLARM networks, computed on the device from the BIEM
// operators of one isolated vesicle (the plain BIEM step is the judge of the
// surrogate: every target is what that step's arithmetic gives for the shape).
//
// For a standardised shape X (newtorch/wrapper_MLARM_batch_compile_N128.py
// :4119-4138) with the self-interaction matrix G (Alpert, poten.py:40-99),
// the tension and divergence matrices Ten, Div (capsules.py:91-206) and
// A = Div G Ten:
//   relax   X+ - X, X+ from the implicit step of tstep_biem.py:181-428 for one
//           vesicle without background flow: [I + dt k G Ben, -dt G Ten;
//           Div, 0] [X+; s] = [X; Div X], Ben the fourth arc derivative of
//           the step's matvec (RelaxNetwork, get_network_torch.py:12-80)
//   selften A^-1 Div G fBend with fBend the step's bending force (the
//           upsampled bending term truncated to N modes, :1007-1013):
//           invTenMatOnSelfBend (:3672-3688)
//   advten  Z[:, 2m+c] = A^-1 Div b_{m+1,c}: the tension of the inextensible
//           response to the Fourier basis velocities b_{k,0} = (cos k th,
//           sin k th)/N and b_{k,1} = (-sin k th, cos k th)/N, k = 1..127, in
//           the layout the step reads (invTenMatOnVback :3632-3669)
//   adv     M b = G Ten Z: the inextensibility correction of the same basis
//           velocities (translateVinfwTorch :3584-3620, dX/dt = (I - M) v)
#include <math.h>

#include "ves_internal.h"

namespace {

constexpr int kModes = 127;

// basis velocities [2N][2 kModes]: rows x (0..N-1) then y, column 2m + c
__global__ void basis_kernel(int N, double* __restrict__ B) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int nc = 2 * kModes;
  if (i >= 2 * N * nc) return;
  const int r = i / nc, col = i % nc;
  const int comp = r >= N, j = r - comp * N;
  const int m = col / 2, c = col % 2;
  const double arg = (2.0 * VES_PI * j / N) * (double)(m + 1);
  const double cs = cos(arg) / N, sn = sin(arg) / N;
  // c = 0: (cos, sin); c = 1: i * (cos + i sin) = (-sin, cos)
  B[i] = c == 0 ? (comp ? sn : cs) : (comp ? cs : -sn);
}

// In-place Gauss-Jordan inverse with partial (row) pivoting of n x n FP64
// matrices, one CTA per matrix held in shared memory (n <= 160).
__global__ void __launch_bounds__(256) gj_inverse_kernel(int n, const double* __restrict__ A,
                                                         double* __restrict__ Ainv, VesDeviceStatus* st) {
  extern __shared__ double sm[];
  double* a = sm;                 // [n][n]
  double* colv = a + n * n;       // [n]
  int* perm = (int*)(colv + n);   // [n]
  __shared__ int prow;
  __shared__ double pval;
  const int k = blockIdx.x;
  const double* Ak = A + (long long)k * n * n;
  for (int i = threadIdx.x; i < n * n; i += blockDim.x) a[i] = Ak[i];
  __syncthreads();
  for (int col = 0; col < n; ++col) {
    if (threadIdx.x < 32) {
      double best = -1.0;
      int br = col;
      for (int r = col + threadIdx.x; r < n; r += 32) {
        const double v = fabs(a[r * n + col]);
        if (v > best) {
          best = v;
          br = r;
        }
      }
      for (int o = 16; o > 0; o >>= 1) {
        const double ob = __shfl_xor_sync(0xffffffffu, best, o);
        const int orr = __shfl_xor_sync(0xffffffffu, br, o);
        if (ob > best || (ob == best && orr < br)) {
          best = ob;
          br = orr;
        }
      }
      if (threadIdx.x == 0) prow = br;
    }
    __syncthreads();
    const int p = prow;
    if (p != col)
      for (int j = threadIdx.x; j < n; j += blockDim.x) {
        const double t = a[col * n + j];
        a[col * n + j] = a[p * n + j];
        a[p * n + j] = t;
      }
    __syncthreads();
    if (threadIdx.x == 0) {
      perm[col] = p;
      pval = a[col * n + col];
    }
    __syncthreads();
    double piv = pval;
    if (piv == 0.0) {
      if (threadIdx.x == 0) ves_set_error(st, VES_ERR_SINGULAR, 40, (long long)k);
      piv = 1.0;
    }
    const double pinv = 1.0 / piv;
    // scale the pivot row (its pivot entry becomes 1/piv) and keep the column
    for (int j = threadIdx.x; j < n; j += blockDim.x) {
      a[col * n + j] = (j == col) ? pinv : a[col * n + j] * pinv;
      colv[j] = a[j * n + col];
    }
    __syncthreads();
    for (int i = threadIdx.x; i < n * n; i += blockDim.x) {
      const int r = i / n, j = i % n;
      if (r == col) continue;
      const double base = (j == col) ? 0.0 : a[i];
      a[i] = base - a[col * n + j] * colv[r];
    }
    __syncthreads();
  }
  // undo the row interchanges as column interchanges, last first
  for (int col = n - 1; col >= 0; --col) {
    const int p = perm[col];
    if (p != col)
      for (int r = threadIdx.x; r < n; r += blockDim.x) {
        const double t = a[r * n + col];
        a[r * n + col] = a[r * n + p];
        a[r * n + p] = t;
      }
    __syncthreads();
  }
  double* out = Ainv + (long long)k * n * n;
  for (int i = threadIdx.x; i < n * n; i += blockDim.x) out[i] = a[i];
}

// out[k][c][r] = in[k][r][c] for rows x cols matrices
__global__ void transpose_kernel(int rows, int cols, const double* __restrict__ in, double* __restrict__ out) {
  const int k = blockIdx.y;
  const long long n = (long long)rows * cols;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const int r = (int)(i / cols), c = (int)(i % cols);
    out[(long long)k * n + (long long)c * rows + r] = in[(long long)k * n + i];
  }
}

// rhs [X + dt vinf; Div X] of the isolated step (vinf NULL: no flow), [nv][3N]
__global__ void relax_rhs_kernel(int nv, int N, const double* __restrict__ X, const double* __restrict__ vinf, double dt,
                                 const double* __restrict__ divx, double* __restrict__ rhs) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (long long)nv * 3 * N) return;
  const long long k = i / (3 * N);
  const int r = (int)(i % (3 * N));
  rhs[i] = r < 2 * N ? X[k * 2 * N + r] + (vinf ? dt * vinf[k * 2 * N + r] : 0.0) : divx[k * N + r - 2 * N];
}

// Ar[k][i][j] = isa[k][i] d1[(i - j) mod N]: the arc derivative of the step's
// matvec (arc_deriv with the Nyquist mode zeroed) as a matrix
__global__ void arc_matrix_kernel(int nv, int N, const double* __restrict__ d1, const double* __restrict__ isa,
                                  double* __restrict__ Ar) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (long long)nv * N * N) return;
  const long long k = i / ((long long)N * N);
  const int r = (int)((i / N) % N), c = (int)(i % N);
  Ar[i] = isa[k * N + r] * d1[((r - c) % N + N) % N];
}

// the self-interaction block of the BIEM matvec (tstep_biem.py:430-610 with no
// other vesicle): [I + dt k G Ben, -dt G Ten; Div, 0], Ben = blockdiag(D4, D4)
// with D4 = Ar^4 the matvec's fourth arc derivative
__global__ void self_block_kernel(int nv, int N, double dt, double kappa, const double* __restrict__ GB,
                                  const double* __restrict__ GT, const double* __restrict__ Div,
                                  double* __restrict__ M) {
  const int n3 = 3 * N, n2 = 2 * N;
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (long long)nv * n3 * n3) return;
  const long long k = i / ((long long)n3 * n3);
  const int r = (int)((i / n3) % n3), c = (int)(i % n3);
  double v;
  if (r < n2)
    v = c < n2 ? (r == c ? 1.0 : 0.0) + dt * kappa * GB[(k * n2 + r) * n2 + c] : -dt * GT[(k * n2 + r) * N + c - n2];
  else
    v = c < n2 ? Div[(k * N + r - n2) * n2 + c] : 0.0;
  M[i] = v;
}

__global__ void relax_dx_kernel(int nv, int N, const double* __restrict__ X, const double* __restrict__ sol,
                                double* __restrict__ dx) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (long long)nv * 2 * N) return;
  const long long k = i / (2 * N);
  const int r = (int)(i % (2 * N));
  dx[i] = sol[k * 3 * N + r] - X[i];
}

int targets_run(ves_ctx* c, int nv, const double* Xs, const double* vinf, double dt, double kappa, int slp,
                double* relax_dx, double* selften, double* advten, double* adv, WsCarver& ws, cudaStream_t s) {
  const int N = c->N;
  const int nc = 2 * kModes;
  const size_t NN = (size_t)N * N;
  double* sa = ws.take<double>((size_t)nv * N);
  double* isa = ws.take<double>((size_t)nv * N);
  double* tang = ws.take<double>((size_t)nv * 2 * N);
  double* G = ws.take<double>((size_t)nv * 4 * NN);
  double* Ten = ws.take<double>((size_t)nv * 2 * NN);
  double* Div = ws.take<double>((size_t)nv * 2 * NN);
  double* M = relax_dx ? ws.take<double>((size_t)nv * 9 * NN) : nullptr;
  double* Ar = relax_dx ? ws.take<double>((size_t)nv * NN) : nullptr;
  double* C2 = relax_dx ? ws.take<double>((size_t)nv * NN) : nullptr;
  double* D4 = relax_dx ? ws.take<double>((size_t)nv * NN) : nullptr;
  double* GB = relax_dx ? ws.take<double>((size_t)nv * 4 * NN) : nullptr;
  int* piv = relax_dx ? ws.take<int>((size_t)nv * 3 * N) : nullptr;
  double* v3 = ws.take<double>((size_t)nv * 3 * N);
  double* x3 = ws.take<double>((size_t)nv * 3 * N);
  double* GT = ws.take<double>((size_t)nv * 2 * NN);
  const bool tens = selften || advten || adv;  // the tension operator A = Div G Ten is needed
  const bool modes = advten || adv;
  double* A = tens ? ws.take<double>((size_t)nv * NN) : nullptr;
  double* Ai = tens ? ws.take<double>((size_t)nv * NN) : nullptr;
  double* Bm = modes ? ws.take<double>((size_t)2 * N * nc) : nullptr;
  double* DB = modes ? ws.take<double>((size_t)nv * N * nc) : nullptr;
  double* Z = modes ? ws.take<double>((size_t)nv * N * nc) : nullptr;
  double* W = adv ? ws.take<double>((size_t)nv * 2 * N * nc) : nullptr;
  // scratch of the Alpert build and the derivative matrices
  size_t scr = 0;
  {
    WsCarver w(nullptr, 0);
    alpert_sl_matrix(c, nv, nullptr, slp, nullptr, w, s);
    scr = w.off;
    WsCarver w2(nullptr, 0);
    derivs_and_precond(c, nv, nullptr, nullptr, nullptr, dt, kappa, nullptr, nullptr, nullptr, nullptr, w2, s);
    scr = std::max(scr, w2.off);
  }
  char* sub = ws.take<char>(scr + 1024);
  if (ws.sizing) return VES_OK;
  if (!ws.ok()) {
    ves_record_error(VES_ERR_WORKSPACE, "mlarm_targets: workspace too small (%zu needed)", ws.off);
    return VES_ERR_WORKSPACE;
  }
  if (nv <= 0) return VES_OK;
  int rc;
  launch_diff_prop(c, 0, nv, Xs, sa, isa, tang, nullptr, s);
  {
    WsCarver w(sub, scr + 1024);
    if ((rc = alpert_sl_matrix(c, nv, Xs, slp, G, w, s))) return rc;
  }
  {
    WsCarver w(sub, scr + 1024);
    if ((rc = derivs_and_precond(c, nv, isa, tang, G, dt, kappa, nullptr, Ten, Div, nullptr, w, s))) return rc;
  }
  const long long sN = (long long)NN;
  launch_bgemm_f64(nv, 2 * N, N, 2 * N, 1.0, G, 2 * N, 4 * sN, Ten, N, 2 * sN, 0.0, GT, N, 2 * sN, s);
  if (relax_dx) {
    // the implicit step of one vesicle: M [X+; s] = [X + dt vinf; Div X]
    ves_count_launch();
    arc_matrix_kernel<<<ceil_div((long long)nv * NN, 256), 256, 0, s>>>(nv, N, c->d1N, isa, Ar);
    launch_bgemm_f64(nv, N, N, N, 1.0, Ar, N, sN, Ar, N, sN, 0.0, C2, N, sN, s);
    launch_bgemm_f64(nv, N, N, N, 1.0, C2, N, sN, C2, N, sN, 0.0, D4, N, sN, s);
    launch_bgemm_f64(nv, 2 * N, N, N, 1.0, G, 2 * N, 4 * sN, D4, N, sN, 0.0, GB, 2 * N, 4 * sN, s);
    launch_bgemm_f64(nv, 2 * N, N, N, 1.0, G + N, 2 * N, 4 * sN, D4, N, sN, 0.0, GB + N, 2 * N, 4 * sN, s);
    ves_count_launch();
    self_block_kernel<<<ceil_div((long long)nv * 9 * NN, 256), 256, 0, s>>>(nv, N, dt, kappa, GB, GT, Div, M);
    launch_surface_div(c, nv, isa, tang, Xs, 2LL * N, v3, N, s);
    ves_count_launch();
    relax_rhs_kernel<<<ceil_div((long long)nv * 3 * N, 256), 256, 0, s>>>(nv, N, Xs, vinf, dt, v3, x3);
    if ((rc = launch_lu_factor(c, nv, 3 * N, M, piv, s))) return rc;
    launch_lu_solve(nv, 3 * N, M, piv, x3, v3, s);
    ves_count_launch();
    relax_dx_kernel<<<ceil_div((long long)nv * 2 * N, 256), 256, 0, s>>>(nv, N, Xs, v3, relax_dx);
  }
  if (!selften && !advten && !adv) return ves_launch_check("mlarm_targets");
  // A = Div G Ten and its inverse
  launch_bgemm_f64(nv, N, N, 2 * N, 1.0, Div, 2 * N, 2 * sN, GT, N, 2 * sN, 0.0, A, N, sN, s);
  {
    const size_t sh = NN * sizeof(double) + (size_t)N * (sizeof(double) + sizeof(int));
    if (N > 160) {
      ves_record_error(VES_ERR_SHAPE, "mlarm_targets: N = %d above 160", N);
      return VES_ERR_SHAPE;
    }
    if ((rc = ves_cuda_status(cudaFuncSetAttribute(gj_inverse_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                   (int)sh), "gj smem")))
      return rc;
    ves_count_launch();
    gj_inverse_kernel<<<nv, 256, sh, s>>>(N, A, Ai, c->status);
  }
  if (selften) {
    // A^-1 Div G fBend
    double* fB = v3;        // [nv][2N] (3N slots per vesicle are enough)
    double* g = x3;
    if ((rc = launch_bend_up(c, nv, Xs, kappa, fB, s))) return rc;
    launch_bgemv_f64(nv, 2 * N, 2 * N, G, fB, 2LL * N, g, 2LL * N, s);
    launch_bgemv_f64(nv, N, 2 * N, Div, g, 2LL * N, fB, N, s);
    launch_bgemv_f64(nv, N, N, Ai, fB, N, selften, N, s);
  }
  if (advten || adv) {
    ves_count_launch();
    basis_kernel<<<ceil_div(2 * N * nc, 256), 256, 0, s>>>(N, Bm);
    // DB = Div B (the basis is shared by every vesicle), Z = A^-1 DB
    launch_bgemm_f64(nv, N, nc, 2 * N, 1.0, Div, 2 * N, 2 * sN, Bm, nc, 0, 0.0, DB, nc, (long long)N * nc, s);
    launch_bgemm_f64(nv, N, nc, N, 1.0, Ai, N, sN, DB, nc, (long long)N * nc, 0.0, Z, nc, (long long)N * nc, s);
    if (advten) {
      ves_count_launch();
      transpose_kernel<<<dim3(ceil_div((long long)N * nc, 256), nv), 256, 0, s>>>(N, nc, Z, advten);
    }
    if (adv) {
      launch_bgemm_f64(nv, 2 * N, nc, N, 1.0, GT, N, 2 * sN, Z, nc, (long long)N * nc, 0.0, W, nc,
                       2LL * N * nc, s);
      ves_count_launch();
      transpose_kernel<<<dim3(ceil_div(2LL * N * nc, 256), nv), 256, 0, s>>>(2 * N, nc, W, adv);
    }
  }
  return ves_launch_check("mlarm_targets");
}

}  // namespace

// dx = X+ - X of the implicit step of non-interacting vesicles with background
// velocity vinf (NULL: none), for callers inside the library (the MLARM
// step's fallback); no status reset, no synchronisation
int isolated_step_run(ves_ctx* c, int nv, const double* X, const double* vinf, double dt, double kappa, int slp,
                      double* dx, WsCarver& ws, cudaStream_t s) {
  return targets_run(c, nv, X, vinf, dt, kappa, slp, dx ? dx : (double*)1, nullptr, nullptr, nullptr, ws, s);
}

extern "C" size_t ves_mlarm_targets_workspace(ves_ctx* c, int nv, int sl_precision) {
  if (!c || nv < 0) return 0;
  WsCarver w(nullptr, 0);
  double* one = (double*)1;
  targets_run(c, nv, nullptr, nullptr, 1e-5, 1.0, sl_precision, one, one, one, one, w, 0);
  return w.off + 256;
}

extern "C" int ves_mlarm_targets(ves_ctx* c, int nv, const double* Xs, double dt, double kappa, int sl_precision,
                                 double* relax_dx, double* selften, double* advten, double* adv, void* ws,
                                 size_t ws_bytes, void* stream) {
  if (!c || !ws || nv < 0 || (nv > 0 && !Xs) || dt <= 0 ||
      (sl_precision != VES_PREC_FP64 && sl_precision != VES_PREC_FP32C)) {
    ves_record_error(VES_ERR_ARG, "mlarm_targets: bad arguments");
    return VES_ERR_ARG;
  }
  cudaStream_t s = (cudaStream_t)stream;
  int rc = ves_reset_status(c, s);
  if (rc) return rc;
  WsCarver w(ws, ws_bytes);
  rc = targets_run(c, nv, Xs, nullptr, dt, kappa, sl_precision, relax_dx, selften, advten, adv, w, s);
  if (rc) return rc;
  return ves_check_status(c, s, "mlarm_targets");
}

namespace {
__global__ void add_kernel(long long n, const double* __restrict__ a, const double* __restrict__ b,
                           double* __restrict__ out) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = a[i] + b[i];
}
}  // namespace

extern "C" size_t ves_isolated_step_workspace(ves_ctx* c, int nv, int sl_precision) {
  if (!c || nv < 0) return 0;
  WsCarver w(nullptr, 0);
  w.take<double>((size_t)nv * 2 * c->N);
  targets_run(c, nv, nullptr, nullptr, 1e-5, 1.0, sl_precision, (double*)1, nullptr, nullptr, nullptr, w, 0);
  return w.off + 256;
}

extern "C" int ves_isolated_step(ves_ctx* c, int nv, const double* X, const double* vinf, double dt, double kappa,
                                 int sl_precision, double* Xout, void* ws, size_t ws_bytes, void* stream) {
  if (!c || !ws || nv < 0 || (nv > 0 && (!X || !Xout)) || dt <= 0 ||
      (sl_precision != VES_PREC_FP64 && sl_precision != VES_PREC_FP32C)) {
    ves_record_error(VES_ERR_ARG, "isolated_step: bad arguments");
    return VES_ERR_ARG;
  }
  cudaStream_t s = (cudaStream_t)stream;
  int rc = ves_reset_status(c, s);
  if (rc) return rc;
  WsCarver w(ws, ws_bytes);
  const long long n = (long long)nv * 2 * c->N;
  double* dx = w.take<double>((size_t)n);
  rc = targets_run(c, nv, X, vinf, dt, kappa, sl_precision, dx, nullptr, nullptr, nullptr, w, s);
  if (rc) return rc;
  if (nv > 0) {
    ves_count_launch();
    add_kernel<<<ceil_div(n, 256), 256, 0, s>>>(n, X, dx, Xout);
  }
  if ((rc = ves_launch_check("isolated_step"))) return rc;
  return ves_check_status(c, s, "isolated_step");
}
