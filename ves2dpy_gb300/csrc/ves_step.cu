// The implicit BIEM time step (TStepBiem.time_step, mytorch/tstep_biem.py:181-428)
// with its GMRES matvec (time_matvec, :430-610) and block-diagonal LU
// preconditioner (preconditionerBD, :653-711).
//
// GMRES restates scipy.sparse.linalg.gmres (the solver the reference calls at
// tstep_biem.py:381): left preconditioning, restart 20, modified Gram-Schmidt,
// LAPACK lartg Givens rotations and SciPy's inner/outer tolerance control.
// Every vector operation runs on the device; the host keeps the (restart+1)
// x restart Hessenberg matrix, whose current column (at most 22 numbers) is
// read back once per inner iteration to decide convergence.
#include <math.h>
#include <string.h>

#include <algorithm>
#include <vector>

#include "ves_internal.h"

namespace {

__global__ void finalize_dot_kernel(const double* __restrict__ partials, int np, double* __restrict__ out,
                                    int take_sqrt) {
  __shared__ double red[512];
  red[threadIdx.x] = threadIdx.x < np ? partials[threadIdx.x] : 0.0;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) *out = take_sqrt ? sqrt(red[0]) : red[0];
}

// w -= h * v with h = sum(partials) (fixed-order), block 0 stores h
__global__ void __launch_bounds__(512) mgs_axpy_kernel(long long n, const double* __restrict__ partials, int np,
                                                       double* __restrict__ w, const double* __restrict__ v,
                                                       double* __restrict__ hout) {
  __shared__ double red[512];
  red[threadIdx.x] = threadIdx.x < np ? partials[threadIdx.x] : 0.0;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
    __syncthreads();
  }
  const double h = red[0];
  if (blockIdx.x == 0 && threadIdx.x == 0) *hout = h;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    w[i] -= h * v[i];
}

// dst = src * (1/scal) unless skip(scal, ref): the "v *= 1/tmp" of SciPy
__global__ void scale_inv_kernel(long long n, double* __restrict__ dst, const double* __restrict__ src,
                                 const double* __restrict__ scal, const double* __restrict__ ref, double eps) {
  const double h1 = *scal;
  const bool brk = ref ? (h1 <= eps * (*ref)) : false;
  const double inv = 1.0 / h1;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    dst[i] = brk ? src[i] : src[i] * inv;
}

__global__ void sub_kernel(long long n, double* __restrict__ r, const double* __restrict__ b,
                           const double* __restrict__ a) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    r[i] = b[i] - a[i];
}

// x += sum_k y[k] V[k]  (accumulated in k order, then added)
__global__ void update_x_kernel(long long n, int cnt, const double* __restrict__ y, const double* __restrict__ V,
                                double* __restrict__ x) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    double t = 0.0;
    for (int k = 0; k < cnt; ++k) t = fma(y[k], V[(long long)k * n + i], t);
    x[i] += t;
  }
}

// pack [X + dt*vinf ; surfaceDiv(X)] and [X ; sigma]
__global__ void pack_kernel(int nv, int N, const double* __restrict__ A2, const double* __restrict__ B1,
                            double* __restrict__ out) {
  const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= (long long)nv * 3 * N) return;
  const long long k = idx / (3 * N), r = idx % (3 * N);
  out[idx] = (r < 2 * N) ? A2[k * 2 * N + r] : B1[k * N + (r - 2 * N)];
}

// rhs1 in the reference's order (tstep_biem.py:242-270), each term scaled by
// 1/alpha (alpha = (1 + visc)/2, 1 without a contrast):
//   X - (Fdlp + D X) / alpha + dt (G rep + nearSingInt_rbf(rep)) / alpha + dt vInf / alpha
__global__ void rhs_pos_kernel(long long n, int N, double dt, const double* __restrict__ X,
                               const double* __restrict__ v, const double* __restrict__ frepG,
                               const double* __restrict__ frepN, const double* __restrict__ fdl,
                               const double* __restrict__ dx, const double* __restrict__ alpha,
                               double* __restrict__ out) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double ia = alpha ? 1.0 / alpha[i / (2 * N)] : 1.0;
  double r = X[i];
  if (fdl) r = r - (fdl[i] + dx[i]) * ia;
  if (frepG) r = r + (dt * (frepG[i] + frepN[i])) * ia;
  out[i] = r + (dt * v[i]) * ia;
}

// alpha = (1 + visc) / 2 (tstep_biem.py:195)
__global__ void alpha_kernel(int nv, const double* __restrict__ visc, double* __restrict__ alpha) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k < nv) alpha[k] = (1.0 + visc[k]) / 2;
}

// vself of the double layer: X jump + D X, jump = (1 - visc)/2 (tstep_biem.py:233-234)
__global__ void dl_self_kernel(long long n, int N, const double* __restrict__ visc, const double* __restrict__ X,
                               long long xs, const double* __restrict__ DX, double* __restrict__ out) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const long long k = i / (2 * N), r = i % (2 * N);
  out[i] = X[k * xs + r] * (0.5 * (1 - visc[k])) + DX[i];
}

// [nv][3][N] -> [nv][2][N] (the positions of a GMRES vector)
__global__ void take_pos_kernel(long long n, int N, const double* __restrict__ v, double* __restrict__ out) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  out[i] = v[(i / (2 * N)) * 3 * N + i % (2 * N)];
}

__global__ void unpack_kernel(int nv, int N, const double* __restrict__ x, double* __restrict__ X,
                              double* __restrict__ sig) {
  const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= (long long)nv * 3 * N) return;
  const long long k = idx / (3 * N), r = idx % (3 * N);
  if (r < 2 * N)
    X[k * 2 * N + r] = x[idx];
  else
    sig[k * N + (r - 2 * N)] = x[idx];
}

// valPos = -(dt Gf)/alpha - D Xm/alpha - (dt LP)/alpha - Fdlp/alpha + Xm
// (tstep_biem.py:541-576; alpha = 1 and no double-layer terms without a contrast)
__global__ void combine_pos_kernel(int nv, int N, double dt, const double* __restrict__ v,
                                   const double* __restrict__ Gf, const double* __restrict__ LP,
                                   const double* __restrict__ alpha, const double* __restrict__ DX,
                                   const double* __restrict__ Fdl, double* __restrict__ out) {
  const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= (long long)nv * 2 * N) return;
  const long long k = idx / (2 * N), r = idx % (2 * N);
  double val;
  if (alpha) {
    const double a = alpha[k];
    val = -((dt * Gf[idx]) / a);
    val -= DX[idx] / a;
    val -= (dt * LP[idx]) / a;
    val -= Fdl[idx] / a;
  } else {
    val = -(dt * Gf[idx]);
    val -= dt * LP[idx];
  }
  val += v[k * 3 * N + r];
  out[k * 3 * N + r] = val;
}

inline unsigned vec_grid(long long n) {
  long long g = (n + 511) / 512;
  if (g > 4096) g = 4096;
  if (g < 1) g = 1;
  return (unsigned)g;
}

// LAPACK dlartg (3.10+): c >= 0, r carries the sign of f.
void lartg(double f, double g, double& c, double& s, double& r) {
  if (g == 0.0) {
    c = 1.0;
    s = 0.0;
    r = f;
  } else if (f == 0.0) {
    c = 0.0;
    s = (g > 0) ? 1.0 : -1.0;
    r = fabs(g);
  } else {
    const double d = sqrt(f * f + g * g);
    c = fabs(f) / d;
    r = (f > 0) ? d : -d;
    s = g / r;
  }
}

struct StepState {
  ves_ctx* c;
  const ves_step_params* prm;
  int nv, N, Nup;
  long long n;
  cudaStream_t s;
  const double* X;  // positions at the start of the step [nv][2][N]
  // geometry of the step
  double *sa, *isa, *tang, *Xup, *sa_up, *G, *LU;
  int* piv;
  // viscosity contrast (null without one): contrasts, alpha, D, upsampled tangents
  const double* visc;
  double *alpha, *D, *tang_up, *Xm, *DX, *vdl, *Fdl;
  ves_near_lists nl;
  double h;
  // matvec temporaries
  double *f, *Gf, *LP;
  char* scratch;
  size_t scratch_bytes;
  int matvecs;
  int dl_scheme;  // near scheme of the double layer: py_hh for the py lists, else the step's
};

// out = A v (time_matvec, tstep_biem.py:430-610), v and out in [nv][3][N]
int matvec(StepState& S, const double* v, double* out) {
  ves_ctx* c = S.c;
  const int nv = S.nv, N = S.N;
  S.matvecs++;
  launch_trac_jump(c, nv, S.prm->kappa, S.isa, S.tang, v, 3LL * N, v + 2 * N, 3LL * N, S.f, S.s);
  launch_bgemv_f64(nv, 2 * N, 2 * N, S.G, S.f, 2LL * N, S.Gf, 2LL * N, S.s);
  WsCarver sub(S.scratch, S.scratch_bytes);
  int rc = near_sing_int_run(c, S.prm->near_scheme, S.prm->farfield_precision, nv, S.X, S.sa_up, S.Xup, S.f, S.Gf,
                             &S.nl, S.h, S.LP, nullptr, sub, S.s);
  if (rc) return rc;
  if (S.visc) {
    // D Xm and the double layer of Xm (tstep_biem.py:489, 497-501)
    const long long n2 = (long long)nv * 2 * N;
    ves_count_launch();
    take_pos_kernel<<<ceil_div(n2, 256), 256, 0, S.s>>>(n2, N, v, S.Xm);
    launch_bgemv_f64(nv, 2 * N, 2 * N, S.D, S.Xm, 2LL * N, S.DX, 2LL * N, S.s);
    ves_count_launch();
    dl_self_kernel<<<ceil_div(n2, 256), 256, 0, S.s>>>(n2, N, S.visc, S.Xm, 2LL * N, S.DX, S.vdl);
    WsCarver sub2(S.scratch, S.scratch_bytes);
    if ((rc = near_sing_int_dl_run(c, S.dl_scheme, S.prm->farfield_precision, nv, S.X, S.Xup, S.tang_up, S.sa_up,
                                   S.visc, S.Xm, S.vdl, &S.nl,
                                   S.h, S.Fdl, nullptr, sub2, S.s)))
      return rc;
  }
  ves_count_launch();
  combine_pos_kernel<<<ceil_div((long long)nv * 2 * N, 256), 256, 0, S.s>>>(nv, N, S.prm->dt, v, S.Gf, S.LP, S.alpha,
                                                                            S.DX, S.Fdl, out);
  launch_surface_div(c, nv, S.isa, S.tang, v, 3LL * N, out + 2 * N, 3LL * N, S.s);
  return ves_launch_check("matvec");
}

// use_preco == 2: the block-diagonal preconditioner built and factored in
// FP32 (no viscosity contrast); otherwise FP64
static bool precond_is_f32(const ves_step_params* prm) { return prm->use_preco == 2 && prm->visc_cont == nullptr; }

int psolve(StepState& S, const double* z, double* out) {
  if (!S.prm->use_preco) {
    return ves_cuda_status(cudaMemcpyAsync(out, z, S.n * sizeof(double), cudaMemcpyDeviceToDevice, S.s), "psolve copy");
  }
  if (precond_is_f32(S.prm))
    launch_lu_solve_f32(S.nv, 3 * S.N, (const float*)S.LU, S.piv, z, out, S.s);
  else
    launch_lu_solve(S.nv, 3 * S.N, S.LU, S.piv, z, out, S.s);
  return ves_launch_check("psolve");
}

struct GmresBufs {
  double *V, *w, *r, *b, *x, *t, *partials, *dsc, *hsc;  // hsc: pinned host scalars
  double* ydev;
};

template <class St>
int device_norm(St& S, GmresBufs& B, const double* a, double* dst) {
  launch_dot_partials(S.n, a, a, B.partials, S.s);
  ves_count_launch();
  finalize_dot_kernel<<<1, 512, 0, S.s>>>(B.partials, dot_partial_blocks(), dst, 1);
  return ves_launch_check("norm");
}

template <class St>
int read_scalars(St& S, GmresBufs& B, const double* src, int count) {
  int rc = ves_cuda_status(cudaMemcpyAsync(B.hsc, src, count * sizeof(double), cudaMemcpyDeviceToHost, S.s), "read");
  if (rc) return rc;
  return ves_cuda_status(cudaStreamSynchronize(S.s), "read sync");
}

// A suspension of several point counts: groups of vesicles, group g with N_g
// points and its own context, in one GMRES system (the groups' [nv][3][N]
// blocks one after the other).  Between groups the far field runs over the
// source group's upsampled points and the near zone and its correction follow
// the MATLAB rules with a separate target set (source group's h).
constexpr int kMaxGroups = 4;

struct MixedState {
  const ves_step_params* prm;
  int ng;
  long long n;
  cudaStream_t s;
  StepState g[kMaxGroups];
  long long off[kMaxGroups + 1];
  double *fup[kMaxGroups], *den[kMaxGroups];
  ves_near_lists xl[kMaxGroups][kMaxGroups];  // [target group][source group]
  double h[kMaxGroups];
  char* scratch;
  size_t scratch_bytes;
  int matvecs;
};

// The far field of every group from every group's upsampled sources (the
// densities M.den of the current matvec), one launch (VES_PREC_FP32M), into
// each group's LP; near-pair exclusions follow the lists of the MATLAB scheme.
int mixed_farfield_merged(MixedState& M, bool sizing = false) {
  int nsrc[kMaxGroups], ns[kMaxGroups], nt[kMaxGroups], ntp[kMaxGroups];
  const double *Xsrc[kMaxGroups], *den[kMaxGroups], *Xtar[kMaxGroups];
  const ves_near_lists* nl[kMaxGroups * kMaxGroups];
  double* out[kMaxGroups];
  const bool lists = M.prm->near_scheme == VES_NEAR_MATLAB;
  for (int g = 0; g < M.ng; ++g) {
    StepState& S = M.g[g];
    nsrc[g] = nt[g] = S.nv;
    ns[g] = S.Nup;
    ntp[g] = S.N;
    Xsrc[g] = S.Xup;
    den[g] = M.den[g];
    Xtar[g] = S.X;
    out[g] = S.LP;
    for (int q = 0; q < M.ng; ++q) nl[g * M.ng + q] = lists ? (q == g ? &S.nl : &M.xl[g][q]) : nullptr;
  }
  FFEnv env;
  env.status = M.g[0].c->status;
  env.N = M.g[0].N;
  env.timing = nullptr;
  WsCarver sub(sizing ? nullptr : M.scratch, sizing ? 0 : M.scratch_bytes);
  const int rc = farfield_mp_groups_run(env, M.ng, nsrc, ns, Xsrc, den, nt, ntp, Xtar, nl, out, sub, M.s);
  if (sizing) M.scratch_bytes = std::max(M.scratch_bytes, sub.off);
  return rc;
}

int matvec(MixedState& M, const double* v, double* out) {
  M.matvecs++;
  const ves_step_params* prm = M.prm;
  for (int q = 0; q < M.ng; ++q) {
    StepState& S = M.g[q];
    const int nv = S.nv, N = S.N;
    const double* vq = v + M.off[q];
    launch_trac_jump(S.c, nv, prm->kappa, S.isa, S.tang, vq, 3LL * N, vq + 2 * N, 3LL * N, S.f, M.s);
    launch_bgemv_f64(nv, 2 * N, 2 * N, S.G, S.f, 2LL * N, S.Gf, 2LL * N, M.s);
    if (M.ng > 1) {
      launch_upsample(S.c, nv, 2, S.f, 2LL * N, M.fup[q], M.s);
      launch_density(nv, S.Nup, M.fup[q], S.sa_up, M.den[q], M.s);
    }
  }
  int rc;
  if (M.ng > 1 && prm->farfield_precision == VES_PREC_FP32M) {
    // every group's far field from every group's sources in one launch, then
    // the near corrections of every (target group, source group) pair in one
    if ((rc = mixed_farfield_merged(M))) return rc;
    if (prm->near_scheme == VES_NEAR_MATLAB) {
      ves_ctx *ct[kMaxGroups * kMaxGroups], *cs[kMaxGroups * kMaxGroups];
      const double *Xt[kMaxGroups * kMaxGroups], *Xs[kMaxGroups * kMaxGroups], *dn[kMaxGroups * kMaxGroups],
          *vs[kMaxGroups * kMaxGroups];
      const ves_near_lists* nl[kMaxGroups * kMaxGroups];
      double hh[kMaxGroups * kMaxGroups];
      double* lp[kMaxGroups * kMaxGroups];
      int np = 0;
      for (int g = 0; g < M.ng; ++g)
        for (int q = 0; q < M.ng; ++q, ++np) {
          StepState& S = M.g[g];
          const StepState& Q = M.g[q];
          ct[np] = S.c;
          cs[np] = Q.c;
          Xt[np] = S.X;
          Xs[np] = Q.Xup;
          dn[np] = M.den[q];
          vs[np] = Q.Gf;
          nl[np] = q == g ? &S.nl : &M.xl[g][q];
          hh[np] = q == g ? S.h : M.h[q];
          lp[np] = S.LP;
        }
      if ((rc = near_correct_matlab_pairs(np, ct, cs, Xt, Xs, dn, vs, nl, hh, lp, M.s))) return rc;
    }
    for (int g = 0; g < M.ng; ++g) {
      StepState& S = M.g[g];
      const int nv = S.nv, N = S.N;
      const double* vg = v + M.off[g];
      double* og = out + M.off[g];
      ves_count_launch();
      combine_pos_kernel<<<ceil_div((long long)nv * 2 * N, 256), 256, 0, M.s>>>(nv, N, prm->dt, vg, S.Gf, S.LP, nullptr,
                                                                                nullptr, nullptr, og);
      launch_surface_div(S.c, nv, S.isa, S.tang, vg, 3LL * N, og + 2 * N, 3LL * N, M.s);
    }
    return ves_launch_check("matvec mixed");
  }
  for (int g = 0; g < M.ng; ++g) {
    StepState& S = M.g[g];
    {
      WsCarver sub(M.scratch, M.scratch_bytes);
      if ((rc = near_sing_int_run(S.c, prm->near_scheme, prm->farfield_precision, S.nv, S.X, S.sa_up, S.Xup, S.f,
                                  S.Gf, &S.nl, S.h, S.LP, nullptr, sub, M.s)))
        return rc;
    }
    for (int q = 0; q < M.ng; ++q) {
      if (q == g) continue;
      const StepState& Q = M.g[q];
      WsCarver sub(M.scratch, M.scratch_bytes);
      if ((rc = near_sing_int_cross_add(S.c, Q.c, prm->near_scheme, prm->farfield_precision, S.nv, S.X, Q.nv, Q.Xup,
                                        M.den[q], Q.Gf, &M.xl[g][q], M.h[q], S.LP, sub, M.s)))
        return rc;
    }
    const int nv = S.nv, N = S.N;
    const double* vg = v + M.off[g];
    double* og = out + M.off[g];
    ves_count_launch();
    combine_pos_kernel<<<ceil_div((long long)nv * 2 * N, 256), 256, 0, M.s>>>(nv, N, prm->dt, vg, S.Gf, S.LP, nullptr,
                                                                              nullptr, nullptr, og);
    launch_surface_div(S.c, nv, S.isa, S.tang, vg, 3LL * N, og + 2 * N, 3LL * N, M.s);
  }
  return ves_launch_check("matvec mixed");
}

int psolve(MixedState& M, const double* z, double* out) {
  if (!M.prm->use_preco) {
    return ves_cuda_status(cudaMemcpyAsync(out, z, M.n * sizeof(double), cudaMemcpyDeviceToDevice, M.s),
                           "psolve copy");
  }
  for (int g = 0; g < M.ng; ++g) {
    if (precond_is_f32(M.prm))
      launch_lu_solve_f32(M.g[g].nv, 3 * M.g[g].N, (const float*)M.g[g].LU, M.g[g].piv, z + M.off[g],
                          out + M.off[g], M.s);
    else
      launch_lu_solve(M.g[g].nv, 3 * M.g[g].N, M.g[g].LU, M.g[g].piv, z + M.off[g], out + M.off[g], M.s);
  }
  return ves_launch_check("psolve mixed");
}

// scipy.sparse.linalg.gmres (scipy/sparse/linalg/_isolve/iterative.py), device vectors
template <class St>
int gmres(St& S, GmresBufs& B, ves_step_result* res) {
  const long long n = S.n;
  const int restart = std::min<long long>(S.prm->gmres_restart > 0 ? S.prm->gmres_restart : 20, n);
  const int maxiter = S.prm->gmres_maxiter > 0 ? S.prm->gmres_maxiter : (int)std::min<long long>(n * 10, 1 << 30);
  const double eps = 2.220446049250313e-16;
  const unsigned g = vec_grid(n);
  // dsc layout: [0..restart+1] current h column, [restart+2] h0, [restart+3] scratch norm
  double* hcol = B.dsc;
  double* h0 = B.dsc + restart + 2;
  double* nrm = B.dsc + restart + 3;
  int rc;
  if ((rc = device_norm(S, B, B.b, nrm))) return rc;
  if ((rc = read_scalars(S, B, nrm, 1))) return rc;
  const double bnrm2 = B.hsc[0];
  const double atol = std::max(0.0, S.prm->gmres_tol * bnrm2);
  res->matvecs = 0;
  res->inner_iters = 0;
  if (bnrm2 == 0.0) {
    rc = ves_cuda_status(cudaMemcpyAsync(B.x, B.b, n * sizeof(double), cudaMemcpyDeviceToDevice, S.s), "x=b");
    res->info = 0;
    res->resid = 0;
    return rc;
  }
  // Mb_nrm2 = ||psolve(b)||
  if ((rc = psolve(S, B.b, B.t))) return rc;
  if ((rc = device_norm(S, B, B.t, nrm))) return rc;
  if ((rc = read_scalars(S, B, nrm, 1))) return rc;
  const double Mb_nrm2 = B.hsc[0];
  double ptol_max_factor = 1.0;
  double ptol = Mb_nrm2 * std::min(ptol_max_factor, atol / bnrm2);
  double presid = 0.0;
  std::vector<double> h((size_t)restart * (restart + 1), 0.0), giv((size_t)restart * 2, 0.0), Sv(restart + 1, 0.0),
      y(restart + 1, 0.0);
  auto H = [&](int col, int k) -> double& { return h[(size_t)col * (restart + 1) + k]; };
  int inner_iter = 0;
  double rnorm = 0.0;
  std::vector<double> rhist;  // true residual after each outer cycle
  bool stagnated = false;
  for (int iteration = 0; iteration < maxiter; ++iteration) {
    if (iteration == 0) {
      // r = b - A x (the initial guess [X; sigma] is nonzero in practice; an
      // all-zero guess gives r = b either way)
      if ((rc = matvec(S, B.x, B.t))) return rc;
      ves_count_launch();
      sub_kernel<<<g, 512, 0, S.s>>>(n, B.r, B.b, B.t);
      if ((rc = device_norm(S, B, B.r, nrm))) return rc;
      if ((rc = read_scalars(S, B, nrm, 1))) return rc;
      if (B.hsc[0] < atol) {
        rnorm = B.hsc[0];
        break;
      }
    }
    double* v0 = B.V;
    if ((rc = psolve(S, B.r, v0))) return rc;
    if ((rc = device_norm(S, B, v0, nrm))) return rc;
    ves_count_launch();
    scale_inv_kernel<<<g, 512, 0, S.s>>>(n, v0, v0, nrm, nullptr, eps);
    if ((rc = read_scalars(S, B, nrm, 1))) return rc;
    std::fill(Sv.begin(), Sv.end(), 0.0);
    Sv[0] = B.hsc[0];
    bool breakdown = false;
    int col = 0;
    for (col = 0; col < restart; ++col) {
      double* vc = B.V + (long long)col * n;
      double* vn = B.V + (long long)(col + 1) * n;
      if ((rc = matvec(S, vc, B.t))) return rc;
      if ((rc = psolve(S, B.t, B.w))) return rc;
      if ((rc = device_norm(S, B, B.w, h0))) return rc;
      for (int k = 0; k <= col; ++k) {
        launch_dot_partials(n, B.V + (long long)k * n, B.w, B.partials, S.s);
        ves_count_launch();
        mgs_axpy_kernel<<<g, 512, 0, S.s>>>(n, B.partials, dot_partial_blocks(), B.w, B.V + (long long)k * n, hcol + k);
      }
      if ((rc = device_norm(S, B, B.w, hcol + col + 1))) return rc;
      ves_count_launch();
      scale_inv_kernel<<<g, 512, 0, S.s>>>(n, vn, B.w, hcol + col + 1, h0, eps);
      if ((rc = ves_launch_check("mgs"))) return rc;
      if ((rc = read_scalars(S, B, B.dsc, restart + 3))) return rc;
      for (int k = 0; k <= col + 1; ++k) H(col, k) = B.hsc[k];
      const double h0v = B.hsc[restart + 2];
      const double h1 = H(col, col + 1);
      if (h1 <= eps * h0v) {
        H(col, col + 1) = 0.0;
        breakdown = true;
      }
      for (int k = 0; k < col; ++k) {
        const double cg = giv[2 * k], sg = giv[2 * k + 1];
        const double n0 = H(col, k), n1 = H(col, k + 1);
        H(col, k) = cg * n0 + sg * n1;
        H(col, k + 1) = -sg * n0 + cg * n1;
      }
      double cg, sg, mag;
      lartg(H(col, col), H(col, col + 1), cg, sg, mag);
      giv[2 * col] = cg;
      giv[2 * col + 1] = sg;
      H(col, col) = mag;
      H(col, col + 1) = 0.0;
      const double tmp = -sg * Sv[col];
      Sv[col] = cg * Sv[col];
      Sv[col + 1] = tmp;
      presid = fabs(tmp);
      inner_iter++;
      if (presid <= ptol || breakdown) break;
    }
    if (col == restart) col = restart - 1;
    if (H(col, col) == 0.0) Sv[col] = 0.0;
    for (int k = 0; k <= col; ++k) y[k] = Sv[k];
    for (int k = col; k > 0; --k) {
      if (y[k] != 0.0) {
        y[k] /= H(k, k);
        const double tmp = y[k];
        for (int j = 0; j < k; ++j) y[j] -= tmp * H(k, j);
      }
    }
    if (y[0] != 0.0) y[0] /= H(0, 0);
    if ((rc = ves_cuda_status(cudaMemcpyAsync(B.ydev, y.data(), (col + 1) * sizeof(double), cudaMemcpyHostToDevice,
                                              S.s),
                              "y upload")))
      return rc;
    ves_count_launch();
    update_x_kernel<<<g, 512, 0, S.s>>>(n, col + 1, B.ydev, B.V, B.x);
    if ((rc = matvec(S, B.x, B.t))) return rc;
    ves_count_launch();
    sub_kernel<<<g, 512, 0, S.s>>>(n, B.r, B.b, B.t);
    if ((rc = device_norm(S, B, B.r, nrm))) return rc;
    if ((rc = read_scalars(S, B, nrm, 1))) return rc;
    rnorm = B.hsc[0];
    if (rnorm <= atol) break;
    if (breakdown) break;
    // Stagnation at the arithmetic's noise floor (e.g. an FP32 all-pairs sum
    // against a 1e-10 tolerance): stop once three outer cycles have not
    // halved the true residual, instead of running to maxiter.
    rhist.push_back(rnorm);
    if (rhist.size() >= 4 && rnorm > 0.5 * rhist[rhist.size() - 4]) {
      stagnated = true;
      break;
    }
    if (presid <= ptol)
      ptol_max_factor = std::max(eps, 0.25 * ptol_max_factor);
    else
      ptol_max_factor = std::min(1.0, 1.5 * ptol_max_factor);
    ptol = presid * std::min(ptol_max_factor, atol / rnorm);
  }
  res->inner_iters = inner_iter;
  res->info = (rnorm <= atol) ? 0 : (stagnated ? -1 : maxiter);
  res->resid = rnorm / bnrm2;
  return VES_OK;
}

}  // namespace

// ---------------------------------------------------------------------------
static int biem_step_impl(ves_ctx* c, const ves_step_params* prm, int nv, const double* X, const double* sigma,
                          double* Xout, double* sigma_out, ves_step_result* res, WsCarver& ws, cudaStream_t s) {
  const int N = c->N, Nup = c->Nup;
  const long long n = 3LL * N * nv;
  const int restart = (int)std::min<long long>(prm->gmres_restart > 0 ? prm->gmres_restart : 20, n > 0 ? n : 1);
  const int maxc = prm->maxc > 0 ? prm->maxc : 64;
  const int maxe = prm->max_entries > 0 ? prm->max_entries : std::max(1024, nv * N);
  StepState S;
  memset(&S, 0, sizeof(S));
  S.c = c;
  S.prm = prm;
  S.nv = nv;
  S.N = N;
  S.Nup = Nup;
  S.n = n;
  S.s = s;
  S.X = X;
  S.sa = ws.take<double>((size_t)nv * N);
  S.isa = ws.take<double>((size_t)nv * N);
  S.tang = ws.take<double>((size_t)nv * 2 * N);
  S.Xup = ws.take<double>((size_t)nv * 2 * Nup);
  S.sa_up = ws.take<double>((size_t)nv * Nup);
  S.G = ws.take<double>((size_t)nv * 4 * N * N);
  S.LU = ws.take<double>((size_t)nv * 9 * N * N);
  S.piv = ws.take<int>((size_t)nv * 3 * N);
  S.f = ws.take<double>((size_t)nv * 2 * N);
  S.Gf = ws.take<double>((size_t)nv * 2 * N);
  S.LP = ws.take<double>((size_t)nv * 2 * N);
  S.nl.maxc = maxc;
  S.nl.cand_count = ws.take<int>(nv);
  S.nl.cand_src = ws.take<int>((size_t)nv * maxc);
  S.nl.excl_mask = ws.take<uint32_t>((size_t)nv * maxc * c->nwords_N);
  S.nl.hh_mask = ws.take<uint32_t>((size_t)nv * maxc * c->nwords_up);
  S.nl.max_entries = maxe;
  S.nl.n_entries = ws.take<int>(1);
  S.nl.ent_tsj = ws.take<int>((size_t)maxe * 3);
  S.nl.ent_icp = ws.take<int>((size_t)maxe);
  S.nl.ent_geo = ws.take<double>((size_t)maxe * 4);
  const bool vc = prm && prm->visc_cont != nullptr;  // viscosity contrast: double-layer terms
  S.visc = vc ? prm->visc_cont : nullptr;
  if (vc) {
    S.alpha = ws.take<double>(nv);
    S.D = ws.take<double>((size_t)nv * 4 * N * N);
    S.tang_up = ws.take<double>((size_t)nv * 2 * Nup);
    S.Xm = ws.take<double>((size_t)nv * 2 * N);
    S.DX = ws.take<double>((size_t)nv * 2 * N);
    S.vdl = ws.take<double>((size_t)nv * 2 * N);
    S.Fdl = ws.take<double>((size_t)nv * 2 * N);
  }
  S.dl_scheme = (prm && (prm->near_scheme == VES_NEAR_PY_HH || prm->near_scheme == VES_NEAR_PY_RBF))
                    ? VES_NEAR_PY_HH
                    : (prm ? prm->near_scheme : VES_NEAR_NONE);
  GmresBufs B;
  B.V = ws.take<double>((size_t)(restart + 1) * n);
  B.w = ws.take<double>(n);
  B.r = ws.take<double>(n);
  B.b = ws.take<double>(n);
  B.x = ws.take<double>(n);
  B.t = ws.take<double>(n);
  B.partials = ws.take<double>(dot_partial_blocks());
  B.dsc = ws.take<double>(restart + 8);
  B.ydev = ws.take<double>(restart + 2);
  double* vinf = ws.take<double>((size_t)nv * 2 * N);
  double* rhs2 = ws.take<double>((size_t)nv * N);
  // one scratch region shared by the sub-stages
  size_t scratch = 0;
  {
    WsCarver w(nullptr, 0);
    alpert_sl_matrix(c, nv, nullptr, prm->sl_precision, nullptr, w, s);
    scratch = std::max(scratch, w.off);
  }
  {
    WsCarver w(nullptr, 0);
    derivs_and_precond(c, nv, nullptr, nullptr, nullptr, 0, 0, nullptr, nullptr, nullptr, (double*)1, w, s);
    w.take<double>((size_t)nv * 4 * N * N);  // Ben
    w.take<double>((size_t)nv * 2 * N * N);  // Ten
    w.take<double>((size_t)nv * 2 * N * N);  // Div
    scratch = std::max(scratch, w.off);
    WsCarver w2(nullptr, 0);
    precond_f32(c, nv, nullptr, nullptr, nullptr, 0, 0, nullptr, w2, s);
    scratch = std::max(scratch, w2.off);
  }
  {
    WsCarver w(nullptr, 0);
    if (prm->near_scheme == VES_NEAR_MATLAB)
      near_zone_matlab(c, nv, nullptr, 0, nullptr, w, s);
    else
      near_zone_py(c, nv, nullptr, (const double*)1, 0, nullptr, w, s);
    scratch = std::max(scratch, w.off);
  }
  {
    WsCarver w(nullptr, 0);
    near_sing_int_run(c, prm->near_scheme, prm->farfield_precision, nv, nullptr, nullptr, nullptr, nullptr, nullptr,
                      nullptr, 0, nullptr, nullptr, w, s);
    scratch = std::max(scratch, w.off);
  }
  if (vc) {
    WsCarver w(nullptr, 0);
    stokes_dl_matrix(c, nv, nullptr, nullptr, prm->sl_precision, nullptr, w, s);
    scratch = std::max(scratch, w.off);
    WsCarver w2(nullptr, 0);
    near_sing_int_dl_run(c, S.dl_scheme, prm->farfield_precision, nv, nullptr, nullptr, nullptr, nullptr, nullptr,
                         nullptr, nullptr, nullptr,
                         0, nullptr, nullptr, w2, s);
    scratch = std::max(scratch, w2.off);
  }
  if (prm->repulsion) {  // force, G force, its near-field integral (RBF), the force's scratch
    WsCarver w(nullptr, 0);
    w.take<double>((size_t)3 * nv * 2 * N);
    w.take<char>(ves_repulsion_force_workspace(nv));
    near_sing_int_run(c, VES_NEAR_PY_RBF, prm->farfield_precision, nv, nullptr, nullptr, nullptr, nullptr, nullptr,
                      nullptr, 0, nullptr, nullptr, w, s);
    scratch = std::max(scratch, w.off);
  }
  S.scratch = ws.take<char>(scratch + 1024);
  S.scratch_bytes = scratch + 1024;
  if (ws.sizing) return VES_OK;
  if (!ws.ok()) {
    ves_record_error(VES_ERR_WORKSPACE, "biem_step: workspace too small (%zu needed)", ws.off);
    return VES_ERR_WORKSPACE;
  }
  if (!prm || !X || !sigma || !Xout || !sigma_out || nv <= 0) {
    ves_record_error(VES_ERR_ARG, "biem_step: bad arguments");
    return VES_ERR_ARG;
  }
  if (prm->near_scheme != VES_NEAR_NONE && prm->near_scheme != VES_NEAR_PY_HH && prm->near_scheme != VES_NEAR_MATLAB &&
      prm->near_scheme != VES_NEAR_PY_RBF) {
    ves_record_error(VES_ERR_ARG, "biem_step: bad near scheme");
    return VES_ERR_ARG;
  }
  if (prm->repulsion && prm->near_scheme != VES_NEAR_PY_HH && prm->near_scheme != VES_NEAR_PY_RBF) {
    ves_record_error(VES_ERR_ARG, "biem_step: repulsion needs the naiveNearZoneInfo lists (near py_hh or py_rbf)");
    return VES_ERR_ARG;
  }
  int rc = ves_reset_status(c, s);
  if (rc) return rc;
  if (restart + 8 > 256) {
    ves_record_error(VES_ERR_ARG, "biem_step: restart %d too large", restart);
    return VES_ERR_ARG;
  }
  B.hsc = c->h_scal;
  // geometry (capsules(X), poten.stokesSLmatrix, near zone)
  launch_diff_prop(c, 0, nv, X, S.sa, S.isa, S.tang, nullptr, s);
  launch_upsample_deriv(c, nv, X, S.Xup, nullptr, S.sa_up, s);
  {
    WsCarver sub(S.scratch, S.scratch_bytes);
    if ((rc = alpert_sl_matrix(c, nv, X, prm->sl_precision, S.G, sub, s))) goto done;
  }
  if (vc) {
    // alpha, the upsampled tangents and poten.stokesDLmatrix (tstep_biem.py:195, 203-205)
    ves_count_launch();
    alpha_kernel<<<ceil_div(nv, 256), 256, 0, s>>>(nv, S.visc, S.alpha);
    launch_upsample_geom(c, nv, X, nullptr, nullptr, S.tang_up, nullptr, s);
    WsCarver sub(S.scratch, S.scratch_bytes);
    if ((rc = stokes_dl_matrix(c, nv, X, S.visc, prm->sl_precision, S.D, sub, s))) goto done;
  }
  S.h = 0.0;
  if (prm->near_scheme == VES_NEAR_MATLAB) {
    WsCarver sub(S.scratch, S.scratch_bytes);
    if ((rc = near_zone_matlab(c, nv, X, 0.0, &S.nl, sub, s))) goto done;
    // h = min length / N (capsules.py:46-47)
    double* len = (double*)S.scratch;
    launch_geom_prop(c, nv, X, nullptr, nullptr, len, s);
    std::vector<double> hl(nv);
    if ((rc = ves_cuda_status(cudaMemcpyAsync(hl.data(), len, nv * sizeof(double), cudaMemcpyDeviceToHost, s), "len")))
      goto done;
    if ((rc = ves_cuda_status(cudaStreamSynchronize(s), "len sync"))) goto done;
    S.h = *std::min_element(hl.begin(), hl.end()) / N;
  } else if (prm->near_scheme == VES_NEAR_PY_HH || prm->near_scheme == VES_NEAR_PY_RBF) {
    WsCarver sub(S.scratch, S.scratch_bytes);
    if ((rc = near_zone_py(c, nv, X, S.Xup, 0.0, &S.nl, sub, s))) goto done;
  }
  // right-hand side [X + dt*vinf; surfaceDiv(X)], with the double layer of X
  // (Fdlp + D X, tstep_biem.py:231-244) and the repulsion when present
  launch_bg_flow(nv, N, prm->flow, prm->speed, prm->chan_width, prm->vortex_size, X, vinf, s);
  if (vc) {
    const long long n2 = (long long)nv * 2 * N;
    launch_bgemv_f64(nv, 2 * N, 2 * N, S.D, X, 2LL * N, S.DX, 2LL * N, s);
    ves_count_launch();
    dl_self_kernel<<<ceil_div(n2, 256), 256, 0, s>>>(n2, N, S.visc, X, 2LL * N, S.DX, S.vdl);
    WsCarver sub(S.scratch, S.scratch_bytes);
    if ((rc = near_sing_int_dl_run(c, S.dl_scheme, prm->farfield_precision, nv, X, S.Xup, S.tang_up, S.sa_up, S.visc,
                                   X, S.vdl, &S.nl, S.h,
                                   S.Fdl, nullptr, sub, s)))
      goto done;
  }
  if (prm->repulsion && nv > 1) {
    // repulsion on the current shapes: G rep + nearSingInt_rbf(rep) (tstep_biem.py:250-264)
    WsCarver sub(S.scratch, S.scratch_bytes);
    double* rp = sub.take<double>((size_t)nv * 2 * N);
    double* rG = sub.take<double>((size_t)nv * 2 * N);
    double* rN = sub.take<double>((size_t)nv * 2 * N);
    const size_t rws = ves_repulsion_force_workspace(nv);
    char* rw = sub.take<char>(rws);
    if ((rc = ves_repulsion_force(N, nv, X, prm->rep_strength, prm->min_dist, rp, rw, rws, s))) goto done;
    launch_bgemv_f64(nv, 2 * N, 2 * N, S.G, rp, 2LL * N, rG, 2LL * N, s);
    if ((rc = near_sing_int_run(c, VES_NEAR_PY_RBF, prm->farfield_precision, nv, X, S.sa_up, S.Xup, rp, rG, &S.nl,
                                S.h, rN, nullptr, sub, s)))
      goto done;
    ves_count_launch();
    rhs_pos_kernel<<<ceil_div((long long)nv * 2 * N, 256), 256, 0, s>>>(
        (long long)nv * 2 * N, N, prm->dt, X, vinf, rG, rN, vc ? S.Fdl : nullptr, S.DX, S.alpha, vinf);
  } else {
    ves_count_launch();
    rhs_pos_kernel<<<ceil_div((long long)nv * 2 * N, 256), 256, 0, s>>>(
        (long long)nv * 2 * N, N, prm->dt, X, vinf, nullptr, nullptr, vc ? S.Fdl : nullptr, S.DX, S.alpha, vinf);
  }
  launch_surface_div(c, nv, S.isa, S.tang, X, 2LL * N, rhs2, N, s);
  ves_count_launch();
  pack_kernel<<<ceil_div(n, 256), 256, 0, s>>>(nv, N, vinf, rhs2, B.b);
  if (prm->use_preco) {
    ves_count_launch();
    pack_kernel<<<ceil_div(n, 256), 256, 0, s>>>(nv, N, X, sigma, B.x);
  } else {
    // without the preconditioner the reference calls gmres without x0 (tstep_biem.py:383)
    if ((rc = ves_cuda_status(cudaMemsetAsync(B.x, 0, n * sizeof(double), s), "x0"))) goto done;
  }
  // preconditioner
  if (prm->use_preco && precond_is_f32(prm)) {
    WsCarver sub(S.scratch, S.scratch_bytes);
    if ((rc = precond_f32(c, nv, S.isa, S.tang, S.G, prm->dt, prm->kappa, (float*)S.LU, sub, s))) goto done;
    if ((rc = launch_lu_factor_f32(c, nv, 3 * N, (float*)S.LU, S.piv, s))) goto done;
  } else if (prm->use_preco) {
    WsCarver sub(S.scratch, S.scratch_bytes);
    double* Ben = nullptr;
    double* Ten = sub.take<double>((size_t)nv * 2 * N * N);
    double* Div = sub.take<double>((size_t)nv * 2 * N * N);
    if ((rc = derivs_and_precond(c, nv, S.isa, S.tang, S.G, prm->dt, prm->kappa, Ben, Ten, Div, S.LU, sub, s,
                                 vc ? S.D : nullptr, vc ? S.alpha : nullptr)))
      goto done;
    if ((rc = launch_lu_factor(c, nv, 3 * N, S.LU, S.piv, s))) goto done;
  }
  if ((rc = ves_check_status(c, s, "biem_step setup"))) goto done;
  S.matvecs = 0;
  rc = gmres(S, B, res);
  if (rc) goto done;
  res->matvecs = S.matvecs;
  ves_count_launch();
  unpack_kernel<<<ceil_div(n, 256), 256, 0, s>>>(nv, N, B.x, Xout, sigma_out);
  {
    int nn = 0;
    if (prm->near_scheme == VES_NEAR_MATLAB)
      cudaMemcpyAsync(&nn, S.nl.n_entries, sizeof(int), cudaMemcpyDeviceToHost, s);
    res->n_near_entries = nn;
  }
  rc = ves_check_status(c, s, "biem_step");
  if (!rc && res->info != 0) {
    ves_record_error(VES_ERR_GMRES_MAXIT, "biem_step: GMRES reached maxiter (resid %.3e)", res->resid);
    rc = VES_ERR_GMRES_MAXIT;
  }
done:
  if (rc == VES_ERR_NEARLIST_OVERFLOW && prm->near_scheme == VES_NEAR_MATLAB && res && S.nl.n_entries) {
    // the MATLAB entry count keeps running past the capacity: report what is needed
    int nn = 0;
    if (cudaMemcpyAsync(&nn, S.nl.n_entries, sizeof(int), cudaMemcpyDeviceToHost, s) == cudaSuccess &&
        cudaStreamSynchronize(s) == cudaSuccess)
      res->n_near_entries = nn;
  }
  return rc;
}

extern "C" size_t ves_biem_step_workspace(ves_ctx* c, const ves_step_params* prm, int nv) {
  if (!c || !prm) return 0;
  WsCarver w(nullptr, 0);
  ves_step_result r;
  biem_step_impl(c, prm, nv, nullptr, nullptr, nullptr, nullptr, &r, w, 0);
  return w.off + 256;
}

extern "C" int ves_biem_step(ves_ctx* c, const ves_step_params* prm, int nv, const double* X, const double* sigma,
                             double* Xout, double* sigma_out, ves_step_result* res, void* ws, size_t ws_bytes,
                             void* stream) {
  if (!c || !prm || !res || !ws) return VES_ERR_ARG;
  memset(res, 0, sizeof(*res));
  WsCarver w(ws, ws_bytes);
  return biem_step_impl(c, prm, nv, X, sigma, Xout, sigma_out, res, w, (cudaStream_t)stream);
}

// ---------------------------------------------------------------------------
// One implicit step of a suspension given as groups of different point counts
// (every group's vesicles in one GMRES system; no viscosity contrast, no
// repulsion; near scheme matlab or none).  Within a group the step is the
// single-N step's; between groups see MixedState.
static int biem_step_mixed_impl(int ng, ves_ctx* const* ctx, const ves_step_params* prm, const int* nvs,
                                const double* const* X, const double* const* sigma, double* const* Xout,
                                double* const* sigma_out, ves_step_result* res, WsCarver& ws, cudaStream_t s) {
  if (ng < 1 || ng > kMaxGroups || !ctx || !prm || !nvs) {
    if (!ws.sizing) ves_record_error(VES_ERR_ARG, "biem_step_mixed: 1 to %d groups", kMaxGroups);
    return VES_ERR_ARG;
  }
  for (int g = 0; g < ng; ++g)
    if (!ctx[g] || nvs[g] < 1) {
      if (!ws.sizing) ves_record_error(VES_ERR_ARG, "biem_step_mixed: bad group %d", g);
      return VES_ERR_ARG;
    }
  const int maxc = prm->maxc > 0 ? prm->maxc : 64;
  MixedState M;
  memset(&M, 0, sizeof(M));
  M.prm = prm;
  M.ng = ng;
  M.s = s;
  M.off[0] = 0;
  for (int g = 0; g < ng; ++g) M.off[g + 1] = M.off[g] + 3LL * ctx[g]->N * nvs[g];
  const long long n = M.off[ng];
  M.n = n;
  const int restart = (int)std::min<long long>(prm->gmres_restart > 0 ? prm->gmres_restart : 20, n > 0 ? n : 1);
  double* vinf[kMaxGroups];
  double* rhs2[kMaxGroups];
  for (int g = 0; g < ng; ++g) {
    ves_ctx* c = ctx[g];
    const int nv = nvs[g], N = c->N, Nup = c->Nup;
    const int maxe = prm->max_entries > 0 ? prm->max_entries : std::max(1024, nv * N);
    StepState& S = M.g[g];
    S.c = c;
    S.prm = prm;
    S.nv = nv;
    S.N = N;
    S.Nup = Nup;
    S.n = 3LL * N * nv;
    S.s = s;
    S.X = X ? X[g] : nullptr;
    S.sa = ws.take<double>((size_t)nv * N);
    S.isa = ws.take<double>((size_t)nv * N);
    S.tang = ws.take<double>((size_t)nv * 2 * N);
    S.Xup = ws.take<double>((size_t)nv * 2 * Nup);
    S.sa_up = ws.take<double>((size_t)nv * Nup);
    S.G = ws.take<double>((size_t)nv * 4 * N * N);
    S.LU = ws.take<double>((size_t)nv * 9 * N * N);
    S.piv = ws.take<int>((size_t)nv * 3 * N);
    S.f = ws.take<double>((size_t)nv * 2 * N);
    S.Gf = ws.take<double>((size_t)nv * 2 * N);
    S.LP = ws.take<double>((size_t)nv * 2 * N);
    S.nl.maxc = maxc;
    S.nl.cand_count = ws.take<int>(nv);
    S.nl.cand_src = ws.take<int>((size_t)nv * maxc);
    S.nl.excl_mask = ws.take<uint32_t>((size_t)nv * maxc * c->nwords_N);
    S.nl.hh_mask = ws.take<uint32_t>((size_t)nv * maxc * c->nwords_up);
    S.nl.max_entries = maxe;
    S.nl.n_entries = ws.take<int>(1);
    S.nl.ent_tsj = ws.take<int>((size_t)maxe * 3);
    S.nl.ent_icp = ws.take<int>((size_t)maxe);
    S.nl.ent_geo = ws.take<double>((size_t)maxe * 4);
    M.fup[g] = ws.take<double>((size_t)nv * 2 * Nup);
    M.den[g] = ws.take<double>((size_t)nv * 2 * Nup);
    vinf[g] = ws.take<double>((size_t)nv * 2 * N);
    rhs2[g] = ws.take<double>((size_t)nv * N);
    for (int q = 0; q < ng; ++q) {
      if (q == g) continue;
      ves_near_lists& L = M.xl[g][q];
      L.maxc = maxc;
      L.cand_count = ws.take<int>(nv);
      L.cand_src = ws.take<int>((size_t)nv * maxc);
      L.excl_mask = ws.take<uint32_t>((size_t)nv * maxc * c->nwords_N);
      L.max_entries = maxe;
      L.n_entries = ws.take<int>(1);
      L.ent_tsj = ws.take<int>((size_t)maxe * 3);
      L.ent_icp = ws.take<int>((size_t)maxe);
      L.ent_geo = ws.take<double>((size_t)maxe * 4);
    }
  }
  GmresBufs B;
  B.V = ws.take<double>((size_t)(restart + 1) * n);
  B.w = ws.take<double>(n);
  B.r = ws.take<double>(n);
  B.b = ws.take<double>(n);
  B.x = ws.take<double>(n);
  B.t = ws.take<double>(n);
  B.partials = ws.take<double>(dot_partial_blocks());
  B.dsc = ws.take<double>(restart + 8);
  B.ydev = ws.take<double>(restart + 2);
  size_t scratch = 0;
  for (int g = 0; g < ng; ++g) {
    ves_ctx* c = ctx[g];
    const int nv = nvs[g], N = c->N;
    {
      WsCarver w(nullptr, 0);
      alpert_sl_matrix(c, nv, nullptr, prm->sl_precision, nullptr, w, s);
      scratch = std::max(scratch, w.off);
    }
    {
      WsCarver w(nullptr, 0);
      derivs_and_precond(c, nv, nullptr, nullptr, nullptr, 0, 0, nullptr, nullptr, nullptr, (double*)1, w, s);
      w.take<double>((size_t)nv * 2 * N * N);  // Ten
      w.take<double>((size_t)nv * 2 * N * N);  // Div
      scratch = std::max(scratch, w.off);
      WsCarver w2(nullptr, 0);
      precond_f32(c, nv, nullptr, nullptr, nullptr, 0, 0, nullptr, w2, s);
      scratch = std::max(scratch, w2.off);
    }
    {
      WsCarver w(nullptr, 0);
      near_zone_matlab(c, nv, nullptr, 0, nullptr, w, s);
      scratch = std::max(scratch, w.off);
    }
    {
      WsCarver w(nullptr, 0);
      near_sing_int_run(c, prm->near_scheme, prm->farfield_precision, nv, nullptr, nullptr, nullptr, nullptr, nullptr,
                        nullptr, 0, nullptr, nullptr, w, s);
      scratch = std::max(scratch, w.off);
    }
    for (int q = 0; q < ng; ++q) {
      if (q == g) continue;
      WsCarver w(nullptr, 0);
      near_zone_matlab_cross(c, ctx[q], nv, nullptr, nvs[q], nullptr, 1.0, nullptr, w, s);
      scratch = std::max(scratch, w.off);
      WsCarver w2(nullptr, 0);
      near_sing_int_cross_add(c, ctx[q], prm->near_scheme, prm->farfield_precision, nv, nullptr, nvs[q], nullptr,
                              nullptr, nullptr, nullptr, 1.0, nullptr, w2, s);
      scratch = std::max(scratch, w2.off);
    }
  }
  if (ng > 1 && prm->farfield_precision == VES_PREC_FP32M) {
    for (int g = 0; g < ng; ++g) {  // shapes only: the sizing pass reads no pointer
      M.g[g].nv = nvs[g];
      M.g[g].N = ctx[g]->N;
      M.g[g].Nup = ctx[g]->Nup;
      M.g[g].c = ctx[g];
    }
    M.scratch_bytes = 0;
    mixed_farfield_merged(M, true);
    scratch = std::max(scratch, M.scratch_bytes);
  }
  M.scratch = ws.take<char>(scratch + 1024);
  M.scratch_bytes = scratch + 1024;
  if (ws.sizing) return VES_OK;
  if (!ws.ok()) {
    ves_record_error(VES_ERR_WORKSPACE, "biem_step_mixed: workspace too small (%zu needed)", ws.off);
    return VES_ERR_WORKSPACE;
  }
  if (!X || !sigma || !Xout || !sigma_out || !res) {
    ves_record_error(VES_ERR_ARG, "biem_step_mixed: bad arguments");
    return VES_ERR_ARG;
  }
  if (prm->near_scheme != VES_NEAR_NONE && prm->near_scheme != VES_NEAR_MATLAB) {
    ves_record_error(VES_ERR_ARG, "biem_step_mixed: near scheme must be matlab or none");
    return VES_ERR_ARG;
  }
  if (prm->visc_cont || prm->repulsion) {
    ves_record_error(VES_ERR_ARG, "biem_step_mixed: no viscosity contrast or repulsion between groups");
    return VES_ERR_ARG;
  }
  if (restart + 8 > 256) {
    ves_record_error(VES_ERR_ARG, "biem_step_mixed: restart %d too large", restart);
    return VES_ERR_ARG;
  }
  int rc = 0;
  for (int g = 0; g < ng; ++g)
    if ((rc = ves_reset_status(ctx[g], s))) return rc;
  B.hsc = ctx[0]->h_scal;
  // geometry, h = min length / N of each group (capsules.py:46-47), in-group zones
  {
    std::vector<double> hl;
    for (int g = 0; g < ng; ++g) {
      StepState& S = M.g[g];
      if (S.nv == 0) continue;
      launch_diff_prop(S.c, 0, S.nv, S.X, S.sa, S.isa, S.tang, nullptr, s);
      launch_upsample_deriv(S.c, S.nv, S.X, S.Xup, nullptr, S.sa_up, s);
      WsCarver sub(M.scratch, M.scratch_bytes);
      if ((rc = alpert_sl_matrix(S.c, S.nv, S.X, prm->sl_precision, S.G, sub, s))) return rc;
      double* len = (double*)M.scratch;
      launch_geom_prop(S.c, S.nv, S.X, nullptr, nullptr, len, s);
      hl.resize(S.nv);
      if ((rc = ves_cuda_status(cudaMemcpyAsync(hl.data(), len, S.nv * sizeof(double), cudaMemcpyDeviceToHost, s),
                                "len")))
        return rc;
      if ((rc = ves_cuda_status(cudaStreamSynchronize(s), "len sync"))) return rc;
      M.h[g] = S.h = *std::min_element(hl.begin(), hl.end()) / S.N;
      if (prm->near_scheme == VES_NEAR_MATLAB) {
        WsCarver sub2(M.scratch, M.scratch_bytes);
        if ((rc = near_zone_matlab(S.c, S.nv, S.X, S.h, &S.nl, sub2, s))) return rc;
      }
    }
  }
  if (prm->near_scheme == VES_NEAR_MATLAB) {
    for (int g = 0; g < ng; ++g)
      for (int q = 0; q < ng; ++q) {
        if (q == g || M.g[g].nv == 0) continue;
        WsCarver sub(M.scratch, M.scratch_bytes);
        if ((rc = near_zone_matlab_cross(ctx[g], ctx[q], M.g[g].nv, X[g], M.g[q].nv, X[q],
                                         M.g[q].nv > 0 ? M.h[q] : 1.0, &M.xl[g][q], sub, s)))
          return rc;
      }
  }
  // right-hand side and initial guess, group by group; the preconditioner blocks
  for (int g = 0; g < ng; ++g) {
    StepState& S = M.g[g];
    const int nv = S.nv, N = S.N;
    if (nv == 0) continue;
    const long long n2 = (long long)nv * 2 * N;
    launch_bg_flow(nv, N, prm->flow, prm->speed, prm->chan_width, prm->vortex_size, S.X, vinf[g], s);
    ves_count_launch();
    rhs_pos_kernel<<<ceil_div(n2, 256), 256, 0, s>>>(n2, N, prm->dt, S.X, vinf[g], nullptr, nullptr, nullptr, nullptr,
                                                     nullptr, vinf[g]);
    launch_surface_div(S.c, nv, S.isa, S.tang, S.X, 2LL * N, rhs2[g], N, s);
    ves_count_launch();
    pack_kernel<<<ceil_div(S.n, 256), 256, 0, s>>>(nv, N, vinf[g], rhs2[g], B.b + M.off[g]);
    if (prm->use_preco) {
      ves_count_launch();
      pack_kernel<<<ceil_div(S.n, 256), 256, 0, s>>>(nv, N, S.X, sigma[g], B.x + M.off[g]);
      WsCarver sub(M.scratch, M.scratch_bytes);
      if (precond_is_f32(prm)) {
        if ((rc = precond_f32(S.c, nv, S.isa, S.tang, S.G, prm->dt, prm->kappa, (float*)S.LU, sub, s))) return rc;
        if ((rc = launch_lu_factor_f32(S.c, nv, 3 * N, (float*)S.LU, S.piv, s))) return rc;
      } else {
        double* Ten = sub.take<double>((size_t)nv * 2 * N * N);
        double* Div = sub.take<double>((size_t)nv * 2 * N * N);
        if ((rc = derivs_and_precond(S.c, nv, S.isa, S.tang, S.G, prm->dt, prm->kappa, nullptr, Ten, Div, S.LU, sub,
                                     s)))
          return rc;
        if ((rc = launch_lu_factor(S.c, nv, 3 * N, S.LU, S.piv, s))) return rc;
      }
    }
  }
  if (!prm->use_preco && n > 0)
    if ((rc = ves_cuda_status(cudaMemsetAsync(B.x, 0, n * sizeof(double), s), "x0"))) return rc;
  for (int g = 0; g < ng; ++g)
    if ((rc = ves_check_status(ctx[g], s, "biem_step_mixed setup"))) {
      if (rc == VES_ERR_NEARLIST_OVERFLOW && prm->near_scheme == VES_NEAR_MATLAB) {
        // report the largest MATLAB entry count met (they run past the capacity)
        int worst = 0;
        for (int a = 0; a < ng; ++a)
          for (int q = 0; q < ng; ++q) {
            const int* ne = (a == q) ? M.g[a].nl.n_entries : M.xl[a][q].n_entries;
            int nn = 0;
            if (M.g[a].nv > 0 && ne && cudaMemcpyAsync(&nn, ne, sizeof(int), cudaMemcpyDeviceToHost, s) == cudaSuccess &&
                cudaStreamSynchronize(s) == cudaSuccess && nn > worst)
              worst = nn;
          }
        res->n_near_entries = worst;
      }
      return rc;
    }
  M.matvecs = 0;
  if ((rc = gmres(M, B, res))) return rc;
  res->matvecs = M.matvecs;
  int nn_total = 0;
  for (int g = 0; g < ng; ++g) {
    StepState& S = M.g[g];
    if (S.nv == 0) continue;
    ves_count_launch();
    unpack_kernel<<<ceil_div(S.n, 256), 256, 0, s>>>(S.nv, S.N, B.x + M.off[g], Xout[g], sigma_out[g]);
    if (prm->near_scheme == VES_NEAR_MATLAB) {
      int nn = 0;
      cudaMemcpyAsync(&nn, S.nl.n_entries, sizeof(int), cudaMemcpyDeviceToHost, s);
      cudaStreamSynchronize(s);
      nn_total += nn;
      for (int q = 0; q < ng; ++q) {
        if (q == g) continue;
        cudaMemcpyAsync(&nn, M.xl[g][q].n_entries, sizeof(int), cudaMemcpyDeviceToHost, s);
        cudaStreamSynchronize(s);
        nn_total += nn;
      }
    }
  }
  res->n_near_entries = nn_total;
  for (int g = 0; g < ng; ++g)
    if ((rc = ves_check_status(ctx[g], s, "biem_step_mixed"))) return rc;
  if (res->info != 0) {
    ves_record_error(VES_ERR_GMRES_MAXIT, "biem_step_mixed: GMRES reached maxiter (resid %.3e)", res->resid);
    return VES_ERR_GMRES_MAXIT;
  }
  return VES_OK;
}

extern "C" size_t ves_biem_step_mixed_workspace(int ngroups, ves_ctx* const* ctx, const ves_step_params* prm,
                                                const int* nv) {
  WsCarver w(nullptr, 0);
  ves_step_result r;
  if (biem_step_mixed_impl(ngroups, ctx, prm, nv, nullptr, nullptr, nullptr, nullptr, &r, w, 0)) return 0;
  return w.off + 256;
}

extern "C" int ves_biem_step_mixed(int ngroups, ves_ctx* const* ctx, const ves_step_params* prm, const int* nv,
                                   const double* const* X, const double* const* sigma, double* const* Xout,
                                   double* const* sigma_out, ves_step_result* res, void* ws, size_t ws_bytes,
                                   void* stream) {
  if (!ctx || !prm || !res || !ws || !nv) return VES_ERR_ARG;
  memset(res, 0, sizeof(*res));
  WsCarver w(ws, ws_bytes);
  return biem_step_mixed_impl(ngroups, ctx, prm, nv, X, sigma, Xout, sigma_out, res, w, (cudaStream_t)stream);
}
