// Internal declarations shared by the ves2d translation units.
#pragma once

#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

#include "../../include/ves2d_gb300.h"
#include "ves_common.cuh"

// Per-N constant tables, resident on one device (created by ves_ctx_create).
struct ves_ctx {
  int N, Nup, m, nquad, device;
  int nwords_N;   // ceil(N/32)
  int nwords_up;  // ceil(Nup/32)
  void* d_buf;    // single allocation holding every table below
  // FP64 tables
  double* d1N;     // [N]    first-derivative circulant on the N grid (Nyquist zeroed)
  double* d1Nup;   // [Nup]  same on the Nup grid
  double* pc;      // [Nup]  N->Nup prolongation circulant: P[u][i] = pc[(u - m i) mod Nup]
  double* pcd;     // [Nup]  its derivative (d/dtheta of the interpolant)
  double* pcdd;    // [Nup]  its second derivative
  double* qw;      // [nquad] Alpert weights (already / 4pi)
  double* cq;      // [14][Nup] coarse cardinal at the 14 off-grid Alpert nodes
  double* adense;  // [14][Nup] Nup-grid trig interpolation rows of the 14 off-grid nodes
  double* Rm;      // [N][Nup] restriction
  double* Pm;      // [Nup][N] prolongation
  double* lag;     // [7][7]  Lagrange interpolation matrix (poten.py:977-990)
  double* cos6;    // [6N]  cos(2 pi r / 6N) (FFT twiddles of the arc-length reparametrisation grid)
  double* sin6;    // [6N]  sin(2 pi r / 6N)
  double* cosU;    // [Nup] cos(2 pi r / Nup)
  double* sinU;    // [Nup] sin(2 pi r / Nup)
  // FP32 copies used by the mixed-precision Alpert build
  float* Rm32;
  float* Pm32;
  float* adense32;
  float* qw32;
  VesDeviceStatus* status;  // device status word (reset per API call)
  VesDeviceStatus* h_status;// pinned host mirror
  double* h_scal;            // pinned host scalars (GMRES read-back), 256 doubles
  int* h_ints;               // pinned host ints (near-list candidate count read-back), 16
  int last_max_cand;         // largest candidate count of the last near-zone build (any vesicle)
  // optional timing of the all-pairs kernel
  int timing;
  int n_ev;                  // recorded event pairs not yet accumulated
  cudaEvent_t ev[2 * 256];
  double ev_pairs[256];
  long long ff_launches;
  double ff_ms, ff_pairs;
  unsigned long long* d_mp;  // multipole path work counters (device, 2), allocated with timing
  // optional timing of the network forward passes (MLARM step)
  int n_nev;
  cudaEvent_t nev[2 * 64];
  double nev_flops[64];
  long long net_launches;
  double net_ms, net_flops;
};

// launch accounting (every kernel launch site calls ves_count_launch)
void ves_count_launch(int n = 1);
// all-pairs kernel timing hooks (no-ops unless timing is on)
void ves_ff_timing_begin(ves_ctx* c, cudaStream_t s);
void ves_ff_timing_end(ves_ctx* c, cudaStream_t s, double pairs);
// network forward timing hooks (no-ops unless timing is on); flops = useful work of the pass
void ves_net_timing_begin(ves_ctx* c, cudaStream_t s);
void ves_net_timing_end(ves_ctx* c, cudaStream_t s, double flops);

// status plumbing -----------------------------------------------------------
int ves_reset_status(ves_ctx* ctx, cudaStream_t s);
int ves_check_status(ves_ctx* ctx, cudaStream_t s, const char* stage);  // syncs the stream
int ves_launch_check(const char* what);                                 // cudaGetLastError

// workspace carving ------------------------------------------------------------
struct WsCarver {
  char* base;
  size_t cap, off;
  bool sizing;  // true: only count bytes
  WsCarver(void* b, size_t c) : base((char*)b), cap(c), off(0), sizing(b == nullptr) {}
  template <typename T>
  T* take(size_t count) {
    off = (off + 255) & ~(size_t)255;
    T* p = sizing ? nullptr : (T*)(base + off);
    off += count * sizeof(T);
    return p;
  }
  bool ok() const { return sizing || off <= cap; }
};

// launchers (implemented in the .cu files) ------------------------------------
// spectral / geometry
void launch_upsample(const ves_ctx* c, int nv, int ncomp, const double* in, long long in_stride,
                     double* out, cudaStream_t s);
void launch_upsample_deriv(const ves_ctx* c, int nv, const double* X, double* Xup, double* dXup,
                           double* sa_up, cudaStream_t s);
void launch_diff_prop(const ves_ctx* c, int grid, int nv, const double* X, double* sa, double* isa,
                      double* tang, double* cur, cudaStream_t s);
// geometry of the Nup-upsampled curve (capsules(interpft(X, Nup))) from the
// derivatives of the trig interpolant: Xup, sa, unit tangent, curvature (any may be null)
void launch_upsample_geom(const ves_ctx* c, int nv, const double* X, double* Xup, double* sa, double* tang,
                          double* cur, cudaStream_t s);
void launch_geom_prop(const ves_ctx* c, int nv, const double* X, double* ra, double* area,
                      double* length, cudaStream_t s);
void launch_trac_jump(const ves_ctx* c, int nv, double kappa, const double* isa, const double* tang,
                      const double* X, long long xs, const double* sig, long long ss, double* f,
                      cudaStream_t s);
void launch_surface_div(const ves_ctx* c, int nv, const double* isa, const double* tang,
                        const double* f, long long fs, double* out, long long os, cudaStream_t s);
void launch_bg_flow(int nv, int N, int flow, double speed, double cw, double vs, const double* X,
                    double* v, cudaStream_t s);
void launch_density(int nv, int ns, const double* f, const double* sa, double* den, cudaStream_t s);
// Dm (or NULL): double-layer matrices [nv][2N][2N]; alpha (or NULL): (1 + visc)/2 per vesicle
int derivs_and_precond(ves_ctx* c, int nv, const double* isa, const double* tang, const double* G,
                       double dt, double kappa, double* Ben, double* Ten, double* Div, double* M,
                       WsCarver& ws, cudaStream_t s, const double* Dm = nullptr, const double* alpha = nullptr);
// the block-diagonal preconditioner of derivs_and_precond built with FP32
// products into M32 [nv][3N][3N] (no viscosity contrast)
int precond_f32(ves_ctx* c, int nv, const double* isa, const double* tang, const double* G, double dt, double kappa,
                float* M32, WsCarver& ws, cudaStream_t s);

// dense per-vesicle algebra
void launch_bgemm_f64(int batch, int M, int N, int K, double alpha, const double* A, int lda,
                      long long sA, const double* B, int ldb, long long sB, double beta, double* C,
                      int ldc, long long sC, cudaStream_t s);
void launch_bgemm_f32(int batch, int M, int N, int K, float alpha, const float* A, int lda,
                      long long sA, const float* B, int ldb, long long sB, float beta, float* C,
                      int ldc, long long sC, cudaStream_t s);
void launch_bgemv_f64(int nv, int m, int n, const double* A, const double* x, long long xs,
                      double* y, long long ys, cudaStream_t s);
int launch_lu_factor(ves_ctx* c, int nv, int n, double* A, int* piv, cudaStream_t s);
void launch_lu_solve(int nv, int n, const double* LU, const int* piv, const double* b, double* x,
                     cudaStream_t s);
// FP32 factorisation / solve with it (FP64 vectors)
int launch_lu_factor_f32(ves_ctx* c, int nv, int n, float* A, int* piv, cudaStream_t s);
void launch_lu_solve_f32(int nv, int n, const float* LU, const int* piv, const double* b, double* x,
                         cudaStream_t s);

// Alpert
int alpert_sl_matrix(ves_ctx* c, int nv, const double* X, int precision, double* G, WsCarver& ws,
                     cudaStream_t s);

// far field
// Execution environment of the all-pairs driver: the device status word, the
// number of target points per column the near-list masks are laid out for,
// and the context whose timing hooks record the launch (may be null).
struct FFEnv {
  VesDeviceStatus* status;
  int N;
  ves_ctx* timing;  // context whose timing hooks and counters record the launch (may be null)
};
int farfield_run_env(const FFEnv& env, int precision, int nsrc, int ns, const double* Xsrc, const double* den,
                     int nt, int ntp, const double* Xtar, const int* self_idx, const ves_near_lists* nl,
                     double* out, WsCarver& ws, cudaStream_t s);
// multipole expansion for separated vesicle pairs, direct FP32 sum for the rest (VES_PREC_FP32M)
int farfield_mp_run(const FFEnv& env, int nsrc, int ns, const double* Xsrc, const double* den, int nt, int ntp,
                    const double* Xtar, const int* self_idx, const ves_near_lists* nl, double* out, WsCarver& ws,
                    cudaStream_t s);
// Every target vesicle of ng point sets (ng <= 4) against every source
// vesicle of the ng sets in one launch (precision VES_PREC_FP32M): targets of
// set g are nt[g] vesicles of ntp[g] points Xtar[g]; sources of set q are
// nsrc[q] vesicles of ns[q] upsampled points Xsrc[q] with densities den[q];
// nl[g*ng + q] is the near list of targets g against sources q (nullptr:
// none); a target's own vesicle (q == g) is skipped; out[g] [nt][2][ntp]
// (overwritten), scaled like farfield_run's.
int farfield_mp_groups_run(const FFEnv& env, int ng, const int* nsrc, const int* ns, const double* const* Xsrc,
                           const double* const* den, const int* nt, const int* ntp, const double* const* Xtar,
                           const ves_near_lists* const* nl, double* const* out, WsCarver& ws, cudaStream_t s);
int farfield_run(ves_ctx* c, int precision, int nsrc, int ns, const double* Xsrc, const double* den,
                 int nt, int ntp, const double* Xtar, const int* self_idx, const ves_near_lists* nl,
                 double* out, WsCarver& ws, cudaStream_t s);

// near zone / near-singular corrections
int near_zone_py(ves_ctx* c, int nv, const double* X, const double* Xup, double thresh,
                 const ves_near_lists* nl, WsCarver& ws, cudaStream_t s);
int near_zone_matlab(ves_ctx* c, int nv, const double* X, double h, const ves_near_lists* nl,
                     WsCarver& ws, cudaStream_t s);
int near_sing_int_run(ves_ctx* c, int scheme, int precision, int nv, const double* X,
                      const double* sa_up, const double* Xup, const double* f, const double* vself,
                      const ves_near_lists* nl, double h, double* LP, double* near_only, WsCarver& ws,
                      cudaStream_t s);
// between two vesicle sets (targets: ct, Xt; sources: cs, Xs / Xup_s, den_s, vself_s)
int near_zone_matlab_cross(ves_ctx* ct, ves_ctx* cs, int nvt, const double* Xt, int nvs, const double* Xs, double h,
                           const ves_near_lists* nl, WsCarver& ws, cudaStream_t s);
// the MATLAB near-singular correction alone, added to LP (the far field
// computed elsewhere); ct == cs for a set against itself
int near_correct_matlab(ves_ctx* ct, ves_ctx* cs, const double* Xt, const double* Xup_s, const double* den_s,
                        const double* vself_s, const ves_near_lists* nl, double h, double* LP, cudaStream_t s);
// several MATLAB corrections (np <= 16 pairs of point sets) in one launch
int near_correct_matlab_pairs(int np, ves_ctx* const* ct, ves_ctx* const* cs, const double* const* Xt,
                              const double* const* Xup_s, const double* const* den_s, const double* const* vself_s,
                              const ves_near_lists* const* nl, const double* h, double* const* LP, cudaStream_t s);
int near_sing_int_cross_add(ves_ctx* ct, ves_ctx* cs, int scheme, int precision, int nvt, const double* Xt, int nvs,
                            const double* Xup_s, const double* den_s, const double* vself_s,
                            const ves_near_lists* nl, double h, double* LP, WsCarver& ws, cudaStream_t s);

// double layer (viscosity contrast)
int stokes_dl_matrix(ves_ctx* c, int nv, const double* X, const double* visc, int precision, double* D, WsCarver& ws,
                     cudaStream_t s);
void launch_dl_density(int nv, int ns, const double* f, const double* sa, const double* visc, double* den,
                       cudaStream_t s);
// precision VES_PREC_FP64: direct FP64 sum; FP32C / FP32M: multipole series for
// separated pairs, direct FP64 for close ones (sa, visc of the sources required)
int farfield_dl_run(ves_ctx* c, int precision, int nsrc, int ns, const double* Xsrc, const double* tang,
                    const double* den, const double* sa, const double* visc, int nt, int ntp, const double* Xtar,
                    const int* self_idx, const ves_near_lists* nl, double* out, WsCarver& ws, cudaStream_t s);
int near_sing_int_dl_run(ves_ctx* c, int scheme, int precision, int nv, const double* X, const double* Xup,
                         const double* tang_up, const double* sa_up, const double* visc, const double* f,
                         const double* vself, const ves_near_lists* nl, double h, double* LP, double* near_only,
                         WsCarver& ws, cudaStream_t s);

// RBF near-field fits (nearSingInt_rbf): adds the fits of the near pairs to LP
int rbf_near_correct(ves_ctx* c, int nv, const double* X, const double* f, const double* vself,
                     const ves_near_lists* nl, double* LP, WsCarver& ws, cudaStream_t s);

// post-step conditioning
int post_redistribute(ves_ctx* c, int nv, const double* X, double* Xout, int* flags, WsCarver& ws,
                      cudaStream_t s);
void launch_align_center_angle(ves_ctx* c, int nv, const double* Xorg, const double* X, double* Xout,
                               double* center, double* angle, cudaStream_t s);
// tol_constraint <= 0: the reference's 1e-2
int post_correct_area_length(ves_ctx* c, int nv, const double* X, const double* area0, const double* length0,
                             double* Xout, int* outer_iters, WsCarver& ws, cudaStream_t s,
                             double tol_constraint = 0.0);

// bending force of the MLARM step: bending of the Nup-upsampled shape truncated to N modes
int launch_bend_up(ves_ctx* c, int nv, const double* X, double kappa, double* fB, cudaStream_t s);

// dx = X+ - X of the implicit BIEM step of non-interacting vesicles (ves_targets.cu);
// dx NULL sizes the workspace only
int isolated_step_run(ves_ctx* c, int nv, const double* X, const double* vinf, double dt, double kappa, int slp,
                      double* dx, WsCarver& ws, cudaStream_t s);

// vector kernels (GMRES)
void launch_dot_partials(long long n, const double* a, const double* b, double* partials,
                         cudaStream_t s);
int dot_partial_blocks();
