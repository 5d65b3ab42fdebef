/*
 * ves2d_gb300.h — C ABI of the GB300 (sm_103a) vesicle-suspension kernels.
 *
 * Every function returns an int status (VES_OK == 0).  All array arguments are
 * caller-owned DEVICE pointers (float64 unless stated) on the device that was
 * current when the context was created; ``stream`` is a cudaStream_t passed as
 * void* (NULL = legacy default stream).  No entry point allocates device memory
 * in a hot call: scratch is passed in as ``ws``/``ws_bytes`` and its size is
 * given by the matching *_workspace() query.  Kernels never trap; device-side
 * failures are reported through the returned status.
 *
 * Device layout ("vesicle-major", the transpose of the reference's X[2N, nv]):
 *   X, f, velocities   [nv][2][n]  x-row then y-row of each vesicle
 *   sigma (tension)    [nv][n]
 *   G (single layer)   [nv][2N][2N] row-major
 *   GMRES unknowns     [nv][3][N]  (x, y, sigma) — the reference's flattening
 *                      torch.cat([X, sigma]).T.reshape(-1)
 *
 * Reference interfaces replaced (paths relative to the Ves2Dpy project):
 *   see the comment above each declaration.
 */
#ifndef VES2D_GB300_H
#define VES2D_GB300_H

#include <stddef.h>
#include <stdint.h>

#if defined(__GNUC__)
#define VES_API __attribute__((visibility("default")))
#else
#define VES_API
#endif

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes --------------------------------------------------------- */
#define VES_OK 0
#define VES_ERR_SHAPE 1            /* bad sizes / unsupported N                  */
#define VES_ERR_NONFINITE 2        /* NaN/Inf (poten.py:77-78 "NaN or Inf")      */
#define VES_ERR_NEARLIST_OVERFLOW 3/* near-zone capacity exceeded               */
#define VES_ERR_GMRES_MAXIT 4      /* GMRES did not reach tolerance (iflag)      */
#define VES_ERR_CUDA 5             /* CUDA runtime error                          */
#define VES_ERR_ARG 6              /* invalid argument (NULL, bad enum, ...)      */
#define VES_ERR_TIMEOUT 7          /* a bounded device-side wait gave up          */
#define VES_ERR_SINGULAR 8         /* zero pivot in a per-vesicle factorisation   */
#define VES_ERR_WORKSPACE 9        /* workspace too small                         */

/* arithmetic of the all-pairs Stokeslet sum */
#define VES_PREC_FP64 0            /* FP64 throughout                              */
#define VES_PREC_FP32C 1           /* FP32 pair terms, per-vesicle-pair centre      */
#define VES_PREC_FP32M 2           /* all-pairs sums only: multipole expansion of   *
                                    * separated source vesicles (truncation below    *
                                    * 1e-10 of the source's density magnitude), the  *
                                    * FP32C direct sum for close pairs               */
                                   /* shift, compensated accumulation              */

/* near-singular schemes */
#define VES_NEAR_NONE 0            /* plain upsampled trapezoid rule, no exclusion */
#define VES_NEAR_PY_HH 1           /* mytorch/poten.py:466-600 + biem_support.py:520-613 */
#define VES_NEAR_MATLAB 2          /* matlab/poten_py.m:495-692 + capsules_py.m:194-643   */
#define VES_NEAR_PY_RBF 3          /* mytorch/poten.py:643-894 (nearSingInt_rbf), py_hh lists */

/* background flows (mytorch/tstep_biem.py:849-952) */
#define VES_FLOW_RELAXATION 0
#define VES_FLOW_EXTENSIONAL 1
#define VES_FLOW_PARABOLIC 2
#define VES_FLOW_TAYLOR_GREEN 3
#define VES_FLOW_SHEAR 4
#define VES_FLOW_VORTEX 5

typedef struct ves_ctx ves_ctx;

/* ---- context (immutable per-N quadrature tables; poten.py:15-37) ---------- */
/* Replaces Poten.__init__ (mytorch/poten.py:15-37): builds, on the current
 * device, the Alpert weights (poten.py:899-974), Fourier restriction and
 * prolongation (fft1.py:209-231), spectral derivative and Lagrange tables. */
VES_API int ves_ctx_create(int N, ves_ctx** out);
VES_API int ves_ctx_destroy(ves_ctx* ctx);
/* N, Nup = N*ceil(sqrt(N)) (poten.py:24), number of Alpert nodes */
VES_API int ves_ctx_info(const ves_ctx* ctx, int* N, int* Nup, int* nquad);
/* Largest number of near-pair candidates (source vesicles whose box comes
 * within the near threshold of one target vesicle's box) met by the near-zone
 * builds since the last call on this context began; the capacity
 * (ves_near_lists.maxc, ves_step_params.maxc, ves_mlarm_params.maxc) a
 * caller needs after VES_ERR_NEARLIST_OVERFLOW.  The reference's
 * naiveNearZoneInfo (biem_support.py:520-613) has no capacity; the device
 * lists have one and report the size they need instead of truncating. */
VES_API int ves_ctx_max_candidates(const ves_ctx* ctx);
/* Text of the last error recorded on this thread (never NULL). */
VES_API const char* ves_last_error(void);

/* ---- curve geometry (curve_batch_compile.py, capsules.py) ------------------ */
/* Curve.diffProp (curve_batch_compile.py:400-423) on the N grid (grid=0) or the
 * upsampled Nup grid (grid=1, X then holds Nup points per vesicle).
 * Outputs sa[nv][n], tang[nv][2][n], cur[nv][n]; any output may be NULL. */
VES_API int ves_diff_prop(ves_ctx* ctx, int grid, int nv, const double* X, double* sa, double* tang,
                  double* cur, void* stream);
/* Curve.geomProp (curve_batch_compile.py:455-473): reduced area, area, length [nv]. */
VES_API int ves_geom_prop(ves_ctx* ctx, int nv, const double* X, double* reduced_area, double* area,
                  double* length, void* stream);
/* interpft_vec (filter.py:192-194) from N to Nup points: in[nv][ncomp][N] ->
 * out[nv][ncomp][Nup]. */
VES_API int ves_upsample(ves_ctx* ctx, int nv, int ncomp, const double* in, double* out, void* stream);
/* capsules.tracJump (capsules.py:54-80): f = -kappa d^4X/ds^4 + d/ds(sigma X_s).
 * X, sigma may be read with per-vesicle strides (GMRES packing): vesicle k's
 * positions start at X + k*x_stride, its tension at sigma + k*s_stride. */
VES_API int ves_trac_jump(ves_ctx* ctx, int nv, double kappa, const double* isa, const double* tang,
                  const double* X, long long x_stride, const double* sigma, long long s_stride,
                  double* f, void* stream);
/* capsules.surfaceDiv (capsules.py:82-89): out[nv][N] = d f/ds . X_s. */
VES_API int ves_surface_div(ves_ctx* ctx, int nv, const double* isa, const double* tang, const double* f,
                    long long f_stride, double* out, long long out_stride, void* stream);
/* capsules.computeDerivs (capsules.py:91-206): Ben[nv][2N][2N], Ten[nv][2N][N],
 * Div[nv][N][2N] (real parts of the complex products, as in the reference). */
VES_API int ves_compute_derivs(ves_ctx* ctx, int nv, const double* isa, const double* tang, double* Ben,
                       double* Ten, double* Div, void* ws, size_t ws_bytes, void* stream);
VES_API size_t ves_compute_derivs_workspace(ves_ctx* ctx, int nv);
/* TStepBiem.bg_flow (tstep_biem.py:849-952): v[nv][2][N] = speed * u(X). */
VES_API int ves_bg_flow(ves_ctx* ctx, int nv, int flow, double speed, double chan_width,
                double vortex_size, const double* X, double* v, void* stream);

/* ---- single-layer self interaction (poten.py:40-99, 213-224) -------------- */
/* Poten.stokesSLmatrix: Alpert log-singular quadrature on the Nup grid,
 * restricted to N (G = R*Gup*P).  precision: VES_PREC_FP64, or VES_PREC_FP32C
 * (kernel values and the R*Gup*P products in FP32, FP64 weights and output). */
VES_API int ves_stokes_sl_matrix(ves_ctx* ctx, int nv, const double* X, int precision, double* G,
                         void* ws, size_t ws_bytes, void* stream);
VES_API size_t ves_stokes_sl_matrix_workspace(ves_ctx* ctx, int nv, int precision);
/* Poten.exactStokesSLdiag: out[k] = G[k] @ f[k], G[nv][m][m]. */
VES_API int ves_sl_diag(int nv, int m, const double* G, const double* f, double* out, void* stream);

/* ---- near zone ------------------------------------------------------------- */
/* Near-pair lists.  Every target vesicle t owns up to ``maxc`` candidate source
 * vesicles (bounding boxes closer than the threshold), in ascending order:
 *   cand_count[nv], cand_src[nv][maxc],
 *   excl_mask[nv][maxc][ceil(N/32)]   bit i: target point i of t is near source s
 *                                     (far-field exclusion; biem_support.py:72,
 *                                      the (ids0, ids1, ids2) of :610-613)
 *   hh_mask  [nv][maxc][Nup/32]       bit u: upsampled point u of s is near a
 *                                     point of t (the (id1_hh, id2_hh) list)
 * MATLAB scheme entries (capsules_py.m:194-467): up to ``max_entries`` records
 *   ent_tsj[max][3] int (target vesicle, source vesicle, target point),
 *   ent_icp[max] int, ent_geo[max][4] double (dist, nearest x, nearest y, theta),
 *   *n_entries (device int). */
typedef struct ves_near_lists {
  int maxc;
  int* cand_count;
  int* cand_src;
  uint32_t* excl_mask;
  uint32_t* hh_mask;
  int max_entries;
  int* n_entries;
  int* ent_tsj;
  int* ent_icp;
  double* ent_geo;
} ves_near_lists;

/* naiveNearZoneInfo (biem_support.py:520-613): threshold 1/N by default
 * (thresh <= 0), Euclidean distance between coarse targets and upsampled
 * sources of every other vesicle. Xup may be NULL (computed into ws). */
VES_API int ves_near_zone_py(ves_ctx* ctx, int nv, const double* X, const double* Xup, double thresh,
                     ves_near_lists* nl, void* ws, size_t ws_bytes, void* stream);
/* capsules_py.m getZone (relate==1) with closestPnt (:581-643): near if the
 * Newton closest point on the 7-point local interpolant is closer than h
 * (h <= 0: min vesicle length / N). */
VES_API int ves_near_zone_matlab(ves_ctx* ctx, int nv, const double* X, double h, ves_near_lists* nl,
                         void* ws, size_t ws_bytes, void* stream);
VES_API size_t ves_near_zone_workspace(ves_ctx* ctx, int nv);

/* ---- layer potentials between vesicles ------------------------------------ */
/* All-pairs Stokeslet sum, allExactStokesSLTarget_compare1/2
 * (biem_support.py:7-272, poten.py:280-336):
 *   u(x) = 1/(4 pi) sum_src [ -1/2 log|r|^2 den + (r.den) r/|r|^2 ],
 *   den = f * sa * 2 pi / ns,
 * sources Xsrc[nsrc][2][ns], den[nsrc][2][ns]; targets Xtar[nt][2][ntp].
 * self_idx[nt] (or NULL): source vesicle skipped for target column t.
 * nl (or NULL): candidate lists whose excl_mask removes (target point, source
 * vesicle) pairs (requires nt == nsrc, ntp == N of ctx).  Result written to
 * out[nt][2][ntp].  precision: VES_PREC_FP64, VES_PREC_FP32C or VES_PREC_FP32M
 * (FP32M: at most 128 target points per column). */
VES_API int ves_farfield(ves_ctx* ctx, int precision, int nsrc, int ns, const double* Xsrc,
                 const double* den, int nt, int ntp, const double* Xtar, const int* self_idx,
                 const ves_near_lists* nl, double* out, void* ws, size_t ws_bytes, void* stream);
VES_API size_t ves_farfield_workspace(ves_ctx* ctx, int precision, int nsrc, int ns, int nt, int ntp);
/* den[nv][2][ns] = f * sa * 2*pi/ns  (biem_support.py:39) */
VES_API int ves_density(int nv, int ns, const double* f, const double* sa, double* den, void* stream);

/* nearSingInt_hh (poten.py:466-600) / nearSingInt (poten_py.m:495-692):
 * LP[nv][2][N] = far field of f over Nup-upsampled sources with the near
 * pairs removed, plus the near correction built from vself = G f.
 * scheme: VES_NEAR_PY_HH, VES_NEAR_PY_RBF (both with the lists of
 * ves_near_zone_py) or VES_NEAR_MATLAB (lists of ves_near_zone_matlab),
 * VES_NEAR_NONE (nl ignored).  near_only (or NULL) receives the correction
 * alone (the reference's second return value; zero for VES_NEAR_PY_RBF, whose
 * reference returns LP only). */
VES_API int ves_near_sing_int(ves_ctx* ctx, int scheme, int precision, int nv, const double* X,
                      const double* sa_up, const double* Xup, const double* f,
                      const double* vself, const ves_near_lists* nl, double h, double* LP,
                      double* near_only, void* ws, size_t ws_bytes, void* stream);
VES_API size_t ves_near_sing_int_workspace(ves_ctx* ctx, int precision, int nv);

/* ---- double layer (viscosity contrast) ------------------------------------ */
/* Geometry of capsules(interpft(X, Nup)): Xup[nv][2][Nup], sa[nv][Nup],
 * tang[nv][2][Nup], cur[nv][Nup] (any output may be NULL), from the first and
 * second derivatives of the trig interpolant at the Nup grid. */
VES_API int ves_upsample_geometry(ves_ctx* ctx, int nv, const double* X, double* Xup, double* sa, double* tang,
                                  double* cur, void* stream);
/* stokesDLmatrix (poten.py:102-175): D[nv][2N][2N] on the Nup-upsampled
 * curve restricted to N points; visc[nv] device viscosity contrasts (D = 0
 * where visc == 1).  precision: VES_PREC_FP64 or VES_PREC_FP32C (kernel
 * values in FP64, the R Dup P products in FP32, as the single-layer build). */
VES_API int ves_stokes_dl_matrix(ves_ctx* ctx, int nv, const double* X, const double* visc, int precision,
                                 double* D, void* ws, size_t ws_bytes, void* stream);
VES_API size_t ves_stokes_dl_matrix_workspace(ves_ctx* ctx, int nv, int precision);
/* den[nv][2][ns] = f * sa * 2*pi/ns * (1 - visc)  (poten.py:411; visc NULL: all 1) */
VES_API int ves_dl_density(int nv, int ns, const double* f, const double* sa, const double* visc, double* den,
                           void* stream);
/* Double-layer sum, exactStokesDL (poten.py:399-441):
 *   u(x) = 1/pi sum_src ((r.n)(r.den)/|r|^4) r,  r = x - y,  n = (ty, -tx),
 * sources Xsrc[nsrc][2][ns] with unit tangents tang[nsrc][2][ns] and den from
 * ves_dl_density; targets Xtar[nt][2][ntp]; self_idx and nl as ves_farfield.
 * precision VES_PREC_FP64: direct FP64 sum (ntp <= 1024, no workspace);
 * VES_PREC_FP32M (or FP32C): multipole series of each source vesicle for the
 * separated pairs, direct FP64 for the others (ntp <= 128; needs the source
 * jacobian sa[nsrc][ns] and contrasts visc[nsrc] of the density, and the
 * workspace of ves_farfield_dl_workspace). */
VES_API int ves_farfield_dl(ves_ctx* ctx, int precision, int nsrc, int ns, const double* Xsrc, const double* tang,
                            const double* den, const double* sa, const double* visc, int nt, int ntp,
                            const double* Xtar, const int* self_idx, const ves_near_lists* nl, double* out,
                            void* ws, size_t ws_bytes, void* stream);
VES_API size_t ves_farfield_dl_workspace(int precision, int nsrc, int nt, int ntp);
/* nearSingInt with kernelDirect = exactStokesDL (tstep_biem.py:236,501;
 * poten_py.m:495-692): double-layer far field over the Nup-upsampled sources
 * (Xup, tang_up, sa_up of the upsampled curve) with the near pairs removed,
 * plus the near correction from vself = jump f + D f.  scheme:
 * VES_NEAR_NONE, VES_NEAR_PY_HH or VES_NEAR_MATLAB; precision as
 * ves_farfield_dl. */
VES_API int ves_near_sing_int_dl(ves_ctx* ctx, int scheme, int precision, int nv, const double* X, const double* Xup,
                                 const double* tang_up, const double* sa_up, const double* visc, const double* f,
                                 const double* vself, const ves_near_lists* nl, double h, double* LP,
                                 double* near_only, void* ws, size_t ws_bytes, void* stream);
VES_API size_t ves_near_sing_int_dl_workspace(ves_ctx* ctx, int nv);

/* ---- the implicit BIEM step (tstep_biem.py:181-428) ------------------------ */
typedef struct ves_step_params {
  double dt;
  double kappa;
  double gmres_tol;      /* relative tolerance (scipy rtol) */
  int gmres_maxiter;     /* outer restart cycles (scipy maxiter) */
  int gmres_restart;     /* 20 = scipy default */
  int use_preco;         /* block-diagonal LU preconditioner (tstep_biem.py:653-711):
                            0 none, 1 FP64, 2 built and factored in FP32 (FP64
                            vectors; GMRES absorbs the difference; FP64 when a
                            viscosity contrast is present) */
  int flow;              /* VES_FLOW_* */
  double speed, chan_width, vortex_size;
  int near_scheme;       /* VES_NEAR_* */
  int farfield_precision;/* VES_PREC_* for the all-pairs sum */
  int sl_precision;      /* VES_PREC_* for the Alpert matrix build */
  int maxc;              /* candidate capacity per vesicle (0 = default 64) */
  int max_entries;       /* MATLAB near entries capacity (0 = default) */
  int repulsion;         /* add the penalty-layer repulsion (tstep_biem.py:250-264);
                            needs near_scheme VES_NEAR_PY_HH or VES_NEAR_PY_RBF */
  double rep_strength;   /* W (prams['repStrength']) */
  double min_dist;       /* eta (prams['minDist']) */
  const double* visc_cont; /* device [nv] viscosity contrasts, or NULL when every
                              vesicle has contrast 1 (no double-layer terms);
                              with contrasts: D, Fdlp and alpha = (1 + visc)/2
                              (tstep_biem.py:195-244, 486-501, 541-560) */
} ves_step_params;

typedef struct ves_step_result {
  int matvecs;           /* number of time_matvec calls (the reference's iter) */
  int inner_iters;       /* GMRES inner iterations */
  int info;              /* 0 converged; maxiter (scipy's code) if the restart
                            cycles ran out; -1 if the true residual stopped
                            decreasing (3 cycles without halving) above the
                            tolerance, i.e. the arithmetic's noise floor */
  double resid;          /* final true residual norm / ||b|| */
  int n_near_pairs;      /* (target point, source vesicle) pairs excluded */
  int n_near_entries;    /* near-correction entries applied */
} ves_step_result;

/* TStepBiem.time_step: X[nv][2][N], sigma[nv][N] -> Xout, sigma_out (may alias
 * the inputs).  Unconfined; optional repulsion and viscosity contrast.
 * Without the preconditioner GMRES starts from zero, as the reference's
 * gmres call without x0 (tstep_biem.py:383). */
VES_API int ves_biem_step(ves_ctx* ctx, const ves_step_params* prm, int nv, const double* X,
                  const double* sigma, double* Xout, double* sigma_out, ves_step_result* res,
                  void* ws, size_t ws_bytes, void* stream);
VES_API size_t ves_biem_step_workspace(ves_ctx* ctx, const ves_step_params* prm, int nv);
/* One implicit step of a suspension of several point counts: ngroups (1-4)
 * groups, group g with nv[g] >= 1 vesicles of ctx[g]->N points, X[g] and
 * sigma[g] in the layout of ves_biem_step.  Every vesicle of every group is
 * in one GMRES system (group blocks in order).  Between groups the far field
 * runs over the source group's upsampled points and the near zone and its
 * correction follow matlab getZone / nearSingInt with a separate target set
 * (matlab/capsules_py.m:194-467, matlab/poten_py.m:495-692), h = the source
 * group's min length / N.  prm->near_scheme VES_NEAR_MATLAB or VES_NEAR_NONE;
 * no viscosity contrast or repulsion (VES_ERR_ARG).  The reference holds one
 * N per suspension (X[2N, nv]); with one group this is ves_biem_step with
 * the MATLAB near rules. */
VES_API int ves_biem_step_mixed(int ngroups, ves_ctx* const* ctx, const ves_step_params* prm, const int* nv,
                                const double* const* X, const double* const* sigma, double* const* Xout,
                                double* const* sigma_out, ves_step_result* res, void* ws, size_t ws_bytes,
                                void* stream);
VES_API size_t ves_biem_step_mixed_workspace(int ngroups, ves_ctx* const* ctx, const ves_step_params* prm,
                                             const int* nv);

/* ---- post-step shape conditioning (curve_batch_compile.py) ---------------- */
/* One redistributeArcLength pass (curve_batch_compile.py:905-972, with
 * my_arcLengthParameter :1039-1092 and the driver's Fourier modes
 * driver_confined.py:240): Xout[nv][2][N] (may alias X); flags[nv]
 * device ints (1 = left unchanged); *all_good (host, may be NULL: no
 * synchronisation) = all flags set.  As in the reference, a vesicle is
 * re-parametrised when the matrix infinity norm of the jacobian deviations
 * of the whole suspension (one scalar, :953) exceeds 1e-5 times its own mean
 * jacobian. */
VES_API int ves_redistribute_arclength(ves_ctx* ctx, int nv, const double* X, double* Xout, int* flags,
                                       int* all_good, void* ws, size_t ws_bytes, void* stream);
VES_API size_t ves_redistribute_arclength_workspace(ves_ctx* ctx, int nv);
/* alignCenterAngle (curve_batch_compile.py:842-901): rigid motion of X onto
 * the physical centre and inclination angle of Xorg. */
VES_API int ves_align_center_angle(ves_ctx* ctx, int nv, const double* Xorg, const double* X, double* Xout,
                                   void* stream);
/* getPhysicalCenter (:84-100) -> center[nv][2]; getIncAngle (:105-194) -> angle[nv]
 * (either may be NULL). */
VES_API int ves_center_angle(ves_ctx* ctx, int nv, const double* X, double* center, double* angle,
                             void* stream);
/* correctAreaAndLengthAugLag (curve_batch_compile.py:590-710): vesicles whose
 * area or length is off by more than 1e-2 are moved to the nearest shape
 * with area0/length0 (augmented Lagrangian, Adam, 100 x 20 iterations at
 * most).  *outer_iters (host, may be NULL) = augmented-Lagrangian updates. */
VES_API int ves_correct_area_length(ves_ctx* ctx, int nv, const double* X, const double* area0,
                                    const double* length0, double* Xout, int* outer_iters, void* ws,
                                    size_t ws_bytes, void* stream);
VES_API size_t ves_correct_area_length_workspace(ves_ctx* ctx, int nv);

/* ---- MLARM surrogate networks (model_zoo/Net_ves_*.py) -------------------- */
/* A network is a chain of blocks of one template applied to ``groups``
 * independent channel groups (grouped convolutions, model_zoo/Net_ves_merge_adv.py:6-191):
 *   A = bn1(relu(conv7,s2,circ pad 3 (x)) ++ relu(conv7,s2,dil 2,circ pad 6 (x)))   2*c1 channels, L/2
 *   B = bn2(the same pair on A)                                                  2*c2 channels, L/4
 *   C = bn3(relu(convT10,s2,pad 4 (B)));  D = bn4(relu(convT10,s2,pad 4 (C)))   2*c2 channels, L/2, L
 *   out = [conv3,zero pad 1 (D) (+ x[0:cmix] if residual)] ++ x[cin-npass:cin]
 * Activations are [nv][groups*channels][length] in the network's precision. */
#define VES_NET_FP64 0             /* CUDA cores, FP64 (parity)                     */
#define VES_NET_FP32 1             /* CUDA cores, FP32 (the reference networks' type) */
#define VES_NET_BF16 2             /* tcgen05 tensor cores: BF16 operands, FP32 accumulation,
                                      FP32 activations between blocks and at the I/O  */
typedef struct ves_net ves_net;
typedef struct ves_net_block {
  int cin, c1, c2, cmix, residual, npass;
} ves_net_block;
/* ``params`` holds 30 host pointers per block, in the reference's full
 * (all-groups) parameter layout and this order: conv1_1.{weight,bias},
 * conv1_2.{..}, conv2_1.{..}, conv2_2.{..}, deconv1.{..}, deconv2.{..},
 * mix.{..}, then bn1..bn4.{weight,bias,running_mean,running_var}
 * (eval-mode batch norm, eps 1e-5).  Replaces the TorchScript models loaded
 * by get_network_torch.py:26-35, 137-142, 217-223, 316-323, 403-415.
 * Allocates the weights on the current device. */
VES_API int ves_net_create(int precision, int groups, int length, int nblocks, const ves_net_block* blocks,
                           const float* const* params, ves_net** out);
VES_API int ves_net_destroy(ves_net* net);
VES_API int ves_net_info(const ves_net* net, int* precision, int* groups, int* length, int* cin, int* cout);
/* Forward pass (model(input), e.g. get_network_torch.py:76): in
 * [nv][groups*cin][length] -> out [nv][groups*cout][length], FP64 for
 * VES_NET_FP64 and FP32 otherwise. */
VES_API int ves_net_forward(const ves_net* net, int nv, const void* in, void* out, void* ws, size_t ws_bytes,
                            void* stream);
VES_API size_t ves_net_forward_workspace(const ves_net* net, int nv);
/* Autotuner of the BF16 tensor-core network (VES_NET_BF16; no effect on
 * the other precisions).  With on != 0, the first forward pass at each
 * vesicle count times every launch shape that fits of each block's three
 * kernels (warp groups per CTA; M = 64 MMAs for layers of at most 64
 * positions on or off) on that call's input, synchronising the stream, and
 * keeps the fastest for later passes at that count.  Results do not depend
 * on the shape.  Concurrent first passes of one network must be serialised
 * by the caller. */
VES_API int ves_net_set_autotune(ves_net* net, int on);

/* ---- MLARM step (newtorch/wrapper_MLARM_batch_compile_N128.py) ------------- */
/* Normalisation constants of the five networks, host FP64, the shapes the
 * reference constructor takes (entry_driver_manyfreeSpaceVesicle_N128.py:120-155). */
typedef struct ves_mlarm_norms {
  const double* adv_in;       /* [127][4] */
  const double* adv_out;      /* [127][4] */
  const double* relax_in;     /* [4]      */
  const double* relax_out;    /* [4]      */
  const double* near_in;      /* [128][4] */
  const double* near_out;     /* [128][2][12] */
  const double* selften_in;   /* [4]      */
  const double* selften_out;  /* [2]      */
  const double* advten_in;    /* [127][4] */
  const double* advten_out;   /* [127][4] */
} ves_mlarm_norms;
typedef struct ves_mlarm ves_mlarm;
/* MLARM_manyfree_py.__init__ (:650-710) for N = 128: binds the context and the
 * five networks (relax [1 group, 2->2, L 128], adv [127, 2->2, L 256],
 * near [128, 2->12, L 128], selften [1, 2->1, L 128], advten [127, 2->2,
 * L 128]; all of one precision) and copies the constants to the device.
 * ``near`` may be NULL when the step never evaluates it. */
VES_API int ves_mlarm_create(ves_ctx* ctx, const ves_net* relax, const ves_net* adv, const ves_net* near,
                             const ves_net* selften, const ves_net* advten, const ves_mlarm_norms* norms,
                             ves_mlarm** out);
VES_API int ves_mlarm_destroy(ves_mlarm* m);
typedef struct ves_mlarm_params {
  double dt, kappa;
  int flow;                   /* background flow when vback is NULL (VES_FLOW_*) */
  double speed, chan_width, vortex_size;
  int farfield_precision;     /* VES_PREC_* of the two all-pairs sums            */
  int eval_near_net;          /* 1: evaluate the near-field network as the reference
                                 does (:1034); its velocities enter the step only
                                 through the repulsion force, zero here          */
  int maxc;                   /* near-pair candidate capacity per vesicle (0: 64) */
  double judge_tol;           /* > 0: the plain BIEM step judges the surrogate and
                                 stands in for it.  A vesicle whose surrogate step
                                 (advection network + relaxation network) changes
                                 its area or its length by more than judge_tol
                                 (relative) takes instead the implicit BIEM step
                                 of the isolated vesicle (tstep_biem.py:181-428
                                 self block) with the step's explicit velocity
                                 vinf + filtered far field; 0: the reference's
                                 step (no judge)                                  */
  int conserve;               /* 1: the advection displacement and the relaxation
                                 network's displacement are made area- and
                                 length-preserving to first order (their
                                 components along n and kappa n removed), as the
                                 exact incompressible, inextensible dynamics is;
                                 0: the reference's step                           */
  double area_len_tol;        /* relative area/length error beyond which the
                                 step's correction acts and down to which it
                                 corrects (correctAreaAndLengthAugLag's
                                 tolConstraint, curve_batch_compile.py:603);
                                 0: the reference's 1e-2                          */
} ves_mlarm_params;
typedef struct ves_mlarm_result {
  int n_near_pairs;           /* excluded (target point, source vesicle) pairs   */
  int auglag_iters;           /* augmented-Lagrangian updates of the correction  */
  int n_fallback;             /* vesicles that took the BIEM step (judge_tol > 0) */
} ves_mlarm_result;
/* Optional device buffers receiving stage outputs of the step (NULL = skip):
 * the standardised shape and its values (:4119-4138), the two far fields
 * (:2495-2675, before filtering), the two tension solves (:3632-3688), the
 * advected shape (:3584-3620, before filtering), the relaxed shape (:3622),
 * and the aligned and corrected shapes (:1160-1179). */
typedef struct ves_mlarm_trace {
  double *Xstand, *scaling, *rotate, *rot_center, *trans;  /* [nv][2][N], [nv], [nv], [nv][2], [nv][2] */
  int* sort_idx;                                           /* [nv][N] */
  double *far1, *far2, *vback_solve, *selfbend_solve;      /* [nv][2][N] x2, [nv][N] x2 */
  double *Xadv, *Xrelax, *Xalign, *Xcorr;                  /* [nv][2][N] */
} ves_mlarm_trace;
/* time_step_many_noinfo(Xold, tenOld, nlayers=3) (:986-1206) without
 * repulsion: X[nv][2][N], ten[nv][N] -> Xout, ten_out.  vback[nv][2][N] is
 * vinf(Xold) (may be NULL: computed from prm->flow).  area0/len0[nv] are the
 * reference area and length of the correction (:1172). */
VES_API int ves_mlarm_step(ves_mlarm* m, const ves_mlarm_params* prm, int nv, const double* X,
                           const double* ten, const double* vback, const double* area0, const double* len0,
                           double* Xout, double* ten_out, ves_mlarm_result* res, const ves_mlarm_trace* trace,
                           void* ws, size_t ws_bytes, void* stream);
VES_API size_t ves_mlarm_step_workspace(ves_mlarm* m, const ves_mlarm_params* prm, int nv);
/* standardizationStep (:4119-4138): five redistribution passes, then the
 * reference values (:4179-4223) and the standardised shape. */
VES_API int ves_mlarm_standardize(ves_ctx* ctx, int nv, const double* X, double* Xstand, double* scaling,
                                  double* rotate, double* rot_center, double* trans, int* sort_idx, void* ws,
                                  size_t ws_bytes, void* stream);
VES_API size_t ves_mlarm_standardize_workspace(ves_ctx* ctx, int nv);

/* ---- training the MLARM networks ------------------------------------------ */
/* The reference loads trained TorchScript models (get_network_torch.py:29,
 * 127, 224, 324, 410) whose weights, data and training code are not in its
 * tree; the MATLAB ground-truth scripts (matlab/relaxation_solve.m,
 * matlab/groundTruth_NearFieldStokesletData.m) generate data with the BIEM
 * operators of one vesicle.  These entry points make that data on the device
 * and train networks of the block template.
 *
 * Training targets for standardised shapes Xs[nv][2][N] (N = 128; the output
 * of ves_mlarm_standardize), each output optional (NULL = skip):
 *   relax_dx[nv][2][N]  X+ - Xs of the implicit step (tstep_biem.py:181-428) of
 *                       the isolated vesicle without flow, time step dt
 *   selften[nv][N]      A^-1 Div G fBend, A = Div G Ten (invTenMatOnSelfBend,
 *                       wrapper_MLARM_batch_compile_N128.py:3672-3688)
 *   advten[nv][254][N]  channel 2m + c: A^-1 Div b_{m+1,c}, b_{k,0} = (cos k th,
 *                       sin k th)/N, b_{k,1} = (-sin k th, cos k th)/N
 *                       (invTenMatOnVback :3632-3669)
 *   adv[nv][254][2N]    channel 2m + c: G Ten A^-1 Div b_{m+1,c} (the M of
 *                       translateVinfwTorch :3584-3620)
 * sl_precision: VES_PREC_FP64 or VES_PREC_FP32C for the Alpert matrix. */
VES_API int ves_mlarm_targets(ves_ctx* ctx, int nv, const double* Xs, double dt, double kappa, int sl_precision,
                              double* relax_dx, double* selften, double* advten, double* adv, void* ws,
                              size_t ws_bytes, void* stream);
VES_API size_t ves_mlarm_targets_workspace(ves_ctx* ctx, int nv, int sl_precision);

/* The implicit step of tstep_biem.py:181-428 for vesicles that do not
 * interact (each solves its own self-interaction block directly):
 * [I + dt k G Ben, -dt G Ten; Div, 0] [Xout; s] = [X + dt vinf; Div X],
 * X, vinf (NULL: no flow), Xout [nv][2][N].  Evolves training shapes under a
 * background flow; the relaxation target above is its vinf = NULL case. */
VES_API int ves_isolated_step(ves_ctx* ctx, int nv, const double* X, const double* vinf, double dt, double kappa,
                              int sl_precision, double* Xout, void* ws, size_t ws_bytes, void* stream);
VES_API size_t ves_isolated_step_workspace(ves_ctx* ctx, int nv, int sl_precision);

/* One channel group of a network of the block template in training
 * (model_zoo/Net_ves_*.py), precision VES_NET_FP32 (training) or VES_NET_FP64
 * (gradient checks): parameters, gradients, Adam moments and the activations
 * of up to max_batch samples.  params: 30 float32 arrays per block in the
 * order conv1_1.{weight,bias}, conv1_2, conv2_1, conv2_2, deconv1, deconv2,
 * mix, then bn1..bn4.{weight, bias, running_mean, running_var} (the state-dict
 * names of the reference modules); batch norm is trained as its
 * evaluation-mode affine map (running statistics fixed). */
typedef struct ves_trainer ves_trainer;
VES_API int ves_trainer_create(int precision, int length, int nblocks, const ves_net_block* blocks,
                               const float* const* params, int max_batch, ves_trainer** out);
VES_API int ves_trainer_destroy(ves_trainer* t);
VES_API long long ves_trainer_num_params(const ves_trainer* t);
/* x[B][cin][L] -> y[B][cout][L] (y may be NULL); keeps the activations */
VES_API int ves_trainer_forward(ves_trainer* t, int batch, const void* x, void* y, void* stream);
/* loss = mean of w_b w_c (y - target)^2 over the last forward's batch
 * (channel weights w_c[cout], sample weights w_b[batch]; NULL: all 1), its
 * gradient through every layer into the parameter gradients (zeroed first);
 * *loss (may be NULL) read back with one stream sync */
VES_API int ves_trainer_backward_mse(ves_trainer* t, int batch, const void* target, const void* channel_weights,
                                     const void* sample_weights, double* loss, void* stream);
/* Adam (bias-corrected, step >= 1) on every trainable parameter */
VES_API int ves_trainer_adam(ves_trainer* t, double lr, double beta1, double beta2, double eps, int step,
                             void* stream);
/* parameters / gradients out as float32 arrays in the order of _create (NULL entries skipped) */
VES_API int ves_trainer_get_params(const ves_trainer* t, float* const* params, void* stream);
VES_API int ves_trainer_get_grads(const ves_trainer* t, float* const* grads, void* stream);
/* the FP64 trainer's gradients as one host array in the same order */
VES_API int ves_trainer_get_grads_f64(const ves_trainer* t, double* out, void* stream);

/* ---- all-pairs sum without allocation (no counterpart in the reference) ---- */
/* The sum of ves_farfield (no near-pair lists) for callers that cannot allocate
 * device memory when they call: applications whose GPU memory is entirely
 * reserved by their own pool allocator, and hosts that call in from a runtime
 * or callback where a cudaMalloc would synchronise the device or is not
 * permitted.  The call takes its scratch from one fixed device array of
 * VES_STATIC_SCRATCH_BYTES bytes that belongs to the library image (held on
 * every GPU that loads the library until the process exits), so it performs
 * no allocation and needs no ves_ctx.  The first call on a device looks up the
 * array's device address (cudaGetSymbolAddress) and keeps it for the life of
 * the device's primary context; make that first call before any stream
 * capture, and make no call after a cudaDeviceReset in the same process (the
 * kept address would be stale).  Sizes whose scratch exceeds the array return
 * VES_ERR_WORKSPACE.  All calls share the one array: calls that overlap on the
 * GPU race and must be serialised by the caller.  Synchronises ``stream``. */
#define VES_STATIC_SCRATCH_BYTES (64u << 20)
VES_API int ves_farfield_static_scratch(int precision, int nsrc, int ns, const double* Xsrc, const double* den,
                                        int nt, int ntp, const double* Xtar, const int* self_idx, double* out,
                                        void* stream);

/* ---- repulsion (capsules.repulsionForce, capsules.py:209-252) ---------------
 * Penalty-layer repulsion between vesicles: X, out [nv][2][N] on the device,
 * strength W, layer thickness eta >= 0 (pairs farther apart than eta add 0).
 * Workspace: ves_repulsion_force_workspace(nv) bytes. */
VES_API size_t ves_repulsion_force_workspace(int nv);
VES_API int ves_repulsion_force(int N, int nv, const double* X, double W, double eta, double* out, void* ws,
                                size_t ws_bytes, void* stream);

/* ---- trajectory files ------------------------------------------------------
 * The reference's binary trajectory format (driver_confined.py:204-206,
 * 294-296; reader newtorch/tools/load_ves2d_file.py:4-72): little-endian
 * float64; N, nv, the initial shapes, then per frame the time and the shapes.
 * Shapes are vesicle by vesicle, N x then N y coordinates: X.T.flatten() of
 * the reference's X[2N, nv] = this library's device layout [nv][2][N]. */
typedef struct ves_traj ves_traj;
/* Create (truncate) ``path`` and write the header and the initial shapes X0
 * ([nv][2][N], on the device when x0_on_device != 0).  ``nslots`` pinned frame
 * buffers (0: 3) decouple the step from the disk. */
VES_API int ves_traj_create(const char* path, int N, int nv, const double* X0, int x0_on_device, int nslots,
                            ves_traj** out);
/* Queue one frame: ``time`` and X ([nv][2][N]).  A device X is copied
 * asynchronously on ``stream`` (it must stay unchanged until that copy has run
 * in stream order); a background thread writes frames in order.  Returns the
 * first earlier write failure, if any. */
VES_API int ves_traj_append(ves_traj* t, double time, const double* X, int on_device, void* stream);
/* Wait until every queued frame is written and flushed; frames written so far. */
VES_API int ves_traj_flush(ves_traj* t, long long* frames_written);
VES_API int ves_traj_close(ves_traj* t);

/* ---- measurement utilities (no counterpart in the reference) -------------- */
typedef struct ves_stats {
  long long kernel_launches;  /* kernels launched through this library (all contexts) */
  long long farfield_launches;/* all-pairs kernel launches timed on this context        */
  double farfield_ms;         /* their summed CUDA-event duration                       */
  double farfield_pairs;      /* (target point, source point) pairs they evaluated      */
  double farfield_mp_terms;   /* VES_PREC_FP32M: series terms evaluated, summed over    *
                               * (target point, source vesicle) pairs (orders + 1)      */
  double farfield_direct_pairs;/* VES_PREC_FP32M: (target point, source point) pairs of *
                               * the direct rule (close vesicle pairs)                  */
  long long networks_launches;/* network forward passes timed on this context (MLARM)  */
  double networks_ms;         /* their summed CUDA-event duration                       */
  double networks_flops;      /* their useful work: 2 x multiply-adds of the layers     */
} ves_stats;
/* Enable/disable CUDA-event timing of the all-pairs kernel and of the MLARM
 * step's network forward passes on ``ctx`` (events are recorded on the
 * launching stream around each launch; off by default). */
VES_API int ves_ctx_set_timing(ves_ctx* ctx, int on);
/* Read (and with reset != 0 clear) the counters; synchronises pending events. */
VES_API int ves_ctx_stats(ves_ctx* ctx, ves_stats* out, int reset);
/* Measurement hook (not part of any step): the MUFU throughput of this GPU,
 * lg2.approx + rcp.approx operations per second over all SMs (a ~0.1 s probe
 * on ``stream``); the denominator of the direct all-pairs kernel's roofline,
 * which no vendor figure gives. */
VES_API int ves_probe_sfu_peak(double* ops_per_second, void* stream);
/* Failure-path check: a kernel waits on an mbarrier that nothing completes,
 * with the bounded wait of the tensor-core kernels (2^20 polls with sleeps:
 * 0.13 s on a GB300); returns VES_ERR_TIMEOUT and leaves the context usable
 * (no trap, no fault). */
VES_API int ves_probe_wait_timeout(ves_ctx* ctx, void* stream);

#ifdef __cplusplus
}
#endif
#endif /* VES2D_GB300_H */
