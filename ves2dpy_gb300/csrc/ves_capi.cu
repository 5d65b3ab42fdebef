// extern "C" entry points of the component operators (the Poten / capsules /
// Curve calls of the reference); the whole step is in ves_step.cu.
#include <string.h>

#include "ves_internal.h"
#include "ves_tc.cuh"

static int finish(ves_ctx* c, cudaStream_t s, const char* what) {
  int rc = ves_launch_check(what);
  if (rc) return rc;
  return ves_check_status(c, s, what);
}

#define VES_REQUIRE(cond, msg)                   \
  do {                                           \
    if (!(cond)) {                               \
      ves_record_error(VES_ERR_ARG, "%s", msg);  \
      return VES_ERR_ARG;                        \
    }                                            \
  } while (0)

extern "C" int ves_diff_prop(ves_ctx* c, int grid, int nv, const double* X, double* sa, double* tang, double* cur,
                             void* stream) {
  VES_REQUIRE(c && X && nv >= 0 && (grid == 0 || grid == 1), "ves_diff_prop: bad arguments");
  cudaStream_t s = (cudaStream_t)stream;
  int rc = ves_reset_status(c, s);
  if (rc) return rc;
  launch_diff_prop(c, grid, nv, X, sa, nullptr, tang, cur, s);
  return finish(c, s, "ves_diff_prop");
}

extern "C" int ves_geom_prop(ves_ctx* c, int nv, const double* X, double* ra, double* area, double* length,
                             void* stream) {
  VES_REQUIRE(c && X && nv >= 0, "ves_geom_prop: bad arguments");
  cudaStream_t s = (cudaStream_t)stream;
  launch_geom_prop(c, nv, X, ra, area, length, s);
  return ves_launch_check("ves_geom_prop");
}

extern "C" int ves_upsample(ves_ctx* c, int nv, int ncomp, const double* in, double* out, void* stream) {
  VES_REQUIRE(c && in && out && nv >= 0 && ncomp > 0, "ves_upsample: bad arguments");
  launch_upsample(c, nv, ncomp, in, (long long)ncomp * c->N, out, (cudaStream_t)stream);
  return ves_launch_check("ves_upsample");
}

extern "C" int ves_trac_jump(ves_ctx* c, int nv, double kappa, const double* isa, const double* tang,
                             const double* X, long long x_stride, const double* sigma, long long s_stride, double* f,
                             void* stream) {
  VES_REQUIRE(c && isa && tang && X && sigma && f && nv >= 0, "ves_trac_jump: bad arguments");
  launch_trac_jump(c, nv, kappa, isa, tang, X, x_stride, sigma, s_stride, f, (cudaStream_t)stream);
  return ves_launch_check("ves_trac_jump");
}

extern "C" int ves_surface_div(ves_ctx* c, int nv, const double* isa, const double* tang, const double* f,
                               long long f_stride, double* out, long long out_stride, void* stream) {
  VES_REQUIRE(c && isa && tang && f && out && nv >= 0, "ves_surface_div: bad arguments");
  launch_surface_div(c, nv, isa, tang, f, f_stride, out, out_stride, (cudaStream_t)stream);
  return ves_launch_check("ves_surface_div");
}

extern "C" size_t ves_compute_derivs_workspace(ves_ctx* c, int nv) {
  if (!c) return 0;
  WsCarver w(nullptr, 0);
  derivs_and_precond(c, nv, nullptr, nullptr, nullptr, 0, 0, nullptr, nullptr, nullptr, nullptr, w, 0);
  return w.off + 256;
}

extern "C" int ves_compute_derivs(ves_ctx* c, int nv, const double* isa, const double* tang, double* Ben,
                                  double* Ten, double* Div, void* ws, size_t ws_bytes, void* stream) {
  VES_REQUIRE(c && isa && tang && Ben && Ten && Div && ws && nv >= 0, "ves_compute_derivs: bad arguments");
  WsCarver w(ws, ws_bytes);
  return derivs_and_precond(c, nv, isa, tang, nullptr, 0, 0, Ben, Ten, Div, nullptr, w, (cudaStream_t)stream);
}

extern "C" int ves_bg_flow(ves_ctx* c, int nv, int flow, double speed, double chan_width, double vortex_size,
                           const double* X, double* v, void* stream) {
  VES_REQUIRE(c && X && v && nv >= 0, "ves_bg_flow: bad arguments");
  VES_REQUIRE(flow >= VES_FLOW_RELAXATION && flow <= VES_FLOW_VORTEX, "ves_bg_flow: unknown flow");
  launch_bg_flow(nv, c->N, flow, speed, chan_width, vortex_size, X, v, (cudaStream_t)stream);
  return ves_launch_check("ves_bg_flow");
}

extern "C" size_t ves_stokes_sl_matrix_workspace(ves_ctx* c, int nv, int precision) {
  if (!c) return 0;
  WsCarver w(nullptr, 0);
  alpert_sl_matrix(c, nv, nullptr, precision, nullptr, w, 0);
  return w.off + 256;
}

extern "C" int ves_stokes_sl_matrix(ves_ctx* c, int nv, const double* X, int precision, double* G, void* ws,
                                    size_t ws_bytes, void* stream) {
  VES_REQUIRE(c && X && G && ws && nv >= 0, "ves_stokes_sl_matrix: bad arguments");
  cudaStream_t s = (cudaStream_t)stream;
  int rc = ves_reset_status(c, s);
  if (rc) return rc;
  WsCarver w(ws, ws_bytes);
  rc = alpert_sl_matrix(c, nv, X, precision, G, w, s);
  if (rc) return rc;
  return ves_check_status(c, s, "ves_stokes_sl_matrix");
}

extern "C" int ves_sl_diag(int nv, int m, const double* G, const double* f, double* out, void* stream) {
  VES_REQUIRE(G && f && out && nv >= 0 && m > 0, "ves_sl_diag: bad arguments");
  launch_bgemv_f64(nv, m, m, G, f, m, out, m, (cudaStream_t)stream);
  return ves_launch_check("ves_sl_diag");
}

extern "C" size_t ves_near_zone_workspace(ves_ctx* c, int nv) {
  if (!c) return 0;
  WsCarver a(nullptr, 0), b(nullptr, 0);
  near_zone_py(c, nv, nullptr, nullptr, 0, nullptr, a, 0);
  near_zone_matlab(c, nv, nullptr, 0, nullptr, b, 0);
  return (a.off > b.off ? a.off : b.off) + 256;
}

extern "C" int ves_near_zone_py(ves_ctx* c, int nv, const double* X, const double* Xup, double thresh,
                                ves_near_lists* nl, void* ws, size_t ws_bytes, void* stream) {
  VES_REQUIRE(c && X && nl && ws && nv >= 0, "ves_near_zone_py: bad arguments");
  cudaStream_t s = (cudaStream_t)stream;
  int rc = ves_reset_status(c, s);
  if (rc) return rc;
  WsCarver w(ws, ws_bytes);
  rc = near_zone_py(c, nv, X, Xup, thresh, nl, w, s);
  if (rc) return rc;
  return finish(c, s, "ves_near_zone_py");
}

extern "C" int ves_near_zone_matlab(ves_ctx* c, int nv, const double* X, double h, ves_near_lists* nl, void* ws,
                                    size_t ws_bytes, void* stream) {
  VES_REQUIRE(c && X && nl && ws && nv >= 0, "ves_near_zone_matlab: bad arguments");
  cudaStream_t s = (cudaStream_t)stream;
  int rc = ves_reset_status(c, s);
  if (rc) return rc;
  WsCarver w(ws, ws_bytes);
  rc = near_zone_matlab(c, nv, X, h, nl, w, s);
  if (rc) return rc;
  return finish(c, s, "ves_near_zone_matlab");
}

extern "C" size_t ves_farfield_workspace(ves_ctx* c, int precision, int nsrc, int ns, int nt, int ntp) {
  if (!c) return 0;
  WsCarver w(nullptr, 0);
  farfield_run(c, precision, nsrc, ns, nullptr, nullptr, nt, ntp, nullptr, nullptr, nullptr, nullptr, w, 0);
  return w.off + 256;
}

extern "C" int ves_farfield(ves_ctx* c, int precision, int nsrc, int ns, const double* Xsrc, const double* den, int nt,
                            int ntp, const double* Xtar, const int* self_idx, const ves_near_lists* nl, double* out,
                            void* ws, size_t ws_bytes, void* stream) {
  VES_REQUIRE(c && Xsrc && den && Xtar && out && ws && nsrc >= 0 && ns > 0 && nt >= 0 && ntp > 0,
              "ves_farfield: bad arguments");
  cudaStream_t s = (cudaStream_t)stream;
  int rc = ves_reset_status(c, s);
  if (rc) return rc;
  WsCarver w(ws, ws_bytes);
  rc = farfield_run(c, precision, nsrc, ns, Xsrc, den, nt, ntp, Xtar, self_idx, nl, out, w, s);
  if (rc) return rc;
  return finish(c, s, "ves_farfield");
}

extern "C" int ves_density(int nv, int ns, const double* f, const double* sa, double* den, void* stream) {
  VES_REQUIRE(f && sa && den && nv >= 0 && ns > 0, "ves_density: bad arguments");
  launch_density(nv, ns, f, sa, den, (cudaStream_t)stream);
  return ves_launch_check("ves_density");
}

extern "C" size_t ves_near_sing_int_workspace(ves_ctx* c, int precision, int nv) {
  if (!c) return 0;
  WsCarver w(nullptr, 0);
  // the largest scheme: the RBF fits add their buffers to the all-pairs scratch
  near_sing_int_run(c, VES_NEAR_PY_RBF, precision, nv, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, 0,
                    nullptr, nullptr, w, 0);
  return w.off + 256;
}

extern "C" int ves_near_sing_int(ves_ctx* c, int scheme, int precision, int nv, const double* X, const double* sa_up,
                                 const double* Xup, const double* f, const double* vself, const ves_near_lists* nl,
                                 double h, double* LP, double* near_only, void* ws, size_t ws_bytes, void* stream) {
  VES_REQUIRE(c && X && sa_up && Xup && f && LP && ws && nv >= 0, "ves_near_sing_int: bad arguments");
  VES_REQUIRE(scheme == VES_NEAR_NONE || vself, "ves_near_sing_int: vself required");
  cudaStream_t s = (cudaStream_t)stream;
  int rc = ves_reset_status(c, s);
  if (rc) return rc;
  WsCarver w(ws, ws_bytes);
  rc = near_sing_int_run(c, scheme, precision, nv, X, sa_up, Xup, f, vself, nl, h, LP, near_only, w, s);
  if (rc) return rc;
  return finish(c, s, "ves_near_sing_int");
}

extern "C" size_t ves_near_sing_int_dl_workspace(ves_ctx* c, int nv) {
  if (!c) return 0;
  WsCarver w(nullptr, 0);
  near_sing_int_dl_run(c, VES_NEAR_PY_HH, VES_PREC_FP32M, nv, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr,
                       nullptr, nullptr, 0, nullptr, nullptr, w, 0);
  return w.off + 256;
}

extern "C" int ves_near_sing_int_dl(ves_ctx* c, int scheme, int precision, int nv, const double* X, const double* Xup,
                                    const double* tang_up, const double* sa_up, const double* visc, const double* f,
                                    const double* vself, const ves_near_lists* nl, double h, double* LP,
                                    double* near_only, void* ws, size_t ws_bytes, void* stream) {
  VES_REQUIRE(c && X && Xup && tang_up && sa_up && visc && f && LP && ws && nv >= 0,
              "ves_near_sing_int_dl: bad arguments");
  VES_REQUIRE(scheme == VES_NEAR_NONE || vself, "ves_near_sing_int_dl: vself required");
  cudaStream_t s = (cudaStream_t)stream;
  int rc = ves_reset_status(c, s);
  if (rc) return rc;
  WsCarver w(ws, ws_bytes);
  rc = near_sing_int_dl_run(c, scheme, precision, nv, X, Xup, tang_up, sa_up, visc, f, vself, nl, h, LP, near_only, w,
                            s);
  if (rc) return rc;
  return finish(c, s, "ves_near_sing_int_dl");
}

extern "C" size_t ves_redistribute_arclength_workspace(ves_ctx* c, int nv) {
  if (!c) return 0;
  WsCarver w(nullptr, 0);
  post_redistribute(c, nv, nullptr, nullptr, nullptr, w, 0);
  return w.off + 256;
}

extern "C" int ves_redistribute_arclength(ves_ctx* c, int nv, const double* X, double* Xout, int* flags,
                                          int* all_good, void* ws, size_t ws_bytes, void* stream) {
  VES_REQUIRE(c && X && Xout && flags && ws && nv >= 0, "ves_redistribute_arclength: bad arguments");
  cudaStream_t s = (cudaStream_t)stream;
  WsCarver w(ws, ws_bytes);
  int rc = post_redistribute(c, nv, X, Xout, flags, w, s);
  if (rc || !all_good) return rc;
  *all_good = 1;
  if (nv == 0) return VES_OK;
  int* h = (int*)c->h_scal;  // pinned scratch, nv ints at most 512 at a time
  for (int k0 = 0; k0 < nv; k0 += 512) {
    const int n = nv - k0 < 512 ? nv - k0 : 512;
    rc = ves_cuda_status(cudaMemcpyAsync(h, flags + k0, n * sizeof(int), cudaMemcpyDeviceToHost, s), "flags");
    if (!rc) rc = ves_cuda_status(cudaStreamSynchronize(s), "flags sync");
    if (rc) return rc;
    for (int i = 0; i < n; ++i)
      if (!h[i]) *all_good = 0;
  }
  return VES_OK;
}

extern "C" int ves_align_center_angle(ves_ctx* c, int nv, const double* Xorg, const double* X, double* Xout,
                                      void* stream) {
  VES_REQUIRE(c && Xorg && X && Xout && nv >= 0, "ves_align_center_angle: bad arguments");
  launch_align_center_angle(c, nv, Xorg, X, Xout, nullptr, nullptr, (cudaStream_t)stream);
  return ves_launch_check("ves_align_center_angle");
}

extern "C" int ves_center_angle(ves_ctx* c, int nv, const double* X, double* center, double* angle, void* stream) {
  VES_REQUIRE(c && X && nv >= 0, "ves_center_angle: bad arguments");
  launch_align_center_angle(c, nv, nullptr, X, nullptr, center, angle, (cudaStream_t)stream);
  return ves_launch_check("ves_center_angle");
}

extern "C" size_t ves_correct_area_length_workspace(ves_ctx* c, int nv) {
  if (!c) return 0;
  WsCarver w(nullptr, 0);
  post_correct_area_length(c, nv, nullptr, nullptr, nullptr, nullptr, nullptr, w, 0);
  return w.off + 256;
}

extern "C" int ves_correct_area_length(ves_ctx* c, int nv, const double* X, const double* area0,
                                       const double* length0, double* Xout, int* outer_iters, void* ws,
                                       size_t ws_bytes, void* stream) {
  VES_REQUIRE(c && X && area0 && length0 && Xout && ws && nv >= 0, "ves_correct_area_length: bad arguments");
  WsCarver w(ws, ws_bytes);
  return post_correct_area_length(c, nv, X, area0, length0, Xout, outer_iters, w, (cudaStream_t)stream);
}

// ---------------------------------------------------------------------------
// Failure-path probe: one thread waits on an mbarrier that nothing completes,
// with the bounded sleeping wait the tensor-core kernels use for MMA
// completion.  The wait gives up, records VES_ERR_TIMEOUT in the context's
// status word and the kernel returns, so the context stays usable.
namespace {
__global__ void wait_probe_kernel(VesDeviceStatus* st) {
  __shared__ uint64_t bar;
  if (threadIdx.x == 0) {
    tc_mbar_init(&bar, 1);
    tc_mbar_fence_init();
  }
  __syncthreads();
  if (threadIdx.x == 0) tc_mbar_wait_sleep(&bar, 0, st, 99);  // phase 0 never completes: nobody arrives
  __syncthreads();
}
}  // namespace

extern "C" int ves_probe_wait_timeout(ves_ctx* c, void* stream) {
  VES_REQUIRE(c, "ves_probe_wait_timeout: bad arguments");
  cudaStream_t s = (cudaStream_t)stream;
  int rc = ves_reset_status(c, s);
  if (rc) return rc;
  ves_count_launch();
  wait_probe_kernel<<<1, 32, 0, s>>>(c->status);
  if ((rc = ves_launch_check("wait probe"))) return rc;
  return ves_check_status(c, s, "wait probe");
}
