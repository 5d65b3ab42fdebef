// Near-zone lists built on the device and the near-singular corrections.
//
// Candidate search: every target vesicle scans all vesicles with one warp,
// testing bounding boxes grown by the near threshold; hits are appended in
// ascending order (warp ballot + popc), so each target vesicle owns a sorted
// candidate list ("bucket") that the far-field kernel walks with a cursor.
// Point-level tests then run one CTA per (target vesicle, candidate).
//
// Two schemes:
// * py_hh — naiveNearZoneInfo (mytorch/biem_support.py:520-613) and
//   nearSingInt_hh (mytorch/poten.py:466-600).  Exclusions: target point i of t
//   is near source vesicle s if any of the Nup upsampled points of s lies
//   closer than the threshold.  Correction: the reference's hedgehog list is
//   indexed by (t, s*Nup + u) but consumed as if it were (k1, k2*N + J); for
//   every such entry with k2 != k1 it adds vself[(icp - 3) mod N, k1] at
//   (J, k2), where icp is the coarse point of k1 closest to upsampled point J
//   of k2 (the last row of the Lagrange matrix is e_0, poten.py:987, so the
//   interpolated value is the first stencil value).
// * matlab — getZone/closestPnt (matlab/capsules_py.m:194-643) and nearSingInt
//   (matlab/poten_py.m:495-692): near if the Newton closest point on the local
//   7-point interpolant of s is closer than h; the trapezoid contribution of s
//   is removed (exclusion) and replaced by the 7-point Lagrange extrapolation
//   along the normal, evaluated at dist/(6*beta*h).
#include "ves_internal.h"

namespace {

__device__ __forceinline__ double horner7(const double* c, double t) {
  double v = 0.0;
#pragma unroll
  for (int i = 0; i < 7; ++i) v = fma(v, t, c[i]);
  return v;
}

// bounding boxes [nv][4] = xmin, xmax, ymin, ymax of n-point curves
__global__ void bbox_kernel(int n, const double* __restrict__ X, double* __restrict__ box) {
  __shared__ double red[4][128];
  const int k = blockIdx.x;
  const double* x = X + (long long)k * 2 * n;
  double a = 1e300, b = -1e300, c = 1e300, d = -1e300;
  for (int j = threadIdx.x; j < n; j += blockDim.x) {
    a = fmin(a, x[j]);
    b = fmax(b, x[j]);
    c = fmin(c, x[n + j]);
    d = fmax(d, x[n + j]);
  }
  red[0][threadIdx.x] = a;
  red[1][threadIdx.x] = b;
  red[2][threadIdx.x] = c;
  red[3][threadIdx.x] = d;
  __syncthreads();
  for (int w = 64; w > 0; w >>= 1) {
    if (threadIdx.x < w) {
      red[0][threadIdx.x] = fmin(red[0][threadIdx.x], red[0][threadIdx.x + w]);
      red[1][threadIdx.x] = fmax(red[1][threadIdx.x], red[1][threadIdx.x + w]);
      red[2][threadIdx.x] = fmin(red[2][threadIdx.x], red[2][threadIdx.x + w]);
      red[3][threadIdx.x] = fmax(red[3][threadIdx.x], red[3][threadIdx.x + w]);
    }
    __syncthreads();
  }
  if (threadIdx.x < 4) box[k * 4 + threadIdx.x] = red[threadIdx.x][0];
}

// one warp per target vesicle; candidates in ascending order.  nt target and
// ns source vesicles; same_set: the two sets are one (a vesicle is not its own
// candidate).
__global__ void candidates_kernel(int nt, int ns, bool same_set, const double* __restrict__ tbox,
                                  const double* __restrict__ sbox, double thr, int maxc, int* __restrict__ cand_count,
                                  int* __restrict__ cand_src, VesDeviceStatus* st) {
  const int t = (blockIdx.x * blockDim.x + threadIdx.x) / 32;
  const int lane = threadIdx.x % 32;
  if (t >= nt) return;
  const double tx0 = tbox[t * 4], tx1 = tbox[t * 4 + 1], ty0 = tbox[t * 4 + 2], ty1 = tbox[t * 4 + 3];
  int count = 0;
  for (int base = 0; base < ns; base += 32) {
    const int s = base + lane;
    bool hit = false;
    if (s < ns && !(same_set && s == t)) {
      const double gx = fmax(0.0, fmax(sbox[s * 4] - tx1, tx0 - sbox[s * 4 + 1]));
      const double gy = fmax(0.0, fmax(sbox[s * 4 + 2] - ty1, ty0 - sbox[s * 4 + 3]));
      hit = gx * gx + gy * gy < thr * thr;
    }
    const unsigned m = __ballot_sync(0xffffffffu, hit);
    const int pos = count + __popc(m & ((1u << lane) - 1u));
    if (hit && pos < maxc) cand_src[(long long)t * maxc + pos] = s;
    count += __popc(m);
  }
  if (lane == 0) {
    cand_count[t] = count < maxc ? count : maxc;
    if (count > maxc) ves_set_error(st, VES_ERR_NEARLIST_OVERFLOW, 20, (long long)t);
  }
}

// py scheme: exclusion bits per target point and hedgehog bits per upsampled point
__global__ void __launch_bounds__(256) py_masks_kernel(int N, int Nup, int maxc, double thr2,
                                                       const double* __restrict__ X, const double* __restrict__ Xup,
                                                       const int* __restrict__ cand_count,
                                                       const int* __restrict__ cand_src,
                                                       uint32_t* __restrict__ excl_mask,
                                                       uint32_t* __restrict__ hh_mask) {
  extern __shared__ double sh[];
  const int t = blockIdx.y, slot = blockIdx.x;
  const int wN = (N + 31) / 32, wU = (Nup + 31) / 32;
  uint32_t* em = excl_mask + ((long long)t * maxc + slot) * wN;
  uint32_t* hm = hh_mask + ((long long)t * maxc + slot) * wU;
  if (slot >= cand_count[t]) return;
  const int s = cand_src[(long long)t * maxc + slot];
  double* tx = sh;
  double* ty = tx + N;
  uint32_t* ebits = (uint32_t*)(ty + N);
  uint32_t* hbits = ebits + wN;
  for (int i = threadIdx.x; i < N; i += blockDim.x) {
    tx[i] = X[(long long)t * 2 * N + i];
    ty[i] = X[(long long)t * 2 * N + N + i];
  }
  for (int i = threadIdx.x; i < wN; i += blockDim.x) ebits[i] = 0;
  for (int i = threadIdx.x; i < wU; i += blockDim.x) hbits[i] = 0;
  __syncthreads();
  const double* xs = Xup + (long long)s * 2 * Nup;
  for (int u = threadIdx.x; u < Nup; u += blockDim.x) {
    const double sx = xs[u], sy = xs[Nup + u];
    bool any = false;
    for (int i = 0; i < N; ++i) {
      const double dx = tx[i] - sx, dy = ty[i] - sy;
      if (dx * dx + dy * dy < thr2) {
        any = true;
        atomicOr(&ebits[i >> 5], 1u << (i & 31));
      }
    }
    if (any) atomicOr(&hbits[u >> 5], 1u << (u & 31));
  }
  __syncthreads();
  for (int i = threadIdx.x; i < wN; i += blockDim.x) em[i] = ebits[i];
  for (int i = threadIdx.x; i < wU; i += blockDim.x) hm[i] = hbits[i];
}

// py_hh correction: one warp per (t, candidate), lanes over hedgehog words
__global__ void hh_apply_kernel(int nv, int N, int Nup, int maxc, const double* __restrict__ X,
                                const double* __restrict__ Xup, const int* __restrict__ cand_count,
                                const int* __restrict__ cand_src, const uint32_t* __restrict__ hh_mask,
                                const double* __restrict__ vself, double* __restrict__ LP,
                                double* __restrict__ near_only, int* __restrict__ counter) {
  const int gw = (blockIdx.x * blockDim.x + threadIdx.x) / 32;
  const int lane = threadIdx.x % 32;
  const int t = gw / maxc, slot = gw % maxc;
  if (t >= nv || slot >= cand_count[t]) return;
  const int s = cand_src[(long long)t * maxc + slot];
  const int wU = (Nup + 31) / 32;
  const uint32_t* hm = hh_mask + ((long long)t * maxc + slot) * wU;
  const double* Xk1 = X + (long long)t * 2 * N;  // k1 = t (coarse vesicle of the pair)
  for (int w = lane; w < wU; w += 32) {
    uint32_t bits = hm[w];
    while (bits) {
      const int b = __ffs(bits) - 1;
      bits &= bits - 1;
      const int u = w * 32 + b;
      const long long id1 = (long long)s * Nup + u;
      const int k2 = (int)(id1 / N), J = (int)(id1 % N);
      if (k2 >= nv || k2 == t) continue;
      // closest coarse point of k1 to upsampled point J of vesicle k2 (first minimum)
      const double px = Xup[(long long)k2 * 2 * Nup + J], py = Xup[(long long)k2 * 2 * Nup + Nup + J];
      double best = 1e300;
      int icp = 0;
      for (int i = 0; i < N; ++i) {
        const double dx = Xk1[i] - px, dy = Xk1[N + i] - py;
        const double d2 = dx * dx + dy * dy;
        if (d2 < best) {
          best = d2;
          icp = i;
        }
      }
      const int pn0 = ((icp - 3) % N + N) % N;
      const double vx = vself[(long long)t * 2 * N + pn0], vy = vself[(long long)t * 2 * N + N + pn0];
      atomicAdd(&LP[(long long)k2 * 2 * N + J], vx);
      atomicAdd(&LP[(long long)k2 * 2 * N + N + J], vy);
      if (near_only) {
        atomicAdd(&near_only[(long long)k2 * 2 * N + J], vx);
        atomicAdd(&near_only[(long long)k2 * 2 * N + N + J], vy);
      }
      if (counter) atomicAdd(counter, 1);
    }
  }
}

// MATLAB scheme: per (target vesicle t, candidate source s) and target point j;
// targets Xt with Nt points per vesicle, sources Xs with Ns (one set: Xt = Xs)
__global__ void __launch_bounds__(128) matlab_zone_kernel(int Nt, int Ns, int maxc, double h,
                                                          const double* __restrict__ Xt,
                                                          const double* __restrict__ Xs,
                                                          const double* __restrict__ lag,
                                                          const int* __restrict__ cand_count,
                                                          const int* __restrict__ cand_src,
                                                          uint32_t* __restrict__ excl_mask, int max_entries,
                                                          int* __restrict__ n_entries, int* __restrict__ ent_tsj,
                                                          int* __restrict__ ent_icp, double* __restrict__ ent_geo,
                                                          VesDeviceStatus* st) {
  extern __shared__ double sh[];
  const int t = blockIdx.y, slot = blockIdx.x;
  const int wN = (Nt + 31) / 32;
  uint32_t* em = excl_mask + ((long long)t * maxc + slot) * wN;
  if (slot >= cand_count[t]) return;
  const int s = cand_src[(long long)t * maxc + slot];
  double* sx = sh;
  double* sy = sx + Ns;
  double* L = sy + Ns;  // 49
  uint32_t* bits = (uint32_t*)(L + 49);
  for (int i = threadIdx.x; i < Ns; i += blockDim.x) {
    sx[i] = Xs[(long long)s * 2 * Ns + i];
    sy[i] = Xs[(long long)s * 2 * Ns + Ns + i];
  }
  for (int i = threadIdx.x; i < 49; i += blockDim.x) L[i] = lag[i];
  for (int i = threadIdx.x; i < wN; i += blockDim.x) bits[i] = 0;
  __syncthreads();
  for (int j = threadIdx.x; j < Nt; j += blockDim.x) {
    const double xt = Xt[(long long)t * 2 * Nt + j], yt = Xt[(long long)t * 2 * Nt + Nt + j];
    double best = 1e300;
    int icp = 0;
    for (int i = 0; i < Ns; ++i) {
      const double dx = xt - sx[i], dy = yt - sy[i];
      const double d2 = dx * dx + dy * dy;
      if (d2 < best) {
        best = d2;
        icp = i;
      }
    }
    if (sqrt(best) >= 2.0 * h) continue;
    // closestPnt: one Newton step from theta = 1/2 on the 7-point interpolant
    double px[7], py[7];
#pragma unroll
    for (int r = 0; r < 7; ++r) {
      double ax = 0, ay = 0;
#pragma unroll
      for (int q = 0; q < 7; ++q) {
        const int idx = ((icp - 3 + q) % Ns + Ns) % Ns;
        ax = fma(L[r * 7 + q], sx[idx], ax);
        ay = fma(L[r * 7 + q], sy[idx], ay);
      }
      px[r] = ax;
      py[r] = ay;
    }
    double dpx[6], dpy[6], d2px[5], d2py[5];
#pragma unroll
    for (int r = 0; r < 6; ++r) {
      dpx[r] = px[r] * (6 - r);
      dpy[r] = py[r] * (6 - r);
    }
#pragma unroll
    for (int r = 0; r < 5; ++r) {
      d2px[r] = dpx[r] * (5 - r);
      d2py[r] = dpy[r] * (5 - r);
    }
    auto hp = [](const double* c, int n, double x) {
      double v = 0;
      for (int i = 0; i < n; ++i) v = fma(v, x, c[i]);
      return v;
    };
    double th = 0.5;
    const double zx = hp(px, 7, th), zy = hp(py, 7, th);
    const double dzx = hp(dpx, 6, th), dzy = hp(dpy, 6, th);
    const double d2zx = hp(d2px, 5, th), d2zy = hp(d2py, 5, th);
    const double num = (zx - xt) * dzx + (zy - yt) * dzy;
    const double den = (zx - xt) * d2zx + (zy - yt) * d2zy + dzx * dzx + dzy * dzy;
    th = th - num / den;
    const double nx = hp(px, 7, th), ny = hp(py, 7, th);
    const double dist = sqrt((nx - xt) * (nx - xt) + (ny - yt) * (ny - yt));
    if (dist < h) {
      atomicOr(&bits[j >> 5], 1u << (j & 31));
      const int e = atomicAdd(n_entries, 1);
      if (e < max_entries) {
        ent_tsj[3 * e] = t;
        ent_tsj[3 * e + 1] = s;
        ent_tsj[3 * e + 2] = j;
        ent_icp[e] = icp;
        ent_geo[4 * e] = dist;
        ent_geo[4 * e + 1] = nx;
        ent_geo[4 * e + 2] = ny;
        ent_geo[4 * e + 3] = th;
      } else {
        ves_set_error(st, VES_ERR_NEARLIST_OVERFLOW, 21, e);
      }
    }
  }
  __syncthreads();
  for (int i = threadIdx.x; i < wN; i += blockDim.x) em[i] = bits[i];
}

// MATLAB correction, one warp per entry.  DL: the layer potential at the
// Lagrange points is the double layer (kernelDirect = exactStokesDL,
// tstep_biem.py:236,501), with normals (ty, -tx) of the upsampled source and
// den already scaled by (1 - visc); otherwise the single layer.
// Targets Xt and LP with Nt points per vesicle; sources with Ns points (vself)
// and Nup upsampled points (Xup, tang_up, den).
template <bool DL>
__global__ void matlab_correct_kernel(int Nt, int Ns, int Nup, double h, const double* __restrict__ Xt,
                                      const double* __restrict__ Xup, const double* __restrict__ tang_up,
                                      const double* __restrict__ den,
                                      const double* __restrict__ vself, const double* __restrict__ lag,
                                      const int* __restrict__ n_entries, int max_entries,
                                      const int* __restrict__ ent_tsj, const int* __restrict__ ent_icp,
                                      const double* __restrict__ ent_geo, double* __restrict__ LP,
                                      double* __restrict__ near_only) {
  const int e = (blockIdx.x * blockDim.x + threadIdx.x) / 32;
  const int lane = threadIdx.x % 32;
  const int ne = min(*n_entries, max_entries);
  if (e >= ne) return;
  const int t = ent_tsj[3 * e], s = ent_tsj[3 * e + 1], j = ent_tsj[3 * e + 2];
  const int icp = ent_icp[e];
  const double dist = ent_geo[4 * e], nxp = ent_geo[4 * e + 1], nyp = ent_geo[4 * e + 2], th = ent_geo[4 * e + 3];
  const double beta = 1.1;
  const double xt = Xt[(long long)t * 2 * Nt + j], yt = Xt[(long long)t * 2 * Nt + Nt + j];
  const double ux = (xt - nxp) / dist, uy = (yt - nyp) / dist;
  // layer potential of source vesicle s at the 6 Lagrange points
  double ax[6], ay[6];
#pragma unroll
  for (int m = 0; m < 6; ++m) ax[m] = ay[m] = 0.0;
  const double* xs = Xup + (long long)s * 2 * Nup;
  const double* ds = den + (long long)s * 2 * Nup;
  for (int u = lane; u < Nup; u += 32) {
    const double sxu = xs[u], syu = xs[Nup + u], dxu = ds[u], dyu = ds[Nup + u];
    double nxu = 0.0, nyu = 0.0;
    if (DL) {
      nxu = tang_up[(long long)s * 2 * Nup + Nup + u];
      nyu = -tang_up[(long long)s * 2 * Nup + u];
    }
#pragma unroll
    for (int m = 0; m < 6; ++m) {
      const double px = nxp + beta * h * ux * (m + 1), py = nyp + beta * h * uy * (m + 1);
      const double rx = px - sxu, ry = py - syu;
      const double r2 = rx * rx + ry * ry;
      if (DL) {
        const double cc = ((rx * nxu + ry * nyu) / (r2 * r2)) * (rx * dxu + ry * dyu);
        ax[m] += cc * rx;
        ay[m] += cc * ry;
      } else {
        const double lg = 0.5 * log(r2);
        const double cc = (rx * dxu + ry * dyu) / r2;
        ax[m] += cc * rx - lg * dxu;
        ay[m] += cc * ry - lg * dyu;
      }
    }
  }
#pragma unroll
  for (int m = 0; m < 6; ++m) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      ax[m] += __shfl_xor_sync(0xffffffffu, ax[m], o);
      ay[m] += __shfl_xor_sync(0xffffffffu, ay[m], o);
    }
  }
  if (lane != 0) return;
  const double kscale = DL ? 1.0 / VES_PI : 1.0 / (4.0 * VES_PI);
  double vals[2];
  for (int comp = 0; comp < 2; ++comp) {
    // on-curve value: Lagrange interpolant of vself around icp at theta
    double coef[7], stencil[7];
    for (int q = 0; q < 7; ++q) stencil[q] = vself[(long long)s * 2 * Ns + comp * Ns + ((icp - 3 + q) % Ns + Ns) % Ns];
    for (int r = 0; r < 7; ++r) {
      double a = 0;
      for (int q = 0; q < 7; ++q) a = fma(lag[r * 7 + q], stencil[q], a);
      coef[r] = a;
    }
    const double vel = horner7(coef, th);
    double pts[7];
    pts[0] = vel;
    for (int m = 0; m < 6; ++m) pts[m + 1] = (comp == 0 ? ax[m] : ay[m]) * kscale;
    for (int r = 0; r < 7; ++r) {
      double a = 0;
      for (int q = 0; q < 7; ++q) a = fma(lag[r * 7 + q], pts[q], a);
      coef[r] = a;
    }
    vals[comp] = horner7(coef, dist / (beta * h * 6.0));
  }
  atomicAdd(&LP[(long long)t * 2 * Nt + j], vals[0]);
  atomicAdd(&LP[(long long)t * 2 * Nt + Nt + j], vals[1]);
  if (near_only) {
    atomicAdd(&near_only[(long long)t * 2 * Nt + j], vals[0]);
    atomicAdd(&near_only[(long long)t * 2 * Nt + Nt + j], vals[1]);
  }
}

__global__ void min_reduce_kernel(int n, const double* __restrict__ a, double* __restrict__ out) {
  __shared__ double red[256];
  double m = 1e300;
  for (int i = threadIdx.x; i < n; i += blockDim.x) m = fmin(m, a[i]);
  red[threadIdx.x] = m;
  __syncthreads();
  for (int w = 128; w > 0; w >>= 1) {
    if (threadIdx.x < w) red[threadIdx.x] = fmin(red[threadIdx.x], red[threadIdx.x + w]);
    __syncthreads();
  }
  if (threadIdx.x == 0) *out = red[0];
}

__global__ void identity_index_kernel(int n, int* __restrict__ idx) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) idx[i] = i;
}

__global__ void add_kernel(long long n, const double* __restrict__ a, double* __restrict__ out) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] += a[i];
}

}  // namespace

int near_zone_py(ves_ctx* c, int nv, const double* X, const double* Xup_in, double thresh,
                 const ves_near_lists* nl, WsCarver& ws, cudaStream_t s) {
  const int N = c->N, Nup = c->Nup;
  double* tbox = ws.take<double>((size_t)nv * 4);
  double* sbox = ws.take<double>((size_t)nv * 4);
  double* Xup = Xup_in ? nullptr : ws.take<double>((size_t)nv * 2 * Nup);
  if (ws.sizing) return VES_OK;
  if (!ws.ok()) {
    ves_record_error(VES_ERR_WORKSPACE, "near_zone_py: workspace too small");
    return VES_ERR_WORKSPACE;
  }
  if (!nl || !nl->cand_count || !nl->cand_src || !nl->excl_mask || !nl->hh_mask || nl->maxc <= 0) {
    ves_record_error(VES_ERR_ARG, "near_zone_py: incomplete near lists");
    return VES_ERR_ARG;
  }
  if (nv <= 0) return VES_OK;
  const double thr = thresh > 0 ? thresh : 1.0 / N;
  if (!Xup_in) launch_upsample(c, nv, 2, X, 2LL * N, Xup, s);
  const double* Xu = Xup_in ? Xup_in : Xup;
  ves_count_launch();
  bbox_kernel<<<nv, 128, 0, s>>>(N, X, tbox);
  ves_count_launch();
  bbox_kernel<<<nv, 128, 0, s>>>(Nup, Xu, sbox);
  ves_count_launch();
  candidates_kernel<<<ceil_div((long long)nv * 32, 256), 256, 0, s>>>(nv, nv, true, tbox, sbox, thr, nl->maxc,
                                                                      nl->cand_count,
                                                                      nl->cand_src, c->status);
  const size_t sh = (size_t)2 * N * sizeof(double) + (c->nwords_N + c->nwords_up) * sizeof(uint32_t);
  dim3 grid(nl->maxc, nv);
  ves_count_launch();
  py_masks_kernel<<<grid, 256, sh, s>>>(N, Nup, nl->maxc, thr * thr, X, Xu, nl->cand_count, nl->cand_src,
                                        nl->excl_mask, nl->hh_mask);
  return ves_launch_check("near_zone_py");
}

int near_zone_matlab(ves_ctx* c, int nv, const double* X, double h, const ves_near_lists* nl, WsCarver& ws,
                     cudaStream_t s) {
  const int N = c->N;
  double* box = ws.take<double>((size_t)nv * 4);
  double* len = ws.take<double>((size_t)nv);
  double* hmin = ws.take<double>(1);
  if (ws.sizing) return VES_OK;
  if (!ws.ok()) {
    ves_record_error(VES_ERR_WORKSPACE, "near_zone_matlab: workspace too small");
    return VES_ERR_WORKSPACE;
  }
  if (!nl || !nl->cand_count || !nl->cand_src || !nl->excl_mask || !nl->n_entries || !nl->ent_tsj ||
      !nl->ent_icp || !nl->ent_geo || nl->maxc <= 0) {
    ves_record_error(VES_ERR_ARG, "near_zone_matlab: incomplete near lists");
    return VES_ERR_ARG;
  }
  if (nv <= 0) return VES_OK;
  if (h <= 0) {
    launch_geom_prop(c, nv, X, nullptr, nullptr, len, s);
    ves_count_launch();
    min_reduce_kernel<<<1, 256, 0, s>>>(nv, len, hmin);
    double lmin = 0;
    int rc = ves_cuda_status(cudaMemcpyAsync(&lmin, hmin, sizeof(double), cudaMemcpyDeviceToHost, s), "hmin");
    if (!rc) rc = ves_cuda_status(cudaStreamSynchronize(s), "hmin sync");
    if (rc) return rc;
    h = lmin / N;
  }
  int rc = ves_cuda_status(cudaMemsetAsync(nl->n_entries, 0, sizeof(int), s), "zero entries");
  if (rc) return rc;
  ves_count_launch();
  bbox_kernel<<<nv, 128, 0, s>>>(N, X, box);
  ves_count_launch();
  candidates_kernel<<<ceil_div((long long)nv * 32, 256), 256, 0, s>>>(nv, nv, true, box, box, 2.0 * h, nl->maxc,
                                                                      nl->cand_count, nl->cand_src, c->status);
  const size_t sh = (size_t)(2 * N + 49) * sizeof(double) + c->nwords_N * sizeof(uint32_t);
  dim3 grid(nl->maxc, nv);
  ves_count_launch();
  matlab_zone_kernel<<<grid, 128, sh, s>>>(N, N, nl->maxc, h, X, X, c->lag, nl->cand_count, nl->cand_src,
                                           nl->excl_mask, nl->max_entries, nl->n_entries, nl->ent_tsj,
                                           nl->ent_icp, nl->ent_geo, c->status);
  return ves_launch_check("near_zone_matlab");
}

int near_sing_int_run(ves_ctx* c, int scheme, int precision, int nv, const double* X, const double* sa_up,
                      const double* Xup, const double* f, const double* vself, const ves_near_lists* nl,
                      double h, double* LP, double* near_only, WsCarver& ws, cudaStream_t s) {
  const int N = c->N, Nup = c->Nup;
  double* fup = ws.take<double>((size_t)nv * 2 * Nup);
  double* den = ws.take<double>((size_t)nv * 2 * Nup);
  int* selfidx = ws.take<int>((size_t)nv);
  const ves_near_lists* excl = (scheme == VES_NEAR_NONE) ? nullptr : nl;
  if (ws.sizing) {
    farfield_run(c, precision, nv, Nup, Xup, den, nv, N, X, selfidx, excl, LP, ws, s);
    if (scheme == VES_NEAR_PY_RBF) rbf_near_correct(c, nv, X, f, vself, nl, LP, ws, s);
    return VES_OK;
  }
  if (!ws.ok()) {
    ves_record_error(VES_ERR_WORKSPACE, "near_sing_int: workspace too small");
    return VES_ERR_WORKSPACE;
  }
  if (scheme != VES_NEAR_NONE && scheme != VES_NEAR_PY_HH && scheme != VES_NEAR_MATLAB && scheme != VES_NEAR_PY_RBF) {
    ves_record_error(VES_ERR_ARG, "near_sing_int: bad scheme %d", scheme);
    return VES_ERR_ARG;
  }
  if (scheme != VES_NEAR_NONE && !nl) {
    ves_record_error(VES_ERR_ARG, "near_sing_int: near lists required");
    return VES_ERR_ARG;
  }
  if (nv <= 0) return VES_OK;
  if (near_only) {
    int rc0 = ves_cuda_status(cudaMemsetAsync(near_only, 0, (size_t)nv * 2 * N * sizeof(double), s), "zero near");
    if (rc0) return rc0;
  }
  if (nv == 1) {  // a single vesicle has no interactions (poten.py:485-486)
    return ves_cuda_status(cudaMemsetAsync(LP, 0, (size_t)2 * N * sizeof(double), s), "zero LP");
  }
  launch_upsample(c, nv, 2, f, 2LL * N, fup, s);
  launch_density(nv, Nup, fup, sa_up, den, s);
  ves_count_launch();
  identity_index_kernel<<<ceil_div(nv, 256), 256, 0, s>>>(nv, selfidx);
  int rc = farfield_run(c, precision, nv, Nup, Xup, den, nv, N, X, selfidx, excl, LP, ws, s);
  if (rc) return rc;
  if (scheme == VES_NEAR_PY_RBF) {
    // nearSingInt_rbf: the far field above plus the fits of the near pairs
    if ((rc = rbf_near_correct(c, nv, X, f, vself, nl, LP, ws, s))) return rc;
  } else if (scheme == VES_NEAR_PY_HH) {
    const long long warps = (long long)nv * nl->maxc;
    ves_count_launch();
    hh_apply_kernel<<<ceil_div(warps * 32, 256), 256, 0, s>>>(nv, N, Nup, nl->maxc, X, Xup, nl->cand_count,
                                                              nl->cand_src, nl->hh_mask, vself, LP, near_only,
                                                              nullptr);
  } else if (scheme == VES_NEAR_MATLAB) {
    const long long warps = nl->max_entries;
    ves_count_launch();
    matlab_correct_kernel<false><<<ceil_div(warps * 32, 256), 256, 0, s>>>(N, N, Nup, h, X, Xup, nullptr, den, vself,
                                                                           c->lag,
                                                                    nl->n_entries, nl->max_entries, nl->ent_tsj,
                                                                    nl->ent_icp, nl->ent_geo, LP, near_only);
  }
  return ves_launch_check("near_sing_int");
}

// Two vesicle sets of different point counts (a mixed suspension): the near
// zone of the target points of one set w.r.t. the source vesicles of the
// other (getZone's NearOther, matlab/capsules_py.m:194-467, with the source
// set's h) and the source set's single layer at the target points with those
// entries corrected (nearSingInt with tEqualS false, matlab/poten_py.m:495-692).
int near_zone_matlab_cross(ves_ctx* ct, ves_ctx* cs, int nvt, const double* Xt, int nvs, const double* Xs, double h,
                           const ves_near_lists* nl, WsCarver& ws, cudaStream_t s) {
  const int Nt = ct->N, Ns = cs->N;
  double* tbox = ws.take<double>((size_t)nvt * 4);
  double* sbox = ws.take<double>((size_t)nvs * 4);
  if (ws.sizing) return VES_OK;
  if (!ws.ok()) {
    ves_record_error(VES_ERR_WORKSPACE, "near_zone_cross: workspace too small");
    return VES_ERR_WORKSPACE;
  }
  if (!nl || !nl->cand_count || !nl->cand_src || !nl->excl_mask || !nl->n_entries || !nl->ent_tsj ||
      !nl->ent_icp || !nl->ent_geo || nl->maxc <= 0 || h <= 0) {
    ves_record_error(VES_ERR_ARG, "near_zone_cross: incomplete near lists or h <= 0");
    return VES_ERR_ARG;
  }
  int rc = ves_cuda_status(cudaMemsetAsync(nl->n_entries, 0, sizeof(int), s), "zero entries");
  if (rc || nvt <= 0) return rc;
  ves_count_launch(nvs > 0 ? 3 : 2);
  bbox_kernel<<<nvt, 128, 0, s>>>(Nt, Xt, tbox);
  if (nvs > 0) bbox_kernel<<<nvs, 128, 0, s>>>(Ns, Xs, sbox);
  candidates_kernel<<<ceil_div((long long)nvt * 32, 256), 256, 0, s>>>(nvt, nvs, false, tbox, sbox, 2.0 * h, nl->maxc,
                                                                       nl->cand_count, nl->cand_src, ct->status);
  const size_t sh = (size_t)(2 * Ns + 49) * sizeof(double) + ct->nwords_N * sizeof(uint32_t);
  dim3 grid(nl->maxc, nvt);
  ves_count_launch();
  matlab_zone_kernel<<<grid, 128, sh, s>>>(Nt, Ns, nl->maxc, h, Xt, Xs, ct->lag, nl->cand_count, nl->cand_src,
                                           nl->excl_mask, nl->max_entries, nl->n_entries, nl->ent_tsj, nl->ent_icp,
                                           nl->ent_geo, ct->status);
  return ves_launch_check("near_zone_cross");
}

int near_sing_int_cross_add(ves_ctx* ct, ves_ctx* cs, int scheme, int precision, int nvt, const double* Xt, int nvs,
                            const double* Xup_s, const double* den_s, const double* vself_s,
                            const ves_near_lists* nl, double h, double* LP, WsCarver& ws, cudaStream_t s) {
  const int Nt = ct->N, Ns = cs->N, Nups = cs->Nup;
  double* tmp = ws.take<double>((size_t)nvt * 2 * Nt);
  const ves_near_lists* excl = (scheme == VES_NEAR_MATLAB) ? nl : nullptr;
  if (ws.sizing) {
    farfield_run(ct, precision, nvs, Nups, Xup_s, den_s, nvt, Nt, Xt, nullptr, excl, tmp, ws, s);
    return VES_OK;
  }
  if (!ws.ok()) {
    ves_record_error(VES_ERR_WORKSPACE, "near_sing_int_cross: workspace too small");
    return VES_ERR_WORKSPACE;
  }
  if (scheme != VES_NEAR_NONE && scheme != VES_NEAR_MATLAB) {
    ves_record_error(VES_ERR_ARG, "near_sing_int_cross: scheme %d (between sets: matlab or none)", scheme);
    return VES_ERR_ARG;
  }
  if (nvt <= 0 || nvs <= 0) return VES_OK;
  int rc = farfield_run(ct, precision, nvs, Nups, Xup_s, den_s, nvt, Nt, Xt, nullptr, excl, tmp, ws, s);
  if (rc) return rc;
  const long long n = (long long)nvt * 2 * Nt;
  ves_count_launch();
  add_kernel<<<ceil_div(n, 256), 256, 0, s>>>(n, tmp, LP);
  if (scheme == VES_NEAR_MATLAB) {
    const long long warps = nl->max_entries;
    ves_count_launch();
    matlab_correct_kernel<false><<<ceil_div(warps * 32, 256), 256, 0, s>>>(
        Nt, Ns, Nups, h, Xt, Xup_s, nullptr, den_s, vself_s, ct->lag, nl->n_entries, nl->max_entries, nl->ent_tsj,
        nl->ent_icp, nl->ent_geo, LP, nullptr);
  }
  return ves_launch_check("near_sing_int_cross");
}

// nearSingInt with kernelDirect = exactStokesDL (tstep_biem.py:236,501;
// matlab/poten_py.m:495-692): the double-layer far field over the Nup
// upsampled sources (den = fup sa_up 2pi/Nup (1 - visc)) with the near pairs
// removed, plus the correction from vself = jump f + D f: the py_hh rule
// (which uses vself only) or the MATLAB Lagrange extrapolation with the
// double layer at the Lagrange points.
int near_sing_int_dl_run(ves_ctx* c, int scheme, int precision, int nv, const double* X, const double* Xup,
                         const double* tang_up, const double* sa_up, const double* visc, const double* f,
                         const double* vself, const ves_near_lists* nl, double h, double* LP, double* near_only,
                         WsCarver& ws, cudaStream_t s) {
  const int N = c->N, Nup = c->Nup;
  double* fup = ws.take<double>((size_t)nv * 2 * Nup);
  double* den = ws.take<double>((size_t)nv * 2 * Nup);
  int* selfidx = ws.take<int>((size_t)nv);
  const ves_near_lists* excl = (scheme == VES_NEAR_NONE) ? nullptr : nl;
  if (ws.sizing) {
    return farfield_dl_run(c, precision, nv, Nup, Xup, tang_up, den, sa_up, visc, nv, N, X, selfidx, excl, LP, ws,
                           s);
  }
  if (!ws.ok()) {
    ves_record_error(VES_ERR_WORKSPACE, "near_sing_int_dl: workspace too small");
    return VES_ERR_WORKSPACE;
  }
  if (scheme != VES_NEAR_NONE && scheme != VES_NEAR_PY_HH && scheme != VES_NEAR_MATLAB) {
    ves_record_error(VES_ERR_ARG, "near_sing_int_dl: scheme %d (the double layer supports none, py_hh, matlab)",
                     scheme);
    return VES_ERR_ARG;
  }
  if (scheme != VES_NEAR_NONE && !nl) {
    ves_record_error(VES_ERR_ARG, "near_sing_int_dl: near lists required");
    return VES_ERR_ARG;
  }
  if (nv <= 0) return VES_OK;
  if (near_only) {
    int rc0 = ves_cuda_status(cudaMemsetAsync(near_only, 0, (size_t)nv * 2 * N * sizeof(double), s), "zero near");
    if (rc0) return rc0;
  }
  if (nv == 1) return ves_cuda_status(cudaMemsetAsync(LP, 0, (size_t)2 * N * sizeof(double), s), "zero LP");
  launch_upsample(c, nv, 2, f, 2LL * N, fup, s);
  launch_dl_density(nv, Nup, fup, sa_up, visc, den, s);
  ves_count_launch();
  identity_index_kernel<<<ceil_div(nv, 256), 256, 0, s>>>(nv, selfidx);
  int rc = farfield_dl_run(c, precision, nv, Nup, Xup, tang_up, den, sa_up, visc, nv, N, X, selfidx, excl, LP, ws,
                           s);
  if (rc) return rc;
  if (scheme == VES_NEAR_PY_HH) {
    const long long warps = (long long)nv * nl->maxc;
    ves_count_launch();
    hh_apply_kernel<<<ceil_div(warps * 32, 256), 256, 0, s>>>(nv, N, Nup, nl->maxc, X, Xup, nl->cand_count,
                                                              nl->cand_src, nl->hh_mask, vself, LP, near_only,
                                                              nullptr);
  } else if (scheme == VES_NEAR_MATLAB) {
    const long long warps = nl->max_entries;
    ves_count_launch();
    matlab_correct_kernel<true><<<ceil_div(warps * 32, 256), 256, 0, s>>>(
        N, N, Nup, h, X, Xup, tang_up, den, vself, c->lag, nl->n_entries, nl->max_entries, nl->ent_tsj, nl->ent_icp,
        nl->ent_geo, LP, near_only);
  }
  return ves_launch_check("near_sing_int_dl");
}
