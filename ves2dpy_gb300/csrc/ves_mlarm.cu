// The MLARM surrogate step for N = 128 (newtorch/wrapper_MLARM_batch_compile_N128.py,
// MLARM_manyfree_py.time_step_many_noinfo :986-1206), on the device.
//
// Geometry and the glue between the networks run in FP64, one CTA per
// vesicle; the networks run through the engine of ves_nets.cu in their own
// precision; the two all-pairs sums use the far-field kernel of
// ves_farfield.cu with the near pairs of the first call excluded in both
// (allExactStokesSLTarget_compare1/2, :429-645).
//
// Work whose result the reference step never reads is not done: the
// Gaussian RBF matrix and its Cholesky factor (:1063-1070, used only when
// use_near_correct is true, :2660), the layer tracer coordinates feeding it
// (:1741-1797) and the near-field velocity contraction (:2499, idem).  The
// near-field network itself is evaluated on request (eval_near_net): its
// velocities reach the step only multiplied by the repulsion force (:2500),
// which is zero without repulsion.
#include <math.h>
#include <string.h>

#include <algorithm>
#include <new>
#include <vector>

#include "ves_internal.h"
#include "ves_fft.cuh"

// engine entry points (ves_nets.cu)
int net_forward_run(const ves_net* net, int nv, const void* in, void* out, WsCarver& ws, VesDeviceStatus* st,
                    cudaStream_t s);
int net_dims(const ves_net* net, int* groups, int* length, int* cin, int* cout);
double net_flops_per_vesicle(const ves_net* net);

namespace {

constexpr int kN = 128;       // shape points the networks were built for
constexpr int kModes = 127;   // Fourier modes 1..127 of the merged networks
constexpr int kNearModes = 128;
constexpr int kNormDoubles = 127 * 4 * 2 + 4 + 4 + 128 * 4 + 128 * 24 + 4 + 2 + 127 * 4 * 2;

__device__ __forceinline__ double circ(const double* __restrict__ d, const double* __restrict__ a, int n, int j) {
  double s = 0.0;
  for (int l = 0; l <= j; ++l) s = fma(d[j - l], a[l], s);
  for (int l = j + 1; l < n; ++l) s = fma(d[j - l + n], a[l], s);
  return s;
}

// deterministic block reductions (blockDim a power of two)
__device__ double bsum(double v, double* red) {
  red[threadIdx.x] = v;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
    __syncthreads();
  }
  const double r = red[0];
  __syncthreads();
  return r;
}

// ---------------------------------------------------------------------------
// fBend (:1007-1013): bending of the shape upsampled to Nup points
// (capsules.bendingTerm, capsules.py:62-68, on capsules(upsample_fft(X, Nup)))
// truncated back to N modes (downsample_fft, filter.py:197-219).  x and y are
// packed as z = x + i y: the arc derivative (isa * ifft(ik fft(.)) with the
// Nyquist mode zeroed) maps real sequences to real ones, so one complex FFT
// pair per derivative serves both; the truncation keeps the real-part
// semantics of each component's Nyquist coefficient separately.
__global__ void bend_up_kernel(int N, int Nup, int m, const double* __restrict__ pc, const double* __restrict__ pcd,
                               const double* __restrict__ cosU, const double* __restrict__ sinU, double kappa,
                               const double* __restrict__ X, double* __restrict__ fB) {
  extern __shared__ double sh[];
  double* is = sh;          // [Nup]
  double* zr = is + Nup;    // [Nup]
  double* zi = zr + Nup;    // [Nup]
  double* tre = zi + Nup;   // [Nup]
  double* tim = tre + Nup;  // [Nup]
  double* xy = tim + Nup;   // [2N]
  const int k = blockIdx.x;
  const double* Xk = X + (long long)k * 2 * N;
  for (int i = threadIdx.x; i < 2 * N; i += blockDim.x) xy[i] = Xk[i];
  __syncthreads();
  // the interpolant and |dXup/dtheta| on the Nup grid
  if (ves_fft_size_ok(N) && Nup % N == 0) {
    // spectral: z = x + i y, FFT of length N (the Nup table read with stride
    // Nup/N), the spectrum zero-padded to Nup with the Nyquist mode split
    // between +N/2 and -N/2 (interpft), inverse FFTs of length Nup of the
    // spectrum times i k (the derivative) and of the spectrum itself
    for (int i = threadIdx.x; i < N; i += blockDim.x) {
      zr[i] = xy[i];
      zi[i] = xy[N + i];
    }
    ves_fft(zr, zi, tre, tim, N, cosU, sinU, -1, Nup / N);
    for (int i = threadIdx.x; i < N; i += blockDim.x) {
      xy[i] = zr[i];  // the spectrum, modes 0..N-1
      xy[N + i] = zi[i];
    }
    __syncthreads();
    const int h = N / 2, top = Nup - N;
    for (int pass = 0; pass < 2; ++pass) {
      for (int u = threadIdx.x; u < Nup; u += blockDim.x) {
        double vr = 0.0, vi = 0.0, kk = 0.0;
        if (u < h) {
          vr = xy[u];
          vi = xy[N + u];
          kk = u;
        } else if (u == h || u == Nup - h) {
          vr = 0.5 * xy[h];
          vi = 0.5 * xy[N + h];
          kk = (u == h) ? (double)h : -(double)h;
        } else if (u > Nup - h) {
          vr = xy[u - top];
          vi = xy[N + u - top];
          kk = (double)(u - Nup);
        }
        if (pass == 0) {  // i k (vr + i vi)
          zr[u] = -kk * vi;
          zi[u] = kk * vr;
        } else {
          zr[u] = vr;
          zi[u] = vi;
        }
      }
      ves_fft(zr, zi, tre, tim, Nup, cosU, sinU, +1);
      for (int u = threadIdx.x; u < Nup; u += blockDim.x) {
        if (pass == 0) {
          const double dx = zr[u] / N, dy = zi[u] / N;
          is[u] = 1.0 / sqrt(dx * dx + dy * dy);
        } else {
          zr[u] /= N;
          zi[u] /= N;
        }
      }
      __syncthreads();
    }
  } else {
    for (int u = threadIdx.x; u < Nup; u += blockDim.x) {
      double x = 0, y = 0, dx = 0, dy = 0;
      int r = u;
      for (int i = 0; i < N; ++i) {
        x = fma(pc[r], xy[i], x);
        y = fma(pc[r], xy[N + i], y);
        dx = fma(pcd[r], xy[i], dx);
        dy = fma(pcd[r], xy[N + i], dy);
        r -= m;
        if (r < 0) r += Nup;
      }
      zr[u] = x;
      zi[u] = y;
      is[u] = 1.0 / sqrt(dx * dx + dy * dy);
    }
  }
  // four arc derivatives: z <- isa * ifft(i k fft(z)), Nyquist zeroed
  for (int it = 0; it < 4; ++it) {
    ves_fft(zr, zi, tre, tim, Nup, cosU, sinU, -1);
    for (int u = threadIdx.x; u < Nup; u += blockDim.x) {
      const double kk = (u < Nup / 2) ? (double)u : (u == Nup / 2 ? 0.0 : (double)(u - Nup));
      const double a = zr[u], b = zi[u];
      zr[u] = -kk * b / Nup;
      zi[u] = kk * a / Nup;
    }
    ves_fft(zr, zi, tre, tim, Nup, cosU, sinU, +1);
    for (int u = threadIdx.x; u < Nup; u += blockDim.x) {
      zr[u] *= is[u];
      zi[u] *= is[u];
    }
  }
  // downsample to N modes: frequencies -N/2+1..N/2-1 as they are, the -N/2
  // slot carrying Re(X_-N/2) + i Re(Y_-N/2) of the two real components
  ves_fft(zr, zi, tre, tim, Nup, cosU, sinU, -1);
  double* wr = is;  // [N]; isa no longer needed
  double* wi = is + N;
  for (int j = threadIdx.x; j < N; j += blockDim.x) {
    if (j < N / 2) {
      wr[j] = zr[j];
      wi[j] = zi[j];
    } else if (j == N / 2) {
      wr[j] = 0.5 * (zr[Nup - N / 2] + zr[N / 2]);
      wi[j] = 0.5 * (zi[Nup - N / 2] + zi[N / 2]);
    } else {
      wr[j] = zr[Nup - N + j];
      wi[j] = zi[Nup - N + j];
    }
  }
  ves_fft(wr, wi, tre, tim, N, cosU, sinU, +1, Nup / N);
  for (int j = threadIdx.x; j < N; j += blockDim.x) {
    fB[(long long)k * 2 * N + j] = -kappa * (wr[j] / Nup);
    fB[(long long)k * 2 * N + N + j] = -kappa * (wi[j] / Nup);
  }
}

// out = base + filterShape(in, 16) (filter.py:287-311): the kept modes
// |m| <= 16 of z = x + iy are symmetric, so x and y are filtered separately
// with one real circulant.
__global__ void filter_kernel(int N, const double* __restrict__ filt, const double* __restrict__ in,
                              const double* __restrict__ base, double* __restrict__ out) {
  extern __shared__ double sh[];
  double* f = sh;
  double* a = f + N;
  const int k = blockIdx.x;
  for (int i = threadIdx.x; i < N; i += blockDim.x) f[i] = filt[i];
  for (int i = threadIdx.x; i < 2 * N; i += blockDim.x) a[i] = in[(long long)k * 2 * N + i];
  __syncthreads();
  for (int i = threadIdx.x; i < 2 * N; i += blockDim.x) {
    const int comp = i >= N, j = i - comp * N;
    const double v = circ(f, a + comp * N, N, j);
    out[(long long)k * 2 * N + i] = base ? base[(long long)k * 2 * N + i] + v : v;
  }
}

__global__ void axpy_kernel(long long n, const double* __restrict__ a, double alpha, const double* __restrict__ b,
                            double* __restrict__ out) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = a[i] + alpha * b[i];
}

// ---------------------------------------------------------------------------
// referenceValues (:4179-4223) and standardize (:4140-4152), one vesicle per CTA

// LAPACK's 2x2 real Schur standardisation (dlanv2, the published scheme of Bai
// & Demmel) and eigenvectors of the triangular factor, as dgeev returns them
// for a 2x2 matrix with real spectrum (torch.linalg.eig on the host).
__device__ void eig2_lapack(double a, double b, double c, double d, double* w0, double* w1, double* v) {
  double cs, sn, aa, bb, dd;
  if (c == 0.0) {
    cs = 1.0; sn = 0.0; aa = a; bb = b; dd = d;
  } else if (b == 0.0) {
    cs = 0.0; sn = 1.0; aa = d; bb = -c; dd = a;
  } else {
    const double p = 0.5 * (a - d);
    const double bcmax = fmax(fabs(b), fabs(c));
    const double bcmis = fmin(fabs(b), fabs(c)) * copysign(1.0, b) * copysign(1.0, c);
    const double scale = fmax(fabs(p), bcmax);
    double z = (p / scale) * p + (bcmax / scale) * bcmis;
    z = p + copysign(sqrt(scale) * sqrt(z), p);
    aa = d + z;
    dd = d - (bcmax / z) * bcmis;
    const double tau = hypot(c, z);
    cs = z / tau;
    sn = c / tau;
    bb = b - c;
  }
  const double x1 = (aa == dd) ? 0.0 : -bb / (aa - dd);
  double v2x = x1 * cs - sn, v2y = x1 * sn + cs;
  const double nrm = sqrt(v2x * v2x + v2y * v2y);
  v2x /= nrm;
  v2y /= nrm;
  *w0 = aa;
  *w1 = dd;
  v[0] = cs;   // column 0
  v[1] = sn;
  v[2] = v2x;  // column 1
  v[3] = v2y;
}

__device__ void phys_center(int N, const double* d, const double* x, const double* y, double* red, double& cx,
                            double& cy) {
  double a = 0, sx = 0, sy = 0;
  for (int j = threadIdx.x; j < N; j += blockDim.x) {
    const double dx = circ(d, x, N, j), dy = circ(d, y, N, j);
    a += x[j] * dy - y[j] * dx;
    sx += x[j] * x[j] * dy;
    sy += y[j] * y[j] * dx;
  }
  const double A = bsum(a, red);
  cx = bsum(sx, red) / A;
  cy = -bsum(sy, red) / A;
}

__global__ void standardize_kernel(int N, const double* __restrict__ d1, const double* __restrict__ X,
                                   double* __restrict__ Xs, double* __restrict__ scaling, double* __restrict__ rotate,
                                   double* __restrict__ rot_center, double* __restrict__ trans,
                                   int* __restrict__ sort_idx) {
  extern __shared__ double sh[];
  double* d = sh;
  double* x = d + N;
  double* y = x + N;
  double* xr = y + N;
  double* yr = xr + N;
  double* red = yr + N;  // [blockDim]
  __shared__ int s_start;
  const int k = blockIdx.x;
  const double* Xk = X + (long long)k * 2 * N;
  for (int i = threadIdx.x; i < N; i += blockDim.x) {
    d[i] = d1[i];
    x[i] = Xk[i];
    y[i] = Xk[N + i];
  }
  __syncthreads();
  double cx, cy;
  phys_center(N, d, x, y, red, cx, cy);
  // principal axes about the centre (curve_batch_compile.py:279-376)
  for (int i = threadIdx.x; i < N; i += blockDim.x) {
    xr[i] = x[i] - cx;
    yr[i] = y[i] - cy;
  }
  __syncthreads();
  double j11 = 0, j12 = 0, j21 = 0, j22 = 0;
  for (int j = threadIdx.x; j < N; j += blockDim.x) {
    const double dx = circ(d, xr, N, j), dy = circ(d, yr, N, j);
    const double jac = sqrt(dx * dx + dy * dy);
    const double nx = dy / jac, ny = -dx / jac;
    const double xc = xr[j], yc = yr[j];
    const double rdn = xc * nx + yc * ny;
    const double rho2 = xc * xc + yc * yc;
    j11 += rdn * (rho2 - xc * xc) * jac;
    j12 += rdn * (-xc * yc) * jac;
    j21 += rdn * (-yc * xc) * jac;
    j22 += rdn * (rho2 - yc * yc) * jac;
  }
  j11 = bsum(j11, red);
  j12 = bsum(j12, red);
  j21 = bsum(j21, red);
  j22 = bsum(j22, red);
  double w0, w1, V[4];
  eig2_lapack(j11, j12, j21, j22, &w0, &w1, V);
  const int pick = (fabs(w1) < fabs(w0)) ? 1 : 0;  // argmin |w|, first on ties
  const double rot = atan2(V[2 * pick], V[2 * pick + 1]);
  const double ct = cos(rot), st = sin(rot);
  __syncthreads();
  for (int i = threadIdx.x; i < N; i += blockDim.x) {
    const double px = x[i] - cx, py = y[i] - cy;
    xr[i] = px * ct - py * st + cx;
    yr[i] = px * st + py * ct + cy;
  }
  __syncthreads();
  double ccx, ccy;
  phys_center(N, d, xr, yr, red, ccx, ccy);
  const double tx = -ccx, ty = -ccy;
  double ls = 0.0;
  for (int j = threadIdx.x; j < N; j += blockDim.x) {
    const double dx = circ(d, xr, N, j), dy = circ(d, yr, N, j);
    ls += sqrt(dx * dx + dy * dy);
  }
  const double length = bsum(ls, red) * 2.0 * VES_PI / N;
  const double sc = 1.0 / length;
  // first point of the sort order: smallest non-negative polar angle
  if (threadIdx.x == 0) {
    double best = 0;
    int bi = -1;
    for (int j = 0; j < N; ++j) {
      double th = atan2(yr[j] + ty, xr[j] + tx);
      if (th < 0) th = 100.0;
      if (bi < 0 || th < best) {
        best = th;
        bi = j;
      }
    }
    s_start = bi;
  }
  __syncthreads();
  const int start = s_start;
  for (int j = threadIdx.x; j < N; j += blockDim.x) {
    const int src = (start + j) % N;
    sort_idx[(long long)k * N + j] = src;
    Xs[(long long)k * 2 * N + j] = sc * (xr[src] + tx);
    Xs[(long long)k * 2 * N + N + j] = sc * (yr[src] + ty);
  }
  if (threadIdx.x == 0) {
    scaling[k] = sc;
    rotate[k] = rot;
    rot_center[2 * k] = cx;
    rot_center[2 * k + 1] = cy;
    trans[2 * k] = tx;
    trans[2 * k + 1] = ty;
  }
}

// ---------------------------------------------------------------------------
// network inputs (model_zoo/get_network_torch.py pre-processing)

// RelaxNetwork / TenSelfNetwork.preProcess (:37-57, :229-253): (x - m_x)/s_x, (y - m_y)/s_y
template <typename Real>
__global__ void prep_xy_kernel(int nv, int N, const double* __restrict__ Xs, const double* __restrict__ p,
                               Real* __restrict__ out) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (long long)nv * 2 * N) return;
  const int comp = (int)((i / N) & 1);
  out[i] = (Real)((Xs[i] - p[2 * comp]) / p[2 * comp + 1]);
}

// MergedTenAdvNetwork / MergedNearFourierNetwork.preProcess (:337-344, :419-432):
// channel 2k + c of mode k is coordinate c normalised by that mode's statistics.
template <typename Real>
__global__ void prep_modes_kernel(int nv, int N, int modes, const double* __restrict__ Xs,
                                  const double* __restrict__ p, Real* __restrict__ out) {
  // one vesicle per blockIdx.y (strided past the grid), [modes][2][N] along x
  const int per = modes * 2 * N;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= per) return;
  const int j = i % N, c = (i / N) & 1, kk = i / (2 * N);
  const double mean = p[4 * kk + 2 * c], sd = p[4 * kk + 2 * c + 1];
  for (long long v = blockIdx.y; v < nv; v += gridDim.y) {
    const double x = Xs[v * 2 * N + c * N + j];
    Real val;
    if (sizeof(Real) == 8)
      val = (Real)((x - mean) / sd);
    else  // FP32 networks: the quotient in FP32 (within an ulp of the rounded FP64 one)
      val = (Real)((float)(x - mean) / (float)sd);
    out[v * per + i] = val;
  }
}

// MergedAdvNetwork.forward input (:150-190): for mode k (Fourier index k+1),
// channel 2k = [x normalised ++ y normalised] (length 2N), channel 2k+1 =
// [cos((2 pi j / N)(k+1)) / N ++ sin(...) / N]; the statistics of mode 63
// (the Nyquist index) have unit std.  FP64 networks: the reference's FP64
// arithmetic; FP32 networks: the quotient in FP32 and the basis from
// sincospif of the exactly reduced argument 2 ((j (k+1)) mod N) / N.
template <typename Real>
__global__ void prep_adv_kernel(int nv, int N, const double* __restrict__ Xs, const double* __restrict__ p,
                                Real* __restrict__ out) {
  const int L = 2 * N;
  const int per = kModes * 2 * L;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= per) return;
  const int jj = i % L, ch = (i / L) & 1, kk = i / (2 * L);
  const int comp = jj >= N, j = jj - comp * N;
  if (ch == 1) {  // the mode's basis function: the same for every vesicle
    Real val;
    if (sizeof(Real) == 8) {
      const double th = ((double)j / N) * (2.0 * VES_PI);
      const double arg = th * (double)(kk + 1);
      val = (Real)((comp ? sin(arg) : cos(arg)) * (1.0 / N));
    } else {
      const int m = (int)(((long long)j * (kk + 1)) % N);
      float sv, cv;
      sincospif(2.0f * (float)m / (float)N, &sv, &cv);
      val = (Real)((comp ? sv : cv) / (float)N);
    }
    for (long long v = blockIdx.y; v < nv; v += gridDim.y) out[v * per + i] = val;
    return;
  }
  const double mean = p[4 * kk + 2 * comp];
  const double sd = (kk == 63) ? 1.0 : p[4 * kk + 2 * comp + 1];
  for (long long v = blockIdx.y; v < nv; v += gridDim.y) {
    const double x = Xs[v * 2 * N + comp * N + j];
    Real val;
    if (sizeof(Real) == 8)
      val = (Real)((x - mean) / sd);
    else
      val = (Real)((float)(x - mean) / (float)sd);
    out[v * per + i] = val;
  }
}

// ---------------------------------------------------------------------------
// contractions of network outputs with the Fourier coefficients of the
// standardised velocity (rotation by the shape angle about the origin and the
// sort order, no translation or scaling: :1829, :3603, :3653).

// fft of the standardised (vx, vy): V1 + i V2, modes 0..N-1, into shared memory
__device__ void stand_fft(int N, const double* __restrict__ v, double rot, const int* __restrict__ sidx,
                          const double* __restrict__ cs, const double* __restrict__ sn, double* __restrict__ sx,
                          double* __restrict__ sy, double* __restrict__ V1, double* __restrict__ V2) {
  const double ct = cos(rot), st = sin(rot);
  for (int j = threadIdx.x; j < N; j += blockDim.x) {
    const int src = sidx[j];
    const double vx = v[src], vy = v[N + src];
    sx[j] = vx * ct - vy * st;
    sy[j] = vx * st + vy * ct;
  }
  __syncthreads();
  for (int kk = threadIdx.x; kk < N; kk += blockDim.x) {
    double re = 0, im = 0;
    int r = 0;
    for (int j = 0; j < N; ++j) {
      re += sx[j] * cs[r] + sy[j] * sn[r];
      im += sy[j] * cs[r] - sx[j] * sn[r];
      r += kk;
      if (r >= N) r -= N;
    }
    V1[kk] = re;
    V2[kk] = im;
  }
  __syncthreads();
}

// invTenMatOnVback (:3632-3669) + invTenMatOnSelfBend (:3672-3688) + tenNew (:1099)
template <typename Real>
__global__ void tension_kernel(int N, const double* __restrict__ vsum, const double* __restrict__ rotate,
                               const int* __restrict__ sort_idx, const double* __restrict__ scaling,
                               const Real* __restrict__ advten, const Real* __restrict__ selften,
                               const double* __restrict__ q_advten, const double* __restrict__ q_selften,
                               const double* __restrict__ tw, double* __restrict__ ten,
                               double* __restrict__ vback_solve, double* __restrict__ selfbend_solve) {
  extern __shared__ double sh[];
  double* sx = sh;
  double* sy = sx + N;
  double* V1 = sy + N;
  double* V2 = V1 + N;
  __shared__ int sidx[kN];
  const int k = blockIdx.x;
  for (int j = threadIdx.x; j < N; j += blockDim.x) sidx[j] = sort_idx[(long long)k * N + j];
  __syncthreads();
  stand_fft(N, vsum + (long long)k * 2 * N, rotate[k], sidx, tw, tw + N, sx, sy, V1, V2);
  const Real* out = advten + (long long)k * 2 * kModes * N;
  const double sc = scaling[k];
  for (int j = threadIdx.x; j < N; j += blockDim.x) {
    double mv = 0;
    for (int kk = 0; kk < kModes; ++kk) {
      const double z1 = (double)out[(2 * kk) * N + j] * q_advten[4 * kk + 1] + q_advten[4 * kk];
      const double z2 = (double)out[(2 * kk + 1) * N + j] * q_advten[4 * kk + 3] + q_advten[4 * kk + 2];
      mv += z1 * V1[kk + 1] + z2 * V2[kk + 1];
    }
    const double sb = ((double)selften[(long long)k * N + j] * q_selften[1] + q_selften[0]) / (sc * sc);
    const int dst = sidx[j];
    ten[(long long)k * N + dst] = -(mv + sb);
    if (vback_solve) vback_solve[(long long)k * N + dst] = mv;
    if (selfbend_solve) selfbend_solve[(long long)k * N + dst] = sb;
  }
}

// translateVinfwTorch (:3584-3620): Xadv = Xold + dt vinf - dt R(-rot) unsort(M vinf_stand)
template <typename Real>
__global__ void translate_kernel(int N, double dt, const double* __restrict__ Xold, const double* __restrict__ vsum,
                                 const double* __restrict__ rotate, const int* __restrict__ sort_idx,
                                 const Real* __restrict__ adv, const double* __restrict__ q,
                                 const double* __restrict__ tw, double* __restrict__ Xadv) {
  extern __shared__ double sh[];
  double* sx = sh;
  double* sy = sx + N;
  double* V1 = sy + N;
  double* V2 = V1 + N;
  double* mx = V2 + N;
  double* my = mx + N;
  __shared__ int sidx[kN];
  const int k = blockIdx.x;
  for (int j = threadIdx.x; j < N; j += blockDim.x) sidx[j] = sort_idx[(long long)k * N + j];
  __syncthreads();
  const double* vk = vsum + (long long)k * 2 * N;
  stand_fft(N, vk, rotate[k], sidx, tw, tw + N, sx, sy, V1, V2);
  const int L = 2 * N;
  const Real* out = adv + (long long)k * 2 * kModes * L;
  for (int j = threadIdx.x; j < N; j += blockDim.x) {
    double ax = 0, ay = 0;
    for (int kk = 0; kk < kModes; ++kk) {
      if (kk == 63) continue;  // xpred_[63] = 0 (get_network_torch.py:185)
      const Real* re = out + (2 * kk) * L;
      const Real* im = out + (2 * kk + 1) * L;
      const double z11 = (double)re[j] * q[4 * kk + 1] + q[4 * kk];
      const double z21 = (double)re[N + j] * q[4 * kk + 1] + q[4 * kk];
      const double z12 = (double)im[j] * q[4 * kk + 3] + q[4 * kk + 2];
      const double z22 = (double)im[N + j] * q[4 * kk + 3] + q[4 * kk + 2];
      ax += z11 * V1[kk + 1] + z12 * V2[kk + 1];
      ay += z21 * V1[kk + 1] + z22 * V2[kk + 1];
    }
    mx[sidx[j]] = ax;
    my[sidx[j]] = ay;
  }
  __syncthreads();
  const double rot = -rotate[k];
  const double ct = cos(rot), st = sin(rot);
  const double* xo = Xold + (long long)k * 2 * N;
  double* xa = Xadv + (long long)k * 2 * N;
  for (int i = threadIdx.x; i < N; i += blockDim.x) {
    const double rx = mx[i] * ct - my[i] * st;
    const double ry = mx[i] * st + my[i] * ct;
    xa[i] = (xo[i] + dt * vk[i]) - dt * rx;
    xa[N + i] = (xo[N + i] + dt * vk[N + i]) - dt * ry;
  }
}

// First-order conservation of a displacement (dx, dy) of the curve (x, y)
// (shared memory, N points, blockDim a power of two): removes the components
// along n and kappa n that change the enclosed area (d A = int n . d X ds) and
// the length (d L = int kappa n . d X ds), so that a surrogate's displacement
// keeps both to first order, as the exact (incompressible, inextensible)
// dynamics does.  tmp: 3N doubles, red: blockDim doubles.
__device__ void conserve_area_length(int N, const double* __restrict__ d1, const double* x, const double* y,
                                     double* dx, double* dy, double* tmp, double* red) {
  double* xp = tmp;
  double* yp = tmp + N;
  double* kap = tmp + 2 * N;
  for (int j = threadIdx.x; j < N; j += blockDim.x) {
    xp[j] = circ(d1, x, N, j);
    yp[j] = circ(d1, y, N, j);
  }
  __syncthreads();
  double m11 = 0, m12 = 0, m22 = 0, r1 = 0, r2 = 0;
  for (int j = threadIdx.x; j < N; j += blockDim.x) {
    const double xpp = circ(d1, xp, N, j), ypp = circ(d1, yp, N, j);
    const double jac = sqrt(xp[j] * xp[j] + yp[j] * yp[j]);
    const double kp = (xp[j] * ypp - yp[j] * xpp) / (jac * jac * jac);
    const double nx = yp[j] / jac, ny = -xp[j] / jac;
    const double dn = nx * dx[j] + ny * dy[j];
    kap[j] = kp;
    m11 += jac;
    m12 += kp * jac;
    m22 += kp * kp * jac;
    r1 += dn * jac;
    r2 += kp * dn * jac;
  }
  m11 = bsum(m11, red);
  m12 = bsum(m12, red);
  m22 = bsum(m22, red);
  r1 = bsum(r1, red);
  r2 = bsum(r2, red);
  const double det = m11 * m22 - m12 * m12;
  double a, b;
  if (det > 1e-12 * m11 * m22) {  // area and length variations independent (not a circle)
    a = (m22 * r1 - m12 * r2) / det;
    b = (m11 * r2 - m12 * r1) / det;
  } else {
    a = r1 / m11;
    b = 0.0;
  }
  for (int j = threadIdx.x; j < N; j += blockDim.x) {
    const double jac = sqrt(xp[j] * xp[j] + yp[j] * yp[j]);
    const double nx = yp[j] / jac, ny = -xp[j] / jac;
    const double c = a + b * kap[j];
    dx[j] -= c * nx;
    dy[j] -= c * ny;
  }
  __syncthreads();
}

// advection displacement Xa - X made first-order area- and length-preserving (in place)
__global__ void conserve_kernel(int N, const double* __restrict__ d1, const double* __restrict__ X,
                                double* __restrict__ Xa) {
  __shared__ double x[kN], y[kN], dx[kN], dy[kN], tmp[3 * kN], red[128];
  const int k = blockIdx.x;
  const long long o = (long long)k * 2 * N;
  for (int j = threadIdx.x; j < N; j += blockDim.x) {
    x[j] = X[o + j];
    y[j] = X[o + N + j];
    dx[j] = Xa[o + j] - x[j];
    dy[j] = Xa[o + N + j] - y[j];
  }
  __syncthreads();
  conserve_area_length(N, d1, x, y, dx, dy, tmp, red);
  for (int j = threadIdx.x; j < N; j += blockDim.x) {
    Xa[o + j] = x[j] + dx[j];
    Xa[o + N + j] = y[j] + dy[j];
  }
}

// RelaxNetwork.forward post-processing (:59-80) and destandardize (:4154-4177);
// d1 non-null: the displacement is first made area- and length-preserving to
// first order in the standardised frame (destandardize is a similarity)
template <typename Real>
__global__ void relax_post_kernel(int N, double dt, const double* __restrict__ Xin, const Real* __restrict__ pred,
                                  const double* __restrict__ q, const double* __restrict__ scaling,
                                  const double* __restrict__ rotate, const double* __restrict__ rot_center,
                                  const double* __restrict__ trans, const int* __restrict__ sort_idx,
                                  double* __restrict__ Xout, const double* __restrict__ d1) {
  __shared__ double ux[kN], uy[kN];
  const int k = blockIdx.x;
  const double sc = scaling[k];
  if (d1) {
    __shared__ double x[kN], y[kN], dx[kN], dy[kN], tmp[3 * kN], red[128];
    const long long o = (long long)k * 2 * N;
    for (int j = threadIdx.x; j < N; j += blockDim.x) {
      x[j] = Xin[o + j];
      y[j] = Xin[o + N + j];
      dx[j] = ((double)pred[o + j] * q[1] + q[0]) / 1e-5 * dt;
      dy[j] = ((double)pred[o + N + j] * q[3] + q[2]) / 1e-5 * dt;
    }
    __syncthreads();
    conserve_area_length(N, d1, x, y, dx, dy, tmp, red);
    for (int j = threadIdx.x; j < N; j += blockDim.x) {
      const int dst = sort_idx[(long long)k * N + j];
      ux[dst] = (x[j] + dx[j]) / sc;
      uy[dst] = (y[j] + dy[j]) / sc;
    }
  } else {
    for (int j = threadIdx.x; j < N; j += blockDim.x) {
      const long long o = (long long)k * 2 * N;
      const double dxs = ((double)pred[o + j] * q[1] + q[0]) / 1e-5 * dt;
      const double dys = ((double)pred[o + N + j] * q[3] + q[2]) / 1e-5 * dt;
      const int dst = sort_idx[(long long)k * N + j];
      ux[dst] = (Xin[o + j] + dxs) / sc;
      uy[dst] = (Xin[o + N + j] + dys) / sc;
    }
  }
  __syncthreads();
  const double cx = rot_center[2 * k], cy = rot_center[2 * k + 1];
  const double tx = trans[2 * k], ty = trans[2 * k + 1];
  const double rot = -rotate[k];
  const double ct = cos(rot), st = sin(rot);
  for (int i = threadIdx.x; i < N; i += blockDim.x) {
    const double px = (ux[i] + -tx) - cx, py = (uy[i] + -ty) - cy;
    Xout[(long long)k * 2 * N + i] = px * ct - py * st + cx;
    Xout[(long long)k * 2 * N + N + i] = px * st + py * ct + cy;
  }
}

// judge: vesicles whose area or length moved by more than tol (relative) in
// the surrogate step are listed for the BIEM fallback
__global__ void judge_kernel(int nv, double tol, const double* __restrict__ a0, const double* __restrict__ l0,
                             const double* __restrict__ a1, const double* __restrict__ l1, int* __restrict__ idx,
                             int* __restrict__ count) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= nv) return;
  const double ea = fabs(a1[k] - a0[k]) / fabs(a0[k]), el = fabs(l1[k] - l0[k]) / fabs(l0[k]);
  if (!(ea <= tol && el <= tol)) idx[atomicAdd(count, 1)] = k;  // NaN counts as a failure
}

__global__ void fb_gather_kernel(int cnt, int N, const int* __restrict__ idx, const double* __restrict__ X,
                                 const double* __restrict__ v, double* __restrict__ Xg, double* __restrict__ vg) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (long long)cnt * 2 * N) return;
  const long long j = i / (2 * N);
  const long long src = (long long)idx[j] * 2 * N + i % (2 * N);
  Xg[i] = X[src];
  vg[i] = v[src];
}

__global__ void fb_scatter_kernel(int cnt, int N, const int* __restrict__ idx, const double* __restrict__ Xg,
                                  const double* __restrict__ dx, double* __restrict__ Xout) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (long long)cnt * 2 * N) return;
  const long long j = i / (2 * N);
  Xout[(long long)idx[j] * 2 * N + i % (2 * N)] = Xg[i] + dx[i];
}

__global__ void count_excl_kernel(long long nwords, const uint32_t* __restrict__ mask, const int* __restrict__ cand_count,
                                  int maxc, int nwords_N, int* __restrict__ total) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  int c = 0;
  if (i < nwords) {
    const long long per_v = (long long)maxc * nwords_N;
    const long long v = i / per_v;
    const int slot = (int)((i % per_v) / nwords_N);
    if (slot < cand_count[v]) c = __popc(mask[i]);
  }
  for (int o = 16; o > 0; o >>= 1) c += __shfl_down_sync(0xffffffffu, c, o);
  if ((threadIdx.x & 31) == 0 && c) atomicAdd(total, c);
}

__global__ void iota_kernel(int n, int* __restrict__ out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = i;
}

}  // namespace

struct ves_mlarm {
  ves_ctx* ctx = nullptr;
  const ves_net *relax = nullptr, *adv = nullptr, *near = nullptr, *selften = nullptr, *advten = nullptr;
  int precision = VES_NET_FP32;
  double* d_const = nullptr;  // norms, filter circulant, twiddles
  double *adv_in, *adv_out, *relax_in, *relax_out, *near_in, *near_out, *selften_in, *selften_out, *advten_in,
      *advten_out, *filt, *tw;
};

namespace {

int check_net(const ves_net* n, const char* name, int groups, int length, int cin, int cout, int* prec) {
  int g, L, ci, co;
  const int p = net_dims(n, &g, &L, &ci, &co);
  if (g != groups || L != length || ci != cin || co != cout) {
    ves_record_error(VES_ERR_ARG, "mlarm_create: %s network is %d groups, L %d, %d -> %d channels; expected %d, %d, "
                     "%d -> %d", name, g, L, ci, co, groups, length, cin, cout);
    return VES_ERR_ARG;
  }
  if (*prec < 0) *prec = p;
  if (p != *prec) {
    ves_record_error(VES_ERR_ARG, "mlarm_create: the networks must share one precision");
    return VES_ERR_ARG;
  }
  return VES_OK;
}

int standardize_run(ves_ctx* c, int nv, const double* X, double* Xs, double* scaling, double* rotate,
                    double* rot_center, double* trans, int* sort_idx, WsCarver& ws, cudaStream_t s) {
  const int N = c->N;
  double* R = ws.take<double>((size_t)nv * 2 * N);
  int* flags = ws.take<int>((size_t)nv);
  size_t need = 0;
  {
    WsCarver w(nullptr, 0);
    post_redistribute(c, nv, nullptr, nullptr, nullptr, w, s);
    need = w.off + 256;
  }
  char* rs = ws.take<char>(need);
  if (ws.sizing) return VES_OK;
  if (!ws.ok()) {
    ves_record_error(VES_ERR_WORKSPACE, "standardize: workspace too small");
    return VES_ERR_WORKSPACE;
  }
  if (nv <= 0) return VES_OK;
  int rc = ves_cuda_status(cudaMemcpyAsync(R, X, (size_t)nv * 2 * N * sizeof(double), cudaMemcpyDeviceToDevice, s),
                           "standardize copy");
  if (rc) return rc;
  // five passes without an early exit (:4125-4128)
  for (int p = 0; p < 5; ++p) {
    WsCarver w2(rs, need);
    if ((rc = post_redistribute(c, nv, R, R, flags, w2, s))) return rc;
  }
  const int threads = 128;
  ves_count_launch();
  standardize_kernel<<<nv, threads, (size_t)(5 * N + threads) * sizeof(double), s>>>(N, c->d1N, R, Xs, scaling,
                                                                                      rotate, rot_center, trans,
                                                                                      sort_idx);
  return ves_launch_check("standardize");
}

template <typename Real>
struct NetBufs {
  Real *in, *out;
};

size_t elem_of(int precision) { return precision == VES_NET_FP64 ? 8 : 4; }

template <typename Real>
int mlarm_step_t(ves_mlarm* m, const ves_mlarm_params* prm, int nv, const double* X, const double* ten,
                 const double* vback_in, const double* area0, const double* len0, double* Xout, double* ten_out,
                 ves_mlarm_result* res, const ves_mlarm_trace* tr, WsCarver& ws, cudaStream_t s) {
  ves_ctx* c = m->ctx;
  const int N = c->N, Nup = c->Nup;
  const size_t n2 = (size_t)nv * 2 * N;
  const int maxc = prm->maxc > 0 ? prm->maxc : 64;
  // geometry and glue buffers
  double* vback = ws.take<double>(n2);
  double* sa = ws.take<double>((size_t)nv * N);
  double* isa = ws.take<double>((size_t)nv * N);
  double* tang = ws.take<double>(n2);
  double* Xup = ws.take<double>((size_t)nv * 2 * Nup);
  double* sa_up = ws.take<double>((size_t)nv * Nup);
  double* fB = ws.take<double>(n2);
  double* fT = ws.take<double>(n2);
  double* trac = ws.take<double>(n2);
  double* far = ws.take<double>(n2);
  double* vsum = ws.take<double>(n2);
  double* tnew = ws.take<double>((size_t)nv * N);
  double* Xs = ws.take<double>(n2);
  double* sv = ws.take<double>((size_t)nv * 6);  // scaling, rotate, rot_center[2], trans[2]
  int* sidx = ws.take<int>((size_t)nv * N);
  double* Xs2 = ws.take<double>(n2);
  double* sv2 = ws.take<double>((size_t)nv * 6);
  int* sidx2 = ws.take<int>((size_t)nv * N);
  double* Xa = ws.take<double>(n2);
  double* Xb = ws.take<double>(n2);
  double* Xc = ws.take<double>(n2);
  int* flags = ws.take<int>((size_t)nv);
  int* counter = ws.take<int>(1);
  double* fup = ws.take<double>((size_t)nv * 2 * Nup);
  double* den = ws.take<double>((size_t)nv * 2 * Nup);
  int* selfidx = ws.take<int>((size_t)nv);
  // judge and fallback (judge_tol > 0): areas and lengths before and after the
  // surrogate step, the listed vesicles, and chunks of their isolated BIEM step
  const bool judge = prm->judge_tol > 0.0;
  const int kFb = std::max(1, std::min(nv, 512));
  double* jgeo = judge ? ws.take<double>((size_t)4 * nv) : nullptr;
  int* fb_idx = judge ? ws.take<int>((size_t)nv + 1) : nullptr;
  double* fbX = judge ? ws.take<double>((size_t)kFb * 2 * N) : nullptr;
  double* fbV = judge ? ws.take<double>((size_t)kFb * 2 * N) : nullptr;
  double* fbD = judge ? ws.take<double>((size_t)kFb * 2 * N) : nullptr;
  ves_near_lists nl;
  memset(&nl, 0, sizeof(nl));
  nl.maxc = maxc;
  nl.cand_count = ws.take<int>((size_t)nv);
  nl.cand_src = ws.take<int>((size_t)nv * maxc);
  nl.excl_mask = ws.take<uint32_t>((size_t)nv * maxc * c->nwords_N);
  nl.hh_mask = ws.take<uint32_t>((size_t)nv * maxc * c->nwords_up);
  // network buffers (one input and one output region shared by the nets)
  const size_t net_in = std::max({(size_t)nv * 2 * N, (size_t)nv * kModes * 2 * 2 * N, (size_t)nv * kNearModes * 2 * N});
  const size_t net_out = std::max({(size_t)nv * kModes * 2 * 2 * N, (size_t)nv * kNearModes * 12 * N});
  Real* nin = ws.take<Real>(net_in);
  Real* nout = ws.take<Real>(net_out);
  Real* nout2 = ws.take<Real>((size_t)nv * N);  // self-tension network output
  // scratch shared by the sub-stages
  size_t scratch = 0;
  {
    const ves_net* nets[5] = {m->relax, m->adv, m->near, m->selften, m->advten};
    for (const ves_net* n : nets) {
      if (!n) continue;
      WsCarver w(nullptr, 0);
      net_forward_run(n, nv, nullptr, nullptr, w, nullptr, s);
      scratch = std::max(scratch, w.off);
    }
    WsCarver w(nullptr, 0);
    near_zone_py(c, nv, nullptr, (const double*)1, 0, nullptr, w, s);
    scratch = std::max(scratch, w.off);
    WsCarver w2(nullptr, 0);
    farfield_run(c, prm->farfield_precision, nv, Nup, nullptr, nullptr, nv, N, nullptr, nullptr, &nl, nullptr, w2, s);
    scratch = std::max(scratch, w2.off);
    WsCarver w3(nullptr, 0);
    standardize_run(c, nv, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, w3, s);
    scratch = std::max(scratch, w3.off);
    WsCarver w4(nullptr, 0);
    post_correct_area_length(c, nv, nullptr, nullptr, nullptr, nullptr, nullptr, w4, s);
    scratch = std::max(scratch, w4.off);
    WsCarver w5(nullptr, 0);
    post_redistribute(c, nv, nullptr, nullptr, nullptr, w5, s);
    scratch = std::max(scratch, w5.off);
    if (judge) {
      WsCarver w6(nullptr, 0);
      isolated_step_run(c, kFb, nullptr, nullptr, prm->dt, prm->kappa, VES_PREC_FP32C, nullptr, w6, s);
      scratch = std::max(scratch, w6.off);
    }
  }
  char* scr = ws.take<char>(scratch + 1024);
  const size_t scr_bytes = scratch + 1024;
  if (ws.sizing) return VES_OK;
  if (!ws.ok()) {
    ves_record_error(VES_ERR_WORKSPACE, "mlarm_step: workspace too small (%zu needed)", ws.off);
    return VES_ERR_WORKSPACE;
  }
  if (nv <= 0) return VES_OK;
  int rc = ves_reset_status(c, s);
  if (rc) return rc;
  const long long nn2 = (long long)n2;
  double *scal = sv, *rot = sv + nv, *rotc = sv + 2 * nv, *trn = sv + 4 * nv;
  double *scal2 = sv2, *rot2 = sv2 + nv, *rotc2 = sv2 + 2 * nv, *trn2 = sv2 + 4 * nv;
  auto sub = [&]() { return WsCarver(scr, scr_bytes); };

  // vinf(Xold), capsules(Xold), capsules(upsample_fft(Xold, Nup))  (:988-1000)
  if (vback_in) {
    rc = ves_cuda_status(cudaMemcpyAsync(vback, vback_in, n2 * sizeof(double), cudaMemcpyDeviceToDevice, s), "vback");
    if (rc) return rc;
  } else {
    launch_bg_flow(nv, N, prm->flow, prm->speed, prm->chan_width, prm->vortex_size, X, vback, s);
  }
  launch_diff_prop(c, 0, nv, X, sa, isa, tang, nullptr, s);
  launch_upsample_deriv(c, nv, X, Xup, nullptr, sa_up, s);
  // fTen = tensionTerm(tenOld); fBend = downsample(bendingTerm on Nup)  (:1007-1013)
  launch_trac_jump(c, nv, 0.0, isa, tang, X, 2LL * N, ten, N, fT, s);
  {
    const size_t sh = (size_t)(5 * Nup + 2 * N) * sizeof(double);
    if (sh > 48 * 1024) {
      rc = ves_cuda_status(cudaFuncSetAttribute(bend_up_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sh),
                           "bend smem");
      if (rc) return rc;
    }
    ves_count_launch();
    bend_up_kernel<<<nv, 256, sh, s>>>(N, Nup, c->m, c->pc, c->pcd, c->cosU, c->sinU, prm->kappa, X, fB);
  }
  const unsigned gb = ceil_div(nn2, 256);
  ves_count_launch();
  axpy_kernel<<<gb, 256, 0, s>>>(nn2, fB, 1.0, fT, trac);
  // standardizationStep(Xold)  (:1019, :4119-4138)
  {
    WsCarver w = sub();
    if ((rc = standardize_run(c, nv, X, Xs, scal, rot, rotc, trn, sidx, w, s))) return rc;
  }
  // near network (predictNearLayers :1726-1812) on request
  if (prm->eval_near_net && m->near) {
    ves_count_launch();
    prep_modes_kernel<Real><<<dim3(ceil_div(kNearModes * 2 * N, 256), std::min(nv, 65535)), 256, 0, s>>>(
        nv, N, kNearModes, Xs, m->near_in, nin);
    WsCarver w = sub();
    ves_net_timing_begin(c, s);
    if ((rc = net_forward_run(m->near, nv, nin, nout, w, c->status, s))) return rc;
    ves_net_timing_end(c, s, net_flops_per_vesicle(m->near) * nv);
  }
  // near pairs (compare1 :429-536): target points of a vesicle closer than 1/N
  // to an upsampled point of another vesicle
  {
    WsCarver w = sub();
    if ((rc = near_zone_py(c, nv, X, Xup, 0.0, &nl, w, s))) return rc;
  }
  ves_count_launch();
  iota_kernel<<<ceil_div(nv, 256), 256, 0, s>>>(nv, selfidx);
  auto far_field = [&](const double* f, double* out) -> int {
    launch_upsample(c, nv, 2, f, 2LL * N, fup, s);
    launch_density(nv, Nup, fup, sa_up, den, s);
    if (nv == 1) return ves_cuda_status(cudaMemsetAsync(out, 0, n2 * sizeof(double), s), "far zero");
    WsCarver w = sub();
    return farfield_run(c, prm->farfield_precision, nv, Nup, Xup, den, nv, N, X, selfidx, &nl, out, w, s);
  };
  const size_t shf = (size_t)3 * N * sizeof(double);
  // first far field, filtered, plus vinf  (:1076-1096)
  if ((rc = far_field(trac, far))) return rc;
  if (tr && tr->far1) cudaMemcpyAsync(tr->far1, far, n2 * sizeof(double), cudaMemcpyDeviceToDevice, s);
  ves_count_launch();
  filter_kernel<<<nv, 128, shf, s>>>(N, m->filt, far, vback, vsum);
  // tension solves (:1099-1113)
  ves_count_launch();
  prep_modes_kernel<Real><<<dim3(ceil_div(kModes * 2 * N, 256), std::min(nv, 65535)), 256, 0, s>>>(
      nv, N, kModes, Xs, m->advten_in, nin);
  {
    WsCarver w = sub();
    ves_net_timing_begin(c, s);
    if ((rc = net_forward_run(m->advten, nv, nin, nout, w, c->status, s))) return rc;
    ves_net_timing_end(c, s, net_flops_per_vesicle(m->advten) * nv);
  }
  ves_count_launch();
  prep_xy_kernel<Real><<<gb, 256, 0, s>>>(nv, N, Xs, m->selften_in, nin);
  {
    WsCarver w = sub();
    ves_net_timing_begin(c, s);
    if ((rc = net_forward_run(m->selften, nv, nin, nout2, w, c->status, s))) return rc;
    ves_net_timing_end(c, s, net_flops_per_vesicle(m->selften) * nv);
  }
  ves_count_launch();
  tension_kernel<Real><<<nv, 128, (size_t)4 * N * sizeof(double), s>>>(
      N, vsum, rot, sidx, scal, nout, nout2, m->advten_out, m->selften_out, m->tw, tnew,
      tr ? tr->vback_solve : nullptr, tr ? tr->selfbend_solve : nullptr);
  // tracJump with the new tension, second far field (:1117-1130)
  launch_trac_jump(c, nv, 0.0, isa, tang, X, 2LL * N, tnew, N, fT, s);
  ves_count_launch();
  axpy_kernel<<<gb, 256, 0, s>>>(nn2, fB, 1.0, fT, trac);
  if ((rc = far_field(trac, far))) return rc;
  if (tr && tr->far2) cudaMemcpyAsync(tr->far2, far, n2 * sizeof(double), cudaMemcpyDeviceToDevice, s);
  ves_count_launch();
  filter_kernel<<<nv, 128, shf, s>>>(N, m->filt, far, vback, vsum);
  // advection (:1150-1160)
  ves_count_launch();
  prep_adv_kernel<Real><<<dim3(ceil_div(kModes * 2 * 2 * N, 256), std::min(nv, 65535)), 256, 0, s>>>(nv, N, Xs,
                                                                                                  m->adv_in, nin);
  {
    WsCarver w = sub();
    ves_net_timing_begin(c, s);
    if ((rc = net_forward_run(m->adv, nv, nin, nout, w, c->status, s))) return rc;
    ves_net_timing_end(c, s, net_flops_per_vesicle(m->adv) * nv);
  }
  ves_count_launch();
  translate_kernel<Real><<<nv, 128, (size_t)6 * N * sizeof(double), s>>>(N, prm->dt, X, vsum, rot, sidx, nout,
                                                                          m->adv_out, m->tw, Xa);
  if (prm->conserve) {
    ves_count_launch();
    conserve_kernel<<<nv, 128, 0, s>>>(N, c->d1N, X, Xa);
  }
  if (tr && tr->Xadv) cudaMemcpyAsync(tr->Xadv, Xa, n2 * sizeof(double), cudaMemcpyDeviceToDevice, s);
  ves_count_launch();
  filter_kernel<<<nv, 128, shf, s>>>(N, m->filt, Xa, nullptr, Xb);
  // relaxation (:1163, :3622-3629)
  {
    WsCarver w = sub();
    if ((rc = standardize_run(c, nv, Xb, Xs2, scal2, rot2, rotc2, trn2, sidx2, w, s))) return rc;
  }
  ves_count_launch();
  prep_xy_kernel<Real><<<gb, 256, 0, s>>>(nv, N, Xs2, m->relax_in, nin);
  {
    WsCarver w = sub();
    ves_net_timing_begin(c, s);
    if ((rc = net_forward_run(m->relax, nv, nin, nout, w, c->status, s))) return rc;
    ves_net_timing_end(c, s, net_flops_per_vesicle(m->relax) * nv);
  }
  ves_count_launch();
  relax_post_kernel<Real><<<nv, 128, 0, s>>>(N, prm->dt, Xs2, nout, m->relax_out, scal2, rot2, rotc2, trn2, sidx2, Xa,
                                             prm->conserve ? c->d1N : nullptr);
  // the plain BIEM step as judge and fallback of the surrogate: vesicles whose
  // area or length the surrogate moved by more than judge_tol take the implicit
  // step of the isolated vesicle with the same explicit velocity vsum
  int nfb = 0;
  if (judge) {
    launch_geom_prop(c, nv, X, nullptr, jgeo, jgeo + nv, s);
    launch_geom_prop(c, nv, Xa, nullptr, jgeo + 2 * nv, jgeo + 3 * nv, s);
    rc = ves_cuda_status(cudaMemsetAsync(fb_idx + nv, 0, sizeof(int), s), "judge count");
    if (rc) return rc;
    ves_count_launch();
    judge_kernel<<<ceil_div(nv, 256), 256, 0, s>>>(nv, prm->judge_tol, jgeo, jgeo + nv, jgeo + 2 * nv, jgeo + 3 * nv,
                                                   fb_idx, fb_idx + nv);
    rc = ves_cuda_status(cudaMemcpyAsync(c->h_ints + 1, fb_idx + nv, sizeof(int), cudaMemcpyDeviceToHost, s),
                         "judge count read");
    if (!rc) rc = ves_cuda_status(cudaStreamSynchronize(s), "judge sync");
    if (rc) return rc;
    nfb = c->h_ints[1];
    for (int a = 0; a < nfb; a += kFb) {
      const int cnt = std::min(kFb, nfb - a);
      const long long ne = (long long)cnt * 2 * N;
      ves_count_launch();
      fb_gather_kernel<<<ceil_div(ne, 256), 256, 0, s>>>(cnt, N, fb_idx + a, X, vsum, fbX, fbV);
      WsCarver w = sub();
      if ((rc = isolated_step_run(c, cnt, fbX, fbV, prm->dt, prm->kappa, VES_PREC_FP32C, fbD, w, s))) return rc;
      ves_count_launch();
      fb_scatter_kernel<<<ceil_div(ne, 256), 256, 0, s>>>(cnt, N, fb_idx + a, fbX, fbD, Xa);
    }
  }
  if (tr && tr->Xrelax) cudaMemcpyAsync(tr->Xrelax, Xa, n2 * sizeof(double), cudaMemcpyDeviceToDevice, s);
  // up to five redistribution passes (stopping once nothing moves is the
  // same as running all five), alignment, area/length correction, filter (:1165-1198)
  rc = ves_cuda_status(cudaMemcpyAsync(Xb, Xa, n2 * sizeof(double), cudaMemcpyDeviceToDevice, s), "copy");
  if (rc) return rc;
  for (int p = 0; p < 5; ++p) {
    WsCarver w = sub();
    if ((rc = post_redistribute(c, nv, Xb, Xb, flags, w, s))) return rc;
  }
  launch_align_center_angle(c, nv, Xa, Xb, Xc, nullptr, nullptr, s);
  if (tr && tr->Xalign) cudaMemcpyAsync(tr->Xalign, Xc, n2 * sizeof(double), cudaMemcpyDeviceToDevice, s);
  int iters = 0;
  {
    WsCarver w = sub();
    if ((rc = post_correct_area_length(c, nv, Xc, area0, len0, Xb, &iters, w, s, prm->area_len_tol))) return rc;
  }
  if (tr && tr->Xcorr) cudaMemcpyAsync(tr->Xcorr, Xb, n2 * sizeof(double), cudaMemcpyDeviceToDevice, s);
  ves_count_launch();
  filter_kernel<<<nv, 128, shf, s>>>(N, m->filt, Xb, nullptr, Xout);
  rc = ves_cuda_status(cudaMemcpyAsync(ten_out, tnew, (size_t)nv * N * sizeof(double), cudaMemcpyDeviceToDevice, s),
                       "ten out");
  if (rc) return rc;
  if (tr) {
    if (tr->Xstand) cudaMemcpyAsync(tr->Xstand, Xs, n2 * sizeof(double), cudaMemcpyDeviceToDevice, s);
    if (tr->scaling) cudaMemcpyAsync(tr->scaling, scal, nv * sizeof(double), cudaMemcpyDeviceToDevice, s);
    if (tr->rotate) cudaMemcpyAsync(tr->rotate, rot, nv * sizeof(double), cudaMemcpyDeviceToDevice, s);
    if (tr->rot_center) cudaMemcpyAsync(tr->rot_center, rotc, 2 * nv * sizeof(double), cudaMemcpyDeviceToDevice, s);
    if (tr->trans) cudaMemcpyAsync(tr->trans, trn, 2 * nv * sizeof(double), cudaMemcpyDeviceToDevice, s);
    if (tr->sort_idx) cudaMemcpyAsync(tr->sort_idx, sidx, (size_t)nv * N * sizeof(int), cudaMemcpyDeviceToDevice, s);
  }
  // excluded pair count for the result record
  rc = ves_cuda_status(cudaMemsetAsync(counter, 0, sizeof(int), s), "count");
  if (rc) return rc;
  {
    const long long nw = (long long)nv * maxc * c->nwords_N;
    ves_count_launch();
    count_excl_kernel<<<ceil_div(nw, 256), 256, 0, s>>>(nw, nl.excl_mask, nl.cand_count, maxc, c->nwords_N, counter);
  }
  int npairs = 0;
  rc = ves_cuda_status(cudaMemcpyAsync(&npairs, counter, sizeof(int), cudaMemcpyDeviceToHost, s), "count read");
  if (rc) return rc;
  rc = ves_check_status(c, s, "mlarm_step");
  if (res) {
    res->n_near_pairs = npairs;
    res->auglag_iters = iters;
    res->n_fallback = nfb;
  }
  return rc;
}

}  // namespace

// fBend of the step (bending of the Nup-upsampled shape, truncated to N modes)
// for callers outside the step (the training targets of ves_targets.cu)
int launch_bend_up(ves_ctx* c, int nv, const double* X, double kappa, double* fB, cudaStream_t s) {
  const int N = c->N, Nup = c->Nup;
  const size_t sh = (size_t)(5 * Nup + 2 * N) * sizeof(double);
  if (sh > 48 * 1024) {
    int rc = ves_cuda_status(cudaFuncSetAttribute(bend_up_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sh),
                             "bend smem");
    if (rc) return rc;
  }
  if (nv <= 0) return VES_OK;
  ves_count_launch();
  bend_up_kernel<<<nv, 256, sh, s>>>(N, Nup, c->m, c->pc, c->pcd, c->cosU, c->sinU, kappa, X, fB);
  return ves_launch_check("bend_up");
}

namespace {

int mlarm_step_run(ves_mlarm* m, const ves_mlarm_params* prm, int nv, const double* X, const double* ten,
                   const double* vback, const double* area0, const double* len0, double* Xout, double* ten_out,
                   ves_mlarm_result* res, const ves_mlarm_trace* tr, WsCarver& ws, cudaStream_t s) {
  if (m->precision == VES_NET_FP64)
    return mlarm_step_t<double>(m, prm, nv, X, ten, vback, area0, len0, Xout, ten_out, res, tr, ws, s);
  return mlarm_step_t<float>(m, prm, nv, X, ten, vback, area0, len0, Xout, ten_out, res, tr, ws, s);
}

}  // namespace

extern "C" int ves_mlarm_create(ves_ctx* ctx, const ves_net* relax, const ves_net* adv, const ves_net* near,
                                const ves_net* selften, const ves_net* advten, const ves_mlarm_norms* nr,
                                ves_mlarm** out) {
  if (!ctx || !relax || !adv || !selften || !advten || !nr || !out) {
    ves_record_error(VES_ERR_ARG, "mlarm_create: bad arguments");
    return VES_ERR_ARG;
  }
  *out = nullptr;
  if (ctx->N != kN || !ves_fft_size_ok(ctx->Nup)) {
    ves_record_error(VES_ERR_SHAPE, "mlarm_create: the networks are built for N = %d, context has N = %d", kN,
                     ctx->N);
    return VES_ERR_SHAPE;
  }
  const double* parts[10] = {nr->adv_in, nr->adv_out, nr->relax_in, nr->relax_out, nr->near_in,
                             nr->near_out, nr->selften_in, nr->selften_out, nr->advten_in, nr->advten_out};
  const int sizes[10] = {127 * 4, 127 * 4, 4, 4, 128 * 4, 128 * 24, 4, 2, 127 * 4, 127 * 4};
  for (int i = 0; i < 10; ++i)
    if (!parts[i] && !(i >= 4 && i <= 5 && !near)) {
      ves_record_error(VES_ERR_ARG, "mlarm_create: normalisation array %d missing", i);
      return VES_ERR_ARG;
    }
  int prec = -1, rc;
  if ((rc = check_net(relax, "relax", 1, 128, 2, 2, &prec))) return rc;
  if ((rc = check_net(adv, "adv", 127, 256, 2, 2, &prec))) return rc;
  if (near && (rc = check_net(near, "near", 128, 128, 2, 12, &prec))) return rc;
  if ((rc = check_net(selften, "selften", 1, 128, 2, 1, &prec))) return rc;
  if ((rc = check_net(advten, "advten", 127, 128, 2, 2, &prec))) return rc;
  ves_mlarm* m = new (std::nothrow) ves_mlarm;
  if (!m) {
    ves_record_error(VES_ERR_CUDA, "mlarm_create: out of host memory");
    return VES_ERR_CUDA;
  }
  m->ctx = ctx;
  m->relax = relax;
  m->adv = adv;
  m->near = near;
  m->selften = selften;
  m->advten = advten;
  m->precision = prec;
  const int N = kN;
  std::vector<double> h;
  std::vector<size_t> off;
  for (int i = 0; i < 10; ++i) {
    off.push_back(h.size());
    for (int j = 0; j < sizes[i]; ++j) h.push_back(parts[i] ? parts[i][j] : 0.0);
  }
  // filterShape(., 16) circulant: (1/N)(1 + 2 sum_{m=1}^{16} cos(2 pi m r / N))
  off.push_back(h.size());
  for (int r = 0; r < N; ++r) {
    double v = 1.0;
    for (int mm = 1; mm <= 16; ++mm) v += 2.0 * cos(2.0 * VES_PI * (double)((mm * r) % N) / N);
    h.push_back(v / N);
  }
  off.push_back(h.size());
  for (int r = 0; r < N; ++r) h.push_back(cos(2.0 * VES_PI * r / N));
  for (int r = 0; r < N; ++r) h.push_back(sin(2.0 * VES_PI * r / N));
  rc = ves_cuda_status(cudaMalloc(&m->d_const, h.size() * sizeof(double)), "mlarm constants");
  if (!rc)
    rc = ves_cuda_status(cudaMemcpy(m->d_const, h.data(), h.size() * sizeof(double), cudaMemcpyHostToDevice),
                         "mlarm constants upload");
  if (rc) {
    if (m->d_const) cudaFree(m->d_const);
    delete m;
    return rc;
  }
  double* b = m->d_const;
  m->adv_in = b + off[0];
  m->adv_out = b + off[1];
  m->relax_in = b + off[2];
  m->relax_out = b + off[3];
  m->near_in = b + off[4];
  m->near_out = b + off[5];
  m->selften_in = b + off[6];
  m->selften_out = b + off[7];
  m->advten_in = b + off[8];
  m->advten_out = b + off[9];
  m->filt = b + off[10];
  m->tw = b + off[11];
  (void)kNormDoubles;
  *out = m;
  return VES_OK;
}

extern "C" int ves_mlarm_destroy(ves_mlarm* m) {
  if (!m) return VES_OK;
  if (m->d_const) cudaFree(m->d_const);
  delete m;
  return VES_OK;
}

extern "C" size_t ves_mlarm_step_workspace(ves_mlarm* m, const ves_mlarm_params* prm, int nv) {
  if (!m || !prm) return 0;
  WsCarver w(nullptr, 0);
  mlarm_step_run(m, prm, nv, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, w, 0);
  return w.off + 256;
}

extern "C" int ves_mlarm_step(ves_mlarm* m, const ves_mlarm_params* prm, int nv, const double* X, const double* ten,
                              const double* vback, const double* area0, const double* len0, double* Xout,
                              double* ten_out, ves_mlarm_result* res, const ves_mlarm_trace* trace, void* ws,
                              size_t ws_bytes, void* stream) {
  if (!m || !prm || !ws || nv < 0 || (nv > 0 && (!X || !ten || !area0 || !len0 || !Xout || !ten_out))) {
    ves_record_error(VES_ERR_ARG, "mlarm_step: bad arguments");
    return VES_ERR_ARG;
  }
  if (prm->farfield_precision != VES_PREC_FP64 && prm->farfield_precision != VES_PREC_FP32C &&
      prm->farfield_precision != VES_PREC_FP32M) {
    ves_record_error(VES_ERR_ARG, "mlarm_step: bad far-field precision");
    return VES_ERR_ARG;
  }
  if (res) memset(res, 0, sizeof(*res));
  WsCarver w(ws, ws_bytes);
  return mlarm_step_run(m, prm, nv, X, ten, vback, area0, len0, Xout, ten_out, res, trace, w, (cudaStream_t)stream);
}

extern "C" size_t ves_mlarm_standardize_workspace(ves_ctx* c, int nv) {
  if (!c) return 0;
  WsCarver w(nullptr, 0);
  standardize_run(c, nv, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, w, 0);
  return w.off + 256;
}

extern "C" int ves_mlarm_standardize(ves_ctx* c, int nv, const double* X, double* Xs, double* scaling,
                                     double* rotate, double* rot_center, double* trans, int* sort_idx, void* ws,
                                     size_t ws_bytes, void* stream) {
  if (!c || !ws || nv < 0 || (nv > 0 && (!X || !Xs || !scaling || !rotate || !rot_center || !trans || !sort_idx))) {
    ves_record_error(VES_ERR_ARG, "mlarm_standardize: bad arguments");
    return VES_ERR_ARG;
  }
  cudaStream_t s = (cudaStream_t)stream;
  int rc = ves_reset_status(c, s);
  if (rc) return rc;
  WsCarver w(ws, ws_bytes);
  rc = standardize_run(c, nv, X, Xs, scaling, rotate, rot_center, trans, sort_idx, w, s);
  if (rc) return rc;
  rc = ves_launch_check("mlarm_standardize");
  if (rc) return rc;
  return ves_check_status(c, s, "mlarm_standardize");
}
