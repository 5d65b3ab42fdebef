// Post-step shape conditioning (FP64), one CTA per vesicle:
//   redistributeArcLength  (curve_batch_compile.py:905-972, 1039-1092)
//   alignCenterAngle       (curve_batch_compile.py:842-901) with
//   getPhysicalCenter      (:84-100) and getIncAngle (:105-194)
//   correctAreaAndLengthAugLag (:590-710): augmented Lagrangian, Adam steps
//   with analytic gradients of area, length and the shape-distance functional.
#include <math.h>

#include <algorithm>
#include <vector>

#include "ves_internal.h"
#include "ves_fft.cuh"

namespace {

__device__ __forceinline__ double circ(const double* __restrict__ d, const double* __restrict__ a, int n, int j) {
  double s = 0.0;
  for (int l = 0; l <= j; ++l) s = fma(d[j - l], a[l], s);
  for (int l = j + 1; l < n; ++l) s = fma(d[j - l + n], a[l], s);
  return s;
}

// deterministic block reductions (blockDim power of two, <= 1024)
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
__device__ double bmax(double v, double* red) {
  red[threadIdx.x] = v;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w) red[threadIdx.x] = fmax(red[threadIdx.x], red[threadIdx.x + w]);
    __syncthreads();
  }
  const double r = red[0];
  __syncthreads();
  return r;
}

int pow2_threads(int n) {
  int t = 32;
  while (t < n && t < 256) t <<= 1;
  return t;
}

// ---------------------------------------------------------------------------
// The redistribution test of curve_batch_compile.py:951-953 compares one
// scalar, the matrix infinity norm of (jac - mean_jac) over the whole (N, nv)
// suspension, with 1e-5 * mean_jac of every vesicle.  Three deterministic
// passes: |jac - mean| per point, partial column sums over chunks of
// vesicles, then the largest row sum.
constexpr int kSpreadChunk = 64;

__global__ void jac_dev_kernel(int N, const double* __restrict__ d1, const double* __restrict__ X,
                               double* __restrict__ dev) {
  extern __shared__ double sh[];
  double* d = sh;
  double* x = d + N;
  double* y = x + N;
  double* jac = y + N;
  double* red = jac + N;
  const int k = blockIdx.x;
  const double* Xk = X + (long long)k * 2 * N;
  for (int i = threadIdx.x; i < N; i += blockDim.x) {
    d[i] = d1[i];
    x[i] = Xk[i];
    y[i] = Xk[N + i];
  }
  __syncthreads();
  double js = 0.0;
  for (int j = threadIdx.x; j < N; j += blockDim.x) {
    const double dx = circ(d, x, N, j), dy = circ(d, y, N, j);
    jac[j] = sqrt(dx * dx + dy * dy);
    js += jac[j];
  }
  const double mean = bsum(js, red) / N;
  for (int j = threadIdx.x; j < N; j += blockDim.x) dev[(long long)k * N + j] = fabs(jac[j] - mean);
}

__global__ void dev_rowsum_kernel(int nv, int N, const double* __restrict__ dev, double* __restrict__ partial) {
  const int b = blockIdx.x;
  const int k0 = b * kSpreadChunk, k1 = min(nv, k0 + kSpreadChunk);
  for (int i = threadIdx.x; i < N; i += blockDim.x) {
    double s = 0.0;
    for (int k = k0; k < k1; ++k) s += dev[(long long)k * N + i];
    partial[(long long)b * N + i] = s;
  }
}

__global__ void spread_kernel(int nchunk, int N, const double* __restrict__ partial, double* __restrict__ spread) {
  __shared__ double red[256];
  double m = 0.0;
  bool nan = false;
  for (int i = threadIdx.x; i < N; i += blockDim.x) {
    double s = 0.0;
    for (int b = 0; b < nchunk; ++b) s += partial[(long long)b * N + i];
    if (s != s) nan = true;
    m = fmax(m, s);
  }
  const int anynan = __syncthreads_or(nan);
  const double r = bmax(m, red);
  if (threadIdx.x == 0) *spread = anynan ? __longlong_as_double(0x7ff8000000000000LL) : r;
}

// one redistributeArcLength pass; flags[k] = 1 if vesicle k was left as is
__global__ void redistribute_kernel(int N, const double* __restrict__ d1, const double* __restrict__ cos6,
                                    const double* __restrict__ sin6, const double* __restrict__ spread_p,
                                    const double* __restrict__ X, double* __restrict__ Xout,
                                    int* __restrict__ flags) {
  extern __shared__ double sh[];
  const int M = 6 * N;  // upsampled grid of the arc-length parameter search
  double* d = sh;
  double* x = d + N;
  double* y = x + N;
  double* are = y + N;     // [M] spectrum work arrays
  double* aim = are + M;   // [M]
  double* tre = aim + M;   // [M] FFT scratch
  double* tim = tre + M;   // [M]
  double* al = tim + M;    // [M]
  double* th = al + M;     // [N]
  double* zr = th + N;     // [N]
  double* zi = zr + N;     // [N]
  double* red = zi + N;    // [blockDim]
  const int k = blockIdx.x;
  const double* Xk = X + (long long)k * 2 * N;
  double* Ok = Xout + (long long)k * 2 * N;
  for (int i = threadIdx.x; i < N; i += blockDim.x) {
    d[i] = d1[i];
    x[i] = Xk[i];
    y[i] = Xk[N + i];
  }
  __syncthreads();
  // jacobian on the N grid: its spread decides, its sum is the length
  double js = 0.0;
  for (int j = threadIdx.x; j < N; j += blockDim.x) {
    const double dx = circ(d, x, N, j), dy = circ(d, y, N, j);
    js += sqrt(dx * dx + dy * dy);
  }
  const double jsum = bsum(js, red);
  const double mean = jsum / N;
  if (!(*spread_p > 1e-5 * mean)) {
    for (int i = threadIdx.x; i < 2 * N; i += blockDim.x) Ok[i] = Xk[i];
    if (threadIdx.x == 0) flags[k] = 1;
    return;
  }
  const double length = jsum * 2.0 * VES_PI / N;
  // zh = fft(x + i y)/N, modes 0..N/2-1, -N/2..-1 (length-N FFT, twiddles
  // from the 6N table); also the coefficients of the final evaluation
  for (int j = threadIdx.x; j < N; j += blockDim.x) {
    zr[j] = x[j];
    zi[j] = y[j];
  }
  ves_fft(zr, zi, tre, tim, N, cos6, sin6, -1, 6);
  for (int m = threadIdx.x; m < N; m += blockDim.x) {
    zr[m] /= N;
    zi[m] /= N;
  }
  __syncthreads();
  // |dX/dt| of the interpolant on the 6N grid: the spectrum i k zh_k placed on
  // the 6N grid and transformed back (the Nyquist mode split in two halves,
  // +-N/2, so that its derivative is that of the real interpolant,
  // -(N/2) c sin(N t / 2)); the same values as the circulant sum of the
  // interpolant's derivative, with O(M log M) instead of O(M N) work
  for (int u = threadIdx.x; u < M; u += blockDim.x) {
    double cr = 0.0, ci = 0.0;
    if (u < N / 2) {  // modes 0 .. N/2-1
      cr = -u * zi[u];
      ci = u * zr[u];
    } else if (u > M - N / 2) {  // modes -(N/2-1) .. -1
      const int k = u - M;
      cr = -k * zi[N + k];
      ci = k * zr[N + k];
    } else if (u == N / 2 || u == M - N / 2) {  // the two halves of the Nyquist mode
      const double h = (u == N / 2 ? 0.25 : -0.25) * N;  // (+-N/2) * 1/2
      cr = -h * zi[N / 2];
      ci = h * zr[N / 2];
    }
    are[u] = cr;
    aim[u] = ci;
  }
  ves_fft(are, aim, tre, tim, M, cos6, sin6, +1);
  for (int u = threadIdx.x; u < M; u += blockDim.x) {
    const double dx = are[u], dy = aim[u];
    are[u] = sqrt(dx * dx + dy * dy);
    aim[u] = 0.0;
  }
  // Fourier coefficients X_k = C_k - i S_k of arc (FFT of length 6N)
  ves_fft(are, aim, tre, tim, M, cos6, sin6, -1);
  const double C0 = are[0];
  // al(t_u) = int_0^{t_u} arc = (C_0/M) t_u + sum_{k=1}^{M/2-1} 2/(k M) [C_k sin(k t_u) - S_k (cos(k t_u) - 1)]
  //         = (C_0/M) t_u + sum_k 2/(k M) S_k + Im sum_k (2/(k M)) X_k e^{i k t_u}
  double cpart = 0.0;
  for (int kk = 1 + threadIdx.x; kk < M / 2; kk += blockDim.x) cpart += 2.0 / ((double)kk * M) * (-aim[kk]);
  const double K0 = bsum(cpart, red);
  for (int kk = threadIdx.x; kk < M; kk += blockDim.x) {
    const double f = (kk >= 1 && kk < M / 2) ? 2.0 / ((double)kk * M) : 0.0;
    are[kk] *= f;
    aim[kk] *= f;
  }
  ves_fft(are, aim, tre, tim, M, cos6, sin6, +1);
  for (int u = threadIdx.x; u < M; u += blockDim.x) al[u] = C0 / M * (2.0 * VES_PI * u / M) + K0 + aim[u];
  __syncthreads();
  // theta: lower_bound of i*L/N in al, linear step with slope 2 pi (the
  // reference's unit-length assumption, curve_batch_compile.py:1085-1087)
  for (int i = threadIdx.x; i < N; i += blockDim.x) {
    if (i == 0) {
      th[0] = 0.0;
      continue;
    }
    const double target = (double)i * length / N;
    int lo = 0, hi = M;
    while (lo < hi) {
      const int mid = (lo + hi) >> 1;
      if (al[mid] < target)
        lo = mid + 1;
      else
        hi = mid;
    }
    const int idx = (lo == 0) ? 0 : lo - 1;  // torch gathers idx-1 (wraps to -1 only if target <= al[0])
    th[i] = 2.0 * VES_PI * idx / M + (target - al[idx]) * (2.0 * VES_PI);
  }
  __syncthreads();
  // z(theta_i) = sum_m zh_m e^{i m theta_i}; powers of e^{i theta} by recurrence
  for (int i = threadIdx.x; i < N; i += blockDim.x) {
    double s1, c1;
    sincos(th[i], &s1, &c1);
    double er = 1.0, ei = 0.0;
    double re = zr[0], im = zi[0];
    for (int kk = 1; kk < N / 2; ++kk) {
      const double nr = er * c1 - ei * s1;
      ei = er * s1 + ei * c1;
      er = nr;
      re += zr[kk] * er - zi[kk] * ei;  // mode +kk
      im += zr[kk] * ei + zi[kk] * er;
      re += zr[N - kk] * er + zi[N - kk] * ei;  // mode -kk: conjugate power
      im += zi[N - kk] * er - zr[N - kk] * ei;
    }
    {
      const double nr = er * c1 - ei * s1;  // mode -N/2
      ei = er * s1 + ei * c1;
      er = nr;
      re += zr[N / 2] * er + zi[N / 2] * ei;
      im += zi[N / 2] * er - zr[N / 2] * ei;
    }
    Ok[i] = re;
    Ok[N + i] = im;
  }
  if (threadIdx.x == 0) flags[k] = 0;
}

// physical centre (curve_batch_compile.py:84-100) and inclination angle (:105-194)
__device__ void center_angle(int N, const double* d, const double* x, const double* y, double* dxb, double* dyb,
                             double* red, double& cx, double& cy, double& ang) {
  for (int j = threadIdx.x; j < N; j += blockDim.x) {
    dxb[j] = circ(d, x, N, j);
    dyb[j] = circ(d, y, N, j);
  }
  __syncthreads();
  double a = 0, sx = 0, sy = 0;
  for (int j = threadIdx.x; j < N; j += blockDim.x) {
    a += x[j] * dyb[j] - y[j] * dxb[j];
    sx += x[j] * x[j] * dyb[j];
    sy += y[j] * y[j] * dxb[j];
  }
  const double A = bsum(a, red);
  cx = bsum(sx, red) / A;
  cy = -bsum(sy, red) / A;
  // centred moments; D annihilates constants, so the derivatives of the
  // centred curve are those of the curve
  double j11 = 0, j12 = 0, j22 = 0;
  for (int j = threadIdx.x; j < N; j += blockDim.x) {
    const double xc = x[j] - cx, yc = y[j] - cy;
    const double jac = sqrt(dxb[j] * dxb[j] + dyb[j] * dyb[j]);
    const double nx = dyb[j] / jac, ny = -dxb[j] / jac;
    const double rdn = xc * nx + yc * ny, rho2 = xc * xc + yc * yc;
    j11 += rdn * (rho2 - xc * xc) * jac;
    j12 += rdn * (-xc * yc) * jac;
    j22 += rdn * (rho2 - yc * yc) * jac;
  }
  const double J11 = bsum(j11, red), J12 = bsum(j12, red), J22 = bsum(j22, red);
  // eigenvector of the symmetric 2x2 moment tensor for the eigenvalue of least magnitude
  const double hm = 0.5 * (J11 + J22), hd = 0.5 * (J11 - J22);
  const double rad = sqrt(hd * hd + J12 * J12);
  const double l1 = hm + rad, l2 = hm - rad;
  const double lam = (fabs(l1) < fabs(l2)) ? l1 : l2;
  double vx, vy;
  if (fabs(lam - J11) + fabs(J12) >= fabs(lam - J22) + fabs(J12) && (fabs(J12) + fabs(lam - J11)) > 0) {
    vx = J12;
    vy = lam - J11;
  } else {
    vx = lam - J22;
    vy = J12;
  }
  if (vx == 0 && vy == 0) {  // isotropic tensor: any direction; take the x axis
    vx = 1;
    vy = 0;
  }
  if (vy < 0) {
    vx = -vx;
    vy = -vy;
  }
  ang = atan2(vy, vx);
}

__global__ void align_kernel(int N, const double* __restrict__ d1, const double* __restrict__ Xorg,
                             const double* __restrict__ X, double* __restrict__ Xout, double* __restrict__ center,
                             double* __restrict__ angle) {
  extern __shared__ double sh[];
  double* d = sh;
  double* x = d + N;
  double* y = x + N;
  double* dxb = y + N;
  double* dyb = dxb + N;
  double* red = dyb + N;
  const int k = blockIdx.x;
  for (int i = threadIdx.x; i < N; i += blockDim.x) d[i] = d1[i];
  double c0x = 0, c0y = 0, a0 = 0;
  if (Xorg) {
    for (int i = threadIdx.x; i < N; i += blockDim.x) {
      x[i] = Xorg[(long long)k * 2 * N + i];
      y[i] = Xorg[(long long)k * 2 * N + N + i];
    }
    __syncthreads();
    center_angle(N, d, x, y, dxb, dyb, red, c0x, c0y, a0);
    __syncthreads();
  }
  for (int i = threadIdx.x; i < N; i += blockDim.x) {
    x[i] = X[(long long)k * 2 * N + i];
    y[i] = X[(long long)k * 2 * N + N + i];
  }
  __syncthreads();
  double c1x, c1y, a1;
  center_angle(N, d, x, y, dxb, dyb, red, c1x, c1y, a1);
  if (!Xorg) {
    if (threadIdx.x == 0) {
      if (center) {
        center[2 * k] = c1x;
        center[2 * k + 1] = c1y;
      }
      if (angle) angle[k] = a1;
    }
    return;
  }
  const double a2 = (a1 > VES_PI) ? a1 - VES_PI : a1 + VES_PI;
  const double anew = (fabs(a0 - a2) < fabs(a0 - a1)) ? a2 : a1;
  const double th = -anew + a0;
  const double ct = cos(th), st = sin(th);
  for (int i = threadIdx.x; i < N; i += blockDim.x) {
    const double xp = x[i] - c1x, yp = y[i] - c1y;
    Xout[(long long)k * 2 * N + i] = xp * ct - yp * st + c0x;
    Xout[(long long)k * 2 * N + N + i] = xp * st + yp * ct + c0y;
  }
}

// ---------------------------------------------------------------------------
// augmented Lagrangian: per corrected vesicle area, length, distance functional
// and the gradient of  mean_k |z_k - X_k|/|X_k|
//   - 1/n sum lam_a (a - a0)/a0 - 1/n sum lam_l (l - l0)/l0
//   + 1/(2 mu) mean((a - a0)^2/a0^2 + (l - l0)^2/l0^2)
__global__ void auglag_eval_kernel(int N, int nc, const double* __restrict__ d1, const double* __restrict__ z,
                                   const double* __restrict__ X0, const double* __restrict__ a0,
                                   const double* __restrict__ l0, const double* __restrict__ lam, double mu,
                                   double* __restrict__ aout, double* __restrict__ lout, double* __restrict__ fout,
                                   double* __restrict__ g) {
  extern __shared__ double sh[];
  double* d = sh;
  double* x = d + N;
  double* y = x + N;
  double* dxb = y + N;
  double* dyb = dxb + N;
  double* tx = dyb + N;
  double* ty = tx + N;
  double* red = ty + N;
  const int k = blockIdx.x;
  const double* zk = z + (long long)k * 2 * N;
  const double* xk = X0 + (long long)k * 2 * N;
  for (int i = threadIdx.x; i < N; i += blockDim.x) {
    d[i] = d1[i];
    x[i] = zk[i];
    y[i] = zk[N + i];
  }
  __syncthreads();
  double sa = 0, sl = 0, sr = 0, sx = 0;
  for (int j = threadIdx.x; j < N; j += blockDim.x) {
    const double dx = circ(d, x, N, j), dy = circ(d, y, N, j);
    dxb[j] = dx;
    dyb[j] = dy;
    const double jac = sqrt(dx * dx + dy * dy);
    tx[j] = dx / jac;
    ty[j] = dy / jac;
    sa += x[j] * dy - y[j] * dx;
    sl += jac;
    const double rx = x[j] - xk[j], ry = y[j] - xk[N + j];
    sr += rx * rx + ry * ry;
    sx += xk[j] * xk[j] + xk[N + j] * xk[N + j];
  }
  const double area = bsum(sa, red) * VES_PI / N;
  const double length = bsum(sl, red) * 2.0 * VES_PI / N;
  const double nr = sqrt(bsum(sr, red));
  const double nx = sqrt(bsum(sx, red));
  if (threadIdx.x == 0) {
    aout[k] = area;
    lout[k] = length;
    fout[k] = nr / nx;
  }
  const double A0 = a0[k], L0 = l0[k];
  const double ca = -lam[k] / A0 / nc + (area - A0) / (A0 * A0) / (mu * nc);
  const double cl = -lam[nc + k] / L0 / nc + (length - L0) / (L0 * L0) / (mu * nc);
  const double cf = (nr > 0) ? 1.0 / (nr * nx * nc) : 0.0;
  const double h = 2.0 * VES_PI / N;
  for (int j = threadIdx.x; j < N; j += blockDim.x) {
    // dA/dx = h D y, dA/dy = -h D x; dL/dx = -h D (Dx/jac), dL/dy = -h D (Dy/jac)
    const double gax = h * dyb[j], gay = -h * dxb[j];
    const double glx = -h * circ(d, tx, N, j), gly = -h * circ(d, ty, N, j);
    g[(long long)k * 2 * N + j] = cf * (x[j] - xk[j]) + ca * gax + cl * glx;
    g[(long long)k * 2 * N + N + j] = cf * (y[j] - xk[N + j]) + ca * gay + cl * gly;
  }
}

// [max |a-a0|/a0, max |l-l0|/l0, mean f]
__global__ void auglag_stats_kernel(int nc, const double* __restrict__ a, const double* __restrict__ l,
                                    const double* __restrict__ f, const double* __restrict__ a0,
                                    const double* __restrict__ l0, double* __restrict__ out) {
  __shared__ double red[3][256];
  double ea = 0, el = 0, sf = 0;
  for (int k = threadIdx.x; k < nc; k += blockDim.x) {
    ea = fmax(ea, fabs(a[k] - a0[k]) / a0[k]);
    el = fmax(el, fabs(l[k] - l0[k]) / l0[k]);
    sf += f[k];
  }
  red[0][threadIdx.x] = ea;
  red[1][threadIdx.x] = el;
  red[2][threadIdx.x] = sf;
  __syncthreads();
  for (int w = 128; w > 0; w >>= 1) {
    if (threadIdx.x < w) {
      red[0][threadIdx.x] = fmax(red[0][threadIdx.x], red[0][threadIdx.x + w]);
      red[1][threadIdx.x] = fmax(red[1][threadIdx.x], red[1][threadIdx.x + w]);
      red[2][threadIdx.x] += red[2][threadIdx.x + w];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    out[0] = red[0][0];
    out[1] = red[1][0];
    out[2] = red[2][0] / nc;
  }
}

// torch.optim.Adam step (betas 0.9/0.999, eps 1e-8, no weight decay)
__global__ void adam_kernel(long long n, int step, double lr, double* __restrict__ z, double* __restrict__ m1,
                            double* __restrict__ m2, const double* __restrict__ g) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double gi = g[i];
  const double a = m1[i] + (gi - m1[i]) * 0.1;  // lerp(m1, g, 1 - beta1)
  const double b = m2[i] * 0.999 + gi * gi * 0.001;
  m1[i] = a;
  m2[i] = b;
  const double bc1 = 1.0 - pow(0.9, step);
  const double bc2 = 1.0 - pow(0.999, step);
  const double denom = sqrt(b) / sqrt(bc2) + 1e-8;
  z[i] -= (lr / bc1) * a / denom;
}

__global__ void auglag_lambda_kernel(int nc, double mu, const double* __restrict__ a, const double* __restrict__ l,
                                     const double* __restrict__ a0, const double* __restrict__ l0,
                                     double* __restrict__ lam) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= nc) return;
  lam[k] -= (1.0 / mu) * ((a[k] - a0[k]) / a0[k]);
  lam[nc + k] -= (1.0 / mu) * ((l[k] - l0[k]) / l0[k]);
}

__global__ void gather_cols_kernel(int N, int nc, const int* __restrict__ idx, const double* __restrict__ X,
                                   double* __restrict__ out) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (long long)nc * 2 * N) return;
  const long long k = i / (2 * N), r = i % (2 * N);
  out[i] = X[(long long)idx[k] * 2 * N + r];
}
__global__ void scatter_cols_kernel(int N, int nc, const int* __restrict__ idx, const double* __restrict__ z,
                                    double* __restrict__ X) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (long long)nc * 2 * N) return;
  const long long k = i / (2 * N), r = i % (2 * N);
  X[(long long)idx[k] * 2 * N + r] = z[i];
}

}  // namespace

int post_redistribute(ves_ctx* c, int nv, const double* X, double* Xout, int* flags, WsCarver& ws,
                      cudaStream_t s) {
  const int N = c->N, M = 6 * N;
  const int nchunk = (nv + kSpreadChunk - 1) / kSpreadChunk;
  double* dev = ws.take<double>((size_t)nv * N);
  double* partial = ws.take<double>((size_t)nchunk * N);
  double* spread = ws.take<double>(1);
  if (ws.sizing) return VES_OK;
  if (!ws.ok()) {
    ves_record_error(VES_ERR_WORKSPACE, "redistribute: workspace too small (%zu needed)", ws.off);
    return VES_ERR_WORKSPACE;
  }
  if (nv <= 0) return VES_OK;
  if (!ves_fft_size_ok(M) || !ves_fft_size_ok(N)) {
    ves_record_error(VES_ERR_SHAPE, "redistribute: N = %d must be a power of two", N);
    return VES_ERR_SHAPE;
  }
  const int threads = pow2_threads(N);
  ves_count_launch(3);
  jac_dev_kernel<<<nv, threads, (size_t)(4 * N + threads) * sizeof(double), s>>>(N, c->d1N, X, dev);
  dev_rowsum_kernel<<<nchunk, 128, 0, s>>>(nv, N, dev, partial);
  spread_kernel<<<1, 256, 0, s>>>(nchunk, N, partial, spread);
  const size_t sh = (size_t)(6 * N + 5 * M + threads) * sizeof(double);
  if (sh > 32 * 1024) {
    int rc = ves_cuda_status(cudaFuncSetAttribute(redistribute_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                  (int)sh),
                             "redistribute smem");
    if (rc) return rc;
  }
  ves_count_launch();
  redistribute_kernel<<<nv, threads, sh, s>>>(N, c->d1N, c->cos6, c->sin6, spread, X, Xout, flags);
  return ves_launch_check("redistribute");
}

void launch_align_center_angle(ves_ctx* c, int nv, const double* Xorg, const double* X, double* Xout,
                               double* center, double* angle, cudaStream_t s) {
  if (nv <= 0) return;
  const int N = c->N;
  const int threads = pow2_threads(N);
  const size_t sh = (size_t)(5 * N + threads) * sizeof(double);
  ves_count_launch();
  align_kernel<<<nv, threads, sh, s>>>(N, c->d1N, Xorg, X, Xout, center, angle);
}

int post_correct_area_length(ves_ctx* c, int nv, const double* X, const double* area0, const double* length0,
                             double* Xout, int* outer_iters, WsCarver& ws, cudaStream_t s, double tol_constraint) {
  const int N = c->N;
  const size_t n2 = (size_t)nv * 2 * N;
  double* z = ws.take<double>(n2);
  double* X0 = ws.take<double>(n2);
  double* m1 = ws.take<double>(n2);
  double* m2 = ws.take<double>(n2);
  double* g = ws.take<double>(n2);
  double* lam = ws.take<double>(2 * (size_t)nv);
  double* a = ws.take<double>(nv);
  double* l = ws.take<double>(nv);
  double* f = ws.take<double>(nv);
  double* a0 = ws.take<double>(nv);
  double* l0 = ws.take<double>(nv);
  int* idx = ws.take<int>(nv);
  double* stats = ws.take<double>(4);
  if (ws.sizing) return VES_OK;
  if (!ws.ok()) {
    ves_record_error(VES_ERR_WORKSPACE, "correct_area_length: workspace too small");
    return VES_ERR_WORKSPACE;
  }
  if (outer_iters) *outer_iters = 0;
  if (nv <= 0) return VES_OK;
  int rc = ves_cuda_status(cudaMemcpyAsync(Xout, X, n2 * sizeof(double), cudaMemcpyDeviceToDevice, s), "copy");
  if (rc) return rc;
  // current area and length; which vesicles violate the tolerance
  launch_geom_prop(c, nv, X, nullptr, a, l, s);
  std::vector<double> ha(nv), hl(nv), ha0(nv), hl0(nv);
  rc = ves_cuda_status(cudaMemcpyAsync(ha.data(), a, nv * sizeof(double), cudaMemcpyDeviceToHost, s), "a");
  if (!rc) rc = ves_cuda_status(cudaMemcpyAsync(hl.data(), l, nv * sizeof(double), cudaMemcpyDeviceToHost, s), "l");
  if (!rc) rc = ves_cuda_status(cudaMemcpyAsync(ha0.data(), area0, nv * sizeof(double), cudaMemcpyDeviceToHost, s), "a0");
  if (!rc) rc = ves_cuda_status(cudaMemcpyAsync(hl0.data(), length0, nv * sizeof(double), cudaMemcpyDeviceToHost, s), "l0");
  if (!rc) rc = ves_cuda_status(cudaStreamSynchronize(s), "sync");
  if (rc) return rc;
  // tolConstraint and tolFunctional (curve_batch_compile.py:603-604); the
  // constraint tolerance may be tightened by the caller
  const double tol_c = tol_constraint > 0 ? tol_constraint : 1e-2, tol_f = 1e-2, lr = 3e-5;
  std::vector<int> hidx;
  double ea = 0, el = 0;
  for (int k = 0; k < nv; ++k) {
    const double eA = fabs((ha[k] - ha0[k]) / ha0[k]), eL = fabs((hl[k] - hl0[k]) / hl0[k]);
    ea = std::max(ea, eA);
    el = std::max(el, eL);
    if (eA > tol_c || eL > tol_c) hidx.push_back(k);
  }
  if (ea < tol_c && el < tol_c) return VES_OK;
  const int nc = (int)hidx.size();
  if (nc == 0) return VES_OK;
  std::vector<double> hA0(nc), hL0(nc);
  for (int k = 0; k < nc; ++k) {
    hA0[k] = ha0[hidx[k]];
    hL0[k] = hl0[hidx[k]];
  }
  rc = ves_cuda_status(cudaMemcpyAsync(idx, hidx.data(), nc * sizeof(int), cudaMemcpyHostToDevice, s), "idx");
  if (!rc) rc = ves_cuda_status(cudaMemcpyAsync(a0, hA0.data(), nc * sizeof(double), cudaMemcpyHostToDevice, s), "a0c");
  if (!rc) rc = ves_cuda_status(cudaMemcpyAsync(l0, hL0.data(), nc * sizeof(double), cudaMemcpyHostToDevice, s), "l0c");
  if (!rc) rc = ves_cuda_status(cudaMemsetAsync(lam, 0, 2 * nc * sizeof(double), s), "lam");
  if (rc) return rc;
  const long long nz = (long long)nc * 2 * N;
  ves_count_launch(2);
  gather_cols_kernel<<<ceil_div(nz, 256), 256, 0, s>>>(N, nc, idx, X, X0);
  gather_cols_kernel<<<ceil_div(nz, 256), 256, 0, s>>>(N, nc, idx, X, z);
  const int threads = pow2_threads(N);
  const size_t sh = (size_t)(7 * N + threads) * sizeof(double);
  double mu = 0.1;
  double hs[3];
  int it = 0;
  for (; it < 100; ++it) {
    rc = ves_cuda_status(cudaMemsetAsync(m1, 0, nz * sizeof(double), s), "m1");
    if (!rc) rc = ves_cuda_status(cudaMemsetAsync(m2, 0, nz * sizeof(double), s), "m2");
    if (rc) return rc;
    bool done = false;
    for (int step = 1; step <= 20; ++step) {
      ves_count_launch(2);
      auglag_eval_kernel<<<nc, threads, sh, s>>>(N, nc, c->d1N, z, X0, a0, l0, lam, mu, a, l, f, g);
      auglag_stats_kernel<<<1, 256, 0, s>>>(nc, a, l, f, a0, l0, stats);
      rc = ves_cuda_status(cudaMemcpyAsync(hs, stats, 3 * sizeof(double), cudaMemcpyDeviceToHost, s), "stats");
      if (!rc) rc = ves_cuda_status(cudaStreamSynchronize(s), "stats sync");
      if (rc) return rc;
      if (hs[2] < tol_f && hs[0] < tol_c && hs[1] < tol_c) {
        done = true;
        break;
      }
      ves_count_launch();
      adam_kernel<<<ceil_div(nz, 256), 256, 0, s>>>(nz, step, lr, z, m1, m2, g);
    }
    if (done) break;
    ves_count_launch();
    auglag_lambda_kernel<<<ceil_div(nc, 256), 256, 0, s>>>(nc, mu, a, l, a0, l0, lam);
    mu *= 0.8;
  }
  if (outer_iters) *outer_iters = it;
  ves_count_launch();
  scatter_cols_kernel<<<ceil_div(nz, 256), 256, 0, s>>>(N, nc, idx, z, Xout);
  return ves_launch_check("correct_area_length");
}
