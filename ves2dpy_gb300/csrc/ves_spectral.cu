// Per-vesicle spectral operators (FP64).  One CTA per vesicle; periodic
// derivatives are circulant convolutions with the Nyquist-free derivative
// stencil held in shared memory, which is the exact operator the reference
// applies through torch.fft (curve_batch_compile.py:379-423, 1188-1200).
#include "ves_internal.h"
#include "ves_fft.cuh"

// y[j] = sum_l d[(j - l) mod n] * a[l]   (a, d in shared memory)
__device__ __forceinline__ double circ_apply(const double* __restrict__ d, const double* __restrict__ a,
                                             int n, int j) {
  double s = 0.0;
  for (int l = 0; l <= j; ++l) s = fma(d[j - l], a[l], s);
  for (int l = j + 1; l < n; ++l) s = fma(d[j - l + n], a[l], s);
  return s;
}

// ----------------------------------------------------------------------------
// interpft N -> Nup: out[u] = sum_i pc[(u - m i) mod Nup] in[i]
__global__ void upsample_kernel(int N, int Nup, int m, const double* __restrict__ pc, int ncomp,
                                const double* __restrict__ in, long long in_stride,
                                double* __restrict__ out) {
  extern __shared__ double sh[];
  double* x = sh;        // [N]
  double* p = sh + N;    // [Nup]
  const int k = blockIdx.x / ncomp, c = blockIdx.x % ncomp;
  const double* src = in + (long long)k * in_stride + (long long)c * N;
  for (int i = threadIdx.x; i < N; i += blockDim.x) x[i] = src[i];
  for (int i = threadIdx.x; i < Nup; i += blockDim.x) p[i] = pc[i];
  __syncthreads();
  double* dst = out + ((long long)k * ncomp + c) * Nup;
  for (int u = threadIdx.x; u < Nup; u += blockDim.x) {
    double s = 0.0;
    int r = u;  // (u - m*i) mod Nup, i = 0
    for (int i = 0; i < N; ++i) {
      s = fma(p[r], x[i], s);
      r -= m;
      if (r < 0) r += Nup;
    }
    dst[u] = s;
  }
}

// interpft N -> Nup of both components of a vesicle at once, as filter.py
// interpft does it (fft, zero-padded spectrum, ifft, times Nup/N): z = x + i y,
// FFT of length N, the Nyquist mode split in half between +N/2 and -N/2 (the
// real part of the reference's one-sided placement, so both components stay
// real), inverse FFT of length Nup, divided by N.
__global__ void __launch_bounds__(256) upsample_fft_kernel(int N, int Nup, const double* __restrict__ cosU,
                                                           const double* __restrict__ sinU,
                                                           const double* __restrict__ in, long long in_stride,
                                                           double* __restrict__ out) {
  extern __shared__ double sh[];
  double* zr = sh;
  double* zi = zr + Nup;
  double* tre = zi + Nup;
  double* tim = tre + Nup;
  const int k = blockIdx.x;
  const double* src = in + (long long)k * in_stride;
  for (int i = threadIdx.x; i < N; i += blockDim.x) {
    zr[i] = src[i];
    zi[i] = src[N + i];
  }
  ves_fft(zr, zi, tre, tim, N, cosU, sinU, -1, Nup / N);
  for (int i = threadIdx.x; i < N; i += blockDim.x) {
    tre[i] = zr[i];
    tim[i] = zi[i];
  }
  __syncthreads();
  const int h = N / 2, top = Nup - N;
  for (int u = threadIdx.x; u < Nup; u += blockDim.x) {
    double vr = 0.0, vi = 0.0;
    if (u < h) {
      vr = tre[u];
      vi = tim[u];
    } else if (u == h || u == Nup - h) {
      vr = 0.5 * tre[h];
      vi = 0.5 * tim[h];
    } else if (u > Nup - h) {
      vr = tre[u - top];
      vi = tim[u - top];
    }
    zr[u] = vr;
    zi[u] = vi;
  }
  ves_fft(zr, zi, tre, tim, Nup, cosU, sinU, +1);
  const double inv = 1.0 / N;
  double* dst = out + (long long)k * 2 * Nup;
  for (int u = threadIdx.x; u < Nup; u += blockDim.x) {
    dst[u] = zr[u] * inv;
    dst[Nup + u] = zi[u] * inv;
  }
}

void launch_upsample(const ves_ctx* c, int nv, int ncomp, const double* in, long long in_stride,
                     double* out, cudaStream_t s) {
  if (nv <= 0) return;
  const int N = c->N, Nup = c->Nup;
  if (ncomp == 2 && in_stride == 2LL * N && N % 2 == 0 && Nup > N && ves_fft_size_ok(N) && ves_fft_size_ok(Nup)) {
    const size_t shf = (size_t)4 * Nup * sizeof(double);
    if (shf > 48 * 1024 &&
        cudaFuncSetAttribute(upsample_fft_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)shf) != cudaSuccess) {
      cudaGetLastError();  // the dense sums below need no opt-in
    } else {
      ves_count_launch();
      upsample_fft_kernel<<<nv, 256, shf, s>>>(N, Nup, c->cosU, c->sinU, in, in_stride, out);
      return;
    }
  }
  size_t sh = (size_t)(N + Nup) * sizeof(double);
  ves_count_launch();
  upsample_kernel<<<nv * ncomp, 256, sh, s>>>(N, Nup, c->m, c->pc, ncomp, in, in_stride, out);
}

// Xup, its parametric derivative and the upsampled jacobian sa_up = |dXup|,
// from the coarse points: derivative of the trig interpolant at the Nup grid.
__global__ void upsample_deriv_kernel(int N, int Nup, int m, const double* __restrict__ pc,
                                      const double* __restrict__ pcd, const double* __restrict__ X,
                                      double* __restrict__ Xup, double* __restrict__ dXup,
                                      double* __restrict__ sa_up) {
  extern __shared__ double sh[];
  double* x = sh;
  double* y = x + N;
  double* p = y + N;
  double* pd = p + Nup;
  const int k = blockIdx.x;
  const double* Xk = X + (long long)k * 2 * N;
  for (int i = threadIdx.x; i < N; i += blockDim.x) {
    x[i] = Xk[i];
    y[i] = Xk[N + i];
  }
  for (int i = threadIdx.x; i < Nup; i += blockDim.x) {
    p[i] = pc[i];
    pd[i] = pcd[i];
  }
  __syncthreads();
  for (int u = threadIdx.x; u < Nup; u += blockDim.x) {
    double sx = 0, sy = 0, dx = 0, dy = 0;
    int r = u;
    for (int i = 0; i < N; ++i) {
      sx = fma(p[r], x[i], sx);
      sy = fma(p[r], y[i], sy);
      dx = fma(pd[r], x[i], dx);
      dy = fma(pd[r], y[i], dy);
      r -= m;
      if (r < 0) r += Nup;
    }
    const long long o = (long long)k * 2 * Nup;
    if (Xup) {
      Xup[o + u] = sx;
      Xup[o + Nup + u] = sy;
    }
    if (dXup) {
      dXup[o + u] = dx;
      dXup[o + Nup + u] = dy;
    }
    if (sa_up) sa_up[(long long)k * Nup + u] = sqrt(dx * dx + dy * dy);
  }
}

// The same by FFT (N power of two or three times one, Nup a multiple of N):
// z = x + i y, FFT of length N (the Nup table read with stride Nup/N), the
// spectrum zero-padded to Nup with the Nyquist mode split between +N/2 and
// -N/2 (interpft), inverse FFTs of length Nup of the spectrum times i k (the
// derivative and the speed) and of the spectrum (the curve).
__global__ void __launch_bounds__(256) upsample_deriv_fft_kernel(int N, int Nup, const double* __restrict__ cosU,
                                                                 const double* __restrict__ sinU,
                                                                 const double* __restrict__ X,
                                                                 double* __restrict__ Xup, double* __restrict__ dXup,
                                                                 double* __restrict__ sa_up) {
  extern __shared__ double sh[];
  double* zr = sh;
  double* zi = zr + Nup;
  double* tre = zi + Nup;
  double* tim = tre + Nup;
  double* spr = tim + Nup;  // [N] the spectrum
  double* spi = spr + N;
  const int k = blockIdx.x;
  const double* Xk = X + (long long)k * 2 * N;
  for (int i = threadIdx.x; i < N; i += blockDim.x) {
    zr[i] = Xk[i];
    zi[i] = Xk[N + i];
  }
  ves_fft(zr, zi, tre, tim, N, cosU, sinU, -1, Nup / N);
  for (int i = threadIdx.x; i < N; i += blockDim.x) {
    spr[i] = zr[i];
    spi[i] = zi[i];
  }
  __syncthreads();
  const int h = N / 2, top = Nup - N;
  const long long o = (long long)k * 2 * Nup;
  for (int pass = 0; pass < 2; ++pass) {
    if (pass == 1 && !Xup) break;
    for (int u = threadIdx.x; u < Nup; u += blockDim.x) {
      double vr = 0.0, vi = 0.0, kk = 0.0;
      if (u < h) {
        vr = spr[u];
        vi = spi[u];
        kk = u;
      } else if (u == h || u == Nup - h) {
        vr = 0.5 * spr[h];
        vi = 0.5 * spi[h];
        kk = (u == h) ? (double)h : -(double)h;
      } else if (u > Nup - h) {
        vr = spr[u - top];
        vi = spi[u - top];
        kk = (double)(u - Nup);
      }
      if (pass == 0) {
        zr[u] = -kk * vi;
        zi[u] = kk * vr;
      } else {
        zr[u] = vr;
        zi[u] = vi;
      }
    }
    ves_fft(zr, zi, tre, tim, Nup, cosU, sinU, +1);
    for (int u = threadIdx.x; u < Nup; u += blockDim.x) {
      const double a = zr[u] / N, b = zi[u] / N;
      if (pass == 0) {
        if (dXup) {
          dXup[o + u] = a;
          dXup[o + Nup + u] = b;
        }
        if (sa_up) sa_up[(long long)k * Nup + u] = sqrt(a * a + b * b);
      } else {
        Xup[o + u] = a;
        Xup[o + Nup + u] = b;
      }
    }
    __syncthreads();
  }
}

// Geometry of the upsampled curve from the first and second derivatives of
// the trig interpolant at the Nup grid.  They equal the FFT derivatives of
// interpft(X, Nup) on its own grid (diffProp of capsules(Xup),
// curve_batch_compile.py:400-423) up to rounding, with an error that does not
// grow with Nup as a fine-grid circulant derivative's does.
__global__ void upsample_geom_kernel(int N, int Nup, int m, const double* __restrict__ pc,
                                     const double* __restrict__ pcd, const double* __restrict__ pcdd,
                                     const double* __restrict__ X, double* __restrict__ Xup,
                                     double* __restrict__ sa, double* __restrict__ tang, double* __restrict__ cur) {
  extern __shared__ double sh[];
  double* x = sh;
  double* y = x + N;
  double* p = y + N;
  double* pd = p + Nup;
  double* pdd = pd + Nup;
  const int k = blockIdx.x;
  const double* Xk = X + (long long)k * 2 * N;
  for (int i = threadIdx.x; i < N; i += blockDim.x) {
    x[i] = Xk[i];
    y[i] = Xk[N + i];
  }
  for (int i = threadIdx.x; i < Nup; i += blockDim.x) {
    p[i] = pc[i];
    pd[i] = pcd[i];
    pdd[i] = pcdd[i];
  }
  __syncthreads();
  for (int u = threadIdx.x; u < Nup; u += blockDim.x) {
    double sx = 0, sy = 0, dx = 0, dy = 0, ddx = 0, ddy = 0;
    int r = u;
    for (int i = 0; i < N; ++i) {
      sx = fma(p[r], x[i], sx);
      sy = fma(p[r], y[i], sy);
      dx = fma(pd[r], x[i], dx);
      dy = fma(pd[r], y[i], dy);
      ddx = fma(pdd[r], x[i], ddx);
      ddy = fma(pdd[r], y[i], ddy);
      r -= m;
      if (r < 0) r += Nup;
    }
    const long long o = (long long)k * 2 * Nup;
    const double jac = sqrt(dx * dx + dy * dy);
    if (Xup) {
      Xup[o + u] = sx;
      Xup[o + Nup + u] = sy;
    }
    if (sa) sa[(long long)k * Nup + u] = jac;
    if (tang) {
      tang[o + u] = dx / jac;
      tang[o + Nup + u] = dy / jac;
    }
    if (cur) cur[(long long)k * Nup + u] = (dx * ddy - dy * ddx) / (jac * jac * jac);
  }
}

void launch_upsample_geom(const ves_ctx* c, int nv, const double* X, double* Xup, double* sa, double* tang,
                          double* cur, cudaStream_t s) {
  if (nv <= 0) return;
  const size_t sh = (size_t)(2 * c->N + 3 * c->Nup) * sizeof(double);
  if (sh > 48 * 1024) cudaFuncSetAttribute(upsample_geom_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sh);
  ves_count_launch();
  upsample_geom_kernel<<<nv, 256, sh, s>>>(c->N, c->Nup, c->m, c->pc, c->pcd, c->pcdd, X, Xup, sa, tang, cur);
}

void launch_upsample_deriv(const ves_ctx* c, int nv, const double* X, double* Xup, double* dXup,
                           double* sa_up, cudaStream_t s) {
  if (nv <= 0) return;
  const int N = c->N, Nup = c->Nup;
  if (N % 2 == 0 && Nup > N && Nup % N == 0 && ves_fft_size_ok(N) && ves_fft_size_ok(Nup)) {
    const size_t shf = (size_t)(4 * Nup + 2 * N) * sizeof(double);
    if (shf <= 48 * 1024 ||
        cudaFuncSetAttribute(upsample_deriv_fft_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)shf) ==
            cudaSuccess) {
      ves_count_launch();
      upsample_deriv_fft_kernel<<<nv, 256, shf, s>>>(N, Nup, c->cosU, c->sinU, X, Xup, dXup, sa_up);
      return;
    }
    cudaGetLastError();  // the dense sums below need no opt-in
  }
  size_t sh = (size_t)(2 * N + 2 * Nup) * sizeof(double);
  ves_count_launch();
  upsample_deriv_kernel<<<nv, 256, sh, s>>>(N, Nup, c->m, c->pc, c->pcd, X, Xup, dXup, sa_up);
}

// ----------------------------------------------------------------------------
// diffProp on an n-point grid (curve_batch_compile.py:400-423)
__global__ void diff_prop_kernel(int n, const double* __restrict__ dstencil,
                                 const double* __restrict__ X, double* __restrict__ sa,
                                 double* __restrict__ isa, double* __restrict__ tang,
                                 double* __restrict__ cur) {
  extern __shared__ double sh[];
  double* d = sh;
  double* x = d + n;
  double* y = x + n;
  double* Dx = y + n;
  double* Dy = Dx + n;
  const int k = blockIdx.x;
  const double* Xk = X + (long long)k * 2 * n;
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    d[i] = dstencil[i];
    x[i] = Xk[i];
    y[i] = Xk[n + i];
  }
  __syncthreads();
  for (int j = threadIdx.x; j < n; j += blockDim.x) {
    Dx[j] = circ_apply(d, x, n, j);
    Dy[j] = circ_apply(d, y, n, j);
  }
  __syncthreads();
  for (int j = threadIdx.x; j < n; j += blockDim.x) {
    const double dx = Dx[j], dy = Dy[j];
    const double jac = sqrt(dx * dx + dy * dy);
    const long long o = (long long)k * n + j;
    if (sa) sa[o] = jac;
    if (isa) isa[o] = 1.0 / jac;
    if (tang) {
      tang[(long long)k * 2 * n + j] = dx / jac;
      tang[(long long)k * 2 * n + n + j] = dy / jac;
    }
    if (cur) {
      const double ddx = circ_apply(d, Dx, n, j);
      const double ddy = circ_apply(d, Dy, n, j);
      cur[o] = (dx * ddy - dy * ddx) / (jac * jac * jac);
    }
  }
}

void launch_diff_prop(const ves_ctx* c, int grid, int nv, const double* X, double* sa, double* isa,
                      double* tang, double* cur, cudaStream_t s) {
  if (nv <= 0) return;
  const int n = grid ? c->Nup : c->N;
  const double* d = grid ? c->d1Nup : c->d1N;
  const int threads = n < 256 ? ((n + 31) / 32) * 32 : 256;
  const size_t sh = (size_t)5 * n * sizeof(double);
  if (sh > 32 * 1024) cudaFuncSetAttribute(diff_prop_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sh);
  ves_count_launch();
  diff_prop_kernel<<<nv, threads, sh, s>>>(n, d, X, sa, isa, tang, cur);
}

// ----------------------------------------------------------------------------
// geomProp (curve_batch_compile.py:455-473); deterministic block reductions
__device__ double block_sum(double v, double* red) {
  const int t = threadIdx.x;
  red[t] = v;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if (t < w) red[t] += red[t + w];
    __syncthreads();
  }
  double r = red[0];
  __syncthreads();
  return r;
}

__global__ void geom_prop_kernel(int n, const double* __restrict__ dstencil,
                                 const double* __restrict__ X, double* ra, double* area,
                                 double* length) {
  extern __shared__ double sh[];
  double* d = sh;
  double* x = d + n;
  double* y = x + n;
  double* red = y + n;  // blockDim
  const int k = blockIdx.x;
  const double* Xk = X + (long long)k * 2 * n;
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    d[i] = dstencil[i];
    x[i] = Xk[i];
    y[i] = Xk[n + i];
  }
  __syncthreads();
  double sl = 0, sa = 0;
  for (int j = threadIdx.x; j < n; j += blockDim.x) {
    const double dx = circ_apply(d, x, n, j), dy = circ_apply(d, y, n, j);
    sl += sqrt(dx * dx + dy * dy);
    sa += x[j] * dy - y[j] * dx;
  }
  const double L = block_sum(sl, red) * 2.0 * VES_PI / n;
  const double A = block_sum(sa, red) * VES_PI / n;
  if (threadIdx.x == 0) {
    if (length) length[k] = L;
    if (area) area[k] = A;
    if (ra) ra[k] = 4.0 * VES_PI * A / (L * L);
  }
}

void launch_geom_prop(const ves_ctx* c, int nv, const double* X, double* ra, double* area,
                      double* length, cudaStream_t s) {
  if (nv <= 0) return;
  const int threads = 128;
  ves_count_launch();
  geom_prop_kernel<<<nv, threads, (size_t)(3 * c->N + threads) * sizeof(double), s>>>(
      c->N, c->d1N, X, ra, area, length);
}

// ----------------------------------------------------------------------------
// tracJump (capsules.py:54-80): f = -kappa (isa D)^4 X + isa D (sigma X_s)
__global__ void trac_jump_kernel(int N, const double* __restrict__ dstencil, double kappa,
                                 const double* __restrict__ isa, const double* __restrict__ tang,
                                 const double* __restrict__ X, long long xs,
                                 const double* __restrict__ sig, long long ss,
                                 double* __restrict__ f) {
  extern __shared__ double sh[];
  double* d = sh;
  double* a = d + N;
  double* b = a + N;
  double* is = b + N;
  const int k = blockIdx.x;
  for (int i = threadIdx.x; i < N; i += blockDim.x) {
    d[i] = dstencil[i];
    is[i] = isa[(long long)k * N + i];
  }
  for (int comp = 0; comp < 2; ++comp) {
    __syncthreads();
    for (int i = threadIdx.x; i < N; i += blockDim.x) a[i] = X[(long long)k * xs + comp * N + i];
    for (int it = 0; it < 4; ++it) {
      __syncthreads();
      for (int j = threadIdx.x; j < N; j += blockDim.x) b[j] = is[j] * circ_apply(d, a, N, j);
      __syncthreads();
      for (int j = threadIdx.x; j < N; j += blockDim.x) a[j] = b[j];
    }
    __syncthreads();
    for (int j = threadIdx.x; j < N; j += blockDim.x)
      b[j] = sig[(long long)k * ss + j] * tang[(long long)k * 2 * N + comp * N + j];
    __syncthreads();
    for (int j = threadIdx.x; j < N; j += blockDim.x) {
      const double ten = is[j] * circ_apply(d, b, N, j);
      f[(long long)k * 2 * N + comp * N + j] = -kappa * a[j] + ten;
    }
  }
}

void launch_trac_jump(const ves_ctx* c, int nv, double kappa, const double* isa, const double* tang,
                      const double* X, long long xs, const double* sig, long long ss, double* f,
                      cudaStream_t s) {
  if (nv <= 0) return;
  const int threads = c->N < 256 ? ((c->N + 31) / 32) * 32 : 256;
  ves_count_launch();
  trac_jump_kernel<<<nv, threads, (size_t)4 * c->N * sizeof(double), s>>>(c->N, c->d1N, kappa, isa,
                                                                            tang, X, xs, sig, ss, f);
}

// surfaceDiv (capsules.py:82-89)
__global__ void surface_div_kernel(int N, const double* __restrict__ dstencil,
                                   const double* __restrict__ isa, const double* __restrict__ tang,
                                   const double* __restrict__ f, long long fs, double* __restrict__ out,
                                   long long os) {
  extern __shared__ double sh[];
  double* d = sh;
  double* fx = d + N;
  double* fy = fx + N;
  const int k = blockIdx.x;
  for (int i = threadIdx.x; i < N; i += blockDim.x) {
    d[i] = dstencil[i];
    fx[i] = f[(long long)k * fs + i];
    fy[i] = f[(long long)k * fs + N + i];
  }
  __syncthreads();
  for (int j = threadIdx.x; j < N; j += blockDim.x) {
    const double is = isa[(long long)k * N + j];
    const double ax = is * circ_apply(d, fx, N, j);
    const double ay = is * circ_apply(d, fy, N, j);
    out[(long long)k * os + j] =
        ax * tang[(long long)k * 2 * N + j] + ay * tang[(long long)k * 2 * N + N + j];
  }
}

void launch_surface_div(const ves_ctx* c, int nv, const double* isa, const double* tang,
                        const double* f, long long fs, double* out, long long os, cudaStream_t s) {
  if (nv <= 0) return;
  const int threads = c->N < 256 ? ((c->N + 31) / 32) * 32 : 256;
  ves_count_launch();
  surface_div_kernel<<<nv, threads, (size_t)3 * c->N * sizeof(double), s>>>(c->N, c->d1N, isa, tang,
                                                                              f, fs, out, os);
}

// ----------------------------------------------------------------------------
// bg_flow (tstep_biem.py:849-952)
__global__ void bg_flow_kernel(int nv, int N, int flow, double speed, double cw, double vs,
                               const double* __restrict__ X, double* __restrict__ v) {
  const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= (long long)nv * N) return;
  const long long k = idx / N, j = idx % N;
  const double x = X[k * 2 * N + j], y = X[k * 2 * N + N + j];
  double vx = 0, vy = 0;
  switch (flow) {
    case VES_FLOW_EXTENSIONAL: vx = -x; vy = y; break;
    case VES_FLOW_PARABOLIC: vx = 1.0 - (y / cw) * (y / cw); vy = 0; break;
    case VES_FLOW_TAYLOR_GREEN: {
      const double sc = VES_PI / vs;
      vx = vs * sin(x * sc) * cos(y * sc);
      vy = -vs * cos(x * sc) * sin(y * sc);
    } break;
    case VES_FLOW_SHEAR: vx = y; vy = 0; break;
    case VES_FLOW_VORTEX:
      vx = sin(x / cw * VES_PI) * cos(y / cw * VES_PI);
      vy = -cos(x / cw * VES_PI) * sin(y / cw * VES_PI);
      break;
    default: break;
  }
  v[k * 2 * N + j] = vx * speed;
  v[k * 2 * N + N + j] = vy * speed;
}

void launch_bg_flow(int nv, int N, int flow, double speed, double cw, double vs, const double* X,
                    double* v, cudaStream_t s) {
  long long n = (long long)nv * N;
  if (n <= 0) return;
  ves_count_launch();
  bg_flow_kernel<<<ceil_div(n, 256), 256, 0, s>>>(nv, N, flow, speed, cw, vs, X, v);
}

// den = f * sa * 2 pi / ns  (biem_support.py:39)
__global__ void density_kernel(int nv, int ns, const double* __restrict__ f,
                               const double* __restrict__ sa, double* __restrict__ den) {
  const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= (long long)nv * 2 * ns) return;
  const long long k = idx / (2 * ns), r = idx % (2 * ns), j = r % ns;
  den[idx] = f[idx] * sa[k * ns + j] * 2.0 * VES_PI / ns;
}

void launch_density(int nv, int ns, const double* f, const double* sa, double* den, cudaStream_t s) {
  long long n = (long long)nv * 2 * ns;
  if (n <= 0) return;
  ves_count_launch();
  density_kernel<<<ceil_div(n, 256), 256, 0, s>>>(nv, ns, f, sa, den);
}

// ----------------------------------------------------------------------------
// computeDerivs (capsules.py:91-206) and the block preconditioner matrix
// (tstep_biem.py:286-352).
//
// A = diag(isa) * D1c with D1c = Dr + i*Di the complex Fourier derivative
// matrix of fft1.fourierDiff (its Nyquist mode -N/2 survives as the
// imaginary rank-one part Di[j][l] = -(1/2)(-1)^(j-l)).  Ben = Re((A A)(A A))
// on both diagonal blocks; Ten/Div use Re(A) = diag(isa) Dr.
__global__ void arc_deriv_matrix_kernel(int N, const double* __restrict__ dstencil,
                                        const double* __restrict__ isa, double* __restrict__ Are,
                                        double* __restrict__ Aim) {
  const int k = blockIdx.y;
  const long long base = (long long)k * N * N;
  for (int idx = blockIdx.x * blockDim.x + threadIdx.x; idx < N * N; idx += gridDim.x * blockDim.x) {
    const int j = idx / N, l = idx % N;
    const double is = isa[(long long)k * N + j];
    const int r = ((j - l) % N + N) % N;
    Are[base + idx] = is * dstencil[r];
    Aim[base + idx] = is * (((j - l) & 1) ? 0.5 : -0.5);
  }
}

// Assemble Ten, Div and M = [I + dt*kappa*G*Ben, -dt*G*Ten; Div, 0]
__global__ void assemble_ten_div_kernel(int N, const double* __restrict__ Are,
                                        const double* __restrict__ tang, double* __restrict__ Ten,
                                        double* __restrict__ Div) {
  const int k = blockIdx.y;
  const long long tb = (long long)k * 2 * N;
  for (int idx = blockIdx.x * blockDim.x + threadIdx.x; idx < N * N; idx += gridDim.x * blockDim.x) {
    const int j = idx / N, l = idx % N;
    const double a = Are[(long long)k * N * N + idx];
    // Ten[j][l] = A[j][l] * xt[l] (x rows), Ten[N+j][l] = A[j][l] * yt[l]
    Ten[(long long)k * 2 * N * N + (long long)j * N + l] = a * tang[tb + l];
    Ten[(long long)k * 2 * N * N + (long long)(N + j) * N + l] = a * tang[tb + N + l];
    // Div[j][l] = xt[j] * A[j][l], Div[j][N+l] = yt[j] * A[j][l]
    Div[(long long)k * N * 2 * N + (long long)j * 2 * N + l] = tang[tb + j] * a;
    Div[(long long)k * N * 2 * N + (long long)j * 2 * N + N + l] = tang[tb + N + j] * a;
  }
}

__global__ void assemble_ben_kernel(int N, const double* __restrict__ D4, double* __restrict__ Ben) {
  const int k = blockIdx.y;
  const int n2 = 2 * N;
  for (int idx = blockIdx.x * blockDim.x + threadIdx.x; idx < n2 * n2; idx += gridDim.x * blockDim.x) {
    const int r = idx / n2, cc = idx % n2;
    double v = 0.0;
    if ((r < N) == (cc < N)) v = D4[(long long)k * N * N + (long long)(r % N) * N + (cc % N)];
    Ben[(long long)k * n2 * n2 + idx] = v;
  }
}

// M[k] (3N x 3N) from GB = G*Ben (2N x 2N), GT = G*Ten (2N x N), Div (N x 2N).
// With a viscosity contrast (Dm, alpha given) the position rows are the
// self-interaction of the matvec, [I - D/alpha + dt*kappa*G*Ben/alpha,
// -dt*G*Ten/alpha]; the reference's own assembly of that case
// (tstep_biem.py:331-334) adds the 2N x N block G*Ten to the 2N x 2N one and
// stops with a shape error.
__global__ void assemble_precond_kernel(int N, double dt, double kappa, const double* __restrict__ GB,
                                        const double* __restrict__ GT, const double* __restrict__ Div,
                                        const double* __restrict__ Dm, const double* __restrict__ alpha,
                                        double* __restrict__ M) {
  const int k = blockIdx.y;
  const int n3 = 3 * N, n2 = 2 * N;
  const double ia = alpha ? 1.0 / alpha[k] : 1.0;
  for (int idx = blockIdx.x * blockDim.x + threadIdx.x; idx < n3 * n3; idx += gridDim.x * blockDim.x) {
    const int r = idx / n3, cc = idx % n3;
    double v;
    if (r < n2) {
      if (cc < n2) {
        v = (r == cc ? 1.0 : 0.0);
        if (Dm) v -= Dm[(long long)k * n2 * n2 + (long long)r * n2 + cc] * ia;
        v += (dt * kappa * GB[(long long)k * n2 * n2 + (long long)r * n2 + cc]) * ia;
      } else {
        v = (-dt * GT[(long long)k * n2 * N + (long long)r * N + (cc - n2)]) * ia;
      }
    } else {
      v = (cc < n2) ? Div[(long long)k * N * n2 + (long long)(r - n2) * n2 + cc] : 0.0;
    }
    M[(long long)k * n3 * n3 + idx] = v;
  }
}

__global__ void arc_deriv_matrix_f32_kernel(int N, const double* __restrict__ dstencil,
                                            const double* __restrict__ isa, float* __restrict__ Are,
                                            float* __restrict__ Aim) {
  const int k = blockIdx.y;
  const long long base = (long long)k * N * N;
  for (int idx = blockIdx.x * blockDim.x + threadIdx.x; idx < N * N; idx += gridDim.x * blockDim.x) {
    const int j = idx / N, l = idx % N;
    const double is = isa[(long long)k * N + j];
    const int r = ((j - l) % N + N) % N;
    Are[base + idx] = (float)(is * dstencil[r]);
    Aim[base + idx] = (float)(is * (((j - l) & 1) ? 0.5 : -0.5));
  }
}

__global__ void ten_div_f32_kernel(int N, const float* __restrict__ Are, const double* __restrict__ tang,
                                   float* __restrict__ Ten, float* __restrict__ Div) {
  const int k = blockIdx.y;
  const long long tb = (long long)k * 2 * N;
  for (int idx = blockIdx.x * blockDim.x + threadIdx.x; idx < N * N; idx += gridDim.x * blockDim.x) {
    const int j = idx / N, l = idx % N;
    const float a = Are[(long long)k * N * N + idx];
    Ten[(long long)k * 2 * N * N + (long long)j * N + l] = a * (float)tang[tb + l];
    Ten[(long long)k * 2 * N * N + (long long)(N + j) * N + l] = a * (float)tang[tb + N + l];
    Div[(long long)k * N * 2 * N + (long long)j * 2 * N + l] = (float)tang[tb + j] * a;
    Div[(long long)k * N * 2 * N + (long long)j * 2 * N + N + l] = (float)tang[tb + N + j] * a;
  }
}

__global__ void to_f32_kernel(long long n, const double* __restrict__ a, float* __restrict__ b) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) b[i] = (float)a[i];
}

__global__ void assemble_precond_f32_kernel(int N, float dt, float kappa, const float* __restrict__ GB,
                                            const float* __restrict__ GT, const float* __restrict__ Div,
                                            float* __restrict__ M) {
  const int k = blockIdx.y;
  const int n3 = 3 * N, n2 = 2 * N;
  for (int idx = blockIdx.x * blockDim.x + threadIdx.x; idx < n3 * n3; idx += gridDim.x * blockDim.x) {
    const int r = idx / n3, cc = idx % n3;
    float v;
    if (r < n2)
      v = cc < n2 ? (r == cc ? 1.0f : 0.0f) + dt * kappa * GB[(long long)k * n2 * n2 + (long long)r * n2 + cc]
                  : -dt * GT[(long long)k * n2 * N + (long long)r * N + (cc - n2)];
    else
      v = (cc < n2) ? Div[(long long)k * N * n2 + (long long)(r - n2) * n2 + cc] : 0.0f;
    M[(long long)k * n3 * n3 + idx] = v;
  }
}

// D4 = Re(C*C) with C = A*A, complex A = Are + i Aim, via real products:
// C = (Are Are - Aim Aim) + i (Are Aim + Aim Are); D4 = Cr Cr - Ci Ci.
int derivs_and_precond(ves_ctx* c, int nv, const double* isa, const double* tang, const double* G,
                       double dt, double kappa, double* Ben, double* Ten, double* Div, double* M,
                       WsCarver& ws, cudaStream_t s, const double* Dm, const double* alpha) {
  const int N = c->N;
  const size_t NN = (size_t)N * N;
  double* Are = ws.take<double>(NN * nv);
  double* Aim = ws.take<double>(NN * nv);
  double* Cr = ws.take<double>(NN * nv);
  double* Ci = ws.take<double>(NN * nv);
  double* D4 = ws.take<double>(NN * nv);
  double* GB = (M != nullptr) ? ws.take<double>(4 * NN * nv) : nullptr;
  double* GT = (M != nullptr) ? ws.take<double>(2 * NN * nv) : nullptr;
  if (ws.sizing) return VES_OK;
  if (!ws.ok()) {
    ves_record_error(VES_ERR_WORKSPACE, "derivs: workspace too small");
    return VES_ERR_WORKSPACE;
  }
  if (nv <= 0) return VES_OK;
  dim3 grid(ceil_div(NN, 256), nv);
  ves_count_launch();
  arc_deriv_matrix_kernel<<<grid, 256, 0, s>>>(N, c->d1N, isa, Are, Aim);
  const long long sN = (long long)NN;
  // Cr = Are*Are - Aim*Aim ; Ci = Are*Aim + Aim*Are
  launch_bgemm_f64(nv, N, N, N, 1.0, Are, N, sN, Are, N, sN, 0.0, Cr, N, sN, s);
  launch_bgemm_f64(nv, N, N, N, -1.0, Aim, N, sN, Aim, N, sN, 1.0, Cr, N, sN, s);
  launch_bgemm_f64(nv, N, N, N, 1.0, Are, N, sN, Aim, N, sN, 0.0, Ci, N, sN, s);
  launch_bgemm_f64(nv, N, N, N, 1.0, Aim, N, sN, Are, N, sN, 1.0, Ci, N, sN, s);
  // D4 = Cr*Cr - Ci*Ci
  launch_bgemm_f64(nv, N, N, N, 1.0, Cr, N, sN, Cr, N, sN, 0.0, D4, N, sN, s);
  launch_bgemm_f64(nv, N, N, N, -1.0, Ci, N, sN, Ci, N, sN, 1.0, D4, N, sN, s);
  dim3 g2(ceil_div(4 * NN, 256), nv);
  if (Ben) {
    ves_count_launch();
    assemble_ben_kernel<<<g2, 256, 0, s>>>(N, D4, Ben);
  }
  ves_count_launch();
  assemble_ten_div_kernel<<<grid, 256, 0, s>>>(N, Are, tang, Ten, Div);
  if (M) {
    // GB = G * Ben: block structure G_ab * D4 for each 2x2 block
    // G rows r (2N), Ben = blockdiag(D4, D4): GB[:, 0:N] = G[:, 0:N] D4, GB[:, N:2N] = G[:, N:2N] D4
    const long long sG = 4 * sN;
    launch_bgemm_f64(nv, 2 * N, N, N, 1.0, G, 2 * N, sG, D4, N, sN, 0.0, GB, 2 * N, sG, s);
    launch_bgemm_f64(nv, 2 * N, N, N, 1.0, G + N, 2 * N, sG, D4, N, sN, 0.0, GB + N, 2 * N, sG, s);
    // GT = G * Ten (2N x 2N)(2N x N)
    launch_bgemm_f64(nv, 2 * N, N, 2 * N, 1.0, G, 2 * N, sG, Ten, N, 2 * sN, 0.0, GT, N, 2 * sN, s);
    dim3 g3(ceil_div(9 * NN, 256), nv);
    ves_count_launch();
    assemble_precond_kernel<<<g3, 256, 0, s>>>(N, dt, kappa, GB, GT, Div, Dm, alpha, M);
  }
  return ves_launch_check("derivs_and_precond");
}

// The preconditioner of derivs_and_precond (tstep_biem.py:653-711) with every
// product in FP32: [I + dt k G Ben, -dt G Ten; Div, 0] in FP32, for an FP32
// factorisation (GMRES only needs an approximate inverse).
int precond_f32(ves_ctx* c, int nv, const double* isa, const double* tang, const double* G, double dt, double kappa,
                float* M32, WsCarver& ws, cudaStream_t s) {
  const int N = c->N;
  const size_t NN = (size_t)N * N;
  float* Are = ws.take<float>(NN * nv);
  float* Aim = ws.take<float>(NN * nv);
  float* Cr = ws.take<float>(NN * nv);
  float* Ci = ws.take<float>(NN * nv);
  float* D4 = ws.take<float>(NN * nv);
  float* Ten = ws.take<float>(2 * NN * nv);
  float* Div = ws.take<float>(2 * NN * nv);
  float* G32 = ws.take<float>(4 * NN * nv);
  float* GB = ws.take<float>(4 * NN * nv);
  float* GT = ws.take<float>(2 * NN * nv);
  if (ws.sizing) return VES_OK;
  if (!ws.ok()) {
    ves_record_error(VES_ERR_WORKSPACE, "precond_f32: workspace too small");
    return VES_ERR_WORKSPACE;
  }
  if (nv <= 0) return VES_OK;
  dim3 grid(ceil_div(NN, 256), nv);
  ves_count_launch(3);
  arc_deriv_matrix_f32_kernel<<<grid, 256, 0, s>>>(N, c->d1N, isa, Are, Aim);
  ten_div_f32_kernel<<<grid, 256, 0, s>>>(N, Are, tang, Ten, Div);
  to_f32_kernel<<<ceil_div((long long)4 * NN * nv, 256), 256, 0, s>>>((long long)4 * NN * nv, G, G32);
  const long long sN = (long long)NN;
  launch_bgemm_f32(nv, N, N, N, 1.0f, Are, N, sN, Are, N, sN, 0.0f, Cr, N, sN, s);
  launch_bgemm_f32(nv, N, N, N, -1.0f, Aim, N, sN, Aim, N, sN, 1.0f, Cr, N, sN, s);
  launch_bgemm_f32(nv, N, N, N, 1.0f, Are, N, sN, Aim, N, sN, 0.0f, Ci, N, sN, s);
  launch_bgemm_f32(nv, N, N, N, 1.0f, Aim, N, sN, Are, N, sN, 1.0f, Ci, N, sN, s);
  launch_bgemm_f32(nv, N, N, N, 1.0f, Cr, N, sN, Cr, N, sN, 0.0f, D4, N, sN, s);
  launch_bgemm_f32(nv, N, N, N, -1.0f, Ci, N, sN, Ci, N, sN, 1.0f, D4, N, sN, s);
  const long long sG = 4 * sN;
  launch_bgemm_f32(nv, 2 * N, N, N, 1.0f, G32, 2 * N, sG, D4, N, sN, 0.0f, GB, 2 * N, sG, s);
  launch_bgemm_f32(nv, 2 * N, N, N, 1.0f, G32 + N, 2 * N, sG, D4, N, sN, 0.0f, GB + N, 2 * N, sG, s);
  launch_bgemm_f32(nv, 2 * N, N, 2 * N, 1.0f, G32, 2 * N, sG, Ten, N, 2 * sN, 0.0f, GT, N, 2 * sN, s);
  dim3 g3(ceil_div(9 * NN, 256), nv);
  ves_count_launch();
  assemble_precond_f32_kernel<<<g3, 256, 0, s>>>(N, (float)dt, (float)kappa, GB, GT, Div, M32);
  return ves_launch_check("precond_f32");
}
