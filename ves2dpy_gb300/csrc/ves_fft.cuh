// FP64 FFT of one sequence in shared memory, by one CTA, for lengths
// M = P or M = 3 P with P a power of two (the arc-length grid 6N and the
// upsampled grid N*ceil(sqrt(N)) for N = 32, 128).  Decimation in time: the
// input is split into R = M / P interleaved subsequences x[R m + r], each
// transformed by an iterative radix-2 FFT of length P, then combined by one
// radix-3 pass.  Twiddles come from a table of cos/sin(2 pi j / M).
//
//   sign = -1:  X[k] = sum_n x[n] exp(-2 pi i k n / M)   (forward, unnormalised)
//   sign = +1:  X[k] = sum_n x[n] exp(+2 pi i k n / M)   (inverse, unnormalised)
#pragma once

#include <cuda_runtime.h>

__host__ __device__ inline bool ves_fft_size_ok(int M) {
  int P = (M % 3 == 0) ? M / 3 : M;
  return P >= 2 && (P & (P - 1)) == 0;
}

__device__ __forceinline__ int ves_bitrev(int v, int bits) { return (int)(__brev((unsigned)v) >> (32 - bits)); }

// re/im: input and output [M]; tre/tim: scratch [M]; cs/sn: cos/sin(2 pi j / (ts M)),
// j < ts M (a table of a longer length ts*M is read with stride ts).
__device__ inline void ves_fft(double* re, double* im, double* tre, double* tim, int M, const double* __restrict__ cs,
                               const double* __restrict__ sn, int sign, int ts = 1) {
  __syncthreads();
  const int R = (M % 3 == 0) ? 3 : 1;
  const int P = M / R;
  const int bits = __ffs(P) - 1;
  // scatter the R subsequences in bit-reversed order: t[r*P + rev(m)] = x[R m + r]
  for (int i = threadIdx.x; i < M; i += blockDim.x) {
    const int r = i % R, m = i / R;
    const int dst = r * P + ves_bitrev(m, bits);
    tre[dst] = re[i];
    tim[dst] = im[i];
  }
  __syncthreads();
  // radix-2 butterflies on each subsequence; stage half-size h: twiddle exp(sign 2 pi i j / (2h))
  for (int h = 1; h < P; h <<= 1) {
    const int stride = ts * (M / (2 * h));  // table step for exp(2 pi i j / (2h))
    for (int b = threadIdx.x; b < R * (P / 2); b += blockDim.x) {
      const int r = b / (P / 2), bb = b % (P / 2);
      const int g = bb / h, j = bb % h;
      const int i0 = r * P + g * 2 * h + j, i1 = i0 + h;
      const double wr = cs[j * stride], wi = sign * sn[j * stride];
      const double vr = tre[i1] * wr - tim[i1] * wi;
      const double vi = tre[i1] * wi + tim[i1] * wr;
      const double ur = tre[i0], ui = tim[i0];
      tre[i0] = ur + vr;
      tim[i0] = ui + vi;
      tre[i1] = ur - vr;
      tim[i1] = ui - vi;
    }
    __syncthreads();
  }
  if (R == 1) {
    for (int i = threadIdx.x; i < M; i += blockDim.x) {
      re[i] = tre[i];
      im[i] = tim[i];
    }
    __syncthreads();
    return;
  }
  // radix-3 combination: X[k + q P] = sum_r w^(r (k + q P)) X_r[k],  w = exp(sign 2 pi i / M)
  for (int k = threadIdx.x; k < P; k += blockDim.x) {
    const double x0r = tre[k], x0i = tim[k];
    const double w1r = cs[ts * k], w1i = sign * sn[ts * k];
    const double w2r = cs[ts * 2 * k], w2i = sign * sn[ts * 2 * k];
    const double y1r = tre[P + k] * w1r - tim[P + k] * w1i, y1i = tre[P + k] * w1i + tim[P + k] * w1r;
    const double y2r = tre[2 * P + k] * w2r - tim[2 * P + k] * w2i, y2i = tre[2 * P + k] * w2i + tim[2 * P + k] * w2r;
    // exp(sign 2 pi i / 3) = -1/2 + sign i sqrt(3)/2
    const double c3 = -0.5, s3 = sign * 0.86602540378443864676;
    const double ar = y1r + y2r, ai = y1i + y2i;       // y1 + y2
    const double dr = y1r - y2r, di = y1i - y2i;       // y1 - y2
    re[k] = x0r + ar;
    im[k] = x0i + ai;
    // q = 1: x0 + y1 w3 + y2 w3^2 = x0 + c3 (y1 + y2) + i s3 (y1 - y2)
    re[k + P] = x0r + c3 * ar - s3 * di;
    im[k + P] = x0i + c3 * ai + s3 * dr;
    // q = 2: x0 + y1 w3^2 + y2 w3^4 = x0 + c3 (y1 + y2) - i s3 (y1 - y2)
    re[k + 2 * P] = x0r + c3 * ar + s3 * di;
    im[k + 2 * P] = x0i + c3 * ai - s3 * dr;
  }
  __syncthreads();
}
