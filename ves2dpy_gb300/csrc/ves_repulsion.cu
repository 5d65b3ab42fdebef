// Artificial repulsion between vesicles (capsules.repulsionForce,
// mytorch/capsules.py:209-252; discrete penalty layers of Grinspun et al.
// 2009).  For target point i of vesicle a:
//
//   rep(i, a) = W * sum_{b != a} sum_j dF(d) * (X(i, a) - X(j, b)),
//   d = sqrt(|X(i, a) - X(j, b)|^2 + 1e-10),  L = floor(eta / d),
//   dF = -L (2L + 1)(L + 1) / 3 + L (L + 1) eta / d.
//
// L = 0 (so dF = 0 exactly) whenever d > eta, so only vesicles whose
// bounding boxes come within eta contribute: one CTA per target vesicle scans
// all bounding boxes, stages each candidate's points in shared memory and
// sums the pairs in FP64.  The reference forms the dense (N, N, nv, nv)
// array; the result differs from it only by summation order.
#include "ves_internal.h"

namespace {

// per-vesicle bounding box [xmin, xmax, ymin, ymax]
__global__ void rep_bbox_kernel(int N, int nv, const double* __restrict__ X, double4* __restrict__ box) {
  const int v = blockIdx.x * blockDim.y + threadIdx.y;
  if (v >= nv) return;
  const double* x = X + (long long)v * 2 * N;
  double x0 = 1e300, x1 = -1e300, y0 = 1e300, y1 = -1e300;
  for (int j = threadIdx.x; j < N; j += 32) {
    x0 = fmin(x0, x[j]);
    x1 = fmax(x1, x[j]);
    y0 = fmin(y0, x[N + j]);
    y1 = fmax(y1, x[N + j]);
  }
  for (int o = 16; o > 0; o >>= 1) {
    x0 = fmin(x0, __shfl_xor_sync(0xffffffffu, x0, o));
    x1 = fmax(x1, __shfl_xor_sync(0xffffffffu, x1, o));
    y0 = fmin(y0, __shfl_xor_sync(0xffffffffu, y0, o));
    y1 = fmax(y1, __shfl_xor_sync(0xffffffffu, y1, o));
  }
  if (threadIdx.x == 0) box[v] = make_double4(x0, x1, y0, y1);
}

// one CTA per target vesicle, one thread per target point (blockDim >= N, a warp multiple)
__global__ void rep_force_kernel(int N, int nv, const double* __restrict__ X, const double4* __restrict__ box,
                                 double W, double eta, double* __restrict__ out) {
  extern __shared__ double srcxy[];  // [2][N] of the candidate
  __shared__ int cand[256];
  __shared__ int ncand;
  const int a = blockIdx.x, i = threadIdx.x;
  const bool valid = i < N;
  const double* xa = X + (long long)a * 2 * N;
  const double xi = valid ? xa[i] : 0.0, yi = valid ? xa[N + i] : 0.0;
  const double4 ba = box[a];
  double ax = 0.0, ay = 0.0;
  for (int b0 = 0; b0 < nv; b0 += 256) {
    if (i == 0) ncand = 0;
    __syncthreads();
    for (int q = i; q < 256 && b0 + q < nv; q += blockDim.x) {
      const int b = b0 + q;
      const double4 bb = box[b];
      // boxes closer than eta in both directions (a pair farther apart contributes exactly 0)
      const bool near = b != a && bb.x <= ba.y + eta && ba.x <= bb.y + eta && bb.z <= ba.w + eta && ba.z <= bb.w + eta;
      if (near) cand[atomicAdd(&ncand, 1)] = b;
    }
    __syncthreads();
    const int nc = ncand;
    for (int c = 0; c < nc; ++c) {
      const double* xb = X + (long long)cand[c] * 2 * N;
      __syncthreads();
      for (int j = i; j < 2 * N; j += blockDim.x) srcxy[j] = xb[j];
      __syncthreads();
      if (valid) {
        for (int j = 0; j < N; ++j) {
          const double dx = xi - srcxy[j], dy = yi - srcxy[N + j];
          const double d = sqrt(dx * dx + dy * dy + 1e-10);
          const double L = floor(eta / d);
          if (L > 0.0) {
            const double dF = -L * (2.0 * L + 1.0) * (L + 1.0) / 3.0 + L * (L + 1.0) * eta / d;
            ax += dF * dx;
            ay += dF * dy;
          }
        }
      }
    }
    __syncthreads();
  }
  if (valid) {
    out[(long long)a * 2 * N + i] = W * ax;
    out[(long long)a * 2 * N + N + i] = W * ay;
  }
}

}  // namespace

extern "C" size_t ves_repulsion_force_workspace(int nv) { return (size_t)(nv > 0 ? nv : 0) * sizeof(double4) + 256; }

extern "C" int ves_repulsion_force(int N, int nv, const double* X, double W, double eta, double* out, void* ws,
                                   size_t ws_bytes, void* stream) {
  if (N <= 0 || nv < 0 || !(eta >= 0.0) || (nv > 0 && (!X || !out || !ws))) {
    ves_record_error(VES_ERR_ARG, "repulsion_force: bad arguments");
    return VES_ERR_ARG;
  }
  if (N > 1024) {
    ves_record_error(VES_ERR_SHAPE, "repulsion_force: at most 1024 points per vesicle");
    return VES_ERR_SHAPE;
  }
  if (ws_bytes < ves_repulsion_force_workspace(nv)) {
    ves_record_error(VES_ERR_WORKSPACE, "repulsion_force: workspace too small");
    return VES_ERR_WORKSPACE;
  }
  if (nv == 0) return VES_OK;
  cudaStream_t s = (cudaStream_t)stream;
  double4* box = reinterpret_cast<double4*>((reinterpret_cast<uintptr_t>(ws) + 31) & ~(uintptr_t)31);
  ves_count_launch(2);
  rep_bbox_kernel<<<ceil_div(nv, 8), dim3(32, 8), 0, s>>>(N, nv, X, box);
  const int threads = ((N + 31) / 32) * 32;
  rep_force_kernel<<<nv, threads, (size_t)2 * N * sizeof(double), s>>>(N, nv, X, box, W, eta, out);
  return ves_launch_check("repulsion_force");
}
