// Shared definitions for the ves2d GB300 kernels (sm_103a).
//
// Device layout used by every kernel (vesicle-major, the transpose of the
// reference's X[2N, nv] column-per-vesicle tensors):
//   positions / densities  [nv][2][n]   (x row then y row of each vesicle)
//   tension                [nv][n]
//   per-vesicle matrices   [nv][rows][cols] row-major
//   GMRES state            [nv][3][N]   (x, y, sigma), the reference's flattening
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/ves2d_gb300.h"

#define VES_PI 3.14159265358979323846

// Device-side status word: kernels never trap; they record the first error
// code here and return.  The host reads it after the stage completes.
struct VesDeviceStatus {
  int code;      // VES_OK or a VES_ERR_* value
  int where;     // kernel-specific location tag
  long long aux; // kernel-specific detail (index that overflowed, ...)
};

__device__ __forceinline__ void ves_set_error(VesDeviceStatus* st, int code, int where, long long aux) {
  if (st == nullptr) return;
  if (atomicCAS(&st->code, VES_OK, code) == VES_OK) {
    st->where = where;
    st->aux = aux;
  }
}

template <typename T>
struct Vec2;
template <>
struct Vec2<float> {
  typedef float2 type;
};
template <>
struct Vec2<double> {
  typedef double2 type;
};

// Hardware approximate reciprocal and base-2 logarithm (MUFU), flush-to-zero.
__device__ __forceinline__ float mufu_rcp(float x) {
  float r;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
}
__device__ __forceinline__ float mufu_lg2(float x) {
  float r;
  asm("lg2.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
}

static inline unsigned ceil_div(long long a, long long b) { return (unsigned)((a + b - 1) / b); }

// Host helper: map a CUDA error to a status code, recording the message.
int ves_cuda_status(cudaError_t e, const char* what);
void ves_record_error(int code, const char* fmt, ...);
