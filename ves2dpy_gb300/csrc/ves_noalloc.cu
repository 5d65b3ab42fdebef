// All-pairs Stokeslet sum for callers that cannot allocate device memory.
//
// Same kernels and arithmetic as ves_farfield (no near-pair lists), but the
// scratch (staged source records, centres, partial sums and the device status
// word) lives in one file-scope device array that is part of the library's
// device image, so a call performs no cudaMalloc/cudaFree and calls no
// allocating library routine.
//
// * The array is VES_STATIC_SCRATCH_BYTES long; every GPU that loads the
//   library holds it until the process exits.
// * Host code cannot use the array's name as a device address.  The first
//   call on each device resolves the address with cudaGetSymbolAddress (with
//   that device current) and caches it for the life of the device's primary
//   context; make that first call before any stream capture, and make no call
//   after a cudaDeviceReset in the same process (the cached address would be
//   stale).
// * Every call shares the array and leaves its contents behind; the status
//   word is cleared at the start of each call and every other byte a call
//   reads is written earlier in the same call.  Calls that overlap on the GPU
//   (other streams or other host threads) race on the array and must be
//   serialised by the caller.
#include <mutex>

#include "ves_internal.h"

static __device__ __align__(256) unsigned char g_static_scratch[VES_STATIC_SCRATCH_BYTES];

namespace {

constexpr int kMaxDevices = 64;
std::mutex g_scratch_mu;
void* g_scratch_addr[kMaxDevices] = {};

// Device address of g_static_scratch on the current device (resolved once).
int static_scratch_address(void** out) {
  int dev = 0;
  int rc = ves_cuda_status(cudaGetDevice(&dev), "cudaGetDevice");
  if (rc) return rc;
  if (dev < 0 || dev >= kMaxDevices) {
    ves_record_error(VES_ERR_ARG, "static scratch: device %d out of range", dev);
    return VES_ERR_ARG;
  }
  std::lock_guard<std::mutex> lock(g_scratch_mu);
  if (!g_scratch_addr[dev]) {
    void* p = nullptr;
    rc = ves_cuda_status(cudaGetSymbolAddress(&p, g_static_scratch), "cudaGetSymbolAddress(static scratch)");
    if (rc) return rc;
    g_scratch_addr[dev] = p;
  }
  *out = g_scratch_addr[dev];
  return VES_OK;
}

}  // namespace

extern "C" int ves_farfield_static_scratch(int precision, int nsrc, int ns, const double* Xsrc, const double* den,
                                           int nt, int ntp, const double* Xtar, const int* self_idx, double* out,
                                           void* stream) {
  if (!Xsrc || !den || !Xtar || !out || nsrc < 0 || ns <= 0 || nt < 0 || ntp <= 0) {
    ves_record_error(VES_ERR_ARG, "ves_farfield_static_scratch: bad arguments");
    return VES_ERR_ARG;
  }
  if (precision != VES_PREC_FP64 && precision != VES_PREC_FP32C && precision != VES_PREC_FP32M) {
    ves_record_error(VES_ERR_ARG, "ves_farfield_static_scratch: bad precision %d", precision);
    return VES_ERR_ARG;
  }
  cudaStream_t s = (cudaStream_t)stream;
  // the first 256 bytes hold the status word, the rest is the workspace
  const size_t cap = VES_STATIC_SCRATCH_BYTES - 256;
  FFEnv env;
  env.status = nullptr;
  env.N = ntp;
  env.timing = nullptr;
  WsCarver sizing(nullptr, 0);
  farfield_run_env(env, precision, nsrc, ns, nullptr, nullptr, nt, ntp, nullptr, nullptr, nullptr, nullptr, sizing, s);
  if (sizing.off > cap) {
    ves_record_error(VES_ERR_WORKSPACE,
                     "ves_farfield_static_scratch: these sizes need %zu bytes of scratch, the static array holds %zu "
                     "(use ves_farfield with a caller-provided workspace)",
                     sizing.off, cap);
    return VES_ERR_WORKSPACE;
  }
  void* base = nullptr;
  int rc = static_scratch_address(&base);
  if (rc) return rc;
  VesDeviceStatus* st = (VesDeviceStatus*)base;
  env.status = st;
  rc = ves_cuda_status(cudaMemsetAsync(st, 0, sizeof(VesDeviceStatus), s), "clear status");
  if (rc) return rc;
  WsCarver w((char*)base + 256, cap);
  rc = farfield_run_env(env, precision, nsrc, ns, Xsrc, den, nt, ntp, Xtar, self_idx, nullptr, out, w, s);
  if (rc) return rc;
  VesDeviceStatus h;
  rc = ves_cuda_status(cudaMemcpyAsync(&h, st, sizeof(h), cudaMemcpyDeviceToHost, s), "read status");
  if (!rc) rc = ves_cuda_status(cudaStreamSynchronize(s), "ves_farfield_static_scratch");
  if (rc) return rc;
  if (h.code != VES_OK) {
    ves_record_error(h.code, "ves_farfield_static_scratch: device status %d at site %d", h.code, h.where);
    return h.code;
  }
  return VES_OK;
}
