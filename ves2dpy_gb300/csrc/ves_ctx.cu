// Context creation: the per-N constant tables of Poten.__init__
// (mytorch/poten.py:15-37), built on the host in double precision from the
// closed-form trigonometric sums and uploaded once.
#include <math.h>
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <vector>

#include "ves_internal.h"

#include <atomic>

static thread_local char g_last_error[512] = "no error";
static std::atomic<long long> g_launches{0};

void ves_count_launch(int n) { g_launches.fetch_add(n, std::memory_order_relaxed); }

static void ff_drain(ves_ctx* c) {
  for (int i = 0; i < c->n_ev; ++i) {
    float ms = 0.f;
    cudaEventSynchronize(c->ev[2 * i + 1]);
    cudaEventElapsedTime(&ms, c->ev[2 * i], c->ev[2 * i + 1]);
    c->ff_ms += ms;
    c->ff_pairs += c->ev_pairs[i];
    c->ff_launches += 1;
  }
  c->n_ev = 0;
}

static void net_drain(ves_ctx* c) {
  for (int i = 0; i < c->n_nev; ++i) {
    float ms = 0.f;
    cudaEventSynchronize(c->nev[2 * i + 1]);
    cudaEventElapsedTime(&ms, c->nev[2 * i], c->nev[2 * i + 1]);
    c->net_ms += ms;
    c->net_flops += c->nev_flops[i];
    c->net_launches += 1;
  }
  c->n_nev = 0;
}

void ves_net_timing_begin(ves_ctx* c, cudaStream_t s) {
  if (!c || !c->timing) return;
  if (c->n_nev == 64) net_drain(c);
  cudaEventRecord(c->nev[2 * c->n_nev], s);
}

void ves_net_timing_end(ves_ctx* c, cudaStream_t s, double flops) {
  if (!c || !c->timing) return;
  cudaEventRecord(c->nev[2 * c->n_nev + 1], s);
  c->nev_flops[c->n_nev] = flops;
  c->n_nev++;
}

void ves_ff_timing_begin(ves_ctx* c, cudaStream_t s) {
  if (!c->timing) return;
  if (c->n_ev == 256) ff_drain(c);
  cudaEventRecord(c->ev[2 * c->n_ev], s);
}

void ves_ff_timing_end(ves_ctx* c, cudaStream_t s, double pairs) {
  if (!c->timing) return;
  cudaEventRecord(c->ev[2 * c->n_ev + 1], s);
  c->ev_pairs[c->n_ev] = pairs;
  c->n_ev++;
}

extern "C" int ves_ctx_set_timing(ves_ctx* c, int on) {
  if (!c) return VES_ERR_ARG;
  if (on && !c->ev[0]) {
    for (int i = 0; i < 2 * 256; ++i) {
      int rc = ves_cuda_status(cudaEventCreate(&c->ev[i]), "cudaEventCreate");
      if (rc) return rc;
    }
  }
  if (on && !c->nev[0]) {
    for (int i = 0; i < 2 * 64; ++i) {
      int rc = ves_cuda_status(cudaEventCreate(&c->nev[i]), "cudaEventCreate");
      if (rc) return rc;
    }
  }
  if (on && !c->d_mp) {
    int rc = ves_cuda_status(cudaMalloc(&c->d_mp, 2 * sizeof(unsigned long long)), "counters");
    if (!rc) rc = ves_cuda_status(cudaMemset(c->d_mp, 0, 2 * sizeof(unsigned long long)), "counters");
    if (rc) return rc;
  }
  if (!on && c->n_ev) ff_drain(c);
  if (!on && c->n_nev) net_drain(c);
  c->timing = on ? 1 : 0;
  return VES_OK;
}

extern "C" int ves_ctx_stats(ves_ctx* c, ves_stats* out, int reset) {
  if (!c || !out) return VES_ERR_ARG;
  ff_drain(c);
  net_drain(c);
  out->kernel_launches = g_launches.load();
  out->networks_launches = c->net_launches;
  out->networks_ms = c->net_ms;
  out->networks_flops = c->net_flops;
  out->farfield_launches = c->ff_launches;
  out->farfield_ms = c->ff_ms;
  out->farfield_pairs = c->ff_pairs;
  out->farfield_mp_terms = 0;
  out->farfield_direct_pairs = 0;
  if (c->d_mp) {
    unsigned long long h[2] = {0, 0};
    int rc = ves_cuda_status(cudaMemcpy(h, c->d_mp, sizeof(h), cudaMemcpyDeviceToHost), "counters");
    if (rc) return rc;
    out->farfield_mp_terms = (double)h[0];
    out->farfield_direct_pairs = (double)h[1];
  }
  if (reset) {
    c->ff_launches = 0;
    c->ff_ms = 0;
    c->ff_pairs = 0;
    c->net_launches = 0;
    c->net_ms = 0;
    c->net_flops = 0;
    if (c->d_mp) cudaMemset(c->d_mp, 0, 2 * sizeof(unsigned long long));
  }
  return VES_OK;
}

// MUFU probe: independent lg2/rcp chains, 8 per thread
__global__ void sfu_probe_kernel(int iters, float seed, float* out) {
  float a[8];
#pragma unroll
  for (int i = 0; i < 8; ++i) a[i] = seed + 0.001f * (threadIdx.x + i);
  for (int it = 0; it < iters; ++it) {
#pragma unroll
    for (int i = 0; i < 8; ++i) {
      float r = mufu_lg2(a[i]);
      a[i] = mufu_rcp(r + 2.0f);
    }
  }
  float s = 0.f;
#pragma unroll
  for (int i = 0; i < 8; ++i) s += a[i];
  if (s == 12345.678f) out[0] = s;  // keep the work alive
}

extern "C" int ves_probe_sfu_peak(double* ops_per_second, void* stream) {
  if (!ops_per_second) return VES_ERR_ARG;
  cudaStream_t s = (cudaStream_t)stream;
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  float* out = nullptr;
  int rc = ves_cuda_status(cudaMallocAsync(&out, sizeof(float), s), "probe alloc");
  if (rc) return rc;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  const int blocks = sms * 8, threads = 256, iters = 4096;
  sfu_probe_kernel<<<blocks, threads, 0, s>>>(64, 1.5f, out);  // warm-up
  cudaEventRecord(e0, s);
  sfu_probe_kernel<<<blocks, threads, 0, s>>>(iters, 1.5f, out);
  cudaEventRecord(e1, s);
  ves_count_launch(2);
  rc = ves_cuda_status(cudaEventSynchronize(e1), "probe");
  float ms = 0.f;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFreeAsync(out, s);
  if (rc) return rc;
  *ops_per_second = (double)blocks * threads * iters * 8 * 2 / (ms * 1e-3);
  return VES_OK;
}

void ves_record_error(int code, const char* fmt, ...) {
  char msg[448];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(msg, sizeof(msg), fmt, ap);
  va_end(ap);
  snprintf(g_last_error, sizeof(g_last_error), "[status %d] %s", code, msg);
}

extern "C" const char* ves_last_error(void) { return g_last_error; }

int ves_cuda_status(cudaError_t e, const char* what) {
  if (e == cudaSuccess) return VES_OK;
  ves_record_error(VES_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
  return VES_ERR_CUDA;
}

int ves_launch_check(const char* what) { return ves_cuda_status(cudaGetLastError(), what); }

int ves_reset_status(ves_ctx* ctx, cudaStream_t s) {
  ctx->last_max_cand = 0;
  return ves_cuda_status(cudaMemsetAsync(ctx->status, 0, sizeof(VesDeviceStatus), s), "reset status");
}

int ves_check_status(ves_ctx* ctx, cudaStream_t s, const char* stage) {
  int rc = ves_cuda_status(
      cudaMemcpyAsync(ctx->h_status, ctx->status, sizeof(VesDeviceStatus), cudaMemcpyDeviceToHost, s),
      stage);
  if (rc) return rc;
  rc = ves_cuda_status(cudaStreamSynchronize(s), stage);
  if (rc) return rc;
  if (ctx->h_status->code != VES_OK) {
    ves_record_error(ctx->h_status->code, "%s: device status %d at site %d (detail %lld)", stage,
                     ctx->h_status->code, ctx->h_status->where, ctx->h_status->aux);
    return ctx->h_status->code;
  }
  return VES_OK;
}

// ---------------------------------------------------------------------------
// closed-form tables

// Cardinal function of N-point trig interpolation with the interpft
// convention (filter.py:221-249): the Nyquist mode -N/2 is kept whole, so its
// real part contributes cos(N/2 t).
static double cardinal(int N, double t) {
  double s = 1.0;
  for (int k = 1; k < N / 2; ++k) s += 2.0 * cos(k * t);
  s += cos(0.5 * N * t);
  return s / N;
}
static double cardinal_deriv(int N, double t) {
  double s = 0.0;
  for (int k = 1; k < N / 2; ++k) s -= 2.0 * k * sin(k * t);
  s -= 0.5 * N * sin(0.5 * N * t);
  return s / N;
}
static double cardinal_deriv2(int N, double t) {
  double s = 0.0;
  for (int k = 1; k < N / 2; ++k) s -= 2.0 * (double)k * k * cos(k * t);
  s -= 0.25 * N * N * cos(0.5 * N * t);
  return s / N;
}
// Entry (node at offset y, grid point r) of sinterpS_ (fft1.py:58-88).  Its
// mode list puts frequency 0 in the Nyquist slot of the FFT, so the Nyquist
// coefficient enters with weight exp(0) = 1: a (-1)^r / n term.
static double sinc_row(int n, double y, int r) {
  const double t = y - 2.0 * VES_PI * r / n;
  double s = 1.0;
  for (int k = 1; k < n / 2; ++k) s += 2.0 * cos(k * t);
  s += (r & 1) ? -1.0 : 1.0;
  return s / n;
}
// First-derivative circulant with the Nyquist mode zeroed (fft1.py:185-196
// modes, used by arcDeriv and getDXY): d[r] = -(2/n) sum_k k sin(2 pi k r / n).
static double deriv_circ(int n, int r) {
  double s = 0.0;
  for (int k = 1; k < n / 2; ++k) s -= 2.0 * k * sin(2.0 * VES_PI * k * r / n);
  return s / n;
}

static const double kAlpertV[7] = {6.531815708567918e-3, 9.086744584657729e-2, 3.967966533375878e-1,
                                   1.027856640525646e+0, 1.945288592909266e+0, 2.980147933889640e+0,
                                   3.998861349951123e+0};
static const double kAlpertU[7] = {2.462194198995203e-2, 1.701315866854178e-1, 4.609256358650077e-1,
                                   7.947291148621895e-1, 1.008710414337933e+0, 1.036093649726216e+0,
                                   1.004787656533285e+0};
static const double kLagrange[49] = {
    64.80,  -388.80, 972.00,  -1296.00, 972.00,  -388.80, 64.80,  -226.80, 1296.00, -3078.00,
    3888.00, -2754.00, 1036.80, -162.00, 315.00, -1674.00, 3699.00, -4356.00, 2889.00, -1026.00,
    153.00, -220.50, 1044.00, -2074.50, 2232.00, -1381.50, 468.00, -67.50,  81.20,   -313.20,
    526.50, -508.00, 297.00,  -97.20,  13.70,   -14.70,  36.00,  -45.00,  40.00,   -22.50,
    7.20,   -1.00,   1.00,    0.00,    0.00,    0.00,    0.00,   0.00,    0.00};

// Offset (relative to the target parameter) of Alpert dense node q in 0..13:
// rows of A1 at v*h and of A2 at 2pi - flip(v*h) (poten.py:938-939).
static double alpert_offset(int q, int Nup) {
  const double h = 2.0 * VES_PI / Nup;
  if (q < 7) return kAlpertV[q] * h;
  return 2.0 * VES_PI - kAlpertV[6 - (q - 7)] * h;
}

extern "C" int ves_ctx_create(int N, ves_ctx** out) {
  if (!out) return VES_ERR_ARG;
  *out = nullptr;
  if (N < 8 || (N % 2) != 0 || N > 1024) {
    ves_record_error(VES_ERR_SHAPE, "N=%d unsupported (even, 8..1024)", N);
    return VES_ERR_SHAPE;
  }
  ves_ctx* c = (ves_ctx*)calloc(1, sizeof(ves_ctx));
  c->N = N;
  c->m = (int)ceil(sqrt((double)N));
  c->Nup = N * c->m;
  const int Nup = c->Nup;
  c->nquad = Nup + 5;
  c->nwords_N = (N + 31) / 32;
  c->nwords_up = (Nup + 31) / 32;
  int rc = ves_cuda_status(cudaGetDevice(&c->device), "cudaGetDevice");
  if (rc) {
    free(c);
    return rc;
  }
  // host tables
  std::vector<double> d1N(N), d1Nup(Nup), pc(Nup), pcd(Nup), pcdd(Nup), qw(c->nquad), cq(14 * Nup),
      ad(14 * Nup), Rm((size_t)N * Nup), Pm((size_t)Nup * N), lag(49), cos6(6 * N),
      sin6(6 * N), cosU(Nup), sinU(Nup);
  for (int r = 0; r < 6 * N; ++r) {
    const double t = 2.0 * VES_PI * r / (6 * N);
    cos6[r] = cos(t);
    sin6[r] = sin(t);
  }
  for (int r = 0; r < N; ++r) d1N[r] = deriv_circ(N, r);
  for (int r = 0; r < Nup; ++r) d1Nup[r] = deriv_circ(Nup, r);
  for (int r = 0; r < Nup; ++r) {
    double t = 2.0 * VES_PI * r / Nup;
    pc[r] = cardinal(N, t);
    pcd[r] = cardinal_deriv(N, t);
    pcdd[r] = cardinal_deriv2(N, t);
    cosU[r] = cos(t);
    sinU[r] = sin(t);
  }
  {
    const double h = 2.0 * VES_PI / Nup;
    const int n = Nup - 2 * 5 + 1;
    int q = 0;
    for (int j = 0; j < 7; ++j) qw[q++] = h * kAlpertU[j] / (4 * VES_PI);
    for (int j = 0; j < n; ++j) qw[q++] = h / (4 * VES_PI);
    for (int j = 0; j < 7; ++j) qw[q++] = h * kAlpertU[6 - j] / (4 * VES_PI);
  }
  for (int q = 0; q < 14; ++q) {
    double y = alpert_offset(q, Nup);
    for (int r = 0; r < Nup; ++r) {
      double t = 2.0 * VES_PI * r / Nup;
      cq[q * Nup + r] = cardinal(N, t + y);    // x(theta_s + y) = sum_i x_i C(theta_s - theta_i + y)
      ad[q * Nup + r] = sinc_row(Nup, y, r);   // weight of grid point r for the node at y
    }
  }
  for (int i = 0; i < N; ++i)
    for (int u = 0; u < Nup; ++u) {
      int r = ((u - c->m * i) % Nup + Nup) % Nup;
      Pm[(size_t)u * N + i] = pc[r];
      Rm[(size_t)i * Nup + u] = pc[r] * (double)N / Nup;
    }
  for (int i = 0; i < 49; ++i) lag[i] = kLagrange[i];

  // one device buffer
  size_t nd = d1N.size() + d1Nup.size() + pc.size() + pcd.size() + pcdd.size() + qw.size() + cq.size() + ad.size() +
              Rm.size() + Pm.size() + lag.size() + 2 * cos6.size() + 2 * cosU.size();
  size_t nf = Rm.size() + Pm.size() + ad.size() + qw.size();
  size_t bytes = nd * sizeof(double) + nf * sizeof(float) + 1024;
  rc = ves_cuda_status(cudaMalloc(&c->d_buf, bytes), "cudaMalloc tables");
  if (rc) {
    free(c);
    return rc;
  }
  double* p = (double*)c->d_buf;
  auto put = [&](std::vector<double>& v) {
    double* d = p;
    cudaMemcpy(d, v.data(), v.size() * sizeof(double), cudaMemcpyHostToDevice);
    p += v.size();
    return d;
  };
  c->d1N = put(d1N);
  c->d1Nup = put(d1Nup);
  c->pc = put(pc);
  c->pcd = put(pcd);
  c->pcdd = put(pcdd);
  c->qw = put(qw);
  c->cq = put(cq);
  c->adense = put(ad);
  c->Rm = put(Rm);
  c->Pm = put(Pm);
  c->lag = put(lag);
  c->cos6 = put(cos6);
  c->sin6 = put(sin6);
  c->cosU = put(cosU);
  c->sinU = put(sinU);
  float* pf = (float*)p;
  auto putf = [&](std::vector<double>& v) {
    std::vector<float> h(v.begin(), v.end());
    float* d = pf;
    cudaMemcpy(d, h.data(), h.size() * sizeof(float), cudaMemcpyHostToDevice);
    pf += h.size();
    return d;
  };
  c->Rm32 = putf(Rm);
  c->Pm32 = putf(Pm);
  c->adense32 = putf(ad);
  c->qw32 = putf(qw);
  rc = ves_cuda_status(cudaMalloc(&c->status, sizeof(VesDeviceStatus)), "cudaMalloc status");
  if (!rc) rc = ves_cuda_status(cudaMemset(c->status, 0, sizeof(VesDeviceStatus)), "memset status");
  if (!rc)
    rc = ves_cuda_status(cudaMallocHost(&c->h_status, sizeof(VesDeviceStatus)), "cudaMallocHost");
  if (!rc) rc = ves_cuda_status(cudaMallocHost(&c->h_scal, 256 * sizeof(double)), "cudaMallocHost scal");
  if (!rc) rc = ves_cuda_status(cudaMallocHost(&c->h_ints, 16 * sizeof(int)), "cudaMallocHost ints");
  if (!rc) rc = ves_cuda_status(cudaDeviceSynchronize(), "table upload");
  if (rc) {
    ves_ctx_destroy(c);
    return rc;
  }
  *out = c;
  return VES_OK;
}

extern "C" int ves_ctx_destroy(ves_ctx* c) {
  if (!c) return VES_OK;
  if (c->d_buf) cudaFree(c->d_buf);
  if (c->status) cudaFree(c->status);
  if (c->h_status) cudaFreeHost(c->h_status);
  if (c->h_scal) cudaFreeHost(c->h_scal);
  if (c->h_ints) cudaFreeHost(c->h_ints);
  if (c->ev[0])
    for (int i = 0; i < 2 * 256; ++i) cudaEventDestroy(c->ev[i]);
  if (c->d_mp) cudaFree(c->d_mp);
  if (c->nev[0])
    for (int i = 0; i < 2 * 64; ++i) cudaEventDestroy(c->nev[i]);
  free(c);
  return VES_OK;
}

extern "C" int ves_ctx_max_candidates(const ves_ctx* c) { return c ? c->last_max_cand : -1; }

extern "C" int ves_ctx_info(const ves_ctx* c, int* N, int* Nup, int* nquad) {
  if (!c) return VES_ERR_ARG;
  if (N) *N = c->N;
  if (Nup) *Nup = c->Nup;
  if (nquad) *nquad = c->nquad;
  return VES_OK;
}
