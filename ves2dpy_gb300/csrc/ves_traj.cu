// Trajectory files in the reference's format (driver_confined.py:204-206
// header and initial shapes, :294-296 one frame per step; read back by
// newtorch/tools/load_ves2d_file.py:4-72): little-endian float64 throughout,
//
//   N, nv, then the initial shapes; per frame: time, then the shapes,
//
// shapes vesicle by vesicle, the N x coordinates then the N y coordinates
// (X.T.flatten() of the reference's X[2N, nv]), which is the device layout
// [nv][2][N] of this library: a frame is one contiguous copy.
//
// Writing never stalls the step: ves_traj_append records an asynchronous
// device-to-host copy of the frame into one of a ring of pinned slots on the
// caller's stream and returns; a background thread waits for each copy and
// writes the frames in order.  The caller blocks only when every slot is
// still waiting for the disk.
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <condition_variable>
#include <deque>
#include <mutex>
#include <new>
#include <thread>
#include <vector>

#include "ves_internal.h"

struct ves_traj {
  FILE* f = nullptr;
  int N = 0, nv = 0;
  size_t frame = 0;  // doubles per frame: time + 2 N nv
  std::vector<double*> slot;
  std::vector<cudaEvent_t> ev;
  std::vector<int> busy;     // 1 while a slot is queued or being written
  std::vector<int> on_dev;   // the slot's data arrives by an asynchronous copy
  std::deque<int> queue;     // slots in write order
  int next = 0;
  std::mutex mu;
  std::condition_variable cv;
  std::thread writer;
  bool stop = false;
  int err = VES_OK;          // first write or copy failure, reported by every later call
  long long frames = 0;
  bool pinned = false;       // slots are pinned (a GPU is present)
};

namespace {

void writer_loop(ves_traj* t) {
  std::unique_lock<std::mutex> lk(t->mu);
  for (;;) {
    t->cv.wait(lk, [t] { return t->stop || !t->queue.empty(); });
    if (t->queue.empty()) return;  // stop requested and nothing left
    const int k = t->queue.front();
    lk.unlock();
    int rc = VES_OK;
    if (t->on_dev[k] && cudaEventSynchronize(t->ev[k]) != cudaSuccess) rc = VES_ERR_CUDA;
    if (rc == VES_OK && fwrite(t->slot[k], sizeof(double), t->frame, t->f) != t->frame) rc = VES_ERR_ARG;
    lk.lock();
    if (rc != VES_OK && t->err == VES_OK) t->err = rc;
    t->queue.pop_front();
    t->busy[k] = 0;
    ++t->frames;
    t->cv.notify_all();
  }
}

void traj_free(ves_traj* t) {
  if (t->writer.joinable()) {
    {
      std::lock_guard<std::mutex> lk(t->mu);
      t->stop = true;
    }
    t->cv.notify_all();
    t->writer.join();
  }
  for (double* p : t->slot)
    if (p) {
      if (t->pinned)
        cudaFreeHost(p);
      else
        free(p);
    }
  for (cudaEvent_t e : t->ev)
    if (e) cudaEventDestroy(e);
  if (t->f) fclose(t->f);
  delete t;
}

int copy_shapes(double* dst, const double* X, size_t n, int on_device) {
  if (on_device) return ves_cuda_status(cudaMemcpy(dst, X, n * sizeof(double), cudaMemcpyDeviceToHost), "traj copy");
  memcpy(dst, X, n * sizeof(double));
  return VES_OK;
}

}  // namespace

extern "C" int ves_traj_create(const char* path, int N, int nv, const double* X0, int x0_on_device, int nslots,
                               ves_traj** out) {
  if (!path || !out || N <= 0 || nv <= 0 || !X0) {
    ves_record_error(VES_ERR_ARG, "traj_create: bad arguments");
    return VES_ERR_ARG;
  }
  *out = nullptr;
  ves_traj* t = new (std::nothrow) ves_traj;
  if (!t) {
    ves_record_error(VES_ERR_ARG, "traj_create: out of host memory");
    return VES_ERR_ARG;
  }
  t->N = N;
  t->nv = nv;
  t->frame = 1 + (size_t)2 * N * nv;
  t->f = fopen(path, "wb");
  if (!t->f) {
    ves_record_error(VES_ERR_ARG, "traj_create: cannot open %s for writing", path);
    traj_free(t);
    return VES_ERR_ARG;
  }
  if (nslots < 1) nslots = 3;
  t->slot.assign(nslots, nullptr);
  t->ev.assign(nslots, nullptr);
  t->busy.assign(nslots, 0);
  t->on_dev.assign(nslots, 0);
  // pinned slots and copy events; without a usable GPU the slots are plain
  // host memory and only host frames can be appended
  int ndev = 0;
  t->pinned = cudaGetDeviceCount(&ndev) == cudaSuccess && ndev > 0;
  if (!t->pinned) cudaGetLastError();
  for (int k = 0; k < nslots; ++k) {
    int rc = VES_OK;
    if (t->pinned) {
      rc = ves_cuda_status(cudaMallocHost(&t->slot[k], (t->frame + 1) * sizeof(double)), "traj pinned slot");
      if (!rc) rc = ves_cuda_status(cudaEventCreateWithFlags(&t->ev[k], cudaEventDisableTiming), "traj event");
    } else {
      t->slot[k] = (double*)malloc((t->frame + 1) * sizeof(double));
      if (!t->slot[k]) {
        ves_record_error(VES_ERR_ARG, "traj_create: out of host memory");
        rc = VES_ERR_ARG;
      }
    }
    if (rc) {
      traj_free(t);
      return rc;
    }
  }
  // header and initial shapes, written now (driver_confined.py:204-206);
  // slots hold frame + 1 doubles for this one
  double* h = t->slot[0];
  h[0] = (double)N;
  h[1] = (double)nv;
  int rc = copy_shapes(h + 2, X0, t->frame - 1, x0_on_device);
  if (!rc && fwrite(h, sizeof(double), t->frame + 1, t->f) != t->frame + 1) {
    ves_record_error(VES_ERR_ARG, "traj_create: write to %s failed", path);
    rc = VES_ERR_ARG;
  }
  if (rc) {
    traj_free(t);
    return rc;
  }
  t->writer = std::thread(writer_loop, t);
  *out = t;
  return VES_OK;
}

extern "C" int ves_traj_append(ves_traj* t, double time, const double* X, int on_device, void* stream) {
  if (!t || !X) {
    ves_record_error(VES_ERR_ARG, "traj_append: bad arguments");
    return VES_ERR_ARG;
  }
  int k;
  {
    std::unique_lock<std::mutex> lk(t->mu);
    if (t->err) {
      ves_record_error(t->err, "traj_append: an earlier frame failed to write");
      return t->err;
    }
    k = t->next;
    t->cv.wait(lk, [t, k] { return !t->busy[k]; });
    t->next = (k + 1) % (int)t->slot.size();
  }
  double* s = t->slot[k];
  s[0] = time;
  const size_t n = t->frame - 1;
  if (on_device && !t->pinned) {
    ves_record_error(VES_ERR_CUDA, "traj_append: device frame without a GPU");
    return VES_ERR_CUDA;
  }
  if (on_device) {
    cudaStream_t st = (cudaStream_t)stream;
    int rc = ves_cuda_status(cudaMemcpyAsync(s + 1, X, n * sizeof(double), cudaMemcpyDeviceToHost, st), "traj copy");
    if (!rc) rc = ves_cuda_status(cudaEventRecord(t->ev[k], st), "traj event");
    if (rc) return rc;
  } else {
    memcpy(s + 1, X, n * sizeof(double));
  }
  {
    std::lock_guard<std::mutex> lk(t->mu);
    t->busy[k] = 1;
    t->on_dev[k] = on_device ? 1 : 0;
    t->queue.push_back(k);
  }
  t->cv.notify_all();
  return VES_OK;
}

extern "C" int ves_traj_flush(ves_traj* t, long long* frames_written) {
  if (!t) return VES_ERR_ARG;
  std::unique_lock<std::mutex> lk(t->mu);
  t->cv.wait(lk, [t] { return t->queue.empty(); });
  if (frames_written) *frames_written = t->frames;
  if (!t->err && fflush(t->f) != 0) t->err = VES_ERR_ARG;
  if (t->err) ves_record_error(t->err, "traj_flush: a frame failed to write");
  return t->err;
}

extern "C" int ves_traj_close(ves_traj* t) {
  if (!t) return VES_OK;
  int rc = ves_traj_flush(t, nullptr);
  traj_free(t);
  return rc;
}
