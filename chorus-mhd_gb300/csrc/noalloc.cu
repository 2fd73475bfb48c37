// noalloc.cu -- the Rusanov point evaluator for callers that cannot allocate device
// memory.
//
// getrusanovflux_gpu stages its host arrays in device buffers it allocates and frees
// on every call.  Two kinds of caller cannot do that: a host that has already handed
// its whole device-memory budget to a pool (a serving process admitting solves under a
// fixed HBM budget, or a coupled code whose framework owns the GPU's memory), where a
// fresh cudaMalloc fails or breaks the pool's accounting; and a host with other work in
// flight on the device that it must not stall, because cudaFree waits for the whole
// device to go idle.  getrusanovflux_noalloc_gpu does the same computation with its
// staging area in a fixed array compiled into this file, so it allocates nothing.
//
// The array holds kNoAllocMaxPoints points (10 MiB of device memory on every GPU that
// loads the library, kept until the process exits).  With CUDA's lazy module loading
// (the default) the array is reserved when this file's module is first used on a
// device, which is the set-up of the first call on that device: that call needs 10 MiB
// of free device memory, so a host that hands all its memory to a pool makes one call
// with n = 0 (set-up only) before it builds the pool.  The set-up, once per device with
// that device current, looks up the array's device address and creates the stream the
// copies and the kernel run on (non-blocking, so a call does not wait for, or hold up,
// the host's own work on other streams); make the first call before any stream capture.
// A CUDA error drops the device's set-up so the next call redoes it; calls made after
// cudaDeviceReset of a device without such an error are not supported.
// All calls share the one array and it keeps the last call's contents: every output
// slot is rewritten for the points of the current call, so nothing needs clearing, but
// calls that overlap on the GPU (from two host threads, or while a previous call is
// still running) race on the array.
#include <cuda_runtime.h>

#include <cstdio>
#include <mutex>

#include "chorus_internal.h"

namespace chorus {
int set_err(int code, const char* fmt, ...);
}

namespace {

constexpr int kNoAllocMaxPoints = 32768;
// per point: Qfl 9 + Qfr 9 + normf 2 + Fnl 8 + Fnr 8 + Az 1 + eigv 1 doubles, and the
// two int32 signs packed into one double slot
constexpr size_t kNoAllocPerPoint = 40;
__device__ __align__(256) double g_rusanov_scratch[kNoAllocMaxPoints * kNoAllocPerPoint];

std::mutex g_scratch_mu;
double* g_scratch_addr[64] = {nullptr};
cudaStream_t g_scratch_stream[64] = {nullptr};

int scratch_for_current_device(double** out, cudaStream_t* st, int* dev_out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return chorus::set_err(CHORUS_ECUDA, "cudaGetDevice: %s", cudaGetErrorString(e));
  if (dev < 0 || dev >= 64) return chorus::set_err(CHORUS_EINVAL, "device %d out of range", dev);
  std::lock_guard<std::mutex> lk(g_scratch_mu);
  if (!g_scratch_addr[dev]) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_rusanov_scratch);
    if (e != cudaSuccess || !p)
      return chorus::set_err(CHORUS_ECUDA, "cudaGetSymbolAddress(scratch) on device %d: %s", dev, cudaGetErrorString(e));
    if (!g_scratch_stream[dev]) {
      e = cudaStreamCreateWithFlags(&g_scratch_stream[dev], cudaStreamNonBlocking);
      if (e != cudaSuccess) {
        g_scratch_stream[dev] = nullptr;
        return chorus::set_err(CHORUS_ECUDA, "cudaStreamCreateWithFlags on device %d: %s", dev, cudaGetErrorString(e));
      }
    }
    g_scratch_addr[dev] = static_cast<double*>(p);
  }
  *out = g_scratch_addr[dev];
  *st = g_scratch_stream[dev];
  *dev_out = dev;
  return CHORUS_OK;
}

// after a CUDA error the next call on the device looks the address up again (the stream
// handle is dropped without destroying it: it may belong to a context that is gone)
void drop_setup(int dev) {
  std::lock_guard<std::mutex> lk(g_scratch_mu);
  g_scratch_addr[dev] = nullptr;
  g_scratch_stream[dev] = nullptr;
}

}  // namespace

extern "C" int getrusanovflux_noalloc_gpu(int32_t n, double gam, const double* Qfl, const double* Qfr, double* Fnl,
                                          double* Fnr, double* Az, const double* normf, const int32_t* sign_l,
                                          const int32_t* sign_r, double* eigv) {
  if (n < 0) return chorus::set_err(CHORUS_EINVAL, "getrusanovflux_noalloc_gpu: n=%d < 0", n);
  if (n > kNoAllocMaxPoints)
    return chorus::set_err(CHORUS_EINVAL, "getrusanovflux_noalloc_gpu: n=%d exceeds the fixed capacity of %d points", n,
                           kNoAllocMaxPoints);
  double* base = nullptr;
  cudaStream_t st = nullptr;
  int dev = 0;
  int rc = scratch_for_current_device(&base, &st, &dev);
  if (rc) return rc;
  if (n == 0) return CHORUS_OK;  // set-up only
  if (!Qfl || !Qfr || !Fnl || !Fnr || !Az || !normf || !sign_l || !sign_r || !eigv)
    return chorus::set_err(CHORUS_EINVAL, "getrusanovflux_noalloc_gpu: null argument");
  const size_t m = (size_t)n;
  double* dQl = base;
  double* dQr = base + 9 * m;
  double* dnf = base + 18 * m;
  double* dFl = base + 20 * m;
  double* dFr = base + 28 * m;
  double* dAz = base + 36 * m;
  double* dev_ = base + 37 * m;
  int* dsl = reinterpret_cast<int*>(base + 38 * m);
  int* dsr = dsl + m;
  cudaError_t e = cudaMemcpyAsync(dQl, Qfl, 9 * m * sizeof(double), cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(dQr, Qfr, 9 * m * sizeof(double), cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(dnf, normf, 2 * m * sizeof(double), cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(dsl, sign_l, m * sizeof(int), cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(dsr, sign_r, m * sizeof(int), cudaMemcpyHostToDevice, st);
  if (e != cudaSuccess) {
    drop_setup(dev);
    return chorus::set_err(CHORUS_ECUDA, "getrusanovflux_noalloc_gpu upload: %s", cudaGetErrorString(e));
  }
  chorus::launch_point_rusanov(n, gam, dQl, dQr, dFl, dFr, dAz, dnf, dsl, dsr, dev_, st);
  e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaMemcpyAsync(Fnl, dFl, 8 * m * sizeof(double), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(Fnr, dFr, 8 * m * sizeof(double), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(Az, dAz, m * sizeof(double), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(eigv, dev_, m * sizeof(double), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) {
    drop_setup(dev);
    return chorus::set_err(CHORUS_ECUDA, "getrusanovflux_noalloc_gpu: %s", cudaGetErrorString(e));
  }
  return CHORUS_OK;
}
