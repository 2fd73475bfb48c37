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
// loads the library, kept until the process exits).  Its device address is looked up
// once per device, with that device current, on the first call made on that device;
// make that first call before any stream capture.  All calls share the one array and it
// keeps the last call's contents: every output slot is rewritten for the points of the
// current call, so nothing needs clearing, but calls that overlap on the GPU (from two
// host threads, or while a previous call is still running) race on the array.
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

int scratch_for_current_device(double** out) {
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
    g_scratch_addr[dev] = static_cast<double*>(p);
  }
  *out = g_scratch_addr[dev];
  return CHORUS_OK;
}

}  // namespace

extern "C" int getrusanovflux_noalloc_gpu(int32_t n, double gam, const double* Qfl, const double* Qfr, double* Fnl,
                                          double* Fnr, double* Az, const double* normf, const int32_t* sign_l,
                                          const int32_t* sign_r, double* eigv) {
  if (n < 0) return chorus::set_err(CHORUS_EINVAL, "getrusanovflux_noalloc_gpu: n=%d < 0", n);
  if (n > kNoAllocMaxPoints)
    return chorus::set_err(CHORUS_EINVAL, "getrusanovflux_noalloc_gpu: n=%d exceeds the fixed capacity of %d points", n,
                           kNoAllocMaxPoints);
  if (n == 0) return CHORUS_OK;
  if (!Qfl || !Qfr || !Fnl || !Fnr || !Az || !normf || !sign_l || !sign_r || !eigv)
    return chorus::set_err(CHORUS_EINVAL, "getrusanovflux_noalloc_gpu: null argument");
  double* base = nullptr;
  int rc = scratch_for_current_device(&base);
  if (rc) return rc;
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
  cudaError_t e = cudaMemcpy(dQl, Qfl, 9 * m * sizeof(double), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(dQr, Qfr, 9 * m * sizeof(double), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(dnf, normf, 2 * m * sizeof(double), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(dsl, sign_l, m * sizeof(int), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(dsr, sign_r, m * sizeof(int), cudaMemcpyHostToDevice);
  if (e != cudaSuccess) return chorus::set_err(CHORUS_ECUDA, "getrusanovflux_noalloc_gpu upload: %s", cudaGetErrorString(e));
  chorus::launch_point_rusanov(n, gam, dQl, dQr, dFl, dFr, dAz, dnf, dsl, dsr, dev_, 0);
  e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaMemcpy(Fnl, dFl, 8 * m * sizeof(double), cudaMemcpyDeviceToHost);
  if (e == cudaSuccess) e = cudaMemcpy(Fnr, dFr, 8 * m * sizeof(double), cudaMemcpyDeviceToHost);
  if (e == cudaSuccess) e = cudaMemcpy(Az, dAz, m * sizeof(double), cudaMemcpyDeviceToHost);
  if (e == cudaSuccess) e = cudaMemcpy(eigv, dev_, m * sizeof(double), cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return chorus::set_err(CHORUS_ECUDA, "getrusanovflux_noalloc_gpu: %s", cudaGetErrorString(e));
  return CHORUS_OK;
}
