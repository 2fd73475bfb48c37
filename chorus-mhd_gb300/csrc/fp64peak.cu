// fp64peak.cu -- the FP64 pipe's fused multiply-add rate of the current GPU, measured.
//
// The residual path is bound by the FP64 pipe rather than by HBM on parts whose FP64
// rate is a small fraction of their FP32 rate, so the benchmark reports its FP64
// instruction rate against this figure: every thread runs kChains independent
// dependency chains of fma(x, a, b) for `iters` iterations, enough warps per SM to hide
// the FMA latency, and the kernel is timed with CUDA events after a warm-up launch.
#include <cuda_runtime.h>

#include <cstdint>

#include "chorus_internal.h"

namespace chorus {
int set_err(int code, const char* fmt, ...);
}

namespace {

constexpr int kChains = 8;
constexpr int kThreads = 256;

__global__ void __launch_bounds__(kThreads) k_dfma_chains(double* out, int iters, double a, double b) {
  const int tid = blockIdx.x * blockDim.x + threadIdx.x;
  double x[kChains];
#pragma unroll
  for (int c = 0; c < kChains; c++) x[c] = 1e-3 * (tid & 1023) + c;
  for (int i = 0; i < iters; i++) {
#pragma unroll
    for (int c = 0; c < kChains; c++) x[c] = fma(x[c], a, b);
  }
  double s = 0.0;
#pragma unroll
  for (int c = 0; c < kChains; c++) s += x[c];
  out[tid] = s;  // keeps the chains live
}

}  // namespace

extern "C" int chorus_gpu_fp64_fma_peak(int32_t device, double* fma_per_s, double* ms_out) {
  if (!fma_per_s) return chorus::set_err(CHORUS_EINVAL, "null argument");
  cudaError_t e = cudaSetDevice(device);
  if (e != cudaSuccess) return chorus::set_err(CHORUS_ECUDA, "cudaSetDevice(%d): %s", device, cudaGetErrorString(e));
  cudaDeviceProp prop;
  e = cudaGetDeviceProperties(&prop, device);
  if (e != cudaSuccess) return chorus::set_err(CHORUS_ECUDA, "cudaGetDeviceProperties: %s", cudaGetErrorString(e));
  const int blocks = prop.multiProcessorCount * 8;  // 64 warps per SM
  const int iters = 4096;
  double* out = nullptr;
  cudaStream_t st = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  float ms = 0.f;
  e = cudaMalloc(&out, sizeof(double) * (size_t)blocks * kThreads);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaEventCreate(&e0);
  if (e == cudaSuccess) e = cudaEventCreate(&e1);
  if (e == cudaSuccess) {
    // a multiplier just below 1 keeps the chains bounded and normal
    const double a = 1.0 - 1.0 / 1048576.0, b = 1.0 / 4096.0;
    k_dfma_chains<<<blocks, kThreads, 0, st>>>(out, iters, a, b);  // warm-up (clocks, module load)
    e = cudaEventRecord(e0, st);
    for (int r = 0; r < 5 && e == cudaSuccess; r++) k_dfma_chains<<<blocks, kThreads, 0, st>>>(out, iters, a, b);
    if (e == cudaSuccess) e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaEventRecord(e1, st);
    if (e == cudaSuccess) e = cudaEventSynchronize(e1);
    if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
  }
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  if (st) cudaStreamDestroy(st);
  if (out) cudaFree(out);
  if (e != cudaSuccess) return chorus::set_err(CHORUS_ECUDA, "fp64 peak: %s", cudaGetErrorString(e));
  const double fmas = 5.0 * blocks * (double)kThreads * kChains * iters;
  *fma_per_s = fmas / (ms * 1e-3);
  if (ms_out) *ms_out = ms;
  return CHORUS_OK;
}
