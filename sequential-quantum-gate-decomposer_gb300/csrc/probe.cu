// Live measurement of the FP64 FMA pipe peak, the roofline denominator of the engine's
// FP64-bound kernels (no HBM figure exists for them).  A grid of 8 CTAs per SM runs
// independent DFMA chains (eight per thread, so latency never limits issue) on the first
// `active_lanes` lanes of every warp, timed with CUDA events on the caller's stream.
#include <cuda_runtime.h>

#include "../../include/sqg.h"
#include "handle.h"

namespace {

__global__ void k_fp64_peak(double* out, int iters, int active_lanes, double a, double b) {
  double x0 = threadIdx.x * 1e-3, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3, x4 = x0 + 4, x5 = x0 + 5, x6 = x0 + 6,
         x7 = x0 + 7;
  if ((int)(threadIdx.x & 31) < active_lanes) {
#pragma unroll 4
  for (int i = 0; i < iters; i++) {
    x0 = fma(x0, a, b); x1 = fma(x1, a, b); x2 = fma(x2, a, b); x3 = fma(x3, a, b);
    x4 = fma(x4, a, b); x5 = fma(x5, a, b); x6 = fma(x6, a, b); x7 = fma(x7, a, b);
  }
  }
  out[blockIdx.x * blockDim.x + threadIdx.x] = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
}

}  // namespace

extern "C" size_t sqg_probe_fp64_scratch_bytes(void) {
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  return (size_t)sms * 8 * 256 * sizeof(double);
}

extern "C" int sqg_probe_fp64_tflops(double* tflops, int active_lanes, void* scratch, size_t scratch_bytes,
                                     void* stream) {
  if (!tflops || !scratch || active_lanes < 1 || active_lanes > 32)
    return sqg::set_error(SQG_ERR_INVALID_ARGUMENT, "null argument or active_lanes outside 1..32");
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const int blocks = sms * 8, threads = 256, iters = 4096;
  if (scratch_bytes < (size_t)blocks * threads * sizeof(double))
    return sqg::set_error(SQG_ERR_WORKSPACE, "probe scratch too small");
  cudaStream_t s = (cudaStream_t)stream;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  k_fp64_peak<<<blocks, threads, 0, s>>>((double*)scratch, iters, active_lanes, 0.9999999, 1e-7);  // warm-up
  cudaEventRecord(e0, s);
  k_fp64_peak<<<blocks, threads, 0, s>>>((double*)scratch, iters, active_lanes, 0.9999999, 1e-7);
  cudaEventRecord(e1, s);
  cudaError_t e = cudaEventSynchronize(e1);
  float ms = 0.f;
  if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (e != cudaSuccess) return sqg::set_error(SQG_ERR_CUDA, cudaGetErrorString(e));
  // flops issued as if every lane were active: with active_lanes < 32 the figure shows
  // whether the pipe is charged per warp instruction or per active lane
  *tflops = 2.0 * 8.0 * iters * (double)blocks * threads / (ms * 1e-3) / 1e12;
  return SQG_OK;
}
