// Measured FP64 FMA throughput of the device: the roofline denominator of the FP64-bound kernels
// (operator products with many right-hand sides, dense front products). GB300 issues far fewer FP64
// than FP32 operations per clock, so these kernels are bounded by it rather than by HBM.
#include <cuda_runtime.h>

#include <cstdint>
#include <mutex>

#include "device.h"

namespace fem2d {

namespace {

// 8 independent FMA chains per thread; the result is stored so the compiler keeps every operation
__global__ void __launch_bounds__(256) fp64_fma_kernel(int iters, double b, double c, double* __restrict__ out) {
  double a[8];
#pragma unroll
  for (int k = 0; k < 8; k++) a[k] = 1.0 + 1e-3 * (threadIdx.x + k);
  for (int i = 0; i < iters; i++) {
#pragma unroll
    for (int k = 0; k < 8; k++) a[k] = fma(a[k], b, c);
  }
  double s = 0.0;
#pragma unroll
  for (int k = 0; k < 8; k++) s += a[k];
  out[blockIdx.x * (int64_t)blockDim.x + threadIdx.x] = s;
}

}  // namespace

double measure_fp64_peak(Ctx& c) {
  const int blocks = c.num_sms * 8, threads = 256, iters = 4096;
  DBuf<double> out;
  out.alloc((size_t)blocks * threads);
  cudaEvent_t e0, e1;
  FEM2D_CUDA(cudaEventCreate(&e0));
  FEM2D_CUDA(cudaEventCreate(&e1));
  fp64_fma_kernel<<<blocks, threads, 0, c.stream>>>(iters, 0.9999999, 1e-7, out.p);   // warm-up
  FEM2D_CUDA(cudaEventRecord(e0, c.stream));
  const int reps = 3;
  for (int r = 0; r < reps; r++) fp64_fma_kernel<<<blocks, threads, 0, c.stream>>>(iters, 0.9999999, 1e-7, out.p);
  FEM2D_CUDA(cudaEventRecord(e1, c.stream));
  FEM2D_CUDA(cudaEventSynchronize(e1));
  FEM2D_CUDA(cudaGetLastError());
  c.launches += 1 + reps;
  float ms = 0;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  const double flops = 2.0 * 8.0 * iters * (double)blocks * threads * reps;
  return flops / (ms * 1e-3) / 1e12;
}

void enable_stream_pool(int device) {
  static std::mutex mu;
  static bool done[256] = {};
  std::lock_guard<std::mutex> lk(mu);
  if (device < 0 || device >= 256 || done[device]) return;
  cudaMemPool_t pool;
  if (cudaDeviceGetDefaultMemPool(&pool, device) == cudaSuccess) {
    uint64_t keep = UINT64_MAX;
    cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
  }
  cudaGetLastError();
  done[device] = true;
}

}  // namespace fem2d
