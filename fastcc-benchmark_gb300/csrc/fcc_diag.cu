// Diagnostics: the FP64 FMA issue rate of the current device, the peak the
// tile kernels are measured against (their every multiply-add is one FP64
// FMA). Eight independent FMA chains per thread, two 1024-thread CTAs per SM,
// timed with CUDA events; nothing is read or written in the timed loop.

#include "fcc_internal.cuh"

namespace {

__global__ void __launch_bounds__(1024) k_fp64_fma(double *sink, int iters, double a, double b) {
  double x[8];
#pragma unroll
  for (int j = 0; j < 8; j++) x[j] = 1e-3 * (threadIdx.x + j);
  for (int i = 0; i < iters; i++) {
#pragma unroll
    for (int j = 0; j < 8; j++) x[j] = fma(x[j], a, b);
  }
  double s = 0;
#pragma unroll
  for (int j = 0; j < 8; j++) s += x[j];
  if (s == 1.2345e300) sink[blockIdx.x] = s;  // keeps the loop alive, never true
}

}  // namespace

extern "C" int fcc_diag_fp64_fma_rate(int32_t device, double *fma_per_second) {
  if (!fma_per_second) return FCC_ERR_ARG;
  *fma_per_second = 0;
  int dev = device;
  if (dev < 0 && cudaGetDevice(&dev) != cudaSuccess) return FCC_ERR_CUDA;
  if (cudaSetDevice(dev) != cudaSuccess) return FCC_ERR_NO_DEVICE;
  int sms = 0;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return FCC_ERR_CUDA;
  double *sink = nullptr;
  if (cudaMalloc(&sink, sizeof(double) * 2 * sms) != cudaSuccess) return FCC_ERR_OOM;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  const int iters = 4096;
  k_fp64_fma<<<2 * sms, 1024>>>(sink, 64, 0.999999, 1e-7);  // warm-up
  cudaEventRecord(e0);
  k_fp64_fma<<<2 * sms, 1024>>>(sink, iters, 0.999999, 1e-7);
  cudaEventRecord(e1);
  cudaError_t err = cudaEventSynchronize(e1);
  float ms = 0;
  if (err == cudaSuccess) err = cudaEventElapsedTime(&ms, e0, e1);
  if (err == cudaSuccess) err = cudaGetLastError();
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(sink);
  if (err != cudaSuccess || ms <= 0) return FCC_ERR_CUDA;
  *fma_per_second = double(2 * sms) * 1024.0 * 8.0 * iters / (double(ms) * 1e-3);
  return FCC_OK;
}
