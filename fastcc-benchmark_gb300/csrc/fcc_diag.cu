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

// Shared-memory FP64 accumulation into a 20,000-double tile (one dense row of
// the benchmark workload), lanes of a warp on distinct positions, four
// updates per iteration. mode 0: built-in atomicAdd(double) of a product;
// 1: compare-and-swap loop around one FMA (the tile kernels' phase 2);
// 2: unsynchronised read-modify-write with FMA (the tile kernels' phase 1,
// exact there because one A entry's positions are distinct).
constexpr int kDiagArea = 20000;

__device__ __forceinline__ unsigned diag_pos(unsigned it, unsigned warp, unsigned lane) {
  const unsigned h = (it * 2654435761u) ^ (warp * 40503u);
  return (h % kDiagArea + lane * 613u) % kDiagArea;  // 613 is prime to 20000: distinct per warp
}

template <int MODE>
__global__ void __launch_bounds__(1024, 1) k_shared_update(double *sink, int iters) {
  extern __shared__ double acc[];
  for (int i = threadIdx.x; i < kDiagArea; i += blockDim.x) acc[i] = 0.0;
  __syncthreads();
  const unsigned lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const double v0 = 1e-3 * (lane + 1);
  for (int it = 0; it < iters; it += 4) {
    const double v = v0 * (1.0 + 1e-9 * it);
#pragma unroll
    for (int q = 0; q < 4; q++) {
      const unsigned p = diag_pos(it + q, warp, lane);
      const double m = 1.0001 + q;
      if (MODE == 0) {
        atomicAdd(&acc[p], v * m);
      } else if (MODE == 1) {
        unsigned long long *a = reinterpret_cast<unsigned long long *>(&acc[p]);
        unsigned long long cur = *reinterpret_cast<volatile unsigned long long *>(a), as;
        do {
          as = cur;
          cur = atomicCAS(a, as, (unsigned long long)__double_as_longlong(fma(v, m, __longlong_as_double((long long)as))));
        } while (cur != as);
      } else {
        acc[p] = fma(v, m, acc[p]);
      }
    }
  }
  __syncthreads();
  if (threadIdx.x == 0) sink[blockIdx.x] = acc[blockIdx.x % kDiagArea];
}

}  // namespace

extern "C" int fcc_diag_shared_update_rate(int32_t mode, double *updates_per_second) {
  if (!updates_per_second || mode < 0 || mode > 2) return FCC_ERR_ARG;
  *updates_per_second = 0;
  int dev = 0, sms = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return FCC_ERR_CUDA;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return FCC_ERR_CUDA;
  double *sink = nullptr;
  if (cudaMalloc(&sink, sizeof(double) * sms) != cudaSuccess) return FCC_ERR_OOM;
  const size_t smem = sizeof(double) * kDiagArea;
  const void *kern = mode == 0 ? reinterpret_cast<const void *>(k_shared_update<0>)
                   : mode == 1 ? reinterpret_cast<const void *>(k_shared_update<1>)
                               : reinterpret_cast<const void *>(k_shared_update<2>);
  cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
  auto launch = [&](int iters) {
    if (mode == 0) k_shared_update<0><<<sms, 1024, smem>>>(sink, iters);
    else if (mode == 1) k_shared_update<1><<<sms, 1024, smem>>>(sink, iters);
    else k_shared_update<2><<<sms, 1024, smem>>>(sink, iters);
  };
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  const int iters = 2048;
  launch(64);
  cudaEventRecord(e0);
  launch(iters);
  cudaEventRecord(e1);
  cudaError_t err = cudaEventSynchronize(e1);
  float ms = 0;
  if (err == cudaSuccess) err = cudaEventElapsedTime(&ms, e0, e1);
  if (err == cudaSuccess) err = cudaGetLastError();
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(sink);
  if (err != cudaSuccess || ms <= 0) return FCC_ERR_CUDA;
  *updates_per_second = double(sms) * 1024.0 * iters / (double(ms) * 1e-3);
  return FCC_OK;
}

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

// The library's stable LSD radix sort on caller data: keys (and their 32- or
// 64-bit payloads) are copied to the device, sorted `reps` times from the
// same unsorted copy, and the sorted pairs come back; *ms_per_sort is the
// mean device time of one sort (CUDA events around the sort alone).
extern "C" int fcc_diag_radix_sort(const void *keys, int32_t key_bytes, const void *vals, int32_t value_bytes,
                                   int64_t n, int32_t nbits, int32_t reps, void *keys_out, void *vals_out,
                                   double *ms_per_sort) {
  using namespace fcc;
  const bool combo = (key_bytes == 8 && (value_bytes == 4 || value_bytes == 8)) || (key_bytes == 4 && value_bytes == 8);
  if (n < 0 || nbits < 0 || nbits > 8 * key_bytes || reps < 1 || !combo ||
      (n > 0 && (!keys || !vals || !keys_out || !vals_out)) || !ms_per_sort || n > i64(0xFFFFFFFFu))
    return FCC_ERR_ARG;
  *ms_per_sort = 0;
  if (n == 0) return FCC_OK;
  const size_t kb = (size_t(key_bytes) * size_t(n) + 255) & ~size_t(255);
  const size_t vb = (size_t(value_bytes) * size_t(n) + 255) & ~size_t(255);
  const size_t kn = size_t(key_bytes) * size_t(n), vn = size_t(value_bytes) * size_t(n);
  const size_t nblk = (size_t(n) + 4095) / 4096;
  const size_t scratch = kb + vb + nblk * 256 * 8 + (size_t(16) << 20);
  char *d = nullptr;
  cudaStream_t st = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  int rc = FCC_OK;
  if (cudaMalloc(&d, 2 * (kb + vb) + scratch + 256) != cudaSuccess) {
    cudaGetLastError();
    return FCC_ERR_OOM;
  }
  try {
    FCC_CUDA(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
    FCC_CUDA(cudaEventCreate(&e0));
    FCC_CUDA(cudaEventCreate(&e1));
    char *k0 = d, *k1 = d + kb;
    char *v0 = d + 2 * kb, *v1 = v0 + vb;
    u32 *err = reinterpret_cast<u32 *>(v1 + vb);
    Arena ar;
    ar.init_fixed(v1 + vb + 256, scratch);
    FCC_CUDA(cudaMemsetAsync(err, 0, sizeof(u32), st));
    FCC_CUDA(cudaMemcpyAsync(k0, keys, kn, cudaMemcpyHostToDevice, st));
    FCC_CUDA(cudaMemcpyAsync(v0, vals, vn, cudaMemcpyHostToDevice, st));
    double total = 0;
    for (int r = 0; r < reps; r++) {
      FCC_CUDA(cudaMemcpyAsync(k1, k0, kn, cudaMemcpyDeviceToDevice, st));
      FCC_CUDA(cudaMemcpyAsync(v1, v0, vn, cudaMemcpyDeviceToDevice, st));
      ar.begin(st);
      FCC_CUDA(cudaEventRecord(e0, st));
      if (key_bytes == 4)
        radix_sort_pairs64(reinterpret_cast<u32 *>(k1), reinterpret_cast<u64 *>(v1), n, nbits, ar, st, err);
      else if (value_bytes == 4)
        radix_sort_pairs(reinterpret_cast<u64 *>(k1), reinterpret_cast<u32 *>(v1), n, nbits, ar, st, err);
      else
        radix_sort_pairs64(reinterpret_cast<u64 *>(k1), reinterpret_cast<u64 *>(v1), n, nbits, ar, st, err);
      FCC_CUDA(cudaEventRecord(e1, st));
      FCC_CUDA(cudaEventSynchronize(e1));
      float ms = 0;
      FCC_CUDA(cudaEventElapsedTime(&ms, e0, e1));
      total += ms;
    }
    FCC_CUDA(cudaMemcpyAsync(keys_out, k1, kn, cudaMemcpyDeviceToHost, st));
    FCC_CUDA(cudaMemcpyAsync(vals_out, v1, vn, cudaMemcpyDeviceToHost, st));
    u32 h_err = 0;
    FCC_CUDA(cudaMemcpyAsync(&h_err, err, sizeof(u32), cudaMemcpyDeviceToHost, st));
    FCC_CUDA(cudaStreamSynchronize(st));
    if (h_err) throw Error{FCC_ERR_CUDA, "radix sort: a bulk-copy wait gave up"};
    *ms_per_sort = total / reps;
  } catch (const fcc::Error &e) {
    rc = e.status;
  }
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  if (st) cudaStreamDestroy(st);
  cudaFree(d);
  return rc;
}
