// Device primitives: workspace arena, exclusive prefix sums and a stable LSD
// radix sort, hand-written for sm_103a. They build the device replacement of
// the reference's per-tile hash index (TileIndexedTensor,
// index_tensors.hpp:491-547): nonzeros are sorted by linearised 64-bit keys
// and grouped into segments by prefix sums of head flags.

#include "fcc_internal.cuh"

namespace fcc {

std::atomic<long long> g_launches{0};

// ---------------------------------------------------------------- arena ----

void Arena::begin(cudaStream_t s) {
  stream_ = s;
  if (fixed_) {
    used_ = total_used_ = 0;
    return;
  }
  bool consolidate = chunks_.size() > 1 || (chunks_.size() == 1 && chunks_[0].size < high_);
  if (consolidate) {
    for (auto &c : chunks_) FCC_CUDA(cudaFreeAsync(c.p, s));
    chunks_.clear();
  }
  if (chunks_.empty() && high_ > 0) {
    size_t sz = (high_ + (size_t(2) << 20) - 1) & ~((size_t(2) << 20) - 1);
    void *p = nullptr;
    p = pool_alloc(pool_, sz, s);
    chunks_.push_back({static_cast<char *>(p), sz});
  }
  used_ = 0;
  total_used_ = 0;
}

// Allocation from a stream-ordered pool that keeps freed blocks cached:
// when a request does not fit, wait for the stream's pending frees, return
// the pool's unused memory to the device and try once more.
void *pool_alloc(cudaMemPool_t pool, size_t bytes, cudaStream_t st) {
  void *p = nullptr;
  cudaError_t e = cudaMallocFromPoolAsync(&p, bytes, pool, st);
  if (e == cudaErrorMemoryAllocation) {
    cudaGetLastError();
    FCC_CUDA(cudaStreamSynchronize(st));
    FCC_CUDA(cudaMemPoolTrimTo(pool, 0));
    e = cudaMallocFromPoolAsync(&p, bytes, pool, st);
  }
  if (e != cudaSuccess) {
    cudaGetLastError();
    throw Error{e == cudaErrorMemoryAllocation ? FCC_ERR_OOM : FCC_ERR_CUDA,
                "device allocation of " + std::to_string(bytes) + " bytes: " + cudaGetErrorString(e)};
  }
  return p;
}

void *Arena::get(size_t bytes) {
  bytes = (bytes + 255) & ~size_t(255);
  if (fixed_) {
    if (used_ + bytes > fsize_)
      throw Error{FCC_ERR_CAPACITY, "the fixed scratch (" + std::to_string(fsize_) +
                                        " bytes) is too small for this contraction"};
    char *p = fbase_ + used_;
    used_ += bytes;
    total_used_ = used_;
    if (used_ > high_) high_ = used_;
    return p;
  }
  if (chunks_.empty() || used_ + bytes > chunks_.back().size) {
    size_t sz = size_t(64) << 20;
    if (!chunks_.empty() && chunks_.back().size > sz) sz = chunks_.back().size;
    if (sz < bytes) sz = bytes;
    void *p = nullptr;
    p = pool_alloc(pool_, sz, stream_);
    chunks_.push_back({static_cast<char *>(p), sz});
    used_ = 0;
  }
  char *p = chunks_.back().p + used_;
  used_ += bytes;
  total_used_ += bytes;
  if (total_used_ > high_) high_ = total_used_;
  return p;
}

void Arena::release_all(cudaStream_t s) {
  if (fixed_) return;
  for (auto &c : chunks_) cudaFreeAsync(c.p, s);
  chunks_.clear();
  used_ = total_used_ = 0;
}

// ----------------------------------------------------------------- scan ----

namespace {

constexpr int kScanThreads = 256;
constexpr int kScanItems = 8;
constexpr int kScanTile = kScanThreads * kScanItems;

template <class T>
__device__ __forceinline__ T warp_inclusive(T x) {
  const int lane = threadIdx.x & 31;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    T y = __shfl_up_sync(kFull, x, o);
    if (lane >= o) x += y;
  }
  return x;
}

// Exclusive scan of one value per thread across the block; *total gets the
// block sum. Ends with a barrier, so `wsum` can be reused afterwards.
template <class T>
__device__ __forceinline__ T block_exclusive(T v, T *wsum, T *total) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int nwarps = blockDim.x >> 5;
  T x = warp_inclusive(v);
  if (lane == 31) wsum[warp] = x;
  __syncthreads();
  if (warp == 0) {
    T w = lane < nwarps ? wsum[lane] : T(0);
    w = warp_inclusive(w);
    if (lane < nwarps) wsum[lane] = w;
  }
  __syncthreads();
  T prefix = warp ? wsum[warp - 1] : T(0);
  if (total) *total = wsum[nwarps - 1];
  __syncthreads();
  return prefix + x - v;
}

template <class Tin, class Tacc>
__global__ void __launch_bounds__(kScanThreads) k_scan_reduce(const Tin *__restrict__ in, i64 n,
                                                              Tacc *__restrict__ part) {
  __shared__ Tacc wsum[32];
  const i64 base = i64(blockIdx.x) * kScanTile;
  Tacc s = 0;
#pragma unroll
  for (int j = 0; j < kScanItems; j++) {
    i64 i = base + j * kScanThreads + threadIdx.x;
    if (i < n) s += Tacc(in[i]);
  }
  Tacc tot;
  block_exclusive<Tacc>(s, wsum, &tot);
  if (threadIdx.x == 0) part[blockIdx.x] = tot;
}

template <class Tin, class Tacc>
__global__ void __launch_bounds__(kScanThreads) k_scan_down(const Tin *__restrict__ in, Tacc *out, i64 n,
                                                            const Tacc *__restrict__ part,
                                                            Tacc *total) {
  __shared__ Tacc tile[kScanTile];
  __shared__ Tacc wsum[32];
  const i64 base = i64(blockIdx.x) * kScanTile;
#pragma unroll
  for (int j = 0; j < kScanItems; j++) {
    int t = j * kScanThreads + threadIdx.x;
    i64 i = base + t;
    tile[t] = i < n ? Tacc(in[i]) : Tacc(0);
  }
  __syncthreads();
  Tacc v[kScanItems];
  Tacc s = 0;
#pragma unroll
  for (int j = 0; j < kScanItems; j++) {
    v[j] = tile[threadIdx.x * kScanItems + j];
    s += v[j];
  }
  Tacc tot;
  Tacc run = block_exclusive<Tacc>(s, wsum, &tot);
  if (part) run += part[blockIdx.x];
#pragma unroll
  for (int j = 0; j < kScanItems; j++) {
    tile[threadIdx.x * kScanItems + j] = run;
    run += v[j];
  }
  if (total && blockIdx.x == gridDim.x - 1 && threadIdx.x == blockDim.x - 1) *total = run;
  __syncthreads();
#pragma unroll
  for (int j = 0; j < kScanItems; j++) {
    int t = j * kScanThreads + threadIdx.x;
    i64 i = base + t;
    if (i < n) out[i] = tile[t];
  }
}

template <class Tin, class Tacc>
void scan_impl(const Tin *in, Tacc *out, i64 n, Tacc *total, Arena &ar, cudaStream_t s) {
  if (n <= 0) {
    if (total) FCC_CUDA(cudaMemsetAsync(total, 0, sizeof(Tacc), s));
    return;
  }
  i64 nblk = (n + kScanTile - 1) / kScanTile;
  Tacc *part = nullptr;
  if (nblk > 1) {
    part = ar.get_n<Tacc>(size_t(nblk));
    k_scan_reduce<Tin, Tacc><<<unsigned(nblk), kScanThreads, 0, s>>>(in, n, part);
    FCC_LAUNCH_CHECK();
    scan_impl<Tacc, Tacc>(part, part, nblk, static_cast<Tacc *>(nullptr), ar, s);
  }
  k_scan_down<Tin, Tacc><<<unsigned(nblk), kScanThreads, 0, s>>>(in, out, n, part, total);
  FCC_LAUNCH_CHECK();
}

}  // namespace

void scan_exclusive(const u32 *in, u32 *out, i64 n, u32 *total, Arena &ar, cudaStream_t s) {
  scan_impl<u32, u32>(in, out, n, total, ar, s);
}
void scan_exclusive(const u64 *in, u64 *out, i64 n, u64 *total, Arena &ar, cudaStream_t s) {
  scan_impl<u64, u64>(in, out, n, total, ar, s);
}
void scan_exclusive_wide(const u32 *in, u64 *out, i64 n, u64 *total, Arena &ar, cudaStream_t s) {
  scan_impl<u32, u64>(in, out, n, total, ar, s);
}

// ----------------------------------------------------------- radix sort ----
//
// One 8-bit digit per pass, three kernels per pass: per-tile digit histograms
// (digit-major, so one exclusive scan yields every tile's output offsets), the
// scan, and a stable scatter. Within a tile each warp ranks its keys with
// __match_any_sync; ranks follow key order (warp, step, lane), which keeps the
// sort stable.

namespace {

constexpr int kRsThreads = 256;
constexpr int kRsWarps = kRsThreads / 32;
constexpr int kRsItems = 16;
constexpr int kRsTile = kRsThreads * kRsItems;  // 4096 keys per tile

__global__ void __launch_bounds__(kRsThreads) k_rs_hist(const u64 *__restrict__ keys, i64 n, int shift,
                                                        u32 *__restrict__ hist, int nblk) {
  __shared__ u32 h[kRsWarps][256];
  for (int i = threadIdx.x; i < kRsWarps * 256; i += kRsThreads) (&h[0][0])[i] = 0;
  __syncthreads();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const i64 base = i64(blockIdx.x) * kRsTile + warp * (kRsItems * 32);
#pragma unroll 4
  for (int j = 0; j < kRsItems; j++) {
    i64 i = base + j * 32 + lane;
    if (i < n) atomicAdd(&h[warp][u32(keys[i] >> shift) & 255u], 1u);
  }
  __syncthreads();
  for (int d = threadIdx.x; d < 256; d += kRsThreads) {
    u32 s = 0;
#pragma unroll
    for (int w = 0; w < kRsWarps; w++) s += h[w][d];
    hist[i64(d) * nblk + blockIdx.x] = s;
  }
}

template <class V>
__global__ void __launch_bounds__(kRsThreads) k_rs_scatter(const u64 *__restrict__ kin,
                                                           const V *__restrict__ vin,
                                                           u64 *__restrict__ kout, V *__restrict__ vout,
                                                           i64 n, int shift, const u32 *__restrict__ offs,
                                                           int nblk) {
  __shared__ u32 wcnt[kRsWarps][256];
  for (int i = threadIdx.x; i < kRsWarps * 256; i += kRsThreads) (&wcnt[0][0])[i] = 0;
  __syncthreads();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const u32 lt_mask = (1u << lane) - 1u;
  const i64 base = i64(blockIdx.x) * kRsTile + warp * (kRsItems * 32);
  u64 k[kRsItems];
  V v[kRsItems];
  u32 r[kRsItems], dg[kRsItems];
#pragma unroll
  for (int j = 0; j < kRsItems; j++) {
    i64 i = base + j * 32 + lane;
    bool valid = i < n;
    k[j] = valid ? kin[i] : 0;
    v[j] = valid ? vin[i] : 0;
    u32 d = valid ? (u32(k[j] >> shift) & 255u) : (256u + lane);
    u32 peers = __match_any_sync(kFull, d);
    u32 before = 0;
    if (valid) before = wcnt[warp][d];
    __syncwarp();
    if (valid && lane == __ffs(peers) - 1) wcnt[warp][d] = before + __popc(peers);
    __syncwarp();
    r[j] = before + __popc(peers & lt_mask);
    dg[j] = d;
  }
  __syncthreads();
  for (int d = threadIdx.x; d < 256; d += kRsThreads) {
    u32 run = offs[i64(d) * nblk + blockIdx.x];
#pragma unroll
    for (int w = 0; w < kRsWarps; w++) {
      u32 c = wcnt[w][d];
      wcnt[w][d] = run;
      run += c;
    }
  }
  __syncthreads();
#pragma unroll
  for (int j = 0; j < kRsItems; j++) {
    i64 i = base + j * 32 + lane;
    if (i < n) {
      u32 pos = wcnt[warp][dg[j]] + r[j];
      kout[pos] = k[j];
      vout[pos] = v[j];
    }
  }
}

}  // namespace

namespace {
template <class V>
void radix_sort_impl(u64 *keys, V *vals, i64 n, int nbits, Arena &ar, cudaStream_t s) {
  if (n <= 1 || nbits <= 0) return;
  if (n > i64(0xFFFFFFFFu)) throw Error{FCC_ERR_ARG, "radix sort: more than 2^32 keys"};
  const int nblk = int((n + kRsTile - 1) / kRsTile);
  u64 *k2 = ar.get_n<u64>(size_t(n));
  V *v2 = ar.get_n<V>(size_t(n));
  u32 *hist = ar.get_n<u32>(size_t(nblk) * 256);
  u64 *ka = keys, *kb = k2;
  V *va = vals, *vb = v2;
  const int passes = (nbits + 7) / 8;
  for (int p = 0; p < passes; p++) {
    const int shift = 8 * p;
    k_rs_hist<<<nblk, kRsThreads, 0, s>>>(ka, n, shift, hist, nblk);
    FCC_LAUNCH_CHECK();
    scan_exclusive(hist, hist, i64(nblk) * 256, nullptr, ar, s);
    k_rs_scatter<V><<<nblk, kRsThreads, 0, s>>>(ka, va, kb, vb, n, shift, hist, nblk);
    FCC_LAUNCH_CHECK();
    std::swap(ka, kb);
    std::swap(va, vb);
  }
  if (ka != keys) {
    FCC_CUDA(cudaMemcpyAsync(keys, ka, sizeof(u64) * size_t(n), cudaMemcpyDeviceToDevice, s));
    FCC_CUDA(cudaMemcpyAsync(vals, va, sizeof(V) * size_t(n), cudaMemcpyDeviceToDevice, s));
  }
}
}  // namespace

void radix_sort_pairs(u64 *keys, u32 *vals, i64 n, int nbits, Arena &ar, cudaStream_t s) {
  radix_sort_impl<u32>(keys, vals, n, nbits, ar, s);
}

void radix_sort_pairs64(u64 *keys, u64 *vals, i64 n, int nbits, Arena &ar, cudaStream_t s) {
  radix_sort_impl<u64>(keys, vals, n, nbits, ar, s);
}

}  // namespace fcc
