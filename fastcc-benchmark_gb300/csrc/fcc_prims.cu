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

void Arena::shrink(cudaStream_t s) {
  if (fixed_) return;
  release_all(s);
  high_ = 0;
  FCC_CUDA(cudaStreamSynchronize(s));
  if (pool_) FCC_CUDA(cudaMemPoolTrimTo(pool_, 0));
}

size_t Arena::available() const {
  size_t fb = 0, tb = 0;
  FCC_CUDA(cudaMemGetInfo(&fb, &tb));
  if (pool_) {
    uint64_t reserved = 0, used = 0;
    FCC_CUDA(cudaMemPoolGetAttribute(pool_, cudaMemPoolAttrReservedMemCurrent, &reserved));
    FCC_CUDA(cudaMemPoolGetAttribute(pool_, cudaMemPoolAttrUsedMemCurrent, &used));
    if (reserved > used) fb += size_t(reserved - used);
  }
  return fb;
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
// sort stable. The scatter keeps each tile in shared memory, ranks it
// block-wide and writes it out in sorted order, so a warp's stores cover runs
// of consecutive positions (a tile holds 16 keys per digit on average)
// instead of one or two keys per digit.

namespace {

constexpr int kRsThreads = 256;
constexpr int kRsWarps = kRsThreads / 32;
constexpr int kRsItems = 16;
constexpr int kRsTile = kRsThreads * kRsItems;  // 4096 keys per tile
static_assert(kRsThreads == 256, "the scatter scans one digit per thread");

template <class K>
__global__ void __launch_bounds__(kRsThreads) k_rs_hist(const K *__restrict__ keys, i64 n, int shift,
                                                        u32 *__restrict__ hist, int nblk) {
  __shared__ u32 h[kRsWarps][256];
  for (int i = threadIdx.x; i < kRsWarps * 256; i += kRsThreads) (&h[0][0])[i] = 0;
  __syncthreads();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const i64 base = i64(blockIdx.x) * kRsTile + warp * (kRsItems * 32);
  K k[kRsItems];  // every load in flight before the first count
#pragma unroll
  for (int j = 0; j < kRsItems; j++) {
    i64 i = base + j * 32 + lane;
    k[j] = i < n ? keys[i] : 0;
  }
#pragma unroll
  for (int j = 0; j < kRsItems; j++)
    if (base + j * 32 + lane < n) atomicAdd(&h[warp][u32(k[j] >> shift) & 255u], 1u);
  __syncthreads();
  for (int d = threadIdx.x; d < 256; d += kRsThreads) {
    u32 s = 0;
#pragma unroll
    for (int w = 0; w < kRsWarps; w++) s += h[w][d];
    hist[i64(d) * nblk + blockIdx.x] = s;
  }
}

// Lanes of the warp whose 9-bit label equals this lane's: one ballot per
// label bit, a lane keeps the lanes that agree with it on every bit.
__device__ __forceinline__ u32 lanes_equal9(u32 label) {
  u32 m = kFull;
#pragma unroll
  for (int bit = 0; bit < 9; bit++) {
    const bool set = (label >> bit) & 1u;
    const u32 v = __ballot_sync(kFull, set);
    m &= set ? v : ~v;
  }
  return m;
}

// Shared memory of the scatter: two tile buffers (the next tile is copied in
// while the current one is ranked), per-warp digit counters, which the tile's
// source order reuses once the ranks are final, and the tile's output bases.
template <class K, class V>
struct RsSmem {
  K keys[2][kRsTile];
  V vals[2][kRsTile];
  union {
    u32 wcnt[kRsWarps][256];
    unsigned short sidx[kRsTile];  // sorted position -> position in the tile
  } u;
  u32 gbase[256];  // output position of the tile's sorted position 0 of each digit
  u32 wsum[kRsWarps];
  unsigned long long full[2];
  u32 fail;
};
static_assert(kRsTile <= 65536, "tile positions are 16-bit");

// Persistent: CTA c takes tiles c, c + gridDim.x, ... Thread 0 starts the
// bulk copy of the next tile's keys and values before the current tile is
// ranked, so the load latency stays off the critical path. Partial tiles (or
// bases that are not 16-byte aligned, bulk == 0) are loaded by all threads.
template <class K, class V>
__global__ void __launch_bounds__(kRsThreads) k_rs_scatter(const K *__restrict__ kin,
                                                           const V *__restrict__ vin,
                                                           K *__restrict__ kout, V *__restrict__ vout,
                                                           i64 n, int shift, const u32 *__restrict__ offs,
                                                           int nblk, int bulk, u32 *err) {
  extern __shared__ __align__(128) unsigned char rs_raw[];
  RsSmem<K, V> &S = *reinterpret_cast<RsSmem<K, V> *>(rs_raw);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const u32 lt_mask = (1u << lane) - 1u;
  const int G = gridDim.x;
  auto tile_cnt = [&](int t) { return int(min(i64(kRsTile), n - i64(t) * kRsTile)); };
  auto staged = [&](int t) { return bulk && tile_cnt(t) == kRsTile; };
  auto issue = [&](int t, int b) {  // thread 0
    if (staged(t)) {
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");  // after the buffer's last generic reads
      mbar_arrive_tx(&S.full[b], u32(kRsTile * (sizeof(K) + sizeof(V))));
      bulk_g2s(S.keys[b], kin + i64(t) * kRsTile, u32(kRsTile * sizeof(K)), &S.full[b]);
      bulk_g2s(S.vals[b], vin + i64(t) * kRsTile, u32(kRsTile * sizeof(V)), &S.full[b]);
    } else {
      mbar_arrive(&S.full[b]);  // completes the phase; the threads load the tile themselves
    }
  };
  if (tid == 0) {
    mbar_init(&S.full[0], 1);
    mbar_init(&S.full[1], 1);
    S.fail = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  }
  __syncthreads();
  if (tid == 0 && int(blockIdx.x) < nblk) issue(blockIdx.x, 0);
  int it = 0;
  for (int t = blockIdx.x; t < nblk; t += G, it++) {
    const int b = it & 1;
    const int cnt = tile_cnt(t);
    if (tid == 0 && t + G < nblk) issue(t + G, b ^ 1);  // its buffer was last read before the loop's end barrier
    const u32 my_off = offs[i64(tid) * nblk + t];          // thread tid: digit tid
    for (int i = tid; i < kRsWarps * 256; i += kRsThreads) (&S.u.wcnt[0][0])[i] = 0;
    if (!staged(t)) {
      for (int i = tid; i < cnt; i += kRsThreads) {
        S.keys[b][i] = kin[i64(t) * kRsTile + i];
        S.vals[b][i] = vin[i64(t) * kRsTile + i];
      }
    }
    if (!mbar_wait(&S.full[b], u32(it >> 1) & 1u)) S.fail = 1;
    __syncthreads();
    if (S.fail) break;
    // Rank within the warp: warp w holds tile positions [512 w, 512 w + 512)
    // in (step, lane) order, so ranks follow input order.
    const int wbase = warp * (kRsItems * 32);
    u32 r[kRsItems], dg[kRsItems];
#pragma unroll
    for (int j = 0; j < kRsItems; j++) {  // digits first (256: no key), then the lanes sharing each
      const int idx = wbase + j * 32 + lane;
      dg[j] = idx < cnt ? (u32(S.keys[b][idx] >> shift) & 255u) : 256u;
    }
#pragma unroll
    for (int j = 0; j < kRsItems; j++) r[j] = lanes_equal9(dg[j]);
    // The per-warp counters are the only chain: one shared read and one
    // write per step.
#pragma unroll
    for (int j = 0; j < kRsItems; j++) {
      const u32 d = dg[j], peers = r[j];
      const bool valid = d < 256u;
      u32 before = 0;
      if (valid) before = S.u.wcnt[warp][d];
      __syncwarp();
      if (valid && lane == __ffs(peers) - 1) S.u.wcnt[warp][d] = before + __popc(peers);
      __syncwarp();
      r[j] = before + __popc(peers & lt_mask);
    }
    __syncthreads();
    // Thread d: the tile's count of digit d, its start in the tile's sorted
    // order (block exclusive scan over digits) and each warp's start within it.
    {
      u32 c[kRsWarps], tot = 0;
#pragma unroll
      for (int w = 0; w < kRsWarps; w++) {
        c[w] = S.u.wcnt[w][tid];
        tot += c[w];
      }
      u32 inc = tot;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const u32 v = __shfl_up_sync(kFull, inc, o);
        if (lane >= o) inc += v;
      }
      if (lane == 31) S.wsum[warp] = inc;
      __syncthreads();
      u32 start = inc - tot;
      for (int w = 0; w < warp; w++) start += S.wsum[w];
      S.gbase[tid] = my_off - start;
#pragma unroll
      for (int w = 0; w < kRsWarps; w++) {
        S.u.wcnt[w][tid] = start;
        start += c[w];
      }
    }
    __syncthreads();
#pragma unroll
    for (int j = 0; j < kRsItems; j++)
      if (dg[j] < 256u) r[j] += S.u.wcnt[warp][dg[j]];
    __syncthreads();  // the counters are dead: their space takes the source order
#pragma unroll
    for (int j = 0; j < kRsItems; j++)
      if (dg[j] < 256u) S.u.sidx[r[j]] = (unsigned short)(wbase + j * 32 + lane);
    __syncthreads();
    // Out in sorted order: consecutive threads write consecutive positions of
    // one digit's run.
#pragma unroll
    for (int q = 0; q < kRsItems; q++) {
      const int i = q * kRsThreads + tid;
      if (i < cnt) {
        const int src = S.u.sidx[i];
        const K key = S.keys[b][src];
        const u32 pos = S.gbase[u32(key >> shift) & 255u] + u32(i);
        kout[pos] = key;
        vout[pos] = S.vals[b][src];
      }
    }
    __syncthreads();
  }
  if (S.fail && tid == 0) {
    atomicOr(err, ERRB_TIMEOUT);
    // The current and the next tile's copies may be in flight: wait for them
    // (bounded) before the CTA's shared memory is released.
    const int t = int(blockIdx.x) + it * G;
    mbar_wait(&S.full[it & 1], u32(it >> 1) & 1u);
    if (t + G < nblk) mbar_wait(&S.full[(it + 1) & 1], u32((it + 1) >> 1) & 1u);
  }
}

}  // namespace

namespace {
template <class K, class V>
int rs_grid(int nblk) {
  static int per_sm[64] = {0}, sms[64] = {0};
  int dev = 0;
  FCC_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= 64) throw Error{FCC_ERR_CUDA, "device ordinal out of range"};
  if (per_sm[dev] == 0) {
    const int smem = int(sizeof(RsSmem<K, V>));
    FCC_CUDA(cudaFuncSetAttribute(k_rs_scatter<K, V>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
    int p = 0;
    FCC_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&p, k_rs_scatter<K, V>, kRsThreads, smem));
    FCC_CUDA(cudaDeviceGetAttribute(&sms[dev], cudaDevAttrMultiProcessorCount, dev));
    if (p < 1) throw Error{FCC_ERR_CUDA, "radix scatter does not fit on an SM"};
    per_sm[dev] = p;
  }
  return std::min(nblk, per_sm[dev] * sms[dev]);
}

template <class K, class V>
void radix_sort_impl(K *keys, V *vals, i64 n, int nbits, Arena &ar, cudaStream_t s, u32 *err) {
  if (n <= 1 || nbits <= 0) return;
  if (n > i64(0xFFFFFFFFu)) throw Error{FCC_ERR_ARG, "radix sort: more than 2^32 keys"};
  const int nblk = int((n + kRsTile - 1) / kRsTile);
  K *k2 = ar.get_n<K>(size_t(n));
  V *v2 = ar.get_n<V>(size_t(n));
  u32 *hist = ar.get_n<u32>(size_t(nblk) * 256);
  K *ka = keys, *kb = k2;
  V *va = vals, *vb = v2;
  const int grid = rs_grid<K, V>(nblk);
  const bool aligned = ((reinterpret_cast<uintptr_t>(keys) | reinterpret_cast<uintptr_t>(vals) |
                         reinterpret_cast<uintptr_t>(k2) | reinterpret_cast<uintptr_t>(v2)) & 15) == 0;
  const int passes = (nbits + 7) / 8;
  for (int p = 0; p < passes; p++) {
    const int shift = 8 * p;
    k_rs_hist<K><<<nblk, kRsThreads, 0, s>>>(ka, n, shift, hist, nblk);
    FCC_LAUNCH_CHECK();
    scan_exclusive(hist, hist, i64(nblk) * 256, nullptr, ar, s);
    k_rs_scatter<K, V><<<grid, kRsThreads, sizeof(RsSmem<K, V>), s>>>(ka, va, kb, vb, n, shift, hist, nblk,
                                                                       aligned ? 1 : 0, err);
    FCC_LAUNCH_CHECK();
    std::swap(ka, kb);
    std::swap(va, vb);
  }
  if (ka != keys) {
    FCC_CUDA(cudaMemcpyAsync(keys, ka, sizeof(K) * size_t(n), cudaMemcpyDeviceToDevice, s));
    FCC_CUDA(cudaMemcpyAsync(vals, va, sizeof(V) * size_t(n), cudaMemcpyDeviceToDevice, s));
  }
}
}  // namespace

void radix_sort_pairs(u64 *keys, u32 *vals, i64 n, int nbits, Arena &ar, cudaStream_t s, u32 *err) {
  radix_sort_impl<u64, u32>(keys, vals, n, nbits, ar, s, err);
}

void radix_sort_pairs64(u64 *keys, u64 *vals, i64 n, int nbits, Arena &ar, cudaStream_t s, u32 *err) {
  radix_sort_impl<u64, u64>(keys, vals, n, nbits, ar, s, err);
}

void radix_sort_pairs64(u32 *keys, u64 *vals, i64 n, int nbits, Arena &ar, cudaStream_t s, u32 *err) {
  if (nbits > 32) throw Error{FCC_ERR_ARG, "radix sort: more bits than a 32-bit key holds"};
  radix_sort_impl<u32, u64>(keys, vals, n, nbits, ar, s, err);
}

}  // namespace fcc
