// Internal declarations shared by the CUDA translation units of
// libfastcc_gpu.so. Not part of the public ABI (include/fastcc_gpu.h is).
#pragma once

#include <cuda_runtime.h>

#include <atomic>
#include <cstdint>
#include <cstdio>
#include <map>
#include <string>
#include <vector>

#include "../../include/fastcc_gpu.h"

namespace fcc {

using u32 = uint32_t;
using u64 = uint64_t;
using i64 = int64_t;

constexpr u32 kFull = 0xFFFFFFFFu;
constexpr u64 kEmptyKey = ~0ull;

// Bits of the device error word. The host maps them to fcc_status.
enum ErrBits : u32 {
  ERRB_COORD = 1u,     // coordinate outside [0, max_index]
  ERRB_OVERFLOW = 2u,  // output capacity exceeded (host retries with the exact count)
  ERRB_HASH = 4u,      // hash probe limit reached
  ERRB_INTERNAL = 8u,  // an invariant of the plan did not hold
  ERRB_TIMEOUT = 16u,  // a bounded wait for a bulk copy (or an injected wait) gave up
};

#ifdef __CUDACC__
// Bulk asynchronous copies (cp.async.bulk) completed on shared-memory
// mbarriers. Every wait polls at most `polls` times (kWaitPolls unless a
// caller passes a shorter limit); a caller whose wait fails flags
// ERRB_TIMEOUT, waits (at the full limit) for its own copies in flight and
// stops.
constexpr long long kWaitPolls = 1ll << 24;

__device__ __forceinline__ u32 smem_addr(const void *p) { return u32(__cvta_generic_to_shared(p)); }

__device__ __forceinline__ bool mbar_wait(unsigned long long *bar, u32 parity, long long polls = kWaitPolls) {
  const u32 a = smem_addr(bar);
  for (long long it = 0; it < polls; it++) {
    u32 done;
    asm volatile("{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
                 : "=r"(done) : "r"(a), "r"(parity) : "memory");
    if (done) return true;
  }
  return false;
}

__device__ __forceinline__ void mbar_init(unsigned long long *bar, u32 count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_arrive(unsigned long long *bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_addr(bar)) : "memory");
}

__device__ __forceinline__ void mbar_arrive_tx(unsigned long long *bar, u32 bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
               : "memory");
}

// Global to shared memory; dst, src and bytes multiples of 16.
__device__ __forceinline__ void bulk_g2s(void *dst, const void *src, u32 bytes, unsigned long long *bar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                   smem_addr(dst)),
               "l"(src), "r"(bytes), "r"(smem_addr(bar))
               : "memory");
}
#endif

// Thrown inside the library and turned into a status at the C ABI.
struct Error {
  int status;
  std::string msg;
};

#define FCC_CUDA(call)                                                                  \
  do {                                                                                  \
    cudaError_t e_ = (call);                                                            \
    if (e_ != cudaSuccess)                                                              \
      throw ::fcc::Error{e_ == cudaErrorMemoryAllocation ? FCC_ERR_OOM : FCC_ERR_CUDA,  \
                         std::string(#call) + ": " + cudaGetErrorString(e_)};           \
  } while (0)

// Every kernel launch is followed by this check; it also counts launches.
extern std::atomic<long long> g_launches;
#define FCC_LAUNCH_CHECK()                                         \
  do {                                                             \
    ::fcc::g_launches.fetch_add(1, std::memory_order_relaxed);     \
    FCC_CUDA(cudaGetLastError());                                  \
  } while (0)

// Grow-only device workspace. Each contraction bump-allocates from one chunk
// taken from the context's stream-ordered memory pool; a call that outgrows it
// takes extra chunks, and the next call replaces them by one chunk of the
// high-water size, so steady-state calls allocate nothing.
//
// A fixed arena (init_fixed) instead bump-allocates from a caller-given
// buffer, never allocates, and reports FCC_ERR_CAPACITY when it runs out.
class Arena {
 public:
  void init(cudaMemPool_t pool) { pool_ = pool; }
  void init_fixed(void *base, size_t size) {
    fixed_ = true;
    fbase_ = static_cast<char *>(base);
    fsize_ = size;
  }
  void begin(cudaStream_t s);  // start of a call: consolidate to high-water size
  void *get(size_t bytes);     // 256-byte aligned, valid until the next begin()
  template <class T> T *get_n(size_t n) { return static_cast<T *>(get(sizeof(T) * (n ? n : 1))); }
  void release_all(cudaStream_t s);
  // release_all, forget the high-water size and return the pool's unused
  // memory to the device (after runs whose workspace says nothing of the
  // next calls', such as the autotuner's trials)
  void shrink(cudaStream_t s);
  // Device memory a call can still allocate: free on the device plus what the
  // pool holds unused.
  size_t available() const;
  size_t high_water() const { return high_; }
  bool is_fixed() const { return fixed_; }

 private:
  struct Chunk { char *p; size_t size; };
  cudaMemPool_t pool_ = nullptr;
  cudaStream_t stream_ = nullptr;
  std::vector<Chunk> chunks_;
  size_t used_ = 0, total_used_ = 0, high_ = 0;
  bool fixed_ = false;
  char *fbase_ = nullptr;  // fixed mode: the caller's buffer
  size_t fsize_ = 0;
};

// What one contraction runs against: a context's stream, workspace and
// scratch words, or the fixed scratch of an allocation-free call.
// Per-context state of the tile scheduler: the learned cost model (device
// copy) and the last contraction's per-tile record, which lives in the
// workspace and stays valid until the next contraction on the context.
struct SchedIo {
  float *model = nullptr;           // FCC_SCHED_MODEL_FLOATS on the device; NULL: none
  u32 ntiles = 0;
  const float *features = nullptr;  // ntiles x FCC_SCHED_FEATURES; NULL unless computed
  const u32 *cls = nullptr;         // class of each tile
  const double *cost = nullptr;     // measured cost of each tile (opts.timing = 2), else NULL
};

// fcc_sched.cu: per-tile features, predicted class costs, measured tile costs.
void tile_features(cudaStream_t st, const u32 *ntiles_p, u32 nmax, const u32 *abeg, const u64 *P, const u32 *nrows,
                   const u32 *lb, u64 LB, float *feat, int num_sms);
void predict_costs(cudaStream_t st, const u32 *ntiles_p, u32 nmax, const float *feat, const float *model,
                   float *pred);
void tile_costs(cudaStream_t st, u32 ntiles, const u32 *corder, const u32 *cls, const u32 *item_off,
                const u32 *t_items, const u64 *item_cyc, const double *occ, const u64 *merge_cyc,
                double merge_occ, double *cost);

struct WaveTune;  // below

struct Runtime {
  explicit Runtime(Arena &a) : arena(a) {}
  Arena &arena;
  cudaStream_t stream = nullptr;
  u32 *d_err = nullptr;            // device error word
  u64 *h_scalars = nullptr;        // host buffer of >= 32 entries
  int num_sms = 0;
  size_t smem_optin = 0;
  cudaEvent_t *ev = nullptr;       // FCC_NUM_PHASES + 1 events; NULL: no timing
  double *phase_ms = nullptr;      // FCC_NUM_PHASES entries or NULL
  cudaMemPool_t pool = nullptr;    // result buffers; NULL: the caller's buffers below
  u32 *out_coords = nullptr;       // caller output: coords SoA with out_stride between modes
  i64 out_stride = 0;
  double *out_vals = nullptr;
  u64 out_cap = 0;
  bool caller_out = false;         // write the output into out_* (any device-accessible memory)
  SchedIo *sched = nullptr;        // NULL: no learned schedule and no per-tile record
  // Streaming a caller output that lives in pinned host memory (NULL: not available):
  cudaStream_t copy_stream = nullptr;  // device-to-host copies of finished output ranges
  cudaEvent_t *wave_ev = nullptr;      // kMaxWaves + 1 events, one per wave and one after the merges
  u64 *h_cursors = nullptr;            // pinned, kMaxWaves + 1 output cursor snapshots
  WaveTune *wave_tune = nullptr;       // the context's choice between one copy and waves (NULL: one copy)
};

// A pinned host output is produced in at most this many waves of tiles.
constexpr int kMaxWaves = 16;

// out_waves 0 with a large pinned host output: the first such call copies
// the output once after the contraction, the second runs kAutoWaves waves
// (copies overlapping the contraction), and later calls take whichever was
// faster. Which one wins depends on the host link: the copies slow the tile
// kernels beside them by a factor that differs from box to box.
constexpr int kAutoWaves = 12;
constexpr unsigned long long kAutoWaveBytes = 1ull << 30;  // outputs below this: one copy
struct WaveTune {
  int trials = 0;    // calls measured so far (0, 1 or 2)
  double ms[2] = {}; // their wall times: one copy, waves
  int pick = 1;      // waves after the trials
};

void set_thread_error(const std::string &msg);
void *pool_alloc(cudaMemPool_t pool, size_t bytes, cudaStream_t st);  // fcc_prims.cu

}  // namespace fcc

struct fcc_ctx {
  int device = 0;
  int num_sms = 0;
  size_t smem_optin = 0;
  cudaStream_t own_stream = nullptr;
  cudaStream_t stream = nullptr;
  cudaMemPool_t pool = nullptr;
  fcc::Arena arena;
  fcc::u32 *d_err = nullptr;       // device error word
  fcc::u64 *h_scalars = nullptr;   // pinned host scalars for read-backs
  cudaEvent_t ev[FCC_NUM_PHASES + 1] = {};
  double phase_ms[FCC_NUM_PHASES] = {};
  cudaStream_t copy_stream = nullptr;          // output waves to pinned host buffers
  cudaEvent_t wave_ev[fcc::kMaxWaves + 1] = {};
  fcc::u64 *h_cursors = nullptr;               // pinned
  fcc::SchedIo sched;
  fcc::WaveTune wave_tune;
  std::map<std::string, std::pair<fcc_options, double>> tuned;  // autotuner cache: signature -> best
  std::string last_error;
};

struct fcc_result {
  int32_t order = 0;
  int64_t nnz = 0;
  int64_t cap = 0;       // stride between coordinate modes
  int64_t products = 0;
  fcc::u32 *d_coords = nullptr;
  double *d_vals = nullptr;
  fcc_ctx *ctx = nullptr;
  bool owned = true;     // false: the buffers belong to the caller
};

namespace fcc {

// ---- primitives (fcc_prims.cu) -------------------------------------------
// Exclusive prefix sums; `out` may alias `in`. When total != nullptr the sum of
// all n inputs is written to *total (device memory).
void scan_exclusive(const u32 *in, u32 *out, i64 n, u32 *total, Arena &ar, cudaStream_t s);
void scan_exclusive(const u64 *in, u64 *out, i64 n, u64 *total, Arena &ar, cudaStream_t s);
// Widening scan: u32 inputs, u64 prefix sums.
void scan_exclusive_wide(const u32 *in, u64 *out, i64 n, u64 *total, Arena &ar, cudaStream_t s);

// Stable LSD radix sort of (key, value) pairs on the low `nbits` bits of the
// keys. keys/vals are sorted in place (ping-ponging through scratch buffers
// taken from the arena).
// Stable LSD radix sort on the low nbits of the keys; err: device error word
// (ERRB_INTERNAL when a copy wait of the scatter gives up).
void radix_sort_pairs(u64 *keys, u32 *vals, i64 n, int nbits, Arena &ar, cudaStream_t s, u32 *err);
void radix_sort_pairs64(u64 *keys, u64 *vals, i64 n, int nbits, Arena &ar, cudaStream_t s,
                        u32 *err);  // 64-bit payload
void radix_sort_pairs64(u32 *keys, u64 *vals, i64 n, int nbits, Arena &ar, cudaStream_t s,
                        u32 *err);  // 32-bit keys (nbits <= 32), 64-bit payload

inline int grid_for(i64 n, int threads, int max_blocks = 1 << 20) {
  i64 b = (n + threads - 1) / threads;
  if (b < 1) b = 1;
  if (b > max_blocks) b = max_blocks;
  return int(b);
}

inline int bits_for(u64 max_value) {  // bits needed to represent max_value
  int b = 0;
  while (b < 64 && (max_value >> b) != 0) b++;
  return b;
}

}  // namespace fcc
