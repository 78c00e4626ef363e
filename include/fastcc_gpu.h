/*
 * fastcc_gpu.h - C ABI of the GB300 (sm_103a) sparse x sparse tensor
 * contraction. Plain pointers and sizes only; no CUDA or C++ types.
 *
 * It replaces the CPU path behind the reference's
 *   template <class AccType, class RES, class RIGHT>
 *   ListTensor<RES> Tensor<DT>::fastcc_multiply(Tensor<RIGHT> &other,
 *       CoOrdinate left_contr, CoOrdinate right_contr, int tile_size = 100)
 * (contract.hpp:824-912 of jianjianh1/fastcc-benchmark). The header-only C++
 * shim in fastcc-benchmark_gb300/host/contract.hpp keeps that call and its
 * types and forwards to fcc_contract below.
 *
 * Semantics kept from the reference:
 *  - operand shape = per-mode max index (Tensor::_infer_shape,
 *    contract.hpp:124-144); radix of a mode = max index + 1;
 *  - contraction modes are paired by position in ctrA/ctrB; the contraction
 *    key is linearised in list order with each operand's own radices
 *    (CoOrdinate::gather_linearize, coordinate.hpp:723-733) unless
 *    FCC_RADIX_SHARED is requested;
 *  - output coordinates: A's non-contracted modes in ascending order, then B's
 *    (CompactCordinate, coordinate.hpp:402-427), decoded with the external
 *    modes' own extents;
 *  - one output per structurally reached (A external, B external) pair, exact
 *    zero sums included (TileAccumulator::drain_into,
 *    index_tensors.hpp:1039-1060); output order is unspecified, as the
 *    reference's per-thread list concatenation leaves it (contract.hpp:906-909).
 * All value arithmetic is IEEE double. Every call returns an fcc_status.
 */
#ifndef FASTCC_GPU_H
#define FASTCC_GPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define FCC_MAX_ORDER 8
#define FCC_ABI_VERSION 5

typedef enum fcc_status {
  FCC_OK = 0,
  FCC_ERR_ARG = 1,       /* invalid argument or coordinate outside [0, max_index] */
  FCC_ERR_OOM = 2,       /* device or pinned-host allocation failed */
  FCC_ERR_HASH_FULL = 3, /* a hash accumulator ran out of slots */
  FCC_ERR_TIMEOUT = 4,   /* a bounded device wait gave up */
  FCC_ERR_CUDA = 5,      /* CUDA runtime error (see fcc_last_error) */
  FCC_ERR_OVERFLOW = 6,  /* an index space or count exceeds 64 bits */
  FCC_ERR_NO_DEVICE = 7, /* no usable sm_103 device */
  FCC_ERR_CAPACITY = 8   /* caller-provided output buffer too small */
} fcc_status;

typedef enum fcc_location { FCC_HOST = 0, FCC_DEVICE = 1 } fcc_location;

/* Accumulator policy. The reference selects it by template argument:
 * TileAccumulator<double> (dense tile, index_tensors.hpp:994-1065) or
 * TileAccumulatorMap<double> (hash, :843-883). Results are identical. */
typedef enum fcc_accumulator {
  FCC_ACC_AUTO = 0,  /* planner picks per contraction */
  FCC_ACC_DENSE = 1, /* shared-memory dense tile (needs the B external span to fit) */
  FCC_ACC_HASH = 2   /* shared-memory open-addressing hash, global hash for split tiles */
} fcc_accumulator;

typedef enum fcc_radix_mode {
  FCC_RADIX_PER_OPERAND = 0, /* the reference's contraction key (own max index per operand) */
  FCC_RADIX_SHARED = 1       /* max over both operands per contracted pair */
} fcc_radix_mode;

/* A COO operand. coords[n*stride_nnz + m*stride_mode] is mode m of nonzero n
 * (AoS: stride_nnz=order, stride_mode=1; SoA: stride_nnz=1, stride_mode=nnz).
 * max_index is always a HOST array of `order` entries; coords and values live
 * where `location` says. Coordinates must lie in [0, max_index[m]]. */
typedef struct fcc_tensor {
  int32_t order;
  int64_t nnz;
  const int32_t *max_index;
  const int32_t *coords;
  int64_t stride_nnz;
  int64_t stride_mode;
  const double *values;
  int32_t location;
} fcc_tensor;

/* Tuning knobs. Zero-initialise for defaults (fcc_options_default). */
typedef struct fcc_options {
  int32_t tile_size;          /* the reference's tile_size; accepted for signature parity, 0 = 100 */
  int32_t accumulator;        /* fcc_accumulator */
  int32_t radix_mode;         /* fcc_radix_mode */
  int32_t rows_per_tile;      /* A external rows per output tile; 0 = planner */
  int64_t products_per_item;  /* multiply-adds per work item; 0 = planner */
  int32_t dense_cap;          /* doubles per shared-memory dense tile; 0 = planner */
  int32_t hash_slots;         /* shared-memory hash slots (power of two); 0 = planner */
  int32_t timing;             /* 1: record per-phase CUDA-event times (fcc_last_timings) */
  int32_t esc_small;          /* expanded pairs reduced in shared memory (esc_reduce): tiles
                                 with at most this many pairs are small (reduced in windows of
                                 consecutive small tiles), larger ones are partitioned by key
                                 blocks first; 0 (default): 4096, the largest allowed */
  int64_t capacity_hint;      /* first output allocation in entries; 0 = planner bound. A
                                 smaller hint is not an error: the device counts every output
                                 and the call retries once with the exact count. */
  int32_t dense_mode;         /* fcc_dense_mode: how a dense tile marks touched positions */
  int32_t tile_threads;       /* threads per tile CTA: dense tiles 640 (default), 512, 768 or
                                 1024; the large hash table 1024 (default), 128, 256 or 512 */
  int32_t hot_columns;        /* per-warp copies of the most frequent B columns in row tiles:
                                 0 or -1 off (default), or a count (multiple of 32) */
  int32_t schedule;           /* fcc_schedule: how each output tile picks its class */
  int32_t dense_fill_log2;    /* FCC_SCHED_RULE: a tile takes the dense class only when its
                                 multiply-adds >= its area / 2^dense_fill_log2; -1: whenever the
                                 tile fits the dense accumulator; 0 (default): 2 when hash tiles
                                 are expanded (hash_esc), else -1 */
  int32_t dense_staging;      /* 0: dense tiles stage the B segments of long A entries in shared
                                 memory with bulk copies when the ring fits beside the tile;
                                 -1: never */
  int32_t sched_mix_margin;   /* FCC_SCHED_LEARNED: 0 (default): per-tile choices; > 0: one class for
                                 every tile unless the model predicts the per-tile mix faster than
                                 the best single class by this many percent */
  int32_t hash_esc;           /* hash tiles expanded to (key, value) pairs, radix-sorted and
                                 reduced instead of accumulated in shared-memory tables, when the
                                 pairs fit in device memory. 2: every hash tile; 1: the tiles
                                 larger than their table (the others run the tables); -1: none
                                 (large tiles split into items merged through a global hash
                                 table); 0 (default): 2, or 1 with a forced hash class, or -1
                                 in allocation-free calls */
  int32_t out_waves;          /* fcc_contract_into with pinned host output buffers: the output is
                                 produced in device memory in this many waves of tiles (1..16),
                                 each wave's outputs copied to the host while the next computes.
                                 0 (default): one wave (the whole output computed, then copied
                                 once), except for outputs of 1 GiB or more: the context's first
                                 such call copies once, its second runs 12 waves, and later calls
                                 take whichever of the two was faster */
  int32_t esc_group;          /* expanded hash tiles are sorted in groups whose keys fit 32 bits;
                                 0 (default): as many tiles per group as that allows; > 0: at
                                 most this many */
  int32_t wait_polls;         /* poll limit of the dense tiles' waits on their staging ring
                                 (consumers waiting for a chunk, the producer waiting for a free
                                 buffer); a wait that runs out ends the call with
                                 FCC_ERR_TIMEOUT. 0 (default): 2^24. The final wait for a CTA's
                                 own copies in flight always uses 2^24 */
  int32_t fault_wait;         /* fault injection for tests: 1 makes the consumer warps of every
                                 staged dense item first wait on an mbarrier that nothing
                                 completes, so that the wait runs out after wait_polls polls and
                                 the call returns FCC_ERR_TIMEOUT; the context stays usable.
                                 0 (default): off */
  int32_t dense_kernel;       /* how a dense tile runs its multiply-adds. 1: two phases (A entries
                                 with long B segments by the whole CTA through a bulk-copy ring
                                 with plain read-modify-writes, the rest by warps, windows of one
                                 entry per lane, compare-and-swap updates); 2: flat (warps take
                                 runs of consecutive multiply-adds, one per lane,
                                 compare-and-swap updates); 3: two phases, the second run flat
                                 with atomic adds. 0 (default): 3, except under the learned
                                 schedule, whose FCC_CLASS_DENSE tiles run 1 (and whose
                                 FCC_CLASS_DENSE_FLAT tiles run 2) */
  int32_t esc_reduce;         /* how expanded pairs (hash_esc) are reduced. 0 (default) or 1: in
                                 shared memory, no sort: small tiles in hash tables over
                                 windows of consecutive small tiles, large ones computed
                                 straight into blocks of 8192 keys, each block reduced densely
                                 or, when sparse, with its sparse neighbours in a hash table;
                                 used where a tile spans at most 2^21 keys and the pairs (each
                                 small tile padded to 8) count in 32 bits, else 2. 2: a radix
                                 sort of groups of tiles whose keys fit 32 bits (64-bit keys
                                 otherwise), then one pass over the runs of equal keys */
} fcc_options;

/* Tile classes: every output tile runs in one of them. The hash classes
 * differ in table size and CTA shape: the small ones run several CTAs per SM
 * so that small tiles overlap their barriers and memory latency. The two
 * dense classes share the tile; they differ in how the CTA runs its
 * multiply-adds (dense_kernel): the rule uses FCC_CLASS_DENSE only, the
 * learned schedule picks between the two per tile. */
enum {
  FCC_CLASS_DENSE = 0,       /* shared-memory dense tile, 640 threads (tile_threads), dense_kernel */
  FCC_CLASS_HASH_L = 1,      /* hash, 8192 slots, 1024 threads (tile_threads), one CTA per SM */
  FCC_CLASS_HASH_M = 2,      /* hash, 4096 slots, 256 threads */
  FCC_CLASS_HASH_S = 3,      /* hash, 2048 slots, 128 threads */
  FCC_CLASS_DENSE_FLAT = 4,  /* the dense tile with flat items (dense_kernel 2) */
  FCC_NUM_CLASSES = 5
};

typedef enum fcc_schedule {
  FCC_SCHED_RULE = 0,     /* dense when the tile fits it (see dense_fill_log2), else the smallest
                             hash table that holds the tile without splitting it */
  FCC_SCHED_LEARNED = 1,  /* the rule's class, overridden per tile where the context's cost model
                             (fcc_sched_set_model) predicts another class at least 25% cheaper
                             (between the two dense classes: at least 5% cheaper); the rule
                             alone, without features or predictions, when no model is set or
                             no tile has a choice (no dense class and every hash tile
                             expanded) */
  FCC_SCHED_FORCE = 2     /* FCC_SCHED_FORCE + class: one class for every tile */
} fcc_schedule;

/* Touched-position tracking of the dense accumulator. Both emit every touched
 * position, exact zero sums included. The sentinel form is used only when no
 * input value is zero or below 1e-150 in magnitude. */
typedef enum fcc_dense_mode {
  FCC_DENSE_AUTO = 0,     /* sentinel when the tiles are well filled */
  FCC_DENSE_BITMASK = 1,  /* a touched bit per position */
  FCC_DENSE_SENTINEL = 2  /* untouched positions hold -0.0 */
} fcc_dense_mode;

typedef struct fcc_ctx fcc_ctx;       /* one device, one stream, one workspace */
typedef struct fcc_result fcc_result; /* device-resident output of one contraction */

/* Phases reported by fcc_last_timings (milliseconds). */
enum {
  FCC_PHASE_UPLOAD = 0,  /* host->device copy of host operands */
  FCC_PHASE_INDEX = 1,   /* linearise + radix sort + segment build + lookup (index_tensors.hpp:506-547) */
  FCC_PHASE_PLAN = 2,    /* tiles, work items, capacity */
  FCC_PHASE_CONTRACT = 3,/* tile contraction + drain (contract.hpp:876-904) */
  FCC_PHASE_MERGE = 4,   /* split-tile merge drain */
  FCC_PHASE_TOTAL = 5,
  FCC_NUM_PHASES = 6
};

/* Context. device < 0 selects the current device. */
int fcc_ctx_create(int32_t device, fcc_ctx **out);
int fcc_ctx_destroy(fcc_ctx *ctx);
/* Use a caller-owned cudaStream_t (passed as void*); NULL restores the ctx stream. */
int fcc_ctx_set_stream(fcc_ctx *ctx, void *cuda_stream);
/* Text of the last error recorded on this context (never NULL). */
const char *fcc_last_error(const fcc_ctx *ctx);
const char *fcc_status_string(int32_t status);
int fcc_options_default(fcc_options *opts);

/*
 * out = A x B contracted over ctrA[i] <-> ctrB[i], i < k.
 * Replaces Tensor<DT>::fastcc_multiply (contract.hpp:824-912). Blocks until
 * the result count is known; the result stays on the device.
 */
int fcc_contract(fcc_ctx *ctx, const fcc_tensor *A, const fcc_tensor *B, const int32_t *ctrA,
                 const int32_t *ctrB, int32_t k, const fcc_options *opts, fcc_result **out);

/*
 * The contraction written into the caller's buffers: coords (mode m at
 * out_coords[m * out_mode_stride + i], uint32, out_mode_stride >=
 * out_capacity) and out_values, out_capacity entries, in any memory the
 * device can write: device memory, or pinned host memory, in which case the
 * output is produced in device memory in waves of tiles (opts->out_waves) and
 * each wave's entries are copied to the host while the next wave computes;
 * the allocation-free context has no copy stream and writes pinned host
 * memory from the kernels. Entry order is unspecified. Returns FCC_ERR_CAPACITY with
 * *out_nnz = the entries needed when the output does not fit (the buffers'
 * contents are then undefined). No counterpart in the reference, whose
 * output goes to a host list.
 */
int fcc_contract_into(fcc_ctx *ctx, const fcc_tensor *A, const fcc_tensor *B, const int32_t *ctrA,
                      const int32_t *ctrB, int32_t k, const fcc_options *opts, uint32_t *out_coords,
                      int64_t out_mode_stride, double *out_values, int64_t out_capacity, int64_t *out_nnz,
                      int64_t *out_products);

/* Result access. Replaces ListTensor's compute_nnz_count/run_through_nnz
 * (index_tensors.hpp:105-114), which are the reference's only accessors. */
int fcc_result_info(const fcc_result *r, int32_t *order, int64_t *nnz, int64_t *products);
/* Device pointers: coords SoA as order arrays of nnz uint32 with stride
 * `*mode_stride` elements between modes; values nnz doubles. */
int fcc_result_device(const fcc_result *r, const uint32_t **coords, int64_t *mode_stride,
                      const double **values);
/* Copies to host buffers; coords gets nnz*order int32 at
 * coords[n*stride_nnz + m*stride_mode]; either pointer may be NULL. */
int fcc_result_copy_to_host(const fcc_result *r, int32_t *coords, int64_t stride_nnz,
                            int64_t stride_mode, double *values);
int fcc_result_free(fcc_result *r);

/* Per-phase times of the last fcc_contract on ctx with opts.timing=1. */
int fcc_last_timings(const fcc_ctx *ctx, double *ms, int32_t n);

/* Multiply-add count sum_c nA(c)*nB(c) (SymbolicTensor::count_ops,
 * index_tensors.hpp:287-303, in 64 bits) computed on the device. */
int fcc_count_products(fcc_ctx *ctx, const fcc_tensor *A, const fcc_tensor *B,
                       const int32_t *ctrA, const int32_t *ctrB, int32_t k,
                       const fcc_options *opts, int64_t *products);

int fcc_abi_version(void);

/*
 * Contraction with batch modes: modes batchA[i] of A and batchB[i] of B
 * (nb pairs) are matched like contracted modes but kept in the output.
 * Replaces Tensor<DT>::multiply(other, left_contr, left_batch, right_contr,
 * right_batch) (contract.hpp:284-367) and its _inner_outer_multiply variant
 * (contract.hpp:1356-1435): output coordinates are the batch modes in
 * batchA order, then A's other non-contracted modes ascending, then B's.
 * Needs order(A) + nb <= FCC_MAX_ORDER.
 */
int fcc_contract_modes(fcc_ctx *ctx, const fcc_tensor *A, const fcc_tensor *B, const int32_t *ctrA,
                       const int32_t *ctrB, int32_t k, const int32_t *batchA, const int32_t *batchB,
                       int32_t nb, const fcc_options *opts, fcc_result **out);

/*
 * Batched contraction: n independent products A[t] x B[t] of one mode
 * pattern (every A[t] of one order, every B[t] of one order, the same ctrA,
 * ctrB, k), run as ONE pipeline: one index build, one tile plan and one
 * persistent tile-kernel launch for the whole batch. The reference has no
 * batched call; it replaces n calls of Tensor<DT>::fastcc_multiply
 * (contract.hpp:824-912) and gives, per instance, exactly their entries.
 *
 * The result has one more mode than a single product: mode 0 is the
 * instance t, followed by t's output coordinates in fcc_contract's order.
 * Entries of all instances are interleaved in no particular order; counts
 * (n int64, may be NULL) receives each instance's entry count. Limits:
 * order(A) <= 6, order(B) <= 7, and per operand at most 2^31-1 nonzeros
 * over the batch. opts->radix_mode is ignored: radices are shared.
 */
int fcc_contract_batch(fcc_ctx *ctx, int32_t n, const fcc_tensor *A, const fcc_tensor *B,
                       const int32_t *ctrA, const int32_t *ctrB, int32_t k, const fcc_options *opts,
                       fcc_result **out, int64_t *counts);

/*
 * fcc_contract_noalloc - the contraction for callers that cannot allocate
 * device memory. It has no counterpart in the reference (whose CPU code
 * allocates freely).
 *
 * Some hosts forbid device allocation after start-up: services that reserve
 * all device memory for their own pool, real-time loops where cudaMalloc's
 * device-wide synchronisation and unbounded latency are not acceptable, or
 * plugins that must leave their host process's device heap alone. They cannot
 * create an fcc_ctx (which allocates a workspace, events and result buffers).
 * This entry point takes the inputs and the OUTPUT buffers from the caller
 * and runs the same kernels, with every temporary taken from one static
 * device array of FCC_NOALLOC_SCRATCH_BYTES (32 MiB) defined in the library.
 * Every GPU that loads the library holds that array until the process exits.
 * It calls no cudaMalloc, cudaFree or other allocating routine.
 *
 * Limits: nnz(A) + nnz(B) <= FCC_NOALLOC_MAX_NNZ, and the contraction's
 * temporaries must fit the array; otherwise FCC_ERR_CAPACITY with a message
 * (fcc_last_error(NULL)). Outputs go to out_coords (mode m at
 * out_coords[m * out_mode_stride + i], uint32) and out_values, device
 * buffers of out_capacity entries; when the output is larger, the call
 * returns FCC_ERR_CAPACITY and *out_nnz holds the count needed.
 *
 * Set-up: the first call on each device looks up the array's device address
 * (cudaGetSymbolAddress, with that device current); make that first call
 * before any stream capture. Work runs on cuda_stream (a cudaStream_t, NULL
 * for the default stream) and the call returns when the result is ready.
 * All calls share the one array and it keeps the last call's contents: calls
 * that overlap on the GPU (other host threads, other streams) race with each
 * other and must be serialised by the caller. opts->timing is ignored.
 */
#define FCC_NOALLOC_SCRATCH_BYTES (32u << 20)
#define FCC_NOALLOC_MAX_NNZ 131072
int fcc_contract_noalloc(const fcc_tensor *A, const fcc_tensor *B, const int32_t *ctrA,
                         const int32_t *ctrB, int32_t k, const fcc_options *opts, void *cuda_stream,
                         uint32_t *out_coords, int64_t out_mode_stride, double *out_values,
                         int64_t out_capacity, int64_t *out_nnz, int64_t *out_products);

/*
 * Autotuner (no counterpart in the reference, whose tile size and
 * accumulator are fixed by the caller). Times the contraction, reps runs
 * after one warm-up, under each candidate: the rule (fill threshold 0 or
 * 2^-6) and the dense class forced, each with 512 and 1024 threads per dense
 * tile, and each hash class forced. *best receives the fastest candidate
 * (base's other fields kept) and *best_ms its mean total time. The winner is
 * cached on ctx under the problem's shape signature (orders, contracted
 * modes, log2 buckets of the nonzero counts and mode extents): a later call
 * on a same-shaped problem returns it without running anything.
 */
int fcc_autotune(fcc_ctx *ctx, const fcc_tensor *A, const fcc_tensor *B, const int32_t *ctrA,
                 const int32_t *ctrB, int32_t k, const fcc_options *base, int32_t reps, fcc_options *best,
                 double *best_ms);
/* The same for a batch (fcc_contract_batch). */
int fcc_autotune_batch(fcc_ctx *ctx, int32_t n, const fcc_tensor *A, const fcc_tensor *B,
                       const int32_t *ctrA, const int32_t *ctrB, int32_t k, const fcc_options *base,
                       int32_t reps, fcc_options *best, double *best_ms);

/*
 * Learned tile schedule. The reference has no scheduler (its tiles all run
 * the one accumulator picked by template argument); these calls serve
 * FCC_SCHED_LEARNED.
 *
 * The cost model is an FP32 MLP, FCC_SCHED_FEATURES -> 64 -> 64 ->
 * FCC_NUM_CLASSES with ReLU, whose outputs are the predicted cost of a tile
 * in each class (log2 of SM cycles); a tile takes the class of lowest
 * prediction. Model layout (FCC_SCHED_MODEL_FLOATS floats): mean[12],
 * scale[12] (inputs are standardised as (x - mean) * scale), W1[12][64],
 * b1[64], W2[64][64], b2[64], W3[64][FCC_NUM_CLASSES], b3[FCC_NUM_CLASSES].
 * Features of a tile, in
 * order: log2(1 + multiply-adds), log2(1 + A entries), log2(rows),
 * log2(column span), log2(area = rows x span), estimated fill
 * min(multiply-adds, area) / area, the fractions of its multiply-adds whose
 * B segment is shorter than 64, 64..1023 and at least 1024 entries long,
 * log2(1 + mean segment length), log2(1 + longest segment), log2(1 +
 * multiply-adds per row).
 */
#define FCC_SCHED_FEATURES 12
#define FCC_SCHED_HIDDEN 64
#define FCC_SCHED_MODEL_FLOATS (2 * 12 + 12 * 64 + 64 + 64 * 64 + 64 + 64 * 5 + 5)
/* Installs (copies to the device) or, with model NULL, removes the model. */
int fcc_sched_set_model(fcc_ctx *ctx, const float *model, int64_t n);
/* Per-tile record of the last contraction on ctx: features (ntiles x 12;
 * computed with opts.timing = 2 or a learned schedule), class, and with
 * opts.timing = 2 the measured cost (SM cycles of its work items divided by
 * the CTAs per SM of its class). Copies min(cap, ntiles) tiles; any pointer
 * may be NULL; *ntiles receives the tile count. */
int fcc_sched_last_tiles(fcc_ctx *ctx, float *features, int32_t *cls, double *cost, int64_t cap,
                         int64_t *ntiles);
/* The MLP on the device (hand-written FP32 kernels). Host arrays, row-major:
 * X n x 12, Y and M (mask, 0 or 1) n x 4. Loss: sum M (y' - y)^2 / sum M. */
int fcc_mlp_predict(fcc_ctx *ctx, const float *X, int64_t n, const float *model, float *Y);
/* Gradient of the loss over all n rows, in model layout (mean and scale
 * entries get 0). */
int fcc_mlp_grad(fcc_ctx *ctx, const float *X, const float *Y, const float *M, int64_t n, const float *model,
                 float *grad, float *loss);
/* Adam (beta 0.9 / 0.999), minibatches of `batch` rows reshuffled every
 * epoch from `seed`; model holds the initial parameters (mean and scale
 * included, kept as given) and receives the trained ones; *loss gets the
 * final loss over all rows. */
int fcc_mlp_train(fcc_ctx *ctx, const float *X, const float *Y, const float *M, int64_t n, int32_t epochs,
                  int32_t batch, float lr, uint64_t seed, float *model, float *loss);

/* Diagnostics: kernels this process has launched through the library so far. */
int64_t fcc_launch_count(void);

/* Diagnostics: measured FP64 FMA rate of a device (FMA instructions per
 * second over all SMs), the compute roofline of the tile kernels, whose every
 * multiply-add is one FP64 FMA. device < 0: the current device. */
int fcc_diag_fp64_fma_rate(int32_t device, double *fma_per_second);

/* Diagnostics: FP64 accumulation rate into a 20,000-double shared-memory
 * tile on the current device (updates per second over all SMs). mode 0: the
 * built-in FP64 atomic add of a product; 1: a compare-and-swap loop around
 * one FMA; 2: an unsynchronised read-modify-write FMA. */
int fcc_diag_shared_update_rate(int32_t mode, double *updates_per_second);

/* Diagnostics: the library's stable LSD radix sort (8-bit digits over the
 * low nbits of each key) on caller data. keys[n] of key_bytes each with
 * payloads vals[n] of value_bytes each (8/4, 8/8 or 4/8), host memory; the
 * sorted pairs are written to keys_out / vals_out, and *ms_per_sort receives
 * the mean device time of one sort over `reps` sorts of the same input. */
int fcc_diag_radix_sort(const void *keys, int32_t key_bytes, const void *vals, int32_t value_bytes, int64_t n,
                        int32_t nbits, int32_t reps, void *keys_out, void *vals_out, double *ms_per_sort);

#ifdef __cplusplus
}
#endif
#endif
