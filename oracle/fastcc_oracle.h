/*
 * fastcc_oracle.h - TEST INFRASTRUCTURE ONLY. CPU restatement of the
 * reference FaSTCC contraction `Tensor<DT>::fastcc_multiply` (contract.hpp:
 * 824-912 of jianjianh1/fastcc-benchmark) used as the parity checker by the
 * tests, by the smoke check and by bench.py's CPU-baseline leg. No product
 * code path links, loads or calls anything in this directory.
 *
 * Parity pin: tests/golden/ holds outputs of the reference's own
 * fastcc_multiply (compiled from its sources with oracle/ref_harness.cpp) and
 * the tests check this restatement against them.
 */
#ifndef FASTCC_ORACLE_H
#define FASTCC_ORACLE_H
#include <stdint.h>
#ifdef __cplusplus
extern "C" {
#endif

typedef struct orc_tensor {
  int32_t order;
  int64_t nnz;
  const int32_t *coords;    /* nnz*order, nonzero-major (the reference's NNZ AoS) */
  const double *values;     /* nnz */
  const int32_t *max_index; /* order entries: the reference's shape[] (contract.hpp:124-144) */
} orc_tensor;

typedef struct orc_result {
  int64_t nnz;
  int32_t order;
  uint64_t *left;   /* A external linear index (the reference's left_index) */
  uint64_t *right;  /* B external linear index (right_index) */
  int32_t *coords;  /* nnz*order decoded output coordinates */
  double *values;
  double *abs_sum;  /* sum of |a*b| per output when requested, else NULL */
  int64_t products; /* multiply-adds performed */
  double index_ms;  /* tile index build (contract.hpp:854-862) */
  double compute_ms;/* tile-pair loop incl. drain (contract.hpp:876-904) */
  double total_ms;  /* the whole call: index, tile-pair loop, concatenation of the
                       per-thread outputs and their coordinate decode */
} orc_result;

/* Max index per mode, as Tensor::_infer_shape (contract.hpp:124-144). */
int orc_infer_shape(const int32_t *coords, int64_t nnz, int32_t order, int32_t *max_index);

/* The reference algorithm with TileAccumulator semantics and a correct drain
 * decode. tile_size as passed to fastcc_multiply (rounded as contract.hpp:844-846
 * and index_tensors.hpp:513-514 do). nthreads <= 0: all hardware threads.
 * Returns 0, or 1 on bad arguments. */
int orc_fastcc_multiply(const orc_tensor *A, const orc_tensor *B, const int32_t *ctrA,
                        const int32_t *ctrB, int32_t k, int32_t tile_size, int32_t nthreads,
                        int32_t want_abs, orc_result *out);

/* Independent check: joins on the contracted coordinate tuples themselves (no
 * linearisation) and returns outputs sorted by coordinates. Small inputs only. */
int orc_bruteforce(const orc_tensor *A, const orc_tensor *B, const int32_t *ctrA,
                   const int32_t *ctrB, int32_t k, orc_result *out);

/* Sum over shared contraction keys of nA(c)*nB(c), 64-bit (SymbolicTensor::
 * count_ops, index_tensors.hpp:287-303). */
int64_t orc_count_products(const orc_tensor *A, const orc_tensor *B, const int32_t *ctrA,
                           const int32_t *ctrB, int32_t k);

void orc_free(orc_result *r);

#ifdef __cplusplus
}
#endif
#endif
