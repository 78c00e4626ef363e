/*
 * fastcc_synth.h - seeded synthetic sparse tensors for the FaSTCC contraction
 * benchmarks and tests.
 *
 * The reference has no generator of its own: its runs read FROSTT `.tns`
 * files (read.hpp:58-106) downloaded by scripts/download_tensors.sh, and its
 * `Tensor(int size, int dims, int *shape)` constructor (contract.hpp:58-65,
 * index_tensors.hpp:168-183) draws unseeded, possibly duplicate coordinates.
 * This generator produces the seeded stand-in workloads instead: distinct COO
 * coordinates, each mode uniform or Zipf-distributed on its finite support,
 * and uniform[-1,1) or sign-random lognormal(0,1) values.
 *
 * Determinism: every draw is a pure function of (seed, stream, counter)
 * (SplitMix64 used as a counter-based generator), and the accepted nonzeros
 * are the first `nnz` distinct candidates in candidate order, so the output
 * does not depend on the number of host threads.
 */
#ifndef FASTCC_SYNTH_H
#define FASTCC_SYNTH_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum fcc_synth_values {
  FCC_SYNTH_UNIFORM = 0,   /* uniform[-1, 1) */
  FCC_SYNTH_LOGNORMAL = 1, /* random sign times exp(N(0,1)) */
};

/*
 * Draws `nnz` distinct coordinates of an `order`-way tensor with the given
 * extents. Mode m is uniform on [0, extents[m]) when zipf_s[m] <= 0, else
 * P(i) proportional to (i+1)^-zipf_s[m] on [0, extents[m]).
 * coords: caller buffer of nnz*order int32, row-major (nonzero-major, AoS).
 * values: caller buffer of nnz doubles.
 * *nnz_out receives the number produced; it is below nnz only when the
 * candidate budget (64*nnz + 2^20 draws) runs out because the support is too
 * small for that many distinct coordinates.
 * Returns 0 on success, 1 on bad arguments (order outside 1..8, extents < 1,
 * or a product of extents that does not fit in 63 bits).
 */
int fcc_synth_coo(uint64_t seed, int32_t order, const int64_t *extents,
                  const double *zipf_s, int64_t nnz, int32_t value_kind,
                  int32_t *coords, double *values, int64_t *nnz_out);

/* The raw counter-based stream: out[i] = splitmix64 draw (seed, stream, i). */
void fcc_synth_raw(uint64_t seed, uint64_t stream, int64_t n, uint64_t *out);

#ifdef __cplusplus
}
#endif
#endif
