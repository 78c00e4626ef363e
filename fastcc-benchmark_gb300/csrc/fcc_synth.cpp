// Seeded synthetic COO tensors (host code). See include/fastcc_synth.h.
//
// Random numbers: SplitMix64 (Steele, Lea, Flood, "Fast splittable
// pseudorandom number generators", OOPSLA 2014) evaluated at a counter, so
// draw i of stream s is mix(seed + (s * 2^40 + i) * gamma) and can be computed
// by any thread in any order.
// Zipf sampling: Walker's alias method in Vose's numerically stable
// construction (M. D. Vose, "A linear algorithm for generating random numbers
// with a given distribution", IEEE TSE 1991): O(extent) set-up, O(1) draws.
// Deduplication: partitioned open-addressing sets, one partition per thread;
// "first occurrence" flags are combined in candidate order so the accepted set
// is the first nnz distinct candidates whatever the thread count.

#include "../../include/fastcc_synth.h"

#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

constexpr uint64_t kGamma = 0x9E3779B97F4A7C15ull;

inline uint64_t mix64(uint64_t z) {
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

inline uint64_t draw(uint64_t seed, uint64_t stream, uint64_t i) {
  return mix64(seed + ((stream << 40) + i + 1) * kGamma);
}

inline double unit53(uint64_t x) {  // [0, 1)
  return double(x >> 11) * (1.0 / 9007199254740992.0);
}

struct Alias {
  int64_t n = 0;
  std::vector<uint32_t> thresh;  // accept own bucket when low32 < thresh
  std::vector<uint32_t> other;
  void build(int64_t n_, double s) {
    n = n_;
    thresh.assign(n, 0xFFFFFFFFu);
    other.resize(n);
    std::vector<double> p(n);
    double tot = 0;
    for (int64_t i = 0; i < n; i++) tot += (p[i] = std::pow(double(i + 1), -s));
    std::vector<int64_t> small, large;
    for (int64_t i = 0; i < n; i++) {
      p[i] = p[i] * double(n) / tot;
      (p[i] < 1.0 ? small : large).push_back(i);
    }
    while (!small.empty() && !large.empty()) {
      int64_t l = small.back(), g = large.back();
      small.pop_back();
      double t = p[l] * 4294967296.0;
      thresh[l] = t >= 4294967295.0 ? 0xFFFFFFFFu : uint32_t(t);
      other[l] = uint32_t(g);
      p[g] = (p[g] + p[l]) - 1.0;
      if (p[g] < 1.0) {
        large.pop_back();
        small.push_back(g);
      }
    }
    for (int64_t i : small) { thresh[i] = 0xFFFFFFFFu; other[i] = uint32_t(i); }
    for (int64_t i : large) { thresh[i] = 0xFFFFFFFFu; other[i] = uint32_t(i); }
  }
  inline int64_t sample(uint64_t x) const {
    int64_t b = int64_t(((x >> 32) * uint64_t(n)) >> 32);
    uint32_t coin = uint32_t(x);
    return coin < thresh[b] ? b : int64_t(other[b]);
  }
};

struct Set64 {  // open addressing, key+1 stored so 0 means empty
  std::vector<uint64_t> slot;
  uint64_t mask = 0, size = 0;
  void init(uint64_t cap) {
    uint64_t c = 1024;
    while (c < cap) c <<= 1;
    slot.assign(c, 0);
    mask = c - 1;
    size = 0;
  }
  bool insert(uint64_t key) {  // true when key was new
    if ((size + 1) * 10 > (mask + 1) * 7) grow();
    uint64_t k = key + 1, h = mix64(key) & mask;
    for (;;) {
      uint64_t v = slot[h];
      if (v == k) return false;
      if (v == 0) { slot[h] = k; size++; return true; }
      h = (h + 1) & mask;
    }
  }
  void grow() {
    std::vector<uint64_t> old;
    old.swap(slot);
    slot.assign(old.size() * 2, 0);
    mask = slot.size() - 1;
    for (uint64_t v : old) {
      if (!v) continue;
      uint64_t h = mix64(v - 1) & mask;
      while (slot[h]) h = (h + 1) & mask;
      slot[h] = v;
    }
  }
};

}  // namespace

extern "C" void fcc_synth_raw(uint64_t seed, uint64_t stream, int64_t n, uint64_t *out) {
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < n; i++) out[i] = draw(seed, stream, uint64_t(i));
}

extern "C" int fcc_synth_coo(uint64_t seed, int32_t order, const int64_t *extents,
                             const double *zipf_s, int64_t nnz, int32_t value_kind,
                             int32_t *coords, double *values, int64_t *nnz_out) {
  if (nnz_out) *nnz_out = 0;
  if (order < 1 || order > 8 || nnz < 0 || !extents || !zipf_s || !nnz_out) return 1;
  unsigned __int128 span = 1;
  for (int m = 0; m < order; m++) {
    if (extents[m] < 1 || extents[m] > (int64_t(1) << 31)) return 1;
    span *= (unsigned __int128)extents[m];
    if (span > ((unsigned __int128)1 << 63)) return 1;
  }
  if (nnz == 0) return 0;
  if (!coords || !values) return 1;

  std::vector<Alias> alias(order);
  for (int m = 0; m < order; m++)
    if (zipf_s[m] > 0) alias[m].build(extents[m], zipf_s[m]);

  int nthreads = 1;
#ifdef _OPENMP
  nthreads = omp_get_max_threads();
#endif
  int nparts = 1;
  while (nparts < nthreads) nparts <<= 1;
  std::vector<Set64> parts(nparts);
  for (auto &p : parts) p.init(uint64_t(2 * nnz / nparts + 1024));

  const int64_t budget = 64 * nnz + (int64_t(1) << 20);
  int64_t produced = 0, next = 0;
  std::vector<uint64_t> lin;
  std::vector<uint8_t> fresh;
  while (produced < nnz && next < budget) {
    int64_t want = nnz - produced;
    int64_t batch = want + want / 4 + 4096;
    if (batch > budget - next) batch = budget - next;
    lin.resize(batch);
    fresh.assign(batch, 0);
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < batch; i++) {
      uint64_t c = uint64_t(next + i), l = 0;
      for (int m = 0; m < order; m++) {
        uint64_t x = draw(seed, uint64_t(m), c);
        int64_t idx = zipf_s[m] > 0 ? alias[m].sample(x)
                                    : int64_t(((x >> 32) * uint64_t(extents[m])) >> 32);
        l = l * uint64_t(extents[m]) + uint64_t(idx);
      }
      lin[i] = l;
    }
#pragma omp parallel
    {
      int t = 0, nt = 1;
#ifdef _OPENMP
      t = omp_get_thread_num();
      nt = omp_get_num_threads();
#endif
      // partition p is owned by thread p % nt; inserts within a partition
      // follow candidate order, so first-occurrence flags are deterministic
      for (int p = t; p < nparts; p += nt) {
        Set64 &mine = parts[p];
        for (int64_t i = 0; i < batch; i++) {
          uint64_t h = mix64(lin[i] ^ 0x5bd1e995u);
          if (int(h & uint64_t(nparts - 1)) != p) continue;
          fresh[i] = mine.insert(lin[i]) ? 1 : 0;
        }
      }
    }
    for (int64_t i = 0; i < batch && produced < nnz; i++) {
      if (!fresh[i]) continue;
      uint64_t l = lin[i];
      int32_t *row = coords + produced * order;
      for (int m = order - 1; m >= 0; m--) {
        row[m] = int32_t(l % uint64_t(extents[m]));
        l /= uint64_t(extents[m]);
      }
      produced++;
    }
    next += batch;
  }

  const uint64_t vstream = 1000;
#pragma omp parallel for schedule(static)
  for (int64_t j = 0; j < produced; j++) {
    uint64_t x = draw(seed, vstream, uint64_t(j));
    if (value_kind == FCC_SYNTH_LOGNORMAL) {
      uint64_t y = draw(seed, vstream + 1, uint64_t(j));
      double u1 = 1.0 - unit53(x);  // (0, 1]
      double u2 = unit53(y);
      double z = std::sqrt(-2.0 * std::log(u1)) * std::cos(6.283185307179586 * u2);
      double v = std::exp(z);
      values[j] = (y & 1) ? -v : v;
    } else {
      values[j] = 2.0 * unit53(x) - 1.0;
    }
  }
  *nnz_out = produced;
  return 0;
}
