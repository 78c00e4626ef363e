// TEST INFRASTRUCTURE ONLY - the CPU oracle for the FaSTCC contraction.
//
// A restatement, in my own code, of the reference's CPU algorithm for
// `Tensor<DT>::fastcc_multiply<TileAccumulator<double>, double>` in
// jianjianh1/fastcc-benchmark. Only tests/, __graft_entry__.smoke() and the
// CPU-baseline leg of bench.py use it, always as the checker or the timed CPU
// baseline, never as part of the product.
//
// What is kept from the reference, step by step:
//  * shape: per-mode max index (Tensor::_infer_shape, contract.hpp:124-144);
//  * external key: Horner over the non-contracted modes in ascending order with
//    radix max+1 (CoOrdinate::remove_linearize, coordinate.hpp:767-781);
//  * contraction key: Horner over the contracted modes in list order with
//    radix max+1 of the operand's own shape (gather_linearize,
//    coordinate.hpp:723-733);
//  * tile width: rounded up to a power of two (contract.hpp:844-846,
//    make_next_power_of_two index_tensors.hpp:476-489), 0 becomes 1
//    (index_tensors.hpp:513-515), ntiles = ceil(span / T) (:524);
//  * tile index: per tile, contraction key -> list of (external % T, value) in
//    nonzero order, keys iterated in first-insertion order, as the
//    insertion-ordered ankerl map of TileIndexedTensor does (:491-547);
//  * tile-pair loop: for every (A tile i, B tile j), for every key of A tile i
//    in insertion order, probe B tile j, and for (li, va) x (ri, vb) add va*vb
//    at li*T + ri (contract.hpp:876-897);
//  * accumulator: dense T x T tile plus first-touch list; drain emits every
//    touched position, exact zero sums included, in first-touch order
//    (TileAccumulator, index_tensors.hpp:994-1060).
// Deliberate differences: the drain decodes positions with pos / T and pos % T
// (the reference shifts by log(T) with the natural log, index_tensors.hpp:1042)
// and decodes external coordinates with the external modes' own extents (the
// reference's sample coordinates carry the leading full-shape bounds,
// contract.hpp:836-843 with coordinate.hpp:544-546); per-thread outputs are
// kept in vectors (the reference's ListTensor::concatenate drops earlier lists
// after an empty one, index_tensors.hpp:115-125). Empty tiles are skipped,
// which changes no result. Summation order per output equals the reference's.

#include "fastcc_oracle.h"

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <map>
#include <unordered_map>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

using u64 = uint64_t;

inline u64 mix64(u64 z) {
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

// make_next_power_of_two on int, including what it does to values <= 0
// (index_tensors.hpp:476-489).
int next_pow2_int(int something) {
  if ((something & (something - 1)) != 0) {
    unsigned u = unsigned(something) - 1u;
    int s = int(u);
    s |= s >> 1; s |= s >> 2; s |= s >> 4; s |= s >> 8; s |= s >> 16;
    something = int(unsigned(s) + 1u);
  }
  return something;
}

struct Operand {
  std::vector<int> ext;        // external modes, ascending
  std::vector<u64> ext_radix;  // max+1
  u64 span = 1;                // product of ext_radix (wraps like the reference)
  std::vector<u64> rem, key;   // per nonzero
};

bool valid_ctr(const orc_tensor *t, const int32_t *ctr, int k) {
  if (!t || t->order < 0 || t->nnz < 0 || k < 0 || k > t->order) return false;
  if (t->nnz > 0 && (!t->coords || !t->values || !t->max_index)) return false;
  for (int i = 0; i < k; i++) {
    if (ctr[i] < 0 || ctr[i] >= t->order) return false;
    for (int j = 0; j < i; j++)
      if (ctr[j] == ctr[i]) return false;
  }
  return true;
}

void prepare(const orc_tensor *t, const int32_t *ctr, int k, Operand &op) {
  std::vector<char> is_ctr(t->order, 0);
  for (int i = 0; i < k; i++) is_ctr[ctr[i]] = 1;
  for (int m = 0; m < t->order; m++)
    if (!is_ctr[m]) {
      op.ext.push_back(m);
      op.ext_radix.push_back(u64(t->max_index[m]) + 1);
      op.span *= u64(t->max_index[m]) + 1;
    }
  op.rem.resize(t->nnz);
  op.key.resize(t->nnz);
  const int d = t->order;
#pragma omp parallel for schedule(static)
  for (int64_t n = 0; n < t->nnz; n++) {
    const int32_t *c = t->coords + n * d;
    u64 r = 0;
    for (size_t e = 0; e < op.ext.size(); e++) r = r * op.ext_radix[e] + u64(c[op.ext[e]]);
    u64 kk = 0;
    for (int i = 0; i < k; i++) kk = kk * (u64(t->max_index[ctr[i]]) + 1) + u64(c[ctr[i]]);
    op.rem[n] = r;
    op.key[n] = kk;
  }
}

// Per-tile insertion-ordered index (TileIndexedTensor, index_tensors.hpp:491-547)
struct TileIndex {
  u64 T = 1;
  std::vector<u64> tile_id;      // non-empty tiles, ascending
  std::vector<int64_t> key_beg;  // per tile -> range in keys
  std::vector<u64> keys;         // insertion order within the tile
  std::vector<int64_t> ent_beg;  // per key -> range in entries
  std::vector<uint32_t> inner;   // external % T
  std::vector<double> val;
  std::vector<int64_t> hbeg;     // per tile -> hash slots
  std::vector<uint32_t> hslot;   // local key id + 1, 0 empty

  int64_t find(size_t t, u64 k) const {
    int64_t hb = hbeg[t];
    u64 mask = u64(hbeg[t + 1] - hb) - 1;
    u64 h = mix64(k) & mask;
    for (;;) {
      uint32_t s = hslot[hb + h];
      if (!s) return -1;
      int64_t id = key_beg[t] + int64_t(s) - 1;
      if (keys[id] == k) return id;
      h = (h + 1) & mask;
    }
  }
};

void build_index(const orc_tensor *t, const Operand &op, u64 T, TileIndex &ix) {
  ix.T = T;
  const int64_t n = t->nnz;
  // stable bucket of nonzeros by tile
  std::vector<std::pair<u64, int64_t>> order(n);
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < n; i++) order[i] = {op.rem[i] / T, i};
  std::stable_sort(order.begin(), order.end(),
                   [](const std::pair<u64, int64_t> &a, const std::pair<u64, int64_t> &b) {
                     return a.first < b.first;
                   });
  std::vector<int64_t> tbeg;
  for (int64_t i = 0; i < n; i++)
    if (i == 0 || order[i].first != order[i - 1].first) {
      ix.tile_id.push_back(order[i].first);
      tbeg.push_back(i);
    }
  tbeg.push_back(n);
  const size_t nt = ix.tile_id.size();
  // per tile: count distinct keys (first pass) to lay out global arrays
  std::vector<int64_t> nkeys(nt + 1, 0), hsize(nt + 1, 0);
  std::vector<std::vector<u64>> tkeys(nt);
  std::vector<std::vector<uint32_t>> tid_of(nt);
#pragma omp parallel for schedule(dynamic, 1)
  for (size_t ti = 0; ti < nt; ti++) {
    int64_t cnt = tbeg[ti + 1] - tbeg[ti];
    u64 cap = 8;
    while (cap < u64(2 * cnt)) cap <<= 1;
    std::vector<uint32_t> slot(cap, 0);
    std::vector<u64> &ks = tkeys[ti];
    std::vector<uint32_t> &ids = tid_of[ti];
    ids.resize(cnt);
    for (int64_t q = 0; q < cnt; q++) {
      u64 k = op.key[order[tbeg[ti] + q].second];
      u64 h = mix64(k) & (cap - 1);
      for (;;) {
        uint32_t s = slot[h];
        if (!s) { ks.push_back(k); slot[h] = uint32_t(ks.size()); ids[q] = uint32_t(ks.size() - 1); break; }
        if (ks[s - 1] == k) { ids[q] = s - 1; break; }
        h = (h + 1) & (cap - 1);
      }
    }
    nkeys[ti] = int64_t(ks.size());
    u64 hc = 8;
    while (hc < u64(2 * ks.size())) hc <<= 1;
    hsize[ti] = int64_t(hc);
  }
  ix.key_beg.assign(nt + 1, 0);
  ix.hbeg.assign(nt + 1, 0);
  for (size_t ti = 0; ti < nt; ti++) {
    ix.key_beg[ti + 1] = ix.key_beg[ti] + nkeys[ti];
    ix.hbeg[ti + 1] = ix.hbeg[ti] + hsize[ti];
  }
  const int64_t K = ix.key_beg[nt];
  ix.keys.resize(K);
  ix.ent_beg.assign(K + 1, 0);
  ix.inner.resize(n);
  ix.val.resize(n);
  ix.hslot.assign(ix.hbeg[nt], 0);
  // entry offsets: entries of a tile are contiguous [tbeg, tbeg+cnt), grouped by key
#pragma omp parallel for schedule(dynamic, 1)
  for (size_t ti = 0; ti < nt; ti++) {
    const int64_t kb = ix.key_beg[ti], cnt = tbeg[ti + 1] - tbeg[ti];
    const std::vector<u64> &ks = tkeys[ti];
    std::vector<int64_t> c(ks.size() + 1, 0);
    for (int64_t q = 0; q < cnt; q++) c[tid_of[ti][q] + 1]++;
    for (size_t j = 0; j < ks.size(); j++) c[j + 1] += c[j];
    for (size_t j = 0; j < ks.size(); j++) {
      ix.keys[kb + j] = ks[j];
      ix.ent_beg[kb + j] = tbeg[ti] + c[j];
    }
    std::vector<int64_t> fill(c.begin(), c.end() - 1);
    for (int64_t q = 0; q < cnt; q++) {
      int64_t src = order[tbeg[ti] + q].second;
      int64_t dst = tbeg[ti] + fill[tid_of[ti][q]]++;
      ix.inner[dst] = uint32_t(op.rem[src] % T);
      ix.val[dst] = t->values[src];
    }
    u64 mask = u64(hsize[ti]) - 1;
    for (size_t j = 0; j < ks.size(); j++) {
      u64 h = mix64(ks[j]) & mask;
      while (ix.hslot[ix.hbeg[ti] + h]) h = (h + 1) & mask;
      ix.hslot[ix.hbeg[ti] + h] = uint32_t(j + 1);
    }
    tkeys[ti].clear(); tkeys[ti].shrink_to_fit();
    tid_of[ti].clear(); tid_of[ti].shrink_to_fit();
  }
  ix.ent_beg[K] = n;
}

void decode_into(const Operand &a, const Operand &b, const u64 *left, const u64 *right, int64_t n,
                 int32_t *coords) {
  const int la = int(a.ext.size()), lb = int(b.ext.size()), d = la + lb;
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < n; i++) {
    u64 l = left[i], r = right[i];
    int32_t *c = coords + i * d;
    for (int e = la - 1; e >= 0; e--) { c[e] = int32_t(l % a.ext_radix[e]); l /= a.ext_radix[e]; }
    for (int e = lb - 1; e >= 0; e--) { c[la + e] = int32_t(r % b.ext_radix[e]); r /= b.ext_radix[e]; }
  }
}

double ms_since(std::chrono::steady_clock::time_point t0) {
  return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
}

}  // namespace

extern "C" int orc_infer_shape(const int32_t *coords, int64_t nnz, int32_t order, int32_t *max_index) {
  if (order < 0 || nnz < 0 || (nnz > 0 && !coords) || !max_index) return 1;
  for (int m = 0; m < order; m++) max_index[m] = 0;
  for (int64_t n = 0; n < nnz; n++)
    for (int m = 0; m < order; m++) max_index[m] = std::max(max_index[m], coords[n * order + m]);
  return 0;
}

extern "C" int orc_fastcc_multiply(const orc_tensor *A, const orc_tensor *B, const int32_t *ctrA,
                                   const int32_t *ctrB, int32_t k, int32_t tile_size,
                                   int32_t nthreads, int32_t want_abs, orc_result *out) {
  if (!out) return 1;
  std::memset(out, 0, sizeof(*out));
  if (!valid_ctr(A, ctrA, k) || !valid_ctr(B, ctrB, k)) return 1;
  if (tile_size > (1 << 30)) return 1;
#ifdef _OPENMP
  int saved = omp_get_max_threads();
  if (nthreads > 0) omp_set_num_threads(nthreads);
#endif
  auto t0 = std::chrono::steady_clock::now();
  Operand oa, ob;
  prepare(A, ctrA, k, oa);
  prepare(B, ctrB, k, ob);
  out->order = int32_t(oa.ext.size() + ob.ext.size());
  // tile width: contract.hpp:844-846 then index_tensors.hpp:513-515
  int ts = tile_size;
  if (ts & (ts - 1)) ts = next_pow2_int(ts);
  u64 T = ts <= 0 ? 1 : u64(ts);
  TileIndex ia, ib;
  build_index(A, oa, T, ia);
  build_index(B, ob, T, ib);
  out->index_ms = ms_since(t0);

  auto t1 = std::chrono::steady_clock::now();
  const int64_t nta = int64_t(ia.tile_id.size()), ntb = int64_t(ib.tile_id.size());
  int nthr = 1;
#ifdef _OPENMP
  nthr = omp_get_max_threads();
#endif
  struct Local {
    std::vector<u64> left, right;
    std::vector<double> val, absv;
    int64_t products = 0;
  };
  std::vector<Local> loc(nthr);
#pragma omp parallel
  {
    int tid = 0;
#ifdef _OPENMP
    tid = omp_get_thread_num();
#endif
    Local &L = loc[tid];
    std::vector<double> acc(T * T, 0.0), aacc;
    if (want_abs) aacc.assign(T * T, 0.0);
    std::vector<uint8_t> touched(T * T, 0);
    std::vector<u64> first_touch;
    first_touch.reserve(1024);
#pragma omp for schedule(dynamic, 1)
    for (int64_t q = 0; q < nta * ntb; q++) {
      const int64_t i = q / ntb, j = q % ntb;
      for (int64_t ka = ia.key_beg[i]; ka < ia.key_beg[i + 1]; ka++) {
        int64_t kb = ib.find(size_t(j), ia.keys[ka]);
        if (kb < 0) continue;
        for (int64_t ea = ia.ent_beg[ka]; ea < ia.ent_beg[ka + 1]; ea++) {
          const u64 base = u64(ia.inner[ea]) * T;
          const double va = ia.val[ea];
          for (int64_t eb = ib.ent_beg[kb]; eb < ib.ent_beg[kb + 1]; eb++) {
            const u64 pos = base + ib.inner[eb];
            const double p = va * ib.val[eb];
            if (!touched[pos]) { touched[pos] = 1; first_touch.push_back(pos); }
            acc[pos] += p;
            if (want_abs) aacc[pos] += std::fabs(p);
          }
          L.products += ib.ent_beg[kb + 1] - ib.ent_beg[kb];
        }
      }
      const u64 lt = ia.tile_id[i], rt = ib.tile_id[j];
      for (u64 pos : first_touch) {
        L.left.push_back(lt * T + pos / T);
        L.right.push_back(rt * T + pos % T);
        L.val.push_back(acc[pos]);
        acc[pos] = 0.0;
        touched[pos] = 0;
        if (want_abs) { L.absv.push_back(aacc[pos]); aacc[pos] = 0.0; }
      }
      first_touch.clear();
    }
  }
  out->compute_ms = ms_since(t1);

  // Concatenate the per-thread outputs (ListTensor::concatenate,
  // contract.hpp:906-909) straight into the result arrays, each thread
  // copying its own range.
  std::vector<int64_t> off(loc.size() + 1, 0);
  for (size_t q = 0; q < loc.size(); q++) {
    off[q + 1] = off[q] + int64_t(loc[q].val.size());
    out->products += loc[q].products;
  }
  const int64_t n = off.back();
  out->nnz = n;
  const size_t cap = size_t(std::max<int64_t>(n, 1));
  out->left = (u64 *)std::malloc(sizeof(u64) * cap);
  out->right = (u64 *)std::malloc(sizeof(u64) * cap);
  out->values = (double *)std::malloc(sizeof(double) * cap);
  out->abs_sum = want_abs ? (double *)std::malloc(sizeof(double) * cap) : nullptr;
  out->coords = (int32_t *)std::malloc(sizeof(int32_t) * std::max<int64_t>(1, n * out->order));
#pragma omp parallel for schedule(static, 1)
  for (int64_t q = 0; q < int64_t(loc.size()); q++) {
    Local &L = loc[q];
    const size_t m = L.val.size();
    if (m) {
      std::memcpy(out->left + off[q], L.left.data(), m * sizeof(u64));
      std::memcpy(out->right + off[q], L.right.data(), m * sizeof(u64));
      std::memcpy(out->values + off[q], L.val.data(), m * sizeof(double));
      if (want_abs) std::memcpy(out->abs_sum + off[q], L.absv.data(), m * sizeof(double));
    }
    std::vector<u64>().swap(L.left);
    std::vector<u64>().swap(L.right);
    std::vector<double>().swap(L.val);
    std::vector<double>().swap(L.absv);
  }
  decode_into(oa, ob, out->left, out->right, n, out->coords);
  out->total_ms = ms_since(t0);
#ifdef _OPENMP
  omp_set_num_threads(saved);
#endif
  return 0;
}

extern "C" int orc_bruteforce(const orc_tensor *A, const orc_tensor *B, const int32_t *ctrA,
                              const int32_t *ctrB, int32_t k, orc_result *out) {
  if (!out) return 1;
  std::memset(out, 0, sizeof(*out));
  if (!valid_ctr(A, ctrA, k) || !valid_ctr(B, ctrB, k)) return 1;
  Operand oa, ob;
  prepare(A, ctrA, k, oa);
  prepare(B, ctrB, k, ob);
  using Tup = std::vector<int32_t>;
  std::map<Tup, std::vector<int64_t>> bidx;
  for (int64_t n = 0; n < B->nnz; n++) {
    Tup t;
    for (int i = 0; i < k; i++) t.push_back(B->coords[n * B->order + ctrB[i]]);
    bidx[t].push_back(n);
  }
  std::map<Tup, std::pair<double, double>> res;
  std::map<Tup, std::pair<u64, u64>> lin;
  int64_t products = 0;
  for (int64_t n = 0; n < A->nnz; n++) {
    Tup t;
    for (int i = 0; i < k; i++) t.push_back(A->coords[n * A->order + ctrA[i]]);
    auto it = bidx.find(t);
    if (it == bidx.end()) continue;
    for (int64_t m : it->second) {
      Tup o;
      for (int e : oa.ext) o.push_back(A->coords[n * A->order + e]);
      for (int e : ob.ext) o.push_back(B->coords[m * B->order + e]);
      double p = A->values[n] * B->values[m];
      auto &r = res[o];
      r.first += p;
      r.second += std::fabs(p);
      lin[o] = {oa.rem[n], ob.rem[m]};
      products++;
    }
  }
  out->order = int32_t(oa.ext.size() + ob.ext.size());
  out->nnz = int64_t(res.size());
  out->products = products;
  const int64_t n = out->nnz;
  out->left = (u64 *)std::malloc(sizeof(u64) * std::max<int64_t>(1, n));
  out->right = (u64 *)std::malloc(sizeof(u64) * std::max<int64_t>(1, n));
  out->values = (double *)std::malloc(sizeof(double) * std::max<int64_t>(1, n));
  out->abs_sum = (double *)std::malloc(sizeof(double) * std::max<int64_t>(1, n));
  out->coords = (int32_t *)std::malloc(sizeof(int32_t) * std::max<int64_t>(1, n * out->order));
  int64_t i = 0;
  for (auto &kv : res) {
    for (int d = 0; d < out->order; d++) out->coords[i * out->order + d] = kv.first[d];
    out->values[i] = kv.second.first;
    out->abs_sum[i] = kv.second.second;
    out->left[i] = lin[kv.first].first;
    out->right[i] = lin[kv.first].second;
    i++;
  }
  return 0;
}

extern "C" int64_t orc_count_products(const orc_tensor *A, const orc_tensor *B, const int32_t *ctrA,
                                      const int32_t *ctrB, int32_t k) {
  if (!valid_ctr(A, ctrA, k) || !valid_ctr(B, ctrB, k)) return -1;
  Operand oa, ob;
  prepare(A, ctrA, k, oa);
  prepare(B, ctrB, k, ob);
  std::unordered_map<u64, int64_t> cb;
  cb.reserve(size_t(B->nnz));
  for (u64 key : ob.key) cb[key]++;
  int64_t s = 0;
  for (u64 key : oa.key) {
    auto it = cb.find(key);
    if (it != cb.end()) s += it->second;
  }
  return s;
}

extern "C" void orc_free(orc_result *r) {
  if (!r) return;
  std::free(r->left);
  std::free(r->right);
  std::free(r->coords);
  std::free(r->values);
  std::free(r->abs_sum);
  std::memset(r, 0, sizeof(*r));
}
