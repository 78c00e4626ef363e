// The GB300 contraction pipeline behind fcc_contract (include/fastcc_gpu.h),
// the device replacement of Tensor<DT>::fastcc_multiply (contract.hpp:824-912).
//
// Reference step                                  -> here
//  TileIndexedTensor over B (index_tensors.hpp:506-547): per tile, hash map
//    contraction key -> (external % T, value)     -> k_linearize + radix sort of
//    B by 64-bit contraction key + segment build (ukey / segbeg): CSF-style
//    segments, one per distinct key, in HBM
//  TileIndexedTensor over A                       -> radix sort of A by its
//    external (row) index; each A nonzero looks up its B segment once
//    (k_lookup) instead of once per B tile (contract.hpp:887)
//  tile-pair loop (contract.hpp:876-897)          -> output tiles of TL A rows
//    x the whole B external span; a tile's multiply-adds are cut into work
//    items of at most `products_per_item`, scheduled dynamically over
//    persistent CTAs
//  TileAccumulator (index_tensors.hpp:994-1060)   -> k_contract_dense: the tile
//    lives in shared memory as doubles plus a touched bitmask; drain emits
//    every touched position (exact zero sums included)
//  TileAccumulatorMap (index_tensors.hpp:843-883) -> k_contract_hash: shared-
//    memory open addressing, for B external spans too wide for a dense tile
//  drain + ListTensor push/concatenate (index_tensors.hpp:90-125,1039-1060)
//    -> block prefix sums reserve an output range with one atomic per tile;
//    warps write coordinates (SoA, uint32) and values coalesced
//  tiles cut into several items                   -> partial tiles are added
//    into a global dense tile or a global per-tile hash region (FP64 atomics)
//    and drained by k_merge_*.

#include <algorithm>
#include <chrono>
#include <cstring>
#include <memory>
#include <type_traits>

#include "fcc_internal.cuh"

namespace fcc {

struct LinSpec {
  int order, n_ext, n_ctr;
  int ext_mode[FCC_MAX_ORDER];
  int ctr_mode[FCC_MAX_ORDER];
  u64 ext_radix[FCC_MAX_ORDER];
  u64 ctr_radix[FCC_MAX_ORDER];
  int32_t max_index[FCC_MAX_ORDER];
};

// Division by a divisor fixed for a whole launch: q = n / d for n, d < 2^32
// as the high half of n * m, m = ceil(2^64 / d) (the round-up method of
// Granlund and Montgomery, "Division by invariant integers using
// multiplication", PLDI 1994). Exact while n * d < 2^64: the error term
// n * (m - 2^64/d) / 2^64 < n / 2^64 stays below 1/d. m = 0 encodes d = 1.
__host__ __device__ __forceinline__ u64 magic_for(u64 d) { return d <= 1 ? 0 : (~0ull) / d + 1; }
__device__ __forceinline__ u32 div_magic(u32 n, u64 m) { return m ? u32(__umul64hi(u64(n), m)) : n; }

struct Decode {
  int na, nb;
  int narrow;  // every radix and both spans < 2^32
  u64 ra[FCC_MAX_ORDER], rb[FCC_MAX_ORDER];
  u64 ma[FCC_MAX_ORDER], mb[FCC_MAX_ORDER];  // magic_for(ra[e]), magic_for(rb[e])
  const u32 *inv_col;  // renumbered B column -> B external index (NULL: identity)
};

struct Out {
  u32 *coords;  // SoA, mode m at coords[m * stride]
  i64 stride;
  double *vals;
  u64 cap;
  u64 *cursor;
};

struct Item {
  u64 p0, p1;  // multiply-adds [p0, p1) of the tile
  u32 tile;
  u32 ea, eb;  // its A entries: ea holds p0, eb is the first entry starting at or after p1
  u32 pad;
};

// ------------------------------------------------------------ helpers ----

__device__ __forceinline__ u32 warp_incl_u32(u32 x) {
  const int lane = threadIdx.x & 31;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    u32 y = __shfl_up_sync(kFull, x, o);
    if (lane >= o) x += y;
  }
  return x;
}

__device__ __forceinline__ u32 hash_slot(u64 key) {
  return u32((key * 0x9E3779B97F4A7C15ull) >> 32) ^ u32(key >> 29);
}

// Output stores are evict-first (st.global.cs): the output streams through
// L2 once and should not push out the B segments the tile kernels re-read.
__device__ __forceinline__ void emit(const Out &o, const Decode &d, u64 idx, u64 row, u64 col,
                                     double v) {
  u32 *c = o.coords;
  if (d.inv_col) col = d.inv_col[col];
  if (d.narrow) {
    u32 r = u32(row);
    for (int e = d.na - 1; e > 0; --e) {
      u32 rad = u32(d.ra[e]), q = div_magic(r, d.ma[e]);
      __stcs(&c[e * o.stride + idx], r - q * rad);
      r = q;
    }
    if (d.na > 0) __stcs(&c[idx], r);
    u32 s = u32(col);
    for (int e = d.nb - 1; e > 0; --e) {
      u32 rad = u32(d.rb[e]), q = div_magic(s, d.mb[e]);
      __stcs(&c[(d.na + e) * o.stride + idx], s - q * rad);
      s = q;
    }
    if (d.nb > 0) __stcs(&c[d.na * o.stride + idx], s);
  } else {
    u64 r = row;
    for (int e = d.na - 1; e > 0; --e) {
      u64 q = r / d.ra[e];
      __stcs(&c[e * o.stride + idx], u32(r - q * d.ra[e]));
      r = q;
    }
    if (d.na > 0) __stcs(&c[idx], u32(r));
    u64 s = col;
    for (int e = d.nb - 1; e > 0; --e) {
      u64 q = s / d.rb[e];
      __stcs(&c[(d.na + e) * o.stride + idx], u32(s - q * d.rb[e]));
      s = q;
    }
    if (d.nb > 0) __stcs(&c[d.na * o.stride + idx], u32(s));
  }
  __stcs(&o.vals[idx], v);
}

// Reserves `total` outputs with one atomic; ~0 marks "over capacity".
__device__ __forceinline__ u64 reserve(const Out &o, u64 total, u32 *err) {
  if (total == 0) return 0;
  u64 b = atomicAdd(reinterpret_cast<unsigned long long *>(o.cursor), (unsigned long long)total);
  if (b + total > o.cap) {
    atomicOr(err, ERRB_OVERFLOW);
    return ~0ull;
  }
  return b;
}

// ------------------------------------------------------ index building ----

__global__ void k_linearize(const int32_t *__restrict__ coords, i64 sn, i64 sm, i64 nnz, LinSpec s,
                            u64 *__restrict__ ext, u64 *__restrict__ key, u32 *__restrict__ iota,
                            u32 *err) {
  for (i64 i = i64(blockIdx.x) * blockDim.x + threadIdx.x; i < nnz; i += i64(gridDim.x) * blockDim.x) {
    const int32_t *c = coords + i * sn;
    bool bad = false;
    u64 e = 0, k = 0;
    for (int q = 0; q < s.n_ext; q++) {
      int32_t v = c[i64(s.ext_mode[q]) * sm];
      bad |= v < 0 || v > s.max_index[s.ext_mode[q]];
      e = e * s.ext_radix[q] + u64(u32(v));
    }
    for (int q = 0; q < s.n_ctr; q++) {
      int32_t v = c[i64(s.ctr_mode[q]) * sm];
      bad |= v < 0 || v > s.max_index[s.ctr_mode[q]];
      k = k * s.ctr_radix[q] + u64(u32(v));
    }
    if (bad) atomicOr(err, ERRB_COORD);
    ext[i] = e;
    key[i] = k;
    iota[i] = u32(i);
  }
}

// |v| below this (zeros included) could make a product round to +-0, so the
// -0.0 "untouched" sentinel of the dense tile cannot be used.
__device__ __forceinline__ bool tiny_value(double v) { return fabs(v) < 1e-150; }

template <class ColT>
__global__ void k_gather_b(const u32 *__restrict__ perm, const u64 *__restrict__ ext,
                           const double *__restrict__ vals, i64 n, ColT *__restrict__ col,
                           double *__restrict__ val, u32 *tiny) {
  bool t = false;
  for (i64 i = i64(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += i64(gridDim.x) * blockDim.x) {
    u32 p = perm[i];
    col[i] = ColT(ext[p]);
    const double v = vals[p];
    val[i] = v;
    t |= tiny_value(v);
  }
  if (__any_sync(kFull, t) && (threadIdx.x & 31) == 0) atomicOr(tiny, 1u);
}

__global__ void k_flag_change(const u64 *__restrict__ key, i64 n, u32 *__restrict__ flag) {
  for (i64 i = i64(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += i64(gridDim.x) * blockDim.x)
    flag[i] = (i == 0 || key[i] != key[i - 1]) ? 1u : 0u;
}

__global__ void k_seg_write(const u64 *__restrict__ key, const u32 *__restrict__ flag,
                            const u32 *__restrict__ idx, i64 n, u64 *__restrict__ ukey,
                            u32 *__restrict__ segbeg) {
  for (i64 i = i64(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += i64(gridDim.x) * blockDim.x) {
    if (flag[i]) {
      ukey[idx[i]] = key[i];
      segbeg[idx[i]] = u32(i);
    }
    if (i == n - 1) segbeg[idx[i] + flag[i]] = u32(n);
  }
}

// Segments per bucket of the key space (key >> shift); an exclusive scan
// turns the counts into bstart[b] = the first segment of bucket b.
__global__ void k_seg_buckets(const u64 *__restrict__ ukey, const u32 *__restrict__ nseg_p, int shift,
                              u32 *__restrict__ count) {
  const u32 nseg = *nseg_p;
  for (i64 i = i64(blockIdx.x) * blockDim.x + threadIdx.x; i < i64(nseg); i += i64(gridDim.x) * blockDim.x) {
    const u64 b = ukey[i] >> shift;
    // A bucket's segments are consecutive: they are counted in pieces that
    // start at the bucket's first segment or at a multiple of 32 and end
    // before the next multiple of 32 (one atomic per piece).
    if (i == 0 || (ukey[i - 1] >> shift) != b || i % 32 == 0) {
      u32 n = 1;
      while (i + n < nseg && (i + n) % 32 != 0 && (ukey[i + n] >> shift) == b) n++;
      atomicAdd(&count[b], n);
    }
  }
}

// For each A nonzero (in row-sorted order) find the B segment of its key:
// a binary search within the key's bucket.
__global__ void k_lookup(const u64 *__restrict__ keyA, const u32 *__restrict__ permA, i64 n,
                         const u64 *__restrict__ ukey, const u32 *__restrict__ nseg_p,
                         const u32 *__restrict__ bstart, int shift, u64 nbuckets,
                         u32 *__restrict__ seg, u32 *__restrict__ flag) {
  const u32 nseg = *nseg_p;
  for (i64 i = i64(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += i64(gridDim.x) * blockDim.x) {
    const u64 k = keyA[permA[i]];
    const u64 b = min(k >> shift, nbuckets - 1);
    u32 lo = bstart[b], hi = bstart[b + 1];  // first index with ukey >= k lies in [lo, hi]
    while (lo < hi) {
      u32 mid = (lo + hi) >> 1;
      if (ukey[mid] < k) lo = mid + 1; else hi = mid;
    }
    bool hit = lo < nseg && ukey[lo] == k;
    seg[i] = lo;
    flag[i] = hit ? 1u : 0u;
  }
}

// Keeps the A entries whose key has a B segment, in row order, with the
// segment's first B entry (sbA) and length.
__global__ void k_compact_a(const u32 *__restrict__ flag, const u32 *__restrict__ idx, i64 n,
                            const u32 *__restrict__ permA, const u64 *__restrict__ rowSorted,
                            const u32 *__restrict__ segTmp, const double *__restrict__ valsA,
                            const u32 *__restrict__ segbeg, u64 *__restrict__ rowA,
                            u32 *__restrict__ sbA, double *__restrict__ valA, u32 *__restrict__ len,
                            u32 *tiny) {
  bool t = false;
  for (i64 i = i64(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += i64(gridDim.x) * blockDim.x) {
    if (!flag[i]) continue;
    const u32 d = idx[i], s = segTmp[i];
    rowA[d] = rowSorted[i];
    sbA[d] = segbeg[s];
    const double v = valsA[permA[i]];
    valA[d] = v;
    t |= tiny_value(v);
    len[d] = segbeg[s + 1] - segbeg[s];
  }
  if (__any_sync(kFull, t) && (threadIdx.x & 31) == 0) atomicOr(tiny, 1u);
}

// ------------------------------------------------------------ planning ----

// Tiles are made of the rows that occur (A's external indices with at least
// one matched entry), not of index ranges: row ranks come from a prefix sum
// over row changes of the row-sorted entries, and a tile holds up to TL
// consecutive ranks of one group. A group is a range of rows sharing
// row / gdiv (the instance of a batched contraction, whose column span lb[g]
// may be narrower than the whole B span); without groups (gdiv == 0) there is
// one group with the whole span.
struct RowGroups {
  u64 gdiv;       // 0: no groups
  const u32 *lb;  // per group: column span (B external columns in use)
  u64 area;       // tile capacity in positions; TL of group g = area / lb[g]
  u64 TL;         // > 0: fixed rows per tile for every group
  u64 LB;         // column span without groups
};

__device__ __forceinline__ u32 group_of(const RowGroups &g, u64 row) { return g.gdiv ? u32(row / g.gdiv) : 0u; }
__device__ __forceinline__ u64 group_lb(const RowGroups &g, u32 grp) { return g.gdiv ? u64(g.lb[grp]) : g.LB; }
__device__ __forceinline__ u64 group_tl(const RowGroups &g, u32 grp) {
  if (g.TL) return g.TL;
  const u64 lb = group_lb(g, grp);
  return lb >= g.area ? 1 : g.area / lb;
}

// rank[e] = rank of entry e's row among the distinct rows; urow[rank] = row;
// gfirst[g] = rank of group g's first row. rflag: row changes, rexcl: their
// exclusive prefix sum.
__global__ void k_row_rank(const u64 *__restrict__ rowA, const u32 *__restrict__ rflag,
                           const u32 *__restrict__ rexcl, i64 n, RowGroups g, u32 *__restrict__ rank,
                           u64 *__restrict__ urow, u32 *__restrict__ gfirst) {
  for (i64 i = i64(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += i64(gridDim.x) * blockDim.x) {
    const u32 r = rexcl[i] + rflag[i] - 1u;
    rank[i] = r;
    if (rflag[i]) {
      urow[r] = rowA[i];
      const u32 grp = group_of(g, rowA[i]);
      if (i == 0 || group_of(g, rowA[i - 1]) != grp) gfirst[grp] = r;
    }
  }
}

// slot[e] = position of e's row inside its tile; flag[e] = 1 where a tile starts.
__global__ void k_row_tiles(const u64 *__restrict__ rowA, const u32 *__restrict__ rflag,
                            const u32 *__restrict__ rank, i64 n, RowGroups g, const u32 *__restrict__ gfirst,
                            u32 *__restrict__ slot, u32 *__restrict__ flag) {
  for (i64 i = i64(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += i64(gridDim.x) * blockDim.x) {
    const u32 grp = group_of(g, rowA[i]);
    const u32 s = u32(u64(rank[i] - gfirst[grp]) % group_tl(g, grp));
    slot[i] = s;
    flag[i] = (rflag[i] && s == 0) ? 1u : 0u;
  }
}

// Per tile: first entry, first row rank and column span.
__global__ void k_tile_write(const u64 *__restrict__ rowA, const u32 *__restrict__ flag,
                             const u32 *__restrict__ idx, const u32 *__restrict__ rank, i64 n, RowGroups g,
                             u32 *__restrict__ abeg, u32 *__restrict__ rank0, u32 *__restrict__ lb) {
  for (i64 i = i64(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += i64(gridDim.x) * blockDim.x) {
    if (flag[i]) {
      const u32 t = idx[i];
      abeg[t] = u32(i);
      rank0[t] = rank[i];
      lb[t] = u32(group_lb(g, group_of(g, rowA[i])));
    }
    if (i == n - 1) abeg[idx[i] + flag[i]] = u32(n);
  }
}

// Row count of each tile, from its last entry's rank.
__global__ void k_tile_nrows(const u32 *__restrict__ ntiles_p, const u32 *__restrict__ abeg,
                             const u32 *__restrict__ rank, const u32 *__restrict__ rank0, u32 *__restrict__ nrows) {
  const u32 ntiles = *ntiles_p;
  for (i64 t = i64(blockIdx.x) * blockDim.x + threadIdx.x; t < ntiles; t += i64(gridDim.x) * blockDim.x)
    nrows[t] = rank[abeg[t + 1] - 1] - rank0[t] + 1;
}

// Tile classes (FCC_CLASS_*): per class whether it may run, its multiply-adds
// per work item and whether it is a hash class.
struct ClassTable {
  u32 enabled[FCC_NUM_CLASSES];
  u32 hash[FCC_NUM_CLASSES];
  u64 pmax[FCC_NUM_CLASSES];
  int forced;     // >= 0: every tile takes this class
  int fill_log2;  // rule: dense only when multiply-adds >= area >> fill_log2 (0: whenever it fits)
  float override_log2;  // learned: leave the rule's class only for a class predicted cheaper by this (log2)
  float dense_switch_log2;  // learned, between the two dense classes (same tile, other kernel)
};

__device__ __forceinline__ u64 tile_area(const u32 *nrows, const u32 *lb, u64 LB, u32 t) {
  return u64(nrows[t]) * (lb ? u64(lb[t]) : LB);
}

// cls[t]: the class of tile t. Forced, or the rule: dense when enabled and
// filled enough, else the smallest hash table holding the tile, else the
// largest. With predicted costs (pred, FCC_NUM_CLASSES log2 costs per tile)
// the tile leaves the rule's class for the cheapest predicted class when that
// is cheaper by more than override_log2 (a tile larger than a class's work
// item is split, as under a forced class). ckey/corder: sort keys for the
// class-order permutation (padding tiles sort last).
__global__ void k_tile_class(const u32 *__restrict__ ntiles_p, i64 nmax, const u32 *__restrict__ abeg,
                             const u64 *__restrict__ P, const u32 *__restrict__ nrows, const u32 *__restrict__ lb,
                             u64 LB, ClassTable ct, const float *__restrict__ pred, u32 *__restrict__ cls,
                             u64 *__restrict__ ckey, u32 *__restrict__ corder) {
  const u32 ntiles = *ntiles_p;
  for (i64 t = i64(blockIdx.x) * blockDim.x + threadIdx.x; t < nmax; t += i64(gridDim.x) * blockDim.x) {
    corder[t] = u32(t);
    if (t >= ntiles) {
      ckey[t] = 7;
      continue;
    }
    const u64 prod = P[abeg[t + 1]] - P[abeg[t]];
    int c = ct.forced;
    if (c < 0) {  // the rule
      const u64 area = tile_area(nrows, lb, LB, u32(t));
      if (ct.enabled[FCC_CLASS_DENSE] && (ct.fill_log2 == 0 || prod >= (area >> ct.fill_log2))) {
        c = FCC_CLASS_DENSE;
      } else {
        c = FCC_CLASS_HASH_L;
        for (int k = FCC_CLASS_HASH_S; k > FCC_CLASS_HASH_L; k--)
          if (ct.enabled[k] && prod <= ct.pmax[k]) { c = k; break; }
        if (!ct.enabled[c]) c = FCC_CLASS_DENSE;  // only dense is enabled
      }
      if (pred) {  // the model overrides the rule where it predicts a clearly cheaper class
        const float *pt = pred + t * FCC_NUM_CLASSES;
        float bestv = 3.0e38f;
        int pick = c;
        for (int k = 0; k < FCC_NUM_CLASSES; k++) {
          if (!ct.enabled[k] || k == c) continue;
          // the other dense class runs the same tile with another kernel: a smaller margin
          const float margin =
              (c == FCC_CLASS_DENSE && k == FCC_CLASS_DENSE_FLAT) ? ct.dense_switch_log2 : ct.override_log2;
          if (pt[k] < pt[c] - margin && pt[k] < bestv) {
            bestv = pt[k];
            pick = k;
          }
        }
        c = pick;
      }
    }
    cls[t] = u32(c);
    ckey[t] = u64(c);
  }
}

// Sums over the tiles of 2^pred: per enabled class (every tile in that class)
// and of the per-tile minimum (a mix). out: FCC_NUM_CLASSES + 1 doubles.
__global__ void k_pred_sums(const u32 *__restrict__ ntiles_p, i64 nmax, const float *__restrict__ pred, ClassTable ct,
                            double *__restrict__ out) {
  const u32 ntiles = *ntiles_p;
  double s[FCC_NUM_CLASSES + 1] = {};
  for (i64 t = i64(blockIdx.x) * blockDim.x + threadIdx.x; t < min(nmax, i64(ntiles));
       t += i64(gridDim.x) * blockDim.x) {
    double mn = 1e300;
    for (int c = 0; c < FCC_NUM_CLASSES; c++) {
      if (!ct.enabled[c]) continue;
      const double v = double(exp2f(pred[t * FCC_NUM_CLASSES + c]));  // FP32 power, FP64 sums
      s[c] += v;
      mn = fmin(mn, v);
    }
    s[FCC_NUM_CLASSES] += mn;
  }
  for (int c = 0; c <= FCC_NUM_CLASSES; c++) {
    double v = s[c];
    for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(kFull, v, o);
    if ((threadIdx.x & 31) == 0 && v != 0.0) atomicAdd(&out[c], v);
  }
}

// Per tile in class order (position i, tile corder[i]): work items, split
// flags (dense / hash), output bound and (split hash tiles) global region size.
__global__ void k_tile_items(const u32 *__restrict__ ntiles_p, i64 nmax, const u32 *__restrict__ corder,
                             const u32 *__restrict__ cls, const u32 *__restrict__ abeg, const u64 *__restrict__ P,
                             const u32 *__restrict__ nrows, const u32 *__restrict__ lb, u64 LB, ClassTable ct,
                             int esc, u32 *__restrict__ nitems, u32 *__restrict__ split_d,
                             u32 *__restrict__ split_h, u64 *__restrict__ cap, u64 *__restrict__ hsz,
                             u32 *__restrict__ esc_flag, u64 *__restrict__ esc_cnt) {
  const u32 ntiles = *ntiles_p;
  for (i64 i = i64(blockIdx.x) * blockDim.x + threadIdx.x; i < nmax; i += i64(gridDim.x) * blockDim.x) {
    if (i >= ntiles) {
      nitems[i] = 0; split_d[i] = 0; split_h[i] = 0; cap[i] = 0; hsz[i] = 0; esc_flag[i] = 0; esc_cnt[i] = 0;
      continue;
    }
    const u32 t = corder[i], c = cls[t];
    const u64 prod = P[abeg[t + 1]] - P[abeg[t]];
    u64 items = (prod + ct.pmax[c] - 1) / ct.pmax[c];
    const u64 area = tile_area(nrows, lb, LB, t);  // rows x LB fits 64 bits (host check)
    const u64 bound = prod < area ? prod : area;
    // esc 1: hash tiles too big for their table; 2: every hash tile
    const bool to_esc = esc && ct.hash[c] && (items > 1 || esc == 2);
    if (to_esc) items = 0;
    nitems[i] = u32(items);
    split_d[i] = (!ct.hash[c] && items > 1) ? 1u : 0u;
    split_h[i] = (ct.hash[c] && items > 1) ? 1u : 0u;
    esc_flag[i] = to_esc ? 1u : 0u;
    esc_cnt[i] = to_esc ? prod : 0;
    cap[i] = bound;
    u64 h = 0;
    if (ct.hash[c] && items > 1) {  // the tile's global table: load <= 0.8 (outputs <= bound)
      h = 64;
      while (h < bound + bound / 4) h <<= 1;
    }
    hsz[i] = h;
  }
}

// First item of each class (ckey sorted by class; out[c] stays ~0 for a class
// without tiles).
__global__ void k_class_bounds(const u32 *__restrict__ ntiles_p, const u64 *__restrict__ ckey,
                               const u32 *__restrict__ item_off, u64 *__restrict__ out) {
  const u32 ntiles = *ntiles_p;
  for (i64 i = i64(blockIdx.x) * blockDim.x + threadIdx.x; i < ntiles; i += i64(gridDim.x) * blockDim.x)
    if (i == 0 || ckey[i] != ckey[i - 1]) out[ckey[i]] = item_off[i];
}

__global__ void k_item_write(const u32 *__restrict__ ntiles_p, const u32 *__restrict__ corder,
                             const u32 *__restrict__ cls, const u32 *__restrict__ abeg, const u64 *__restrict__ P,
                             const u32 *__restrict__ item_off, ClassTable ct, Item *__restrict__ items,
                             const u32 *__restrict__ split_d, const u32 *__restrict__ split_h,
                             const u32 *__restrict__ split_d_idx, const u32 *__restrict__ split_h_idx,
                             int *__restrict__ split_of_tile, u32 *__restrict__ split_tiles_d,
                             u32 *__restrict__ split_tiles_h, const u64 *__restrict__ hoff_i,
                             const u64 *__restrict__ hsz_i, u64 *__restrict__ hoff_t, u64 *__restrict__ hsz_t,
                             const u32 *__restrict__ esc_flag, const u32 *__restrict__ esc_idx,
                             const u64 *__restrict__ esc_off, u32 *__restrict__ esc_tiles,
                             u64 *__restrict__ esc_base) {
  const u32 ntiles = *ntiles_p;
  for (i64 i = i64(blockIdx.x) * blockDim.x + threadIdx.x; i < ntiles; i += i64(gridDim.x) * blockDim.x) {
    const u32 t = corder[i];
    if (esc_flag[i]) {  // expanded, sorted and reduced instead of run as items
      esc_tiles[esc_idx[i]] = t;
      esc_base[esc_idx[i]] = esc_off[i];
      split_of_tile[t] = -1;
      hoff_t[t] = 0;
      hsz_t[t] = 0;
      continue;
    }
    const u64 pmax = ct.pmax[cls[t]];
    const u32 alo = abeg[t], ahi = abeg[t + 1];
    const u64 b = P[alo], e = P[ahi];
    u32 o = item_off[i];
    u32 ea = alo;
    for (u64 p = b; p < e; p += pmax) {
      Item it;
      it.p0 = p;
      it.p1 = (e - p > pmax) ? p + pmax : e;
      it.tile = t;
      it.ea = ea;
      u32 lo = ea, hi = ahi;  // first entry with P[entry] >= p1
      while (lo < hi) {
        const u32 mid = (lo + hi) >> 1;
        if (P[mid] < it.p1) lo = mid + 1; else hi = mid;
      }
      it.eb = lo;
      it.pad = 0;
      items[o++] = it;
      ea = (lo > alo && P[lo] > it.p1) ? lo - 1 : lo;  // the entry holding the next item's p0
    }
    split_of_tile[t] = -1;
    if (split_d[i]) {
      split_of_tile[t] = int(split_d_idx[i]);
      split_tiles_d[split_d_idx[i]] = t;
    }
    if (split_h[i]) {
      split_of_tile[t] = int(split_h_idx[i]);
      split_tiles_h[split_h_idx[i]] = t;
    }
    hoff_t[t] = hoff_i[i];
    hsz_t[t] = hsz_i[i];
  }
}

// ------------------------------------------------- hot-column remap ----
//
// B external indices are renumbered by descending frequency so that "one of
// the `hot` most frequent columns" is the test q < hot in the tile kernels;
// inv_col maps back when outputs are written.

template <class ColT>
__global__ void k_col_hist(const ColT *__restrict__ col, i64 n, u32 *__restrict__ count) {
  for (i64 i = i64(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += i64(gridDim.x) * blockDim.x) {
    const u32 c = u32(col[i]);
    const u32 peers = __match_any_sync(__activemask(), c);
    if ((threadIdx.x & 31) == u32(__ffs(peers) - 1)) atomicAdd(&count[c], u32(__popc(peers)));
  }
}

__global__ void k_col_sortkeys(const u32 *__restrict__ count, u64 LB, int bits, u64 *__restrict__ key,
                               u32 *__restrict__ idx) {
  for (u64 c = u64(blockIdx.x) * blockDim.x + threadIdx.x; c < LB; c += u64(gridDim.x) * blockDim.x) {
    key[c] = (u64(~count[c]) << bits) | c;  // ascending = most frequent first
    idx[c] = u32(c);
  }
}

__global__ void k_col_tables(const u64 *__restrict__ key, u64 LB, int bits, u32 hot, u32 *__restrict__ colmap,
                             u32 *__restrict__ inv, unsigned long long *hot_count) {
  u64 part = 0;
  for (u64 r = u64(blockIdx.x) * blockDim.x + threadIdx.x; r < LB; r += u64(gridDim.x) * blockDim.x) {
    const u32 c = u32(key[r] & ((u64(1) << bits) - 1));
    colmap[c] = u32(r);
    inv[r] = c;
    if (r < hot) part += u64(~u32(key[r] >> bits));
  }
  part = __reduce_add_sync(kFull, u32(part));  // hot counts fit 32 bits per warp (nnz < 2^31)
  if ((threadIdx.x & 31) == 0 && part) atomicAdd(hot_count, (unsigned long long)part);
}

template <class ColT>
__global__ void k_apply_colmap(ColT *__restrict__ col, i64 n, const u32 *__restrict__ colmap) {
  for (i64 i = i64(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += i64(gridDim.x) * blockDim.x)
    col[i] = ColT(colmap[u32(col[i])]);
}

// --------------------------------------------------------- tile kernels ----
//
// Work: an item is a range [p0, p1) of the global multiply-add index space
// (A sorted by row; the multiply-adds of A entry e are P[e] .. P[e+1]-1, one
// per nonzero of its B segment). An item never crosses an output tile. The
// CTA that takes an item cuts it into chunks; its warps pull chunks from a
// shared counter. Within a chunk a warp walks the A entries in order:
//  * a run of >= kLongRun multiply-adds of one entry streams its B segment,
//    32 lanes x kBatch loads in flight before the accumulator updates;
//  * shorter entries go one per lane, up to 32 at once, so rows made of many
//    rare keys (hub rows of Zipf tensors) keep every lane busy.

constexpr int kDefaultDenseMode = 3;  // fcc_options.dense_kernel 0 means this
constexpr int kTileThreads = 640;   // dense tiles by default (20 warps in 96 registers); 512, 768, 1024 on request
constexpr int kMergeThreads = 512;  // merges of split tiles
constexpr int kBatch = 4;
constexpr u32 kLongRun = 64;
constexpr u64 kNegZero = 0x8000000000000000ull;

struct ProdSrc {
  const u64 *P;        // multiply-add prefix per compacted A entry (nA2 + 1)
  const u32 *slotA;    // the entry's row inside its tile
  const u32 *sbA;      // first B entry of the entry's segment
  const double *valA;
  const double *valB;
};

// Lanes that run different A entries can update the same output position at
// once (Zipf hub columns sit in most segments). Colliding lanes are summed
// with shuffles first; only the lowest lane of each group keeps an update.
// Returns true for the lanes whose (key, *v) must still be applied.
// An update adds m * x: normally m = va, x = vb. A group leader carries
// m = 1 and x = the group's sum of products.
template <class KeyT>
__device__ __forceinline__ bool aggregate_lanes(KeyT key, double *m, double *x) {
  const u32 lane = threadIdx.x & 31;
  const u32 peers = __match_any_sync(__activemask(), key);
  if (peers == (1u << lane)) return true;
  const int leader = __ffs(peers) - 1;
  const double p = *m * *x;
  double s = p;
  for (u32 rest = peers & (peers - 1); rest; rest &= rest - 1) {
    const double y = __shfl_sync(peers, p, __ffs(rest) - 1);
    if (int(lane) == leader) s += y;
  }
  *m = 1.0;
  *x = s;
  return int(lane) == leader;
}

constexpr u64 kNoSkip = ~0ull;
constexpr u32 kNoEntry = 0xFFFFFFFFu;

// Multiply-adds of A entry e that fall inside [p0, p1).
__device__ __forceinline__ u64 coverage(const u64 *__restrict__ P, u32 e, u64 p0, u64 p1) {
  const u64 lo = max(__ldg(&P[e]), p0), hi = min(__ldg(&P[e + 1]), p1);
  return hi > lo ? hi - lo : 0;
}

// One warp runs the multiply-adds [q0, q1) of an item [p0, p1), in windows of
// 32 consecutive A entries (entry e + lane in each lane). Entries with >= skip
// multiply-adds in the item were run by the whole CTA and are left out; the
// others overlapping [q0, q1) are either streamed by the whole warp, one after
// another (>= kLongRun multiply-adds in the chunk), or run one per lane.
// e0: the entry holding q0, or kNoEntry to search for it.
template <class ColT, class KeyT, class Add>
__device__ __forceinline__ void products_chunk(const ProdSrc &s, const ColT *__restrict__ colB, u32 alo,
                                               u32 ahi, u32 e0, u64 q0, u64 q1, u64 p0, u64 p1, u64 skip,
                                               u64 LB, Add &add) {
  const u32 lane = threadIdx.x & 31;
  u32 e = e0;
  if (e == kNoEntry) {
    u32 lo = alo, hi = ahi;  // last entry with P[e] <= q0
    while (hi - lo > 1) {
      const u32 mid = (lo + hi) >> 1;
      if (__ldg(&s.P[mid]) <= q0) lo = mid; else hi = mid;
    }
    e = lo;
  }
  for (;; e += 32) {
    const u32 el = e + lane;
    u64 sg = 0, tg = 0, pl = 0;
    if (el < ahi) {
      pl = __ldg(&s.P[el]);
      const u64 pr = __ldg(&s.P[el + 1]);
      sg = max(pl, q0);
      tg = min(pr, q1);
      if (sg > tg) sg = tg;
      if (skip != kNoSkip && min(pr, p1) - max(pl, p0) >= skip) tg = sg;  // run by the CTA
    }
    const bool any_left = __any_sync(kFull, el < ahi && pl < q1);
    const u64 n = tg - sg;
    u32 stream = __ballot_sync(kFull, n >= kLongRun);
    const bool mine = n > 0 && n < kLongRun;
    double va = 0.0;
    KeyT base = 0;
    u32 b0 = 0;
    if (n > 0) {
      va = __ldg(&s.valA[el]);
      base = KeyT(u64(__ldg(&s.slotA[el])) * LB);
      b0 = __ldg(&s.sbA[el]) + u32(sg - pl);
    }
    while (stream) {  // warp-wide runs
      const int j = __ffs(stream) - 1;
      stream &= stream - 1;
      const double wva = __shfl_sync(kFull, va, j);
      const KeyT wbase = __shfl_sync(kFull, base, j);
      const u32 wb0 = __shfl_sync(kFull, b0, j);
      const u32 wn = u32(__shfl_sync(kFull, n, j));
      for (u32 o = 0; o < wn; o += 32 * kBatch) {
        ColT c[kBatch];
        double v[kBatch];
#pragma unroll
        for (int k = 0; k < kBatch; k++) {
          const u32 i = o + k * 32 + lane;
          if (i < wn) { c[k] = __ldg(&colB[wb0 + i]); v[k] = __ldg(&s.valB[wb0 + i]); }
        }
        KeyT key[kBatch];
        double m[kBatch];
        u32 valid = 0;
#pragma unroll
        for (int k = 0; k < kBatch; k++) {
          const u32 i = o + k * 32 + lane;
          key[k] = wbase + KeyT(c[k]);
          m[k] = wva;
          if (i < wn) valid |= 1u << k;
        }
        add.batch(key, m, v, valid, true, false);
      }
    }
    if (mine) {  // one entry per lane
      const u32 cnt = u32(n);
      for (u32 o = 0; o < cnt; o += kBatch) {
        ColT c[kBatch];
        double v[kBatch];
#pragma unroll
        for (int k = 0; k < kBatch; k++)
          if (o + k < cnt) { c[k] = __ldg(&colB[b0 + o + k]); v[k] = __ldg(&s.valB[b0 + o + k]); }
        KeyT key[kBatch];
        double m[kBatch];
        u32 valid = 0;
#pragma unroll
        for (int k = 0; k < kBatch; k++) {
          key[k] = base + KeyT(c[k]);
          m[k] = va;
          if (o + k < cnt && aggregate_lanes(key[k], &m[k], &v[k])) valid |= 1u << k;
        }
        add.batch(key, m, v, valid, false, false);
      }
    }
    if (!any_left) break;
    // the window's last entry reaches past q1: done
    const u64 last_end = __shfl_sync(kFull, (el < ahi) ? __ldg(&s.P[el + 1]) : ~0ull, 31);
    if (last_end >= q1) break;
  }
}

// ---- dense items in two phases ----
//
// Phase 1: an A entry with >= kCtaRun multiply-adds in the item is run by the
// whole CTA. Its B segment holds distinct columns, so every tile position gets
// at most one update from it and a plain FMA read-modify-write is exact;
// barriers separate consecutive entries. On Zipf operands these entries hold
// most multiply-adds (85% on the 10M-nonzero benchmark tensor).
// Phase 2: the other entries, by warps pulling chunks, with compare-and-swap
// FMAs. The item plan (built by one pass over the item's entries) lists the
// phase-1 entries and the first entry of every chunk, so chunks start without
// a search.

constexpr u32 kCtaRun = 1024;
constexpr int kCtaPer = 8;
constexpr u32 kListMax = 1024;   // items hold at most kListMax * kCtaRun multiply-adds
constexpr u32 kChunkMax = 2048;

template <u32 kLong, u32 kChunks>
struct PlanT {
  static constexpr u32 kLongMax = kLong, kChunkCap = kChunks, kRows = kChunks / 2;
  u32 ea, eb, nlong, nchunk, next;
  u64 chunk;
  u32 list[kLong];
  alignas(16) u32 start[kChunks];  // also the drain's row cache (kRows u64)
};
using ItemPlan = PlanT<kListMax, kChunkMax>;  // dense items: long-entry list, many chunks
using HashPlan = PlanT<1, 512>;               // hash items (<= 4096 multiply-adds)
constexpr u32 kRowCache = ItemPlan::kRows;

// ea/eb: the item's entries (Item::ea, Item::eb). Chunks hold at least
// min_chunk multiply-adds.
template <class Plan>
__device__ void build_item_plan(const u64 *__restrict__ P, u32 ea, u32 eb, u64 p0, u64 p1, u64 min_chunk,
                                Plan &pl) {
  const u32 tid = threadIdx.x, nwarps = blockDim.x >> 5;
  if (tid == 0) {
    pl.ea = ea;
    pl.eb = eb;
    const u64 np = p1 - p0;
    u64 chunk = np / (4 * nwarps);
    chunk = chunk < min_chunk ? min_chunk : (chunk > 4096 ? 4096 : chunk);
    if ((np + chunk - 1) / chunk > Plan::kChunkCap) chunk = (np + Plan::kChunkCap - 1) / Plan::kChunkCap;
    pl.chunk = chunk;
    pl.nchunk = u32((np + chunk - 1) / chunk);
    pl.nlong = 0;
    pl.next = 0;
  }
  __syncthreads();
  const u64 chunk = pl.chunk;
  for (u32 e = pl.ea + tid; e < pl.eb; e += blockDim.x) {
    const u64 lo = max(__ldg(&P[e]), p0), hi = min(__ldg(&P[e + 1]), p1);
    if (hi <= lo) continue;
    if (hi - lo >= kCtaRun) {
      const u32 i = atomicAdd(&pl.nlong, 1u);
      if (i < Plan::kLongMax) pl.list[i] = e;
    }
    for (u64 c = (lo - p0 + chunk - 1) / chunk; c < (hi - p0 + chunk - 1) / chunk; c++) pl.start[c] = e;
  }
  __syncthreads();
}

// ---- phase 1 with bulk-copy staging ----
//
// Warp 0 (one lane) produces: it reads each long entry's metadata and copies
// the entry's B segment, in chunks of kStageCh multiply-adds, from global
// memory into a ring of kStageBufs shared-memory buffers with cp.async.bulk,
// completion tracked by an mbarrier per buffer ("full"). The other warps
// consume: wait for a chunk, apply its plain FMA read-modify-writes, and
// release the buffer through a second mbarrier ("empty", one arrival per
// consumer warp). Chunks of one entry touch distinct columns, so consumers
// wait for each other only where a new entry starts. The producer runs up
// to kStageBufs chunks ahead, so segment loads and entry metadata overlap the
// accumulation. Every wait, including the consumers' wait between entries,
// is an mbarrier poll with a bounded count (DenseArgs::wait_polls); on timeout
// the kernel flags ERRB_TIMEOUT, stops issuing, waits (at the full limit) for
// its copies in flight and skips its remaining phase-1 work. With
// DenseArgs::fault_wait the consumers first wait on `never`, an mbarrier that
// nothing arrives at: the injected wait that tests make run out.
constexpr u32 kStageCh = 1824;  // 3 x 608 consumer threads of a 640-thread tile: no partial round
constexpr u32 kStageBufs = 2;
constexpr u32 kStageValBytes = (kStageCh + 2) * 8;  // 16-byte multiple: room for a 1-element head
constexpr u32 kStageColBytes = (kStageCh + 4) * 4;  // 16-byte multiple: room for a 3-element head
constexpr u32 kStageBufBytes = kStageValBytes + kStageColBytes;
constexpr u32 kStageBytes = kStageBufs * kStageBufBytes;

struct StageHdr {  // one staged chunk (written by the producer before the copies)
  double va;
  u32 base, cnt, sc, sv;  // tile offset of the entry's row, multiply-adds, col / val head skip
  u32 first, more;        // first chunk of an entry after the item's first; another chunk follows
};

struct StageCtl {
  unsigned long long full[kStageBufs], empty[kStageBufs];
  unsigned long long never;  // never completed: the target of an injected wait
  StageHdr hdr[kStageBufs];
  u32 seq;    // chunks staged so far by this CTA (sets buffer and mbarrier parity)
  u32 fail;   // a wait timed out: skip the remaining work
};

__device__ __forceinline__ void stage_init(StageCtl &c, u32 consumers) {
  if (threadIdx.x == 0) {
    for (u32 b = 0; b < kStageBufs; b++) {
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_addr(&c.full[b])) : "memory");
      asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(&c.empty[b])), "r"(consumers)
                   : "memory");
    }
    mbar_init(&c.never, 1);
    c.seq = 0;
    c.fail = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  }
  __syncthreads();
}

// Phase 1 of a dense item with staging (all threads call; ends with a barrier).
template <bool kSentinel>
__device__ void dense_phase1_staged(const ProdSrc &s, const u32 *__restrict__ colB, u64 p0, u64 p1, u32 LB,
                                    double *acc, u32 *mask, const ItemPlan &pl, unsigned char *stage,
                                    StageCtl &ctl, u32 *err, long long polls, u32 fault_wait) {
  const u32 nlong = min(pl.nlong, kListMax);
  const u32 tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const u32 nconsumers = blockDim.x - 32;
  u32 seq = ctl.seq;  // every role advances it by one per chunk
  if (nlong == 0 || ctl.fail) {
    __syncthreads();
    return;
  }
  u32 issued_last[kStageBufs] = {};  // producer: last chunk copied into each buffer by this item
  bool issued[kStageBufs] = {};
  if (warp == 0) {
    if (lane == 0) {  // producer
      bool ok = true;
      // entry metadata one entry ahead: its loads overlap this entry's copies
      u32 e = pl.list[0];
      u64 npb = __ldg(&s.P[e]), npe = __ldg(&s.P[e + 1]);
      double nva = __ldg(&s.valA[e]);
      u32 nslot = __ldg(&s.slotA[e]), nsb = __ldg(&s.sbA[e]);
      for (u32 li = 0; li < nlong && ok; li++) {
        const u64 pb = npb;
        const u64 lo = max(pb, p0), hi = min(npe, p1);
        const double va = nva;
        const u32 base = nslot * LB;
        const u32 b0 = nsb + u32(lo - pb);
        const u32 n = u32(hi - lo);
        if (li + 1 < nlong) {
          e = pl.list[li + 1];
          npb = __ldg(&s.P[e]);
          npe = __ldg(&s.P[e + 1]);
          nva = __ldg(&s.valA[e]);
          nslot = __ldg(&s.slotA[e]);
          nsb = __ldg(&s.sbA[e]);
        }
        for (u32 off = 0; off < n; off += kStageCh, seq++) {
          const u32 b = seq % kStageBufs;
          if (seq >= kStageBufs && !mbar_wait(&ctl.empty[b], ((seq / kStageBufs) - 1) & 1, polls)) {
            ok = false;
            break;
          }
          const u32 cnt = min(kStageCh, n - off), g = b0 + off;
          const u32 sc = g & 3u, sv = g & 1u;
          const u32 cbytes = ((sc + cnt + 3u) & ~3u) * 4u, vbytes = ((sv + cnt + 1u) & ~1u) * 8u;
          StageHdr &h = ctl.hdr[b];
          h.va = va;
          h.base = base;
          h.cnt = cnt;
          h.sc = sc;
          h.sv = sv;
          h.first = (off == 0 && li > 0) ? 1u : 0u;
          h.more = (li + 1 < nlong || off + kStageCh < n) ? 1u : 0u;
          unsigned char *buf = stage + b * kStageBufBytes;
          asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(&ctl.full[b])),
                       "r"(cbytes + vbytes)
                       : "memory");
          bulk_g2s(buf, s.valB + (g - sv), vbytes, &ctl.full[b]);
          bulk_g2s(buf + kStageValBytes, colB + (g - sc), cbytes, &ctl.full[b]);
          issued[b] = true;
          issued_last[b] = seq;
        }
      }
      if (!ok) {  // stop issuing
        atomicOr(err, ERRB_TIMEOUT);
        ctl.fail = 1;
      }
      ctl.seq = seq;
    }
  } else {  // consumers
    const u32 ctid = tid - 32;
    if (fault_wait && !mbar_wait(&ctl.never, 0, polls)) {  // injected: always runs out
      atomicOr(err, ERRB_TIMEOUT);
      ctl.fail = 1;
    }
    while (!ctl.fail) {
      const u32 b = seq % kStageBufs;
      if (!mbar_wait(&ctl.full[b], (seq / kStageBufs) & 1, polls)) {
        atomicOr(err, ERRB_TIMEOUT);
        ctl.fail = 1;
        break;
      }
      const StageHdr h = ctl.hdr[b];
      // a new entry may share columns with the previous one: wait until every
      // consumer warp has released the previous chunk (a bounded wait, unlike
      // a named barrier)
      if (h.first) {
        const u32 pseq = seq - 1, pb = pseq % kStageBufs;
        if (!mbar_wait(&ctl.empty[pb], (pseq / kStageBufs) & 1, polls)) {
          atomicOr(err, ERRB_TIMEOUT);
          ctl.fail = 1;
          break;
        }
      }
      const double *val = reinterpret_cast<const double *>(stage + b * kStageBufBytes) + h.sv;
      const u32 *col = reinterpret_cast<const u32 *>(stage + b * kStageBufBytes + kStageValBytes) + h.sc;
      for (u32 i = ctid; i < h.cnt; i += nconsumers) {
        const u32 q = h.base + col[i];
        acc[q] = fma(h.va, val[i], acc[q]);
        if (!kSentinel) atomicOr(&mask[q >> 5], 1u << (q & 31));
      }
      __syncwarp();
      if (lane == 0) asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_addr(&ctl.empty[b])) : "memory");
      seq++;
      if (!h.more) break;
    }
  }
  __syncthreads();
  // After a failed wait (here or in another role) copies of this item may
  // still be in flight, unconsumed: the producer lets them land (full limit)
  // before the CTA can reuse or release the ring.
  if (ctl.fail && tid == 0)
    for (u32 b = 0; b < kStageBufs; b++)
      if (issued[b]) mbar_wait(&ctl.full[b], (issued_last[b] / kStageBufs) & 1);
  __syncthreads();
}

// ---- dense items, flat ----
//
// The item's multiply-adds [p0, p1) are numbered by the prefix P over its A
// entries; warps pull chunks of consecutive numbers and give each lane one
// multiply-add per round, kBatch rounds at a time (their loads in flight
// together). The A entries of a chunk are read 32 at a time into a window
// (lane k: entry e + k's end, first B element, row slot and value). A batch
// that lies inside one entry (the long entries that hold most multiply-adds)
// takes that entry's data by one shuffle each; a batch that crosses entries
// finds each lane's entry by a five-step search over the shuffled ends. So
// every lane is busy whatever the entries' lengths, and B is read coalesced
// along each segment. Updates are compare-and-swap FMAs (other warps run other
// entries of the same tile); lanes of one round that fall into different
// entries may share a column and are combined first. The most frequent
// columns (renumbered to [0, hot)) go to the warp's private copy with plain
// read-modify-writes (see DenseAdd).
__device__ __forceinline__ u32 window_count_le(u64 endk, u64 x) {  // window ends <= x (at most 31 for x < end[31])
  u32 j = 0;
#pragma unroll
  for (u32 step = 16; step >= 1; step >>= 1) {
    const u64 v = __shfl_sync(kFull, endk, j + step - 1);
    if (v <= x) j += step;
  }
  return j;
}

// Warps pull the item plan's chunks and run their multiply-adds flat. Entries
// with at least `skip` multiply-adds in [p0, p1) are left out (phase 1 of a
// two-phase item ran them); kNoSkip runs every entry.
template <class Add>
__device__ void flat_chunks(const ProdSrc &s, const u32 *__restrict__ colB, u32 ahi, u64 p0, u64 p1, u32 LB,
                            ItemPlan &pl, Add &add, u64 skip, bool add_tile) {
  const u32 lane = threadIdx.x & 31;
  const u64 chunk = pl.chunk;
  const u32 nch = pl.nchunk;
  constexpr u64 kSpan = 32 * kBatch;
  for (;;) {
    u32 c = 0;
    if (lane == 0) c = atomicAdd(&pl.next, 1u);
    c = __shfl_sync(kFull, c, 0);
    if (c >= nch) break;
    u64 q = p0 + u64(c) * chunk;
    const u64 q1 = min(q + chunk, p1);
    u32 e = pl.start[c];  // the entry holding q
    while (q < q1) {
      // window: entries e .. e + 31
      const u32 ek = e + lane;
      u64 endk = ~0ull, begk = ~0ull;
      u32 sbk = 0, basek = 0, longk = 0;
      double vak = 0.0;
      if (ek < ahi) {
        begk = __ldg(&s.P[ek]);
        endk = __ldg(&s.P[ek + 1]);
        sbk = __ldg(&s.sbA[ek]);
        basek = __ldg(&s.slotA[ek]) * LB;
        vak = __ldg(&s.valA[ek]);
        longk = skip != kNoSkip && min(endk, p1) - max(begk, p0) >= skip;
      }
      const u64 wend = min(__shfl_sync(kFull, endk, 31), q1);  // the window covers [q, wend)
      u32 jc = window_count_le(endk, q);                       // the entry holding q
      while (q < wend) {
        const u64 ec = __shfl_sync(kFull, endk, jc);
        if (__shfl_sync(kFull, longk, jc)) {  // run by phase 1
          q = min(ec, wend);
          if (q == ec) jc++;
          continue;
        }
        const u64 bend = min(q + kSpan, wend);
        u32 key[kBatch];
        double m[kBatch], x[kBatch];
        u32 valid = 0;
        if (ec >= bend) {  // the batch lies inside entry jc: distinct columns
          const u64 bj = __shfl_sync(kFull, begk, jc);
          const u32 g0 = __shfl_sync(kFull, sbk, jc) + u32(q - bj) + lane;
          const u32 basej = __shfl_sync(kFull, basek, jc);
          const double vaj = __shfl_sync(kFull, vak, jc);
          const u32 n = u32(bend - q);
#pragma unroll
          for (int r = 0; r < kBatch; r++) {
            const u32 i = u32(r) * 32 + lane;
            key[r] = 0;
            x[r] = 0.0;
            m[r] = vaj;
            if (i < n) {
              key[r] = basej + __ldg(&colB[g0 + u32(r) * 32]);
              x[r] = __ldg(&s.valB[g0 + u32(r) * 32]);
              valid |= 1u << r;
            }
          }
          add.batch(key, m, x, valid, true, true, add_tile);
          q = bend;
          if (q == ec) jc++;
        } else {  // the batch crosses entries: each lane finds its own
#pragma unroll
          for (int r = 0; r < kBatch; r++) {
            const u64 pr = q + u64(r) * 32 + lane;
            u32 j = window_count_le(endk, pr);  // every lane shuffles; lanes past the batch keep jc
            if (pr >= bend) j = jc;
            const u64 bj = __shfl_sync(kFull, begk, j);
            const u32 sbj = __shfl_sync(kFull, sbk, j);
            const u32 basej = __shfl_sync(kFull, basek, j);
            const double vaj = __shfl_sync(kFull, vak, j);
            const u32 lj = __shfl_sync(kFull, longk, j);
            key[r] = 0;
            x[r] = 0.0;
            m[r] = vaj;
            if (pr < bend && !lj) {
              const u32 g = sbj + u32(pr - bj);
              key[r] = basej + __ldg(&colB[g]);
              x[r] = __ldg(&s.valB[g]);
              valid |= 1u << r;
            }
          }
#pragma unroll
          for (int r = 0; r < kBatch; r++)
            if (((valid >> r) & 1u) && !aggregate_lanes(key[r], &m[r], &x[r])) valid &= ~(1u << r);
          __syncwarp();
          add.batch(key, m, x, valid, false, true, add_tile);
          q = bend;
          if (q < wend) jc = window_count_le(endk, q);
        }
      }
      e += 32;
    }
  }
}

template <class Add>
__device__ void dense_item_flat(const ProdSrc &s, const u32 *__restrict__ colB, u32 ahi, u64 p0, u64 p1, u32 ea,
                                u32 eb, u32 LB, ItemPlan &pl, Add &add) {
  build_item_plan(s.P, ea, eb, p0, p1, 256, pl);
  flat_chunks(s, colB, ahi, p0, p1, LB, pl, add, kNoSkip, false);
}

// kFlat2: phase 2 runs flat (flat_chunks, the phase-1 entries left out)
// instead of products_chunk's windows of one entry per lane.
template <bool kSentinel, bool kFlat2, class Add>
__device__ void dense_item(const ProdSrc &s, const u32 *__restrict__ colB, u32 alo, u32 ahi, u64 p0, u64 p1,
                           u32 ea, u32 eb, u32 LB, double *acc, u32 *mask, ItemPlan &pl, Add &add,
                           unsigned char *stage, StageCtl &ctl, u32 *err, long long polls, u32 fault_wait) {
  build_item_plan(s.P, ea, eb, p0, p1, 256, pl);
  const u32 tid = threadIdx.x, lane = tid & 31;
  const u32 nlong = stage ? 0u : min(pl.nlong, kListMax);
  if (stage) dense_phase1_staged<kSentinel>(s, colB, p0, p1, LB, acc, mask, pl, stage, ctl, err, polls, fault_wait);
  for (u32 li = 0; li < nlong; li++) {
    const u32 e = pl.list[li];
    const u64 pb = __ldg(&s.P[e]);
    const u64 lo = max(pb, p0), hi = min(__ldg(&s.P[e + 1]), p1);
    const double va = __ldg(&s.valA[e]);
    const u32 base = __ldg(&s.slotA[e]) * LB;
    const u32 b0 = __ldg(&s.sbA[e]) + u32(lo - pb);
    const u32 n = u32(hi - lo);
    for (u32 o = 0; o < n; o += blockDim.x * kCtaPer) {
      u32 c[kCtaPer];
      double v[kCtaPer];
#pragma unroll
      for (int k = 0; k < kCtaPer; k++) {
        const u32 i = o + k * blockDim.x + tid;
        if (i < n) { c[k] = __ldg(&colB[b0 + i]); v[k] = __ldg(&s.valB[b0 + i]); }
      }
#pragma unroll
      for (int k = 0; k < kCtaPer; k++) {
        const u32 i = o + k * blockDim.x + tid;
        if (i < n) {
          const u32 q = base + c[k];
          acc[q] = fma(va, v[k], acc[q]);
          if (!kSentinel) atomicOr(&mask[q >> 5], 1u << (q & 31));
        }
      }
    }
    __syncthreads();
  }
  // phase 2
  if (kFlat2) {
    flat_chunks(s, colB, ahi, p0, p1, LB, pl, add, u64(kCtaRun), true);
    return;
  }
  const u64 chunk = pl.chunk;
  const u32 nch = pl.nchunk;
  for (;;) {
    u32 c = 0;
    if (lane == 0) c = atomicAdd(&pl.next, 1u);
    c = __shfl_sync(kFull, c, 0);
    if (c >= nch) break;
    const u64 q0 = p0 + u64(c) * chunk;
    const u64 q1 = min(q0 + chunk, p1);
    products_chunk<u32, u32>(s, colB, alo, ahi, pl.start[c], q0, q1, p0, p1, u64(kCtaRun), LB, add);
  }
}

struct DenseArgs {
  const Item *items;
  u32 nitems;
  u32 *counter;
  const u32 *tile_abeg;
  const u32 *tile_rank0;  // first row rank
  const u32 *tile_lb;     // column span
  const u32 *tile_nrows;
  const u64 *urow;        // row rank -> A external index
  const int *split_of_tile;
  const u32 *split_tiles;
  u32 nsplit;
  ProdSrc src;
  const u32 *colB;
  u32 area, words;        // tile capacity (positions, mask words)
  u32 hot;  // renumbered columns [0, hot) are accumulated per warp (row tiles only)
  double *gacc;
  u32 *gmask;
  Out out;
  Decode dec;
  u32 *err;
  u64 *item_cyc;  // per item: SM cycles from fetch to drained (NULL: not recorded)
  u32 stage_off;  // byte offset of phase 1's staging ring in dynamic shared memory; 0: no staging
  u64 *merge_cyc; // per tile: SM cycles of its split-tile merge (NULL: not recorded)
  long long wait_polls = kWaitPolls;  // poll limit of the staging ring's waits
  u32 fault_wait = 0;                 // 1: injected wait that runs out (tests)
};

// The touched mask of positions [32w, 32w+32) of a dense tile, in every lane.
// With kSentinel the tile holds -0.0 at untouched positions and the mask is a
// ballot.
template <bool kSentinel>
__device__ __forceinline__ u32 group_mask(const double *acc, const u32 *mask, u32 area, u32 w) {
  if (!kSentinel) return mask[w];
  const u32 pos = w * 32 + (threadIdx.x & 31);
  const bool t = pos < area && u64(__double_as_longlong(acc[pos])) != kNegZero;
  return __ballot_sync(kFull, t);
}

// Exclusive prefix sum of v over the block; *total gets the sum. s_warp holds
// 32 entries. Ends with a barrier.
__device__ __forceinline__ u32 block_excl_u32(u32 v, u32 *s_warp, u32 *total) {
  const u32 lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
  const u32 incl = warp_incl_u32(v);
  if (lane == 31) s_warp[warp] = incl;
  __syncthreads();
  if (warp == 0) {
    u32 x = lane < nwarps ? s_warp[lane] : 0u;
    x = warp_incl_u32(x);
    if (lane < nwarps) s_warp[lane] = x;
  }
  __syncthreads();
  const u32 before = warp ? s_warp[warp - 1] : 0u;
  *total = s_warp[nwarps - 1];
  __syncthreads();
  return before + incl - v;
}

// Emits every touched position among the first `used` of a dense tile with
// its value and resets it (mask words to 0; values to 0.0, or -0.0 with
// kSentinel). Position p holds row urow[rank0 + p / LB], column p % LB
// (lbm = magic_for(LB)). Pass 1 counts the touched positions of each
// 32-position group, one prefix sum over the groups reserves the output
// range, pass 2 writes each group's outputs contiguously. s_cnt holds
// ceil(used / 32) (<= 4 * blockDim.x) entries.
template <bool kSentinel>
__device__ void drain_dense(double *acc, u32 *mask, u32 used, u32 LB, u64 lbm, const u64 *__restrict__ urow,
                            u32 rank0, const Out &out, const Decode &dec, u32 *err, u32 *s_cnt, u32 *s_warp,
                            u64 *s_base, u64 *s_rows) {
  const u32 tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nwarps = blockDim.x >> 5;
  const u32 words = (used + 31) / 32, area = used;
  // the tile's rows, staged once (the barrier after pass 1 publishes them)
  const u32 nrows = div_magic(used, lbm);
  const bool cached = nrows <= kRowCache;
  if (cached)
    for (u32 i = tid; i < nrows; i += blockDim.x) s_rows[i] = __ldg(&urow[rank0 + i]);
  for (u32 w = warp; w < words; w += nwarps) {
    const u32 b = group_mask<kSentinel>(acc, mask, area, w);
    if (lane == 0) s_cnt[w] = __popc(b);
  }
  __syncthreads();
  const u32 ipt = (words + blockDim.x - 1) / blockDim.x;  // groups per thread (<= 4)
  u32 loc[4], sum = 0;
#pragma unroll
  for (int j = 0; j < 4; j++) {
    const u32 w = tid * ipt + j;
    loc[j] = (u32(j) < ipt && w < words) ? s_cnt[w] : 0u;
    sum += loc[j];
  }
  u32 total;
  u32 run = block_excl_u32(sum, s_warp, &total);
#pragma unroll
  for (int j = 0; j < 4; j++) {
    const u32 w = tid * ipt + j;
    if (u32(j) < ipt && w < words) s_cnt[w] = run;
    run += loc[j];
  }
  if (tid == 0) *s_base = reserve(out, total, err);
  __syncthreads();
  const u64 base = *s_base;
  const bool write = base != ~0ull;
  const double reset = kSentinel ? __longlong_as_double((long long)kNegZero) : 0.0;
  const u32 lt = (1u << lane) - 1u;
  for (u32 w = warp; w < words; w += nwarps) {
    const u32 b = group_mask<kSentinel>(acc, mask, area, w);
    if ((b >> lane) & 1u) {
      const u32 pos = w * 32 + lane;
      const double v = acc[pos];
      acc[pos] = reset;
      const u32 slot = div_magic(pos, lbm);
      const u64 row = cached ? s_rows[slot] : __ldg(&urow[rank0 + slot]);
      if (write) emit(out, dec, base + s_cnt[w] + __popc(b & lt), row, pos - slot * LB, v);
    }
    if (!kSentinel) {
      __syncwarp();
      if (lane == 0) mask[w] = 0u;
    }
  }
}

// Adds a partial tile into its global split-tile buffer and resets it.
template <bool kSentinel>
__device__ void flush_dense(double *acc, u32 *mask, u32 used, double *gacc, u32 *gmask) {
  const u32 lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
  const u32 words = (used + 31) / 32, area = used;
  const double reset = kSentinel ? __longlong_as_double((long long)kNegZero) : 0.0;
  for (u32 w = warp; w < words; w += nwarps) {
    const u32 pos = w * 32 + lane;
    bool t;
    if (kSentinel) t = pos < area && u64(__double_as_longlong(acc[pos])) != kNegZero;
    else t = (mask[w] >> lane) & 1u;
    const u32 b = __ballot_sync(kFull, t);
    if (t) {
      atomicAdd(&gacc[pos], acc[pos]);
      acc[pos] = reset;
    }
    if (lane == 0 && b) atomicOr(&gmask[w], b);
    if (!kSentinel && lane == 0) mask[w] = 0u;
  }
}

// Shared-memory FP64 accumulation. On this GPU the FP64 issue rate bounds the
// tile kernels (measured: ~1.55 FP64 instructions per clock per SM), so each
// multiply-add is one FMA inside a compare-and-swap loop: acc = fma(m, x, acc).
// The built-in FP64 atomic add costs a separate multiply plus its own add
// (measured 0.56 updates per clock per SM against 0.81 for this loop and 0.91
// for an unsynchronised read-modify-write with FMA).
__device__ __forceinline__ void fma_shared(double *p, double m, double x) {
  unsigned long long *a = reinterpret_cast<unsigned long long *>(p);
  unsigned long long cur = *reinterpret_cast<volatile unsigned long long *>(a), assumed;
  do {
    assumed = cur;
    cur = atomicCAS(a, assumed,
                    (unsigned long long)__double_as_longlong(fma(m, x, __longlong_as_double((long long)assumed))));
  } while (cur != assumed);
}

//
// Zipf-like operands send most multiply-adds of a row to a few columns (for
// Zipf(1.2) over 20,000 columns, ~70% land in the 64 most frequent). Updates
// to one address from many warps retry their compare-and-swap, so the most
// frequent columns (renumbered to [0, hot) on the host) can get a private
// copy per warp, summed into the tile before the drain.
template <bool kSentinel>
struct DenseAdd {
  double *acc;
  u32 *mask;
  double *priv;  // this warp's copy of the hot columns
  u32 *pmask;    // its touched bits (bitmask mode)
  u32 hot;
  // Applies a lane's kBatch updates (key[k] += m[k] * x[k] where valid).
  // distinct: the warp's updates of this batch have distinct keys (one A
  // entry's B segment); otherwise only the lanes of one round k are distinct
  // (combined beforehand). plain_priv: the whole warp calls converged, so
  // its private hot-column copy, which no other warp touches, takes plain
  // read-modify-writes (rounds of different keys ordered by __syncwarp);
  // otherwise it takes compare-and-swap like the shared tile. add_tile: the
  // shared tile takes the built-in FP64 atomic add of the product (a multiply
  // and an atomic, no retry loop) instead of a compare-and-swap loop around
  // one FMA; measured faster for the short entries of two-phase items (phase
  // 2 run flat), slower for whole flat items.
  __device__ __forceinline__ void batch(const u32 (&key)[kBatch], const double (&m)[kBatch],
                                        const double (&x)[kBatch], u32 valid, bool distinct,
                                        bool plain_priv, bool add_tile = false) const {
#pragma unroll
    for (int k = 0; k < kBatch; k++) {
      if ((valid >> k) & 1u) {
        const u32 q = key[k];
        if (q < hot) {
          if (plain_priv) priv[q] = fma(m[k], x[k], priv[q]);
          else fma_shared(&priv[q], m[k], x[k]);
          if (!kSentinel) atomicOr(&pmask[q >> 5], 1u << (q & 31));
        } else {
          if (add_tile) atomicAdd(&acc[q], m[k] * x[k]);
          else fma_shared(&acc[q], m[k], x[k]);
          if (!kSentinel) atomicOr(&mask[q >> 5], 1u << (q & 31));
        }
      }
      if (plain_priv && !distinct && hot) __syncwarp();
    }
    if (plain_priv && distinct && hot) __syncwarp();  // before the warp's next batch
  }
};

// Sums the per-warp hot-column copies into tile positions [0, hot) and resets
// them. Call between barriers.
template <bool kSentinel>
__device__ __forceinline__ void merge_hot_dense(double *acc, u32 *mask, double *priv, u32 *pmask, u32 hot) {
  const u32 nwarps = blockDim.x >> 5, pw = hot / 32;
  const double init = kSentinel ? __longlong_as_double((long long)kNegZero) : 0.0;
  for (u32 i = threadIdx.x; i < hot; i += blockDim.x) {
    double s = init;
    u32 touched = 0;
    for (u32 w = 0; w < nwarps; w++) {
      s += priv[w * hot + i];
      priv[w * hot + i] = init;
      if (!kSentinel) touched |= (pmask[w * pw + i / 32] >> (i & 31)) & 1u;
    }
    acc[i] += s;  // -0.0 + -0.0 stays the untouched sentinel
    if (!kSentinel && touched) atomicOr(&mask[i >> 5], 1u << (i & 31));
  }
  __syncthreads();
  if (!kSentinel)
    for (u32 i = threadIdx.x; i < nwarps * pw; i += blockDim.x) pmask[i] = 0u;
}

// kMode 1: two-phase items (dense_item); 2: flat items (dense_item_flat);
// 3: two-phase items whose phase 2 runs flat.
template <bool kSentinel, int kThreads, int kMode>
__global__ void __launch_bounds__(kThreads, 1) k_contract_dense(DenseArgs a) {
  extern __shared__ __align__(16) unsigned char smem[];
  // layout: acc[area] | mask[words] (bitmask mode) | priv[nwarps*hot] | pmask[nwarps*hot/32]
  double *acc = reinterpret_cast<double *>(smem);
  u32 *mask = reinterpret_cast<u32 *>(acc + a.area);
  const u32 nwarps = blockDim.x >> 5, warp = threadIdx.x >> 5;
  const size_t off = (size_t(a.area) * 8 + (kSentinel ? 0 : size_t(a.words) * 4) + 15) & ~size_t(15);
  double *priv = reinterpret_cast<double *>(smem + off);
  u32 *pmask = reinterpret_cast<u32 *>(priv + size_t(nwarps) * a.hot);
  __shared__ u32 s_item;
  __shared__ u32 s_warp[32];
  __shared__ u32 s_cnt[1024];
  __shared__ u64 s_base;
  __shared__ ItemPlan plan;
  __shared__ StageCtl ctl;
  const int tid = threadIdx.x;
  unsigned char *stage = a.stage_off ? smem + a.stage_off : nullptr;
  if (stage) stage_init(ctl, nwarps - 1);
  const double init = kSentinel ? __longlong_as_double((long long)kNegZero) : 0.0;
  for (u32 i = tid; i < a.area; i += blockDim.x) acc[i] = init;
  if (!kSentinel)
    for (u32 i = tid; i < a.words; i += blockDim.x) mask[i] = 0u;
  for (u32 i = tid; i < nwarps * a.hot; i += blockDim.x) priv[i] = init;
  if (!kSentinel)
    for (u32 i = tid; i < nwarps * (a.hot / 32); i += blockDim.x) pmask[i] = 0u;
  DenseAdd<kSentinel> add{acc, mask, priv + size_t(warp) * a.hot, pmask + size_t(warp) * (a.hot / 32), a.hot};
  for (;;) {
    const long long c0 = clock64();
    if (tid == 0) s_item = atomicAdd(a.counter, 1u);
    __syncthreads();
    const u32 it = s_item;
    if (it >= a.nitems) break;
    const Item item = a.items[it];
    const u32 t = item.tile;
    const u32 LB = a.tile_lb[t], used = a.tile_nrows[t] * LB;
    if constexpr (kMode == 2)
      dense_item_flat(a.src, a.colB, a.tile_abeg[t + 1], item.p0, item.p1, item.ea, item.eb, LB, plan, add);
    else
      dense_item<kSentinel, kMode == 3>(a.src, a.colB, a.tile_abeg[t], a.tile_abeg[t + 1], item.p0, item.p1,
                                        item.ea, item.eb, LB, acc, mask, plan, add, stage, ctl, a.err,
                                        a.wait_polls, a.fault_wait);
    __syncthreads();
    if (a.hot) {
      merge_hot_dense<kSentinel>(acc, mask, priv, pmask, a.hot);
      __syncthreads();
    }
    const int sidx = a.split_of_tile[t];
    if (sidx < 0)
      drain_dense<kSentinel>(acc, mask, used, LB, magic_for(LB), a.urow, a.tile_rank0[t], a.out, a.dec, a.err,
                             s_cnt, s_warp, &s_base, reinterpret_cast<u64 *>(plan.start));  // plan is idle
    else
      flush_dense<kSentinel>(acc, mask, used, a.gacc + u64(sidx) * a.area, a.gmask + u64(sidx) * a.words);
    __syncthreads();
    if (a.item_cyc && tid == 0) a.item_cyc[it] = u64(clock64() - c0);
  }
}

__global__ void __launch_bounds__(kMergeThreads) k_merge_dense(DenseArgs a) {
  __shared__ u32 s_warp[32];
  __shared__ u32 s_cnt[1024];
  __shared__ u64 s_base;
  __shared__ u64 s_rows[kRowCache];
  for (u32 s = blockIdx.x; s < a.nsplit; s += gridDim.x) {
    const long long c0 = clock64();
    const u32 t = a.split_tiles[s];
    const u32 LB = a.tile_lb[t];
    drain_dense<false>(a.gacc + u64(s) * a.area, a.gmask + u64(s) * a.words, a.tile_nrows[t] * LB, LB,
                       magic_for(LB), a.urow, a.tile_rank0[t], a.out, a.dec, a.err, s_cnt, s_warp, &s_base, s_rows);
    __syncthreads();
    if (a.merge_cyc && threadIdx.x == 0) a.merge_cyc[t] = u64(clock64() - c0);
  }
}

using DenseKernel = void (*)(DenseArgs);

// The dense tile kernel for a tile shape: touched positions by sentinel or
// bitmask, threads per CTA, two-phase or flat items.
template <int kMode>
DenseKernel dense_kernel_for(bool sentinel, int threads) {
  switch (threads) {
    case 512: return sentinel ? k_contract_dense<true, 512, kMode> : k_contract_dense<false, 512, kMode>;
    case 768: return sentinel ? k_contract_dense<true, 768, kMode> : k_contract_dense<false, 768, kMode>;
    case 1024: return sentinel ? k_contract_dense<true, 1024, kMode> : k_contract_dense<false, 1024, kMode>;
    default: return sentinel ? k_contract_dense<true, 640, kMode> : k_contract_dense<false, 640, kMode>;
  }
}

// ---------------------------------------------------------- hash tiles ----

template <class ColT>
struct HashArgs {
  const Item *items;
  u32 nitems;
  u32 *counter;
  const u32 *tile_rank0;  // first row rank
  const u64 *urow;        // row rank -> A external index
  const u32 *tile_nrows;
  const u32 *tile_abeg;
  const int *split_of_tile;
  const u32 *split_tiles;
  u32 nsplit;
  ProdSrc src;
  const ColT *colB;
  u64 LB;
  u32 TL;
  u32 slots;        // shared-memory slots (power of two)
  u32 hot;          // renumbered columns [0, hot) accumulated per warp (TL == 1 only)
  const u64 *hoff;  // per tile: first slot of its global region (split tiles)
  const u64 *hsz;   // per tile: global region size, a power of two (split tiles)
  u64 *gkeys;
  double *gvals;
  Out out;
  Decode dec;
  u32 *err;
  u64 *item_cyc;  // per item: SM cycles from fetch to drained (NULL: not recorded)
  u64 *merge_cyc; // per tile: SM cycles of its split-tile merge (NULL: not recorded)
};

// Emits occupied slots of an open-addressing table, coalesced per warp, and
// resets them. Key k holds row urow[rank0 + k / LB], column k % LB (column k
// of row urow[rank0] when TL == 1).
__device__ void drain_hash(u64 *keys, double *vals, u64 nslots, u64 LB, u32 TL, u32 rank0, u32 nrows,
                           const u64 *__restrict__ urow, const Out &out, const Decode &dec, u32 *err,
                           u32 *s_wcnt, u64 *s_base, u64 *s_rows, u32 row_cap) {
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nwarps = blockDim.x >> 5;
  // the tile's rows, staged once (the barrier after the count publishes them)
  const bool cached = nrows <= row_cap;
  if (cached)
    for (u32 i = tid; i < nrows; i += blockDim.x) s_rows[i] = __ldg(&urow[rank0 + i]);
  const u64 spw = ((nslots + nwarps - 1) / nwarps + 31) & ~u64(31);
  const u64 s0 = min(nslots, u64(warp) * spw), s1 = min(nslots, s0 + spw);
  u32 c = 0;
  for (u64 s = s0 + lane; s < s1; s += 32) c += keys[s] != kEmptyKey ? 1u : 0u;
  c = __reduce_add_sync(kFull, c);
  if (lane == 0) s_wcnt[warp] = c;
  __syncthreads();
  if (tid == 0) {
    u32 run = 0;
    for (int w = 0; w < nwarps; w++) {
      const u32 x = s_wcnt[w];
      s_wcnt[w] = run;
      run += x;
    }
    *s_base = reserve(out, run, err);
  }
  __syncthreads();
  const u64 base = *s_base;
  const bool write = base != ~0ull;
  u64 run = write ? base + s_wcnt[warp] : 0;
  const u32 lt = (1u << lane) - 1u;
  for (u64 cs = s0; cs < s1; cs += 32) {
    const u64 s = cs + lane;
    const u64 key = s < s1 ? keys[s] : kEmptyKey;
    const bool occ = key != kEmptyKey;
    const u32 bal = __ballot_sync(kFull, occ);
    if (occ) {
      const double v = vals[s];
      u64 slot = 0, col = key;
      if (TL > 1) { slot = key / LB; col = key % LB; }
      const u64 row = cached ? s_rows[slot] : __ldg(&urow[rank0 + slot]);
      if (write) emit(out, dec, run + __popc(bal & lt), row, col, v);
    }
    if (s < s1) { keys[s] = kEmptyKey; vals[s] = 0.0; }
    run += __popc(bal);
  }
}

__device__ __forceinline__ void global_hash_add(u64 *gk, double *gv, u64 hs, u64 key, double v, u32 *err) {
  u64 h = u64(hash_slot(key)) & (hs - 1);
  for (u64 probe = 0; probe < hs; probe++) {
    const u64 cur = atomicCAS(reinterpret_cast<unsigned long long *>(&gk[h]), kEmptyKey, key);
    if (cur == kEmptyKey || cur == key) {
      atomicAdd(&gv[h], v);
      return;
    }
    h = (h + 1) & (hs - 1);
  }
  atomicOr(err, ERRB_HASH);
}

struct HashAdd {
  u64 *hk;
  double *hv;
  u32 hmask;
  u32 *err;
  double *priv;  // this warp's copy of the hot columns (keys [0, hot) when TL == 1)
  u32 *pmask;
  u32 hot;
  __device__ __forceinline__ void operator()(u64 key, double m, double x) const {
    if (key < hot) {
      fma_shared(&priv[key], m, x);
      atomicOr(&pmask[key >> 5], 1u << (key & 31));
      return;
    }
    insert(key, m, x);
  }
  __device__ __forceinline__ void insert(u64 key, double m, double x) const {
    u32 h = hash_slot(key) & hmask;
    for (u32 probe = 0; probe <= hmask; ++probe) {
      const u64 cur = *reinterpret_cast<volatile u64 *>(&hk[h]);
      if (cur == key) { fma_shared(&hv[h], m, x); return; }
      if (cur == kEmptyKey) {
        const u64 old = atomicCAS(reinterpret_cast<unsigned long long *>(&hk[h]), kEmptyKey, key);
        if (old == kEmptyKey || old == key) { fma_shared(&hv[h], m, x); return; }
      }
      h = (h + 1) & hmask;
    }
    atomicOr(err, ERRB_HASH);
  }
  __device__ __forceinline__ void batch(const u64 (&key)[kBatch], const double (&m)[kBatch],
                                        const double (&x)[kBatch], u32 valid, bool /*distinct*/,
                                        bool /*plain_priv*/, bool /*add_tile*/ = false) const {
#pragma unroll
    for (int k = 0; k < kBatch; k++)
      if ((valid >> k) & 1u) (*this)(key[k], m[k], x[k]);
  }
};

// kThreads 256 and 128 run three and six CTAs per SM (the shared-memory
// limits of the 4096- and 2048-slot tables): independent items overlap their
// barriers and memory latency.
template <class ColT, int kThreads>
__global__ void __launch_bounds__(kThreads, kThreads == 128 ? 6 : kThreads == 256 ? 3 : 1)
    k_contract_hash(HashArgs<ColT> a) {
  extern __shared__ __align__(16) unsigned char smem[];
  // layout: hk[slots] | hv[slots] | priv[nwarps*hot] | pmask[nwarps*hot/32]
  u64 *hk = reinterpret_cast<u64 *>(smem);
  double *hv = reinterpret_cast<double *>(hk + a.slots);
  const u32 nwarps = blockDim.x >> 5, warp = threadIdx.x >> 5, pw = a.hot / 32;
  double *priv = hv + a.slots;
  u32 *pmask = reinterpret_cast<u32 *>(priv + size_t(nwarps) * a.hot);
  __shared__ u32 s_item;
  __shared__ u32 s_wcnt[32];
  __shared__ u64 s_base;
  __shared__ HashPlan plan;
  const int tid = threadIdx.x, lane = tid & 31;
  for (u32 i = tid; i < a.slots; i += blockDim.x) { hk[i] = kEmptyKey; hv[i] = 0.0; }
  for (u32 i = tid; i < nwarps * a.hot; i += blockDim.x) priv[i] = 0.0;
  for (u32 i = tid; i < nwarps * pw; i += blockDim.x) pmask[i] = 0u;
  for (;;) {
    const long long c0 = clock64();
    if (tid == 0) s_item = atomicAdd(a.counter, 1u);
    __syncthreads();
    const u32 it = s_item;
    if (it >= a.nitems) break;
    const Item item = a.items[it];
    const u32 t = item.tile;
    const u64 np = item.p1 - item.p0;
    u32 hsl = 64;
    while (u64(hsl) < 2 * np && hsl < a.slots) hsl <<= 1;
    HashAdd add{hk, hv, hsl - 1, a.err, priv + size_t(warp) * a.hot, pmask + size_t(warp) * pw, a.hot};
    // chunks of the item's multiply-adds, each starting at a known entry
    build_item_plan(a.src.P, item.ea, item.eb, item.p0, item.p1, 256, plan);
    for (;;) {
      u32 c = 0;
      if (lane == 0) c = atomicAdd(&plan.next, 1u);
      c = __shfl_sync(kFull, c, 0);
      if (c >= plan.nchunk) break;
      const u64 q0 = item.p0 + u64(c) * plan.chunk, q1 = min(q0 + plan.chunk, item.p1);
      products_chunk<ColT, u64>(a.src, a.colB, item.ea, item.eb, plan.start[c], q0, q1, item.p0, item.p1, kNoSkip,
                                a.LB, add);
    }
    __syncthreads();
    if (a.hot) {  // per-warp hot columns -> the table (their keys were counted in np)
      for (u32 i = tid; i < a.hot; i += blockDim.x) {
        double sum = 0.0;
        u32 touched = 0;
        for (u32 w = 0; w < nwarps; w++) {
          sum += priv[w * a.hot + i];
          priv[w * a.hot + i] = 0.0;
          touched |= (pmask[w * pw + i / 32] >> (i & 31)) & 1u;
        }
        if (touched) add.insert(i, 1.0, sum);
      }
      __syncthreads();
      for (u32 i = tid; i < nwarps * pw; i += blockDim.x) pmask[i] = 0u;
      __syncthreads();
    }
    const int sidx = a.split_of_tile[t];
    if (sidx < 0) {
      drain_hash(hk, hv, hsl, a.LB, a.TL, a.tile_rank0[t], a.tile_nrows[t], a.urow, a.out, a.dec, a.err, s_wcnt,
                 &s_base, reinterpret_cast<u64 *>(plan.start), HashPlan::kRows);  // the plan is idle
    } else {
      const u64 off = a.hoff[t], hs = a.hsz[t];
      for (u32 s = tid; s < hsl; s += blockDim.x) {
        const u64 key = hk[s];
        if (key != kEmptyKey) {
          global_hash_add(a.gkeys + off, a.gvals + off, hs, key, hv[s], a.err);
          hk[s] = kEmptyKey;
          hv[s] = 0.0;
        }
      }
    }
    __syncthreads();
    if (a.item_cyc && tid == 0) a.item_cyc[it] = u64(clock64() - c0);
  }
}

template <class ColT>
__global__ void __launch_bounds__(kMergeThreads) k_merge_hash(HashArgs<ColT> a) {
  __shared__ u32 s_wcnt[32];
  __shared__ u64 s_base;
  __shared__ u64 s_rows[kRowCache];
  for (u32 s = blockIdx.x; s < a.nsplit; s += gridDim.x) {
    const long long c0 = clock64();
    const u32 t = a.split_tiles[s];
    const u64 off = a.hoff[t];
    drain_hash(a.gkeys + off, a.gvals + off, a.hsz[t], a.LB, a.TL, a.tile_rank0[t], a.tile_nrows[t], a.urow,
               a.out, a.dec, a.err, s_wcnt, &s_base, s_rows, kRowCache);
    __syncthreads();
    if (a.merge_cyc && threadIdx.x == 0) a.merge_cyc[t] = u64(clock64() - c0);
  }
}

// ---------------------------------------------- expand, sort, reduce ----
//
// Hash tiles (by default all of them; with a forced hash class only those
// with more multiply-adds than a table holds) are not
// accumulated in shared-memory tables: their products are expanded into
// (key, value) pairs, key = esc index x span + slot x LB + column (the esc
// index local to a group of tiles whose keys fit 32 bits), radix-sorted
// (stable, so equal keys keep the products' order) and reduced run by run:
// every output written once, no atomics.

struct EscArgs {
  const u32 *tiles;     // esc index -> tile
  const u64 *base;      // esc index -> first pair (counted from the first pair of all groups)
  u32 n;                // esc tiles
  u64 span, LB;         // key = s * span + slot * LB + col, span = rows * LB
  u64 rows;
  u64 lbm;              // magic_for(LB) (used with 32-bit keys)
  u64 rowsm;            // magic_for(rows) (used with 32-bit keys)
  u64 pair0;            // base[0]: this group's first pair
  void *keys;           // u32 when every key fits 32 bits, else u64
  u64 *vals;            // the products' bits (double), sorted along with the keys
  u64 total;            // pairs
};

// Flat over all expanded pairs: each lane writes eight consecutive pairs.
// The lane finds the esc tile and the A entry of its first pair by binary
// search (over the tiles' first pairs, then over the tile's product prefix)
// and advances both linearly from there. Hub rows have many A entries with
// short B segments, so a warp per entry would leave most lanes idle.
constexpr u32 kEscExpandPer = 8;  // a multiple of 4: vector stores

template <class ColT, class KeyT>
__global__ void __launch_bounds__(256) k_esc_expand(EscArgs a, const ProdSrc src, const ColT *__restrict__ colB,
                                                    const u32 *__restrict__ tile_abeg) {
  KeyT *keys = static_cast<KeyT *>(a.keys);
  const u64 nth = u64(gridDim.x) * blockDim.x;
  for (u64 q0 = (u64(blockIdx.x) * blockDim.x + threadIdx.x) * kEscExpandPer; q0 < a.total;
       q0 += nth * kEscExpandPer) {
    // esc tile: the last s with base[s] <= q0
    u32 lo = 0, hi = a.n;  // base[lo] <= q0 < base[hi] (base[n] = total), relative to pair0
    while (hi - lo > 1) {
      const u32 m = (lo + hi) >> 1;
      if (__ldg(&a.base[m]) - a.pair0 <= q0) lo = m;
      else hi = m;
    }
    u32 s = lo;
    u64 tb = __ldg(&a.base[s]) - a.pair0, tnext = s + 1 < a.n ? __ldg(&a.base[s + 1]) - a.pair0 : a.total;
    u32 t = a.tiles[s];
    u32 ea = tile_abeg[t], eb = tile_abeg[t + 1];
    u64 p0 = __ldg(&src.P[ea]);
    // A entry: the last e with P[e] <= p
    auto find_entry = [&](u64 p) {
      u32 l = ea, h = eb;  // P[l] <= p < P[h]
      while (h - l > 1) {
        const u32 m = (l + h) >> 1;
        if (__ldg(&src.P[m]) <= p) l = m;
        else h = m;
      }
      return l;
    };
    u32 e = find_entry(p0 + (q0 - tb));
    u64 pe = __ldg(&src.P[e]), pn = __ldg(&src.P[e + 1]);
    u32 sb = __ldg(&src.sbA[e]);
    double va = __ldg(&src.valA[e]);
    u64 kb = u64(s) * a.span + u64(__ldg(&src.slotA[e])) * a.LB;
    KeyT kk[kEscExpandPer];
    double vv[kEscExpandPer];
    const u32 cnt = u32(min(u64(kEscExpandPer), a.total - q0));
#pragma unroll
    for (u32 i = 0; i < kEscExpandPer; i++) {
      if (i < cnt) {
        const u64 q = q0 + i;
        if (q == tnext) {  // the next esc tile (every esc tile has pairs)
          s++;
          tb = tnext;
          tnext = s + 1 < a.n ? __ldg(&a.base[s + 1]) - a.pair0 : a.total;
          t = a.tiles[s];
          ea = tile_abeg[t];
          eb = tile_abeg[t + 1];
          p0 = __ldg(&src.P[ea]);
          e = ea;
          pe = p0;
          pn = __ldg(&src.P[e + 1]);
          sb = __ldg(&src.sbA[e]);
          va = __ldg(&src.valA[e]);
          kb = u64(s) * a.span + u64(__ldg(&src.slotA[e])) * a.LB;
        }
        const u64 p = p0 + (q - tb);
        while (p >= pn) {  // next A entry of the tile
          e++;
          pe = pn;
          pn = __ldg(&src.P[e + 1]);
          sb = __ldg(&src.sbA[e]);
          va = __ldg(&src.valA[e]);
          kb = u64(s) * a.span + u64(__ldg(&src.slotA[e])) * a.LB;
        }
        const u32 j = sb + u32(p - pe);
        kk[i] = KeyT(kb + u64(__ldg(&colB[j])));
        vv[i] = va * __ldg(&src.valB[j]);
      }
    }
    if (cnt == kEscExpandPer) {  // 32 or 64 aligned bytes of keys, 64 of values
      if (sizeof(KeyT) == 4) {
        uint4 *dk = reinterpret_cast<uint4 *>(keys + q0);
#pragma unroll
        for (u32 i = 0; i < kEscExpandPer / 4; i++)
          dk[i] = make_uint4(u32(kk[4 * i]), u32(kk[4 * i + 1]), u32(kk[4 * i + 2]), u32(kk[4 * i + 3]));
      } else {
        ulonglong2 *dk = reinterpret_cast<ulonglong2 *>(keys + q0);
#pragma unroll
        for (u32 i = 0; i < kEscExpandPer / 2; i++) dk[i] = make_ulonglong2(u64(kk[2 * i]), u64(kk[2 * i + 1]));
      }
      double2 *dv = reinterpret_cast<double2 *>(a.vals + q0);
#pragma unroll
      for (u32 i = 0; i < kEscExpandPer / 2; i++) dv[i] = make_double2(vv[2 * i], vv[2 * i + 1]);
    } else {
      for (u32 i = 0; i < cnt; i++) {
        keys[q0 + i] = kk[i];
        a.vals[q0 + i] = u64(__double_as_longlong(vv[i]));
      }
    }
  }
}

// The sorted pairs are read in chunks of 256 positions, one warp per chunk,
// eight consecutive positions per lane. A run of equal keys starts at a
// "head" (position 0 or a key change); runs are numbered in key order by the
// heads before them.
constexpr u32 kEscPer = 8;
constexpr u64 kEscChunk = 32 * kEscPer;

struct EscLane {  // one lane's eight positions
  u64 k[kEscPer];
  u32 heads;  // bit q: position q starts a run
};

template <class KeyT>
__device__ __forceinline__ EscLane esc_load_keys(const EscArgs &a, u64 c, u32 lane) {
  static_assert(sizeof(KeyT) == 4 || sizeof(KeyT) == 8, "32- or 64-bit keys");
  const KeyT *keys = static_cast<const KeyT *>(a.keys);
  EscLane L;
  const u64 p0 = c * kEscChunk + lane * kEscPer;
  if (p0 + kEscPer <= a.total) {  // 32 or 64 aligned bytes
    if (sizeof(KeyT) == 8) {
      const ulonglong2 *src = reinterpret_cast<const ulonglong2 *>(keys + p0);
#pragma unroll
      for (u32 q = 0; q < kEscPer / 2; q++) {
        const ulonglong2 w = src[q];
        L.k[2 * q] = w.x;
        L.k[2 * q + 1] = w.y;
      }
    } else {
      const uint4 *src = reinterpret_cast<const uint4 *>(keys + p0);
#pragma unroll
      for (u32 q = 0; q < kEscPer / 4; q++) {
        const uint4 w = src[q];
        L.k[4 * q] = w.x;
        L.k[4 * q + 1] = w.y;
        L.k[4 * q + 2] = w.z;
        L.k[4 * q + 3] = w.w;
      }
    }
  } else {
#pragma unroll
    for (u32 q = 0; q < kEscPer; q++) L.k[q] = p0 + q < a.total ? u64(keys[p0 + q]) : ~0ull;
  }
  u64 prev = __shfl_up_sync(kFull, L.k[kEscPer - 1], 1);
  if (lane == 0 && c > 0) prev = keys[c * kEscChunk - 1];
  L.heads = 0;
#pragma unroll
  for (u32 q = 0; q < kEscPer; q++) {
    const u64 pk = q ? L.k[q - 1] : prev;
    if (p0 + q < a.total && (p0 + q == 0 || L.k[q] != pk)) L.heads |= 1u << q;
  }
  return L;
}

// Heads per chunk (the runs' numbering, after an exclusive scan).
template <class KeyT>
__global__ void __launch_bounds__(256) k_esc_count(EscArgs a, u32 *__restrict__ chunk_heads) {
  const u32 lane = threadIdx.x & 31;
  const u64 nchunks = (a.total + kEscChunk - 1) / kEscChunk;
  const u64 nw = (u64(gridDim.x) * blockDim.x) >> 5;
  for (u64 c = (u64(blockIdx.x) * blockDim.x + threadIdx.x) >> 5; c < nchunks; c += nw) {
    const EscLane L = esc_load_keys<KeyT>(a, c, lane);
    u32 n = __popc(L.heads);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) n += __shfl_xor_sync(kFull, n, o);
    if (lane == 0) chunk_heads[c] = n;
  }
}

// First pair of each group of G expanded tiles.
__global__ void k_esc_group_starts(const u64 *__restrict__ base, u32 G, u32 ngroups, u64 *__restrict__ start) {
  for (u32 g = blockIdx.x * blockDim.x + threadIdx.x; g < ngroups; g += gridDim.x * blockDim.x)
    start[g] = base[u64(g) * G];
}

__global__ void k_esc_reserve(const Out out, const u32 *__restrict__ nruns, u64 *__restrict__ base, u32 *err) {
  if (threadIdx.x == 0 && blockIdx.x == 0) *base = reserve(out, *nruns, err);
}

// Output row and column of a key. key / LB = s * rows + slot names the row;
// consecutive runs mostly share it, so the lane keeps the last one.
struct EscRowCache {
  u64 q = ~0ull, row = 0;
};

template <class KeyT>
__device__ __forceinline__ void esc_emit(const EscArgs &a, const u32 *__restrict__ tile_rank0,
                                         const u64 *__restrict__ urow, const Out &out, const Decode &dec,
                                         EscRowCache &rc, u64 idx, u64 key, double v) {
  u64 q;
  if (sizeof(KeyT) == 4) q = div_magic(u32(key), a.lbm);  // exact: key, LB < 2^32
  else q = key / a.LB;
  const u64 col = key - q * a.LB;
  if (q != rc.q) {
    const u64 s = sizeof(KeyT) == 4 ? u64(div_magic(u32(q), a.rowsm)) : q / a.rows, slot = q - s * a.rows;
    rc.q = q;
    rc.row = __ldg(&urow[tile_rank0[a.tiles[s]] + slot]);
  }
  emit(out, dec, idx, rc.row, col, v);
}

// Each run is summed and emitted (at base + its number) by the lane holding
// its head: its values in that lane in order, then the following lanes'
// values up to the next head (a segmented suffix sum over the lanes), then,
// for the chunk's last run, the positions after the chunk up to the next key
// change, found by a galloping search over the sorted keys and summed by the
// warp. A chunk's positions before its first head belong to an earlier run.
template <class KeyT>
__global__ void __launch_bounds__(256) k_esc_reduce(EscArgs a, const u32 *__restrict__ chunk_off,
                                                    const u64 *__restrict__ base_p,
                                                    const u32 *__restrict__ tile_rank0,
                                                    const u64 *__restrict__ urow, const Out out, const Decode dec) {
  // the chunk's finished runs, staged so that the warp emits them together
  __shared__ u64 s_key[8][kEscChunk];
  __shared__ double s_val[8][kEscChunk];
  const u64 base = *base_p;
  if (base == ~0ull) return;  // over capacity: counted by the cursor, retried by the host
  const u32 lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  u64 *sk = s_key[wib];
  double *sv = s_val[wib];
  EscRowCache rc;
  const u64 nchunks = (a.total + kEscChunk - 1) / kEscChunk;
  const u64 nw = (u64(gridDim.x) * blockDim.x) >> 5;
  for (u64 c = (u64(blockIdx.x) * blockDim.x + threadIdx.x) >> 5; c < nchunks; c += nw) {
    const EscLane L = esc_load_keys<KeyT>(a, c, lane);
    const u64 p0 = c * kEscChunk + lane * kEscPer;
    double v[kEscPer];
    if (p0 + kEscPer <= a.total) {
      const double2 *src = reinterpret_cast<const double2 *>(a.vals + p0);
#pragma unroll
      for (u32 q = 0; q < kEscPer / 2; q++) {
        const double2 w = src[q];
        v[2 * q] = w.x;
        v[2 * q + 1] = w.y;
      }
    } else {
#pragma unroll
      for (u32 q = 0; q < kEscPer; q++)
        v[q] = p0 + q < a.total ? __longlong_as_double((long long)a.vals[p0 + q]) : 0.0;
    }
    const u32 nh = __popc(L.heads);
    u32 incl = nh;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const u32 t = __shfl_up_sync(kFull, incl, o);
      if (lane >= o) incl += t;
    }
    const u32 nruns = __shfl_sync(kFull, incl, 31);  // runs starting in the chunk
    u32 run = incl - nh;                             // the lane's first run, within the chunk
    // In-lane runs; the lane's last run stays open.
    double lead = 0.0, acc = 0.0;
    u64 key = 0;
    bool open = false;
#pragma unroll
    for (u32 q = 0; q < kEscPer; q++) {
      if ((L.heads >> q) & 1u) {
        if (open) {
          sk[run] = key;
          sv[run] = acc;
          run++;
        }
        open = true;
        key = L.k[q];
        acc = v[q];
      } else if (open) {
        acc += v[q];
      } else {
        lead += v[q];
      }
    }
    // Suffix over lanes: t = this lane's lead plus, while no head stops it,
    // the leads of the lanes after it.
    double t = lead;
    bool f = nh > 0;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const double to = __shfl_down_sync(kFull, t, o);
      const bool fo = __shfl_down_sync(kFull, f ? 1u : 0u, o) != 0;
      if (lane + o < 32) {
        if (!f) t += to;
        f = f || fo;
      }
    }
    double cont = __shfl_down_sync(kFull, t, 1);
    bool stops = __shfl_down_sync(kFull, f ? 1u : 0u, 1) != 0;
    if (lane == 31) {
      cont = 0.0;
      stops = false;
    }
    if (open) acc += cont;
    // The chunk's last run may continue past the chunk.
    const bool walk = open && !stops;
    const u32 wm = __ballot_sync(kFull, walk);
    if (wm) {
      const u32 wl = __ffs(wm) - 1;
      const u64 k0 = __shfl_sync(kFull, key, wl);
      const u64 q0 = (c + 1) * kEscChunk;
      u64 end = q0;  // first position after the run
      if (lane == wl) {
        const KeyT *keys = static_cast<const KeyT *>(a.keys);
        u64 step = 1, lo = q0;  // keys[lo - 1] == k0 (or lo == q0)
        while (lo < a.total && keys[lo] == k0) {
          const u64 hi = min(a.total, lo + step);
          if (keys[hi - 1] == k0) {
            lo = hi;
            step <<= 1;
          } else {
            u64 l = lo, h = hi - 1;  // keys[l] == k0, keys[h] != k0
            while (h - l > 1) {
              const u64 m = l + (h - l) / 2;
              if (keys[m] == k0) l = m;
              else h = m;
            }
            lo = h;
            break;
          }
        }
        end = lo;
      }
      end = __shfl_sync(kFull, end, wl);
      double sum = 0.0;
      for (u64 i = q0 + lane; i < end; i += 32) sum += __longlong_as_double((long long)a.vals[i]);
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) sum += __shfl_xor_sync(kFull, sum, o);
      if (lane == wl) acc += sum;
    }
    if (open) {
      sk[run] = key;
      sv[run] = acc;
    }
    __syncwarp();
    const u64 first = base + chunk_off[c];
    for (u32 r = lane; r < nruns; r += 32) esc_emit<KeyT>(a, tile_rank0, urow, out, dec, rc, first + r, sk[r], sv[r]);
    __syncwarp();
  }
}

// ------------------------------- expanded pairs reduced in shared memory ----
//
// Instead of being sorted, the expanded pairs are reduced in shared memory:
//  * small tiles (at most small_max pairs): windows of kBinWindow
//    positions over this region, each taking the tiles that start in it
//    (fewer than kBinWindow + small_max positions and at most
//    kBinWindow / 8 + 1 tiles, one contiguous range), are reduced in
//    shared-memory hash tables. Their pairs are written tile by tile, each
//    tile padded to a multiple of eight pairs (padding keys are kBinEmpty);
//    a small tile's key is its rank among the window's tiles x span + its
//    local key (slot x LB + column);
//  * the large tiles (hub rows) are expanded straight into blocks of
//    kBinWidth consecutive local keys (slot x LB + column), keyed by the
//    local key alone: every chunk of kBinChunk of a tile's products counts
//    its pairs per block, one exclusive scan over (tile, block, chunk) gives
//    every chunk its positions, and the chunk computes its products again
//    and writes each pair there. A block with more than kBinDenseMin pairs
//    is reduced in a dense kBinWidth-entry accumulator (untouched entries
//    hold -0.0), runs of consecutive sparser blocks together in one hash
//    table. Every first update of a slot appends it to a list of occupied
//    slots, from which the outputs are written.
// Every reduced window or block reserves its outputs with one atomic and
// writes them. Every pair is written once and read once; keys never need
// more than 32 bits, so every expanded tile goes through one set of launches.

constexpr u32 kBinBits = 13;
constexpr u32 kBinWidth = 1u << kBinBits;  // local keys per block: 8192 doubles, 64 KB
constexpr u32 kBinMaxBlocks = 256;         // blocks per tile: spans up to 2^21 keys
constexpr u32 kBinChunk = 4096;            // products per partition chunk (a multiple of 8)
constexpr u32 kBinWindow = 2048;           // small-tile positions per window
constexpr u32 kBinSmallMax = 4096;         // default (and largest) small tile; a multiple of 8
constexpr u32 kBinDenseMin = 2048;         // a block with more pairs is reduced densely
constexpr u32 kBinHashPairs = 4096;        // sparse blocks merged up to this many pairs
constexpr u32 kBinSlots = 8192;            // hash slots: > 4/3 x (kBinWindow + kBinSmallMax - 1)
constexpr int kBinThreads = 512;
constexpr u32 kBinEmpty = 0xFFFFFFFFu;     // padding / free slot (keys stay below 257 x 2^21)
// values, keys, and the list of occupied slots
constexpr size_t kBinSmem = size_t(kBinSlots) * (sizeof(double) + sizeof(u32) + sizeof(uint16_t));
constexpr u32 kBinPer = 8;                 // the tiles' padding unit
constexpr int kBinIlp = 4;                 // pairs per thread in flight in the reductions

struct BinJob {  // a dense block, or a run of sparse blocks, of one large tile
  u32 s;         // esc index
  uint16_t b0, b1;  // blocks [b0, b1)
};

struct BinArgs {
  u32 n;                  // expanded tiles
  u32 small_max;          // tiles with more pairs are large
  u32 nb;                 // blocks per tile: ceil(span / kBinWidth)
  u32 span, LB, rows;     // local key = slot x LB + column < span = rows x LB
  u64 spanm, lbm;         // magic_for(span), magic_for(LB)
  const u32 *tiles;       // esc index -> tile
  const u64 *base;        // esc index -> first pair (base[0] = 0)
  u64 total;              // pairs
  u32 *keys;              // the small tiles' pairs, padded
  u64 *vals;
  u32 *nch;               // per esc tile: partition chunks if large, else 0
  u32 *spp, *chpre, *srk; // exclusive scans over the tiles (n + 1 entries each) of the small tiles'
                          // padded pairs, of nch, and of the small tiles' count
  u32 *small_list;        // small tiles in esc order
  u32 *chunk_tile;        // chunk -> esc index
  u32 *first;             // window -> first esc index s with spp[s] >= window start
  u64 max_windows;
  u32 *hist;              // pairs per (tile, block, chunk), at nb * chpre[s] + b * nch[s] + c
  u32 *hpre;              // exclusive scan of hist, hist_len + 1 entries
  u64 hist_len;
  u32 *bkeys;             // the large tiles' pairs, partitioned
  u64 *bvals;
  BinJob *jobs;
  u32 *njobs;             // large-tile jobs
  u32 *work;              // the reduction's job counter
};

__device__ __forceinline__ u64 bin_tile_pairs(const BinArgs &b, u32 s) {
  return (s + 1 < b.n ? __ldg(&b.base[s + 1]) : b.total) - __ldg(&b.base[s]);
}

// Every tile's place in the small region (spp), its partition chunks
// (chpre) and the small tiles' ranks (srk), as exclusive scans over the
// tiles: each CTA scans 1024 tiles and writes its totals (k_bin_prep), one
// CTA scans the totals (k_bin_prep_totals), and every tile adds its CTA's
// offset (k_bin_prep_add).
constexpr int kPrepThreads = 1024;
constexpr int kPrepVals = 3;
__global__ void __launch_bounds__(kPrepThreads) k_bin_prep(BinArgs b, u32 *__restrict__ bsum) {
  __shared__ u32 wsum[kPrepVals][kPrepThreads / 32];
  const u32 lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const u32 s = blockIdx.x * kPrepThreads + threadIdx.x;
  u32 v[kPrepVals] = {0, 0, 0};  // padded pairs if small; chunks if large; 1 if small
  if (s < b.n) {
    const u32 p = u32(bin_tile_pairs(b, s));
    const bool large = p > b.small_max;
    v[0] = large ? 0u : (p + kBinPer - 1) / kBinPer * kBinPer;
    v[1] = large ? (p + kBinChunk - 1) / kBinChunk : 0u;
    v[2] = large ? 0u : 1u;
    b.nch[s] = v[1];
  }
  u32 incl[kPrepVals];
#pragma unroll
  for (int k = 0; k < kPrepVals; k++) {
    incl[k] = warp_incl_u32(v[k]);
    if (lane == 31) wsum[k][warp] = incl[k];
  }
  __syncthreads();
  if (warp < kPrepVals) {  // warp k scans the warp sums of value k
    const u32 x = wsum[warp][lane], xi = warp_incl_u32(x);
    wsum[warp][lane] = xi - x;
    if (lane == 31) bsum[u64(warp) * gridDim.x + blockIdx.x] = xi;
  }
  __syncthreads();
  u32 *dst[kPrepVals] = {b.spp, b.chpre, b.srk};
#pragma unroll
  for (int k = 0; k < kPrepVals; k++)
    if (s < b.n) dst[k][s] = wsum[k][warp] + incl[k] - v[k];
}

// Exclusive scan of the CTA totals in place (nblk per value); the grand
// totals go to entry n of each scan.
__global__ void __launch_bounds__(kPrepThreads) k_bin_prep_totals(BinArgs b, u32 *__restrict__ bsum, u32 nblk) {
  __shared__ u32 wsum[kPrepThreads / 32];
  __shared__ u32 carry;
  const u32 lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  u32 *dst[kPrepVals] = {b.spp, b.chpre, b.srk};
  for (int k = 0; k < kPrepVals; k++) {
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    u32 *t = bsum + u64(k) * nblk;
    for (u32 c0 = 0; c0 < nblk; c0 += kPrepThreads) {
      const u32 i = c0 + threadIdx.x;
      const u32 v = i < nblk ? t[i] : 0u, incl = warp_incl_u32(v);
      if (lane == 31) wsum[warp] = incl;
      __syncthreads();
      if (warp == 0) {
        const u32 x = wsum[lane], xi = warp_incl_u32(x);
        wsum[lane] = xi - x;
      }
      __syncthreads();
      if (i < nblk) t[i] = carry + wsum[warp] + incl - v;
      __syncthreads();
      if (threadIdx.x == kPrepThreads - 1) carry += wsum[warp] + incl;
      __syncthreads();
    }
    if (threadIdx.x == 0) dst[k][b.n] = carry;
    __syncthreads();
  }
}

__global__ void __launch_bounds__(kPrepThreads) k_bin_prep_add(BinArgs b, const u32 *__restrict__ bsum) {
  const u32 s = blockIdx.x * kPrepThreads + threadIdx.x;
  if (s >= b.n) return;
  u32 *dst[kPrepVals] = {b.spp, b.chpre, b.srk};
#pragma unroll
  for (int k = 0; k < kPrepVals; k++) dst[k][s] += bsum[u64(k) * gridDim.x + blockIdx.x];
}

// chunk_tile for the large tiles' chunks; small_list; first[w] = the first
// esc index s with spp[s] >= w * kBinWindow (n when none), for every window
// and one past.
__global__ void k_bin_index(BinArgs b) {
  const u64 i0 = u64(blockIdx.x) * blockDim.x + threadIdx.x, nth = u64(gridDim.x) * blockDim.x;
  for (u64 s = i0; s < b.n; s += nth) {
    const u32 c0 = b.chpre[s], nc = b.nch[s];
    for (u32 c = 0; c < nc; c++) b.chunk_tile[c0 + c] = u32(s);
    if (nc == 0) b.small_list[b.srk[s]] = u32(s);
  }
  const u64 nwin = (u64(b.spp[b.n]) + kBinWindow - 1) / kBinWindow;
  for (u64 w = i0; w <= nwin && w < b.max_windows; w += nth) {
    const u64 x = w * kBinWindow;
    u32 lo = 0, hi = b.n;  // the first s in [lo, hi] with spp[s] >= x (spp[n] = the region's size)
    while (lo < hi) {
      const u32 m = (lo + hi) >> 1;
      if (u64(b.spp[m]) >= x) hi = m;
      else lo = m + 1;
    }
    b.first[w] = lo;
  }
}

// The A entry holding product p of a tile whose entries are [ea, eb).
__device__ __forceinline__ u32 bin_entry_of(const u64 *__restrict__ P, u32 ea, u32 eb, u64 p) {
  u32 l = ea, h = eb;  // P[l] <= p < P[h]
  while (h - l > 1) {
    const u32 m = (l + h) >> 1;
    if (__ldg(&P[m]) <= p) l = m;
    else h = m;
  }
  return l;
}

// A lane's walk over the products of one tile, forward only.
struct BinWalk {
  u32 e = kNoEntry, sb = 0, kb = 0;
  u64 pe = 0, pn = 0;
  double va = 0.0;
  __device__ __forceinline__ void load(const ProdSrc &src, u32 kt, u32 LB) {
    pe = __ldg(&src.P[e]);
    pn = __ldg(&src.P[e + 1]);
    sb = __ldg(&src.sbA[e]);
    va = __ldg(&src.valA[e]);
    kb = kt + __ldg(&src.slotA[e]) * LB;
  }
  // key kb + column and value of product p (p at or after the current entry's
  // first). Entries it passes over cost one load each (their ends); the
  // entry it stops at loads the rest once.
  template <bool kVal, class ColT>
  __device__ __forceinline__ void at(const ProdSrc &src, const ColT *__restrict__ colB, u32 kt, u32 LB, u64 p,
                                     u32 &key, double &v) {
    if (p >= pn) {
      do {
        e++;
        pe = pn;
        pn = __ldg(&src.P[e + 1]);
      } while (p >= pn);
      sb = __ldg(&src.sbA[e]);
      if (kVal) va = __ldg(&src.valA[e]);
      kb = kt + __ldg(&src.slotA[e]) * LB;
    }
    const u32 j = sb + u32(p - pe);
    key = kb + u32(__ldg(&colB[j]));
    v = kVal ? va * __ldg(&src.valB[j]) : 0.0;
  }
};

// Expansion of the small tiles into their padded region. A warp takes 256
// consecutive positions, lane l the positions l, l + 32, ...: lanes next to
// each other read B entries next to each other (one A entry's segment) and
// store next to each other. The warp finds the tile of its first position
// by binary search; lanes walk forward from there.
template <class ColT>
__global__ void __launch_bounds__(256) k_bin_expand(BinArgs b, const ProdSrc src, const ColT *__restrict__ colB,
                                                    const u32 *__restrict__ tile_abeg) {
  const u64 ptot = b.spp[b.n];
  const u32 lane = threadIdx.x & 31;
  const u64 nwarps = (u64(gridDim.x) * blockDim.x) >> 5;
  for (u64 c = (u64(blockIdx.x) * blockDim.x + threadIdx.x) >> 5; c * 256 < ptot; c += nwarps) {
    // the last s with spp[s] <= c * 256: a small tile (large tiles tie with the small tile after them)
    u32 s;
    {
      u32 lo = 0, hi = b.n;  // spp[lo] <= x < spp[hi] (spp[n] = ptot)
      const u64 x = c * 256;
      while (hi - lo > 1) {
        const u32 m = (lo + hi) >> 1;
        if (u64(__ldg(&b.spp[m])) <= x) lo = m;
        else hi = m;
      }
      s = lo;
    }
    u64 tb = 0, te = 0, cnt = 0, p0 = 0;  // the tile: padded [tb, te), pairs, first product
    u32 ea = 0, eb = 0, kt = 0;           // its A entries; its key offset (rank in the window x span)
    BinWalk wk;
    bool fresh = true;
#pragma unroll 1
    for (u32 i = 0; i < 8; i++) {
      const u64 q = c * 256 + 32 * i + lane;
      if (q >= ptot) break;
      if (fresh || q >= te) {  // this lane's next tile
        while (u64(__ldg(&b.spp[s + 1])) <= q) s++;
        fresh = false;
        tb = __ldg(&b.spp[s]);
        te = __ldg(&b.spp[s + 1]);
        cnt = bin_tile_pairs(b, s);
        kt = (__ldg(&b.srk[s]) - __ldg(&b.srk[__ldg(&b.first[u32(tb / kBinWindow)])])) * b.span;
        const u32 t = b.tiles[s];
        ea = tile_abeg[t];
        eb = tile_abeg[t + 1];
        p0 = __ldg(&src.P[ea]);
        wk.e = kNoEntry;
      }
      const u64 o = q - tb;
      u32 key = kBinEmpty;
      double v = 0.0;
      if (o < cnt) {
        const u64 p = p0 + o;
        if (wk.e == kNoEntry) {
          wk.e = bin_entry_of(src.P, ea, eb, p);
          wk.load(src, kt, b.LB);
        }
        wk.at<true>(src, colB, kt, b.LB, p, key, v);
      }
      b.keys[q] = key;
      b.vals[q] = u64(__double_as_longlong(v));
    }
  }
}

// Chunk g of the large tiles: tile s, chunk c, its products [p0 + o0, p0 + o1)
// (tile offsets). Warp w of the CTA takes offsets o0 + 512 w + [0, 512),
// lane l every 32nd from l; f(valid, local key, value) is called by every
// lane of the warp at each step.
template <class ColT, bool kVal, class F>
__device__ __forceinline__ void bin_chunk_pairs(const BinArgs &b, const ProdSrc &src, const ColT *__restrict__ colB,
                                                const u32 *__restrict__ tile_abeg, u32 s, u32 c, F &&f) {
  const u32 lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const u64 cnt = bin_tile_pairs(b, s);
  const u64 w0 = u64(c) * kBinChunk + u64(warp) * (kBinChunk / 8);
  if (w0 >= cnt) return;  // warp-uniform
  const u64 w1 = min(cnt, w0 + kBinChunk / 8);
  const u32 t = b.tiles[s];
  const u32 ea = tile_abeg[t], eb = tile_abeg[t + 1];
  const u64 p0 = __ldg(&src.P[ea]);
  BinWalk wk;
  wk.e = bin_entry_of(src.P, ea, eb, p0 + w0);  // the warp's first product; lanes walk on from it
  wk.load(src, 0u, b.LB);
  for (u64 o = w0 + lane; o - lane < w1; o += 32) {
    const bool valid = o < w1;
    u32 key = kBinEmpty;
    double v = 0.0;
    if (valid) wk.at<kVal>(src, colB, 0u, b.LB, p0 + o, key, v);
    f(valid, key, v);
  }
}

// Pairs per block of each chunk of the large tiles: a shared histogram per
// warp, summed at the end (faster than combining equal blocks across lanes).
template <class ColT>
__global__ void __launch_bounds__(256) k_bin_count(BinArgs b, const ProdSrc src, const ColT *__restrict__ colB,
                                                   const u32 *__restrict__ tile_abeg) {
  __shared__ u32 h[8][kBinMaxBlocks];  // one histogram per warp (256 threads)
  const u32 nchunks = b.chpre[b.n];
  const u32 warp = threadIdx.x >> 5;
  for (u32 g = blockIdx.x; g < nchunks; g += gridDim.x) {
    for (u32 i = threadIdx.x; i < 8 * kBinMaxBlocks; i += blockDim.x) (&h[0][0])[i] = 0;
    __syncthreads();
    const u32 s = b.chunk_tile[g], c = g - b.chpre[s];
    bin_chunk_pairs<ColT, false>(b, src, colB, tile_abeg, s, c, [&](bool valid, u32 key, double) {
      if (valid) atomicAdd(&h[warp][key >> kBinBits], 1u);
    });
    __syncthreads();
    const u64 r = u64(b.nb) * b.chpre[s] + c;
    const u32 nc = b.nch[s];
    for (u32 i = threadIdx.x; i < b.nb; i += blockDim.x) {
      u32 t = 0;
#pragma unroll
      for (int w = 0; w < 8; w++) t += h[w][i];
      b.hist[r + u64(i) * nc] = t;
    }
    __syncthreads();
  }
}

// Each chunk's pairs, computed again, to their block's positions; lanes of
// one block take consecutive positions with one shared atomic (measured
// faster here than an atomic per lane, unlike the counting pass).
template <class ColT>
__global__ void __launch_bounds__(256) k_bin_place(BinArgs b, const ProdSrc src, const ColT *__restrict__ colB,
                                                   const u32 *__restrict__ tile_abeg) {
  __shared__ u32 cur[kBinMaxBlocks];
  const u32 nchunks = b.chpre[b.n];
  const u32 lane = threadIdx.x & 31;
  for (u32 g = blockIdx.x; g < nchunks; g += gridDim.x) {
    const u32 s = b.chunk_tile[g], c = g - b.chpre[s];
    const u64 r = u64(b.nb) * b.chpre[s] + c;
    const u32 nc = b.nch[s];
    for (u32 i = threadIdx.x; i < b.nb; i += blockDim.x) cur[i] = b.hpre[r + u64(i) * nc];
    __syncthreads();
    bin_chunk_pairs<ColT, true>(b, src, colB, tile_abeg, s, c, [&](bool valid, u32 key, double v) {
      const u32 bin = valid ? key >> kBinBits : kBinMaxBlocks;
      const u32 peers = __match_any_sync(kFull, bin);
      const u32 leader = __ffs(peers) - 1;
      u32 pos = 0;
      if (lane == leader && bin < kBinMaxBlocks) pos = atomicAdd(&cur[bin], u32(__popc(peers)));
      pos = __shfl_sync(kFull, pos, leader) + __popc(peers & ((1u << lane) - 1u));
      if (valid) {
        b.bkeys[pos] = key;
        b.bvals[pos] = u64(__double_as_longlong(v));
      }
    });
    __syncthreads();
  }
}

// Jobs of each large tile: every block with more than kBinDenseMin pairs
// alone (dense), runs of consecutive sparser blocks up to kBinHashPairs pairs
// together (hash).
__global__ void k_bin_jobs(BinArgs b) {
  for (u32 s = blockIdx.x * blockDim.x + threadIdx.x; s < b.n; s += gridDim.x * blockDim.x) {
    const u32 nc = b.nch[s];
    if (nc == 0) continue;
    const u64 r = u64(b.nb) * b.chpre[s];
    u32 run0 = 0, runp = 0;
    auto push = [&](u32 b0, u32 b1) {
      const u32 j = atomicAdd(b.njobs, 1u);
      b.jobs[j] = BinJob{s, uint16_t(b0), uint16_t(b1)};
    };
    u32 prev = b.hpre[r];
    for (u32 blk = 0; blk < b.nb; blk++) {
      const u32 next = b.hpre[r + u64(blk + 1) * nc];  // blk + 1 == nb: the next tile's (or the end's) start
      const u32 cnt = next - prev;
      prev = next;
      if (cnt > kBinDenseMin) {
        if (runp > 0) push(run0, blk);
        push(blk, blk + 1);
        run0 = blk + 1;
        runp = 0;
      } else if (runp + cnt > kBinHashPairs) {
        push(run0, blk);
        run0 = blk;
        runp = cnt;
      } else {
        runp += cnt;
      }
    }
    if (runp > 0) push(run0, b.nb);
  }
}

// Lanes holding the same key (hub columns reach a block or a window from
// many A entries at once) are summed first; returns true for the lane that
// keeps the key with the group's sum in *v. Every lane of the warp calls it
// (kBinEmpty for no pair).
__device__ __forceinline__ bool bin_aggregate(u32 key, double *v) {
  const u32 lane = threadIdx.x & 31;
  const u32 peers = __match_any_sync(kFull, key);
  if (key == kBinEmpty) return false;
  if (peers == (1u << lane)) return true;
  const u32 leader = __ffs(peers) - 1;
  double sum = *v;
  for (u32 rest = peers & (peers - 1); rest; rest &= rest - 1) {
    const double y = __shfl_sync(peers, *v, __ffs(rest) - 1);
    if (lane == leader) sum += y;
  }
  *v = sum;
  return lane == leader;
}

// Shared-memory hash insert: linear probing from a multiplicative hash, the
// table never full (slots > pairs); a slot's key is read before it is
// claimed. Returns true when this call claimed the slot (*slot).
__device__ __forceinline__ bool bin_insert(u32 *tk, double *tv, u32 mask, u32 lg, u32 key, double v, u32 *slot) {
  u32 h = (key * 2654435761u) >> (32 - lg);
  bool claimed = false;
  for (;;) {
    u32 cur = reinterpret_cast<volatile u32 *>(tk)[h];
    if (cur == kBinEmpty) {
      cur = atomicCAS(&tk[h], kBinEmpty, key);
      claimed = cur == kBinEmpty;
    }
    if (cur == kBinEmpty || cur == key) break;
    h = (h + 1) & mask;
  }
  atomicAdd(&tv[h], v);  // under contention the built-in add beats a compare-and-swap loop
  *slot = h;
  return claimed;
}

// Appends the slots this warp's lanes claimed to the CTA's list of occupied
// slots (one shared atomic per warp). Every lane of the warp calls it.
__device__ __forceinline__ void bin_list_append(bool claimed, u32 slot, uint16_t *list, u32 *nocc) {
  const u32 m = __ballot_sync(kFull, claimed);
  if (!m) return;
  const u32 lane = threadIdx.x & 31, leader = __ffs(m) - 1;
  u32 base = 0;
  if (lane == leader) base = atomicAdd(nocc, u32(__popc(m)));
  base = __shfl_sync(kFull, base, leader);
  if (claimed) list[base + __popc(m & ((1u << lane) - 1u))] = uint16_t(slot);
}

// Output row and column of a reduced key: a window's key is the tile's rank
// in the window x span + the local key, a large tile's key the local key.
struct BinWho {
  bool window;
  u32 s;      // large tile: its esc index
  u32 rank0;  // window: the rank of its first small tile
};

struct BinRowCache {
  u32 s = kBinEmpty, slot = 0;
  u64 row = 0;
};

__device__ __forceinline__ void bin_emit_one(const BinArgs &b, const u32 *__restrict__ tile_rank0,
                                             const u64 *__restrict__ urow, const Out &out, const Decode &dec,
                                             const BinWho &who, BinRowCache &rc, u64 idx, u32 key, double v) {
  u32 s = who.s, loc = key;
  if (who.window) {
    const u32 r = div_magic(key, b.spanm);
    loc = key - r * b.span;
    s = __ldg(&b.small_list[who.rank0 + r]);
  }
  const u32 slot = b.rows > 1 ? div_magic(loc, b.lbm) : 0u;
  const u32 col = loc - slot * b.LB;
  if (s != rc.s || slot != rc.slot) {
    rc.s = s;
    rc.slot = slot;
    rc.row = __ldg(&urow[tile_rank0[b.tiles[s]] + slot]);
  }
  emit(out, dec, idx, rc.row, col, v);
}

// Emits the nocc slots of the list (key tk[slot], or k0 + slot for a dense
// block; value tv[slot]) with one reservation for the CTA: consecutive
// threads write consecutive outputs.
__device__ __forceinline__ void bin_emit(const BinArgs &b, const u32 *__restrict__ tile_rank0,
                                         const u64 *__restrict__ urow, const Out &out, const Decode &dec, u32 *err,
                                         const BinWho &who, const uint16_t *list, u32 nocc, const u32 *tk,
                                         const double *tv, bool dense, u32 k0, u64 *s_base) {
  if (threadIdx.x == 0) *s_base = reserve(out, nocc, err);
  __syncthreads();
  const u64 base = *s_base;
  if (base != ~0ull) {  // else over capacity: counted by the cursor, retried by the host
    BinRowCache rc;
    for (u32 i = threadIdx.x; i < nocc; i += blockDim.x) {
      const u32 slot = list[i];
      bin_emit_one(b, tile_rank0, urow, out, dec, who, rc, base + i, dense ? k0 + slot : tk[slot], tv[slot]);
    }
  }
  __syncthreads();
}

// Hash-reduces positions [lo, hi) of (keys, vals), padding skipped.
__device__ __forceinline__ void bin_hash(const u32 *__restrict__ keys, const u64 *__restrict__ vals, u64 lo, u64 hi,
                                         u32 *tk, double *tv, uint16_t *list, u32 *nocc) {
  const u32 np = u32(hi - lo);
  u32 lg = 5;
  while ((1u << lg) < np + np / 3 + 1) lg++;
  const u32 slots = 1u << lg;
  for (u32 i = threadIdx.x; i < slots; i += blockDim.x) {
    tk[i] = kBinEmpty;
    tv[i] = 0.0;
  }
  if (threadIdx.x == 0) *nocc = 0;
  __syncthreads();
  for (u64 q0 = lo; q0 < hi; q0 += u64(blockDim.x) * kBinIlp) {  // the same trip count in every lane
    u32 k[kBinIlp];
    double v[kBinIlp];
#pragma unroll
    for (int i = 0; i < kBinIlp; i++) {  // every load in flight first
      const u64 q = q0 + u64(i) * blockDim.x + threadIdx.x;
      k[i] = q < hi ? keys[q] : kBinEmpty;
      v[i] = q < hi ? __longlong_as_double((long long)vals[q]) : 0.0;
    }
#pragma unroll
    for (int i = 0; i < kBinIlp; i++) {
      u32 slot = 0;
      const bool claimed = bin_aggregate(k[i], &v[i]) && bin_insert(tk, tv, slots - 1, lg, k[i], v[i], &slot);
      bin_list_append(claimed, slot, list, nocc);
    }
  }
  __syncthreads();
}

// Persistent CTAs take jobs from a counter (the next one fetched while the
// current one runs): first the large tiles' jobs (dense blocks and runs of
// sparse blocks, from the partitioned pairs), then the windows of small tiles.
__global__ void __launch_bounds__(kBinThreads) k_bin_reduce(BinArgs b, const u32 *__restrict__ tile_rank0,
                                                            const u64 *__restrict__ urow, const Out out,
                                                            const Decode dec, u32 *err) {
  extern __shared__ __align__(16) unsigned char bin_smem[];
  double *tv = reinterpret_cast<double *>(bin_smem);               // kBinSlots values (dense: the block)
  u32 *tk = reinterpret_cast<u32 *>(tv + kBinSlots);                // kBinSlots keys (hash)
  uint16_t *list = reinterpret_cast<uint16_t *>(tk + kBinSlots);   // occupied slots
  __shared__ u32 s_job, s_nocc;
  __shared__ u64 s_base;
  const u32 nbig = *b.njobs;
  const u64 nwin = (u64(b.spp[b.n]) + kBinWindow - 1) / kBinWindow;
  const u64 njobs = u64(nbig) + nwin;
  if (threadIdx.x == 0) s_job = atomicAdd(b.work, 1u);
  __syncthreads();
  for (;;) {
    const u64 j = s_job;
    __syncthreads();
    if (j >= njobs) break;
    u32 next = 0;
    if (threadIdx.x == 0) next = atomicAdd(b.work, 1u);  // consumed after this job
    if (j < nbig) {
      const BinJob jb = b.jobs[j];
      const BinWho who{false, jb.s, 0};
      const u32 nc = b.nch[jb.s];
      const u64 r = u64(b.nb) * b.chpre[jb.s];
      const u32 lo = b.hpre[r + u64(jb.b0) * nc], hi = b.hpre[r + u64(jb.b1) * nc];
      if (jb.b1 == jb.b0 + 1 && hi - lo > kBinDenseMin) {  // dense block
        // Untouched positions hold -0.0 and every update adds a value that is
        // not -0.0 (a -0.0 product is added as +0.0): a sum never returns to
        // -0.0 in round-to-nearest, so "touched" is "not -0.0", with no
        // bitmap to maintain.
        const u32 k0 = u32(jb.b0) * kBinWidth;
        for (u32 i = threadIdx.x; i < kBinWidth; i += blockDim.x) tv[i] = -0.0;
        if (threadIdx.x == 0) s_nocc = 0;
        __syncthreads();
        for (u32 q0 = lo; q0 < hi; q0 += blockDim.x * kBinIlp) {  // the same trip count in every lane
          u32 loc[kBinIlp];
          double v[kBinIlp];
#pragma unroll
          for (int i = 0; i < kBinIlp; i++) {
            const u32 q = q0 + u32(i) * blockDim.x + threadIdx.x;
            loc[i] = q < hi ? b.bkeys[q] - k0 : kBinEmpty;
            v[i] = q < hi ? __longlong_as_double((long long)b.bvals[q]) : 0.0;
          }
#pragma unroll
          for (int i = 0; i < kBinIlp; i++) {
            bool first = false;
            if (bin_aggregate(loc[i], &v[i]))
              first = __double_as_longlong(atomicAdd(&tv[loc[i]], v[i] + 0.0)) == (long long)0x8000000000000000ull;
            bin_list_append(first, loc[i], list, &s_nocc);
          }
        }
        __syncthreads();
        bin_emit(b, tile_rank0, urow, out, dec, err, who, list, s_nocc, tk, tv, true, k0, &s_base);
      } else {  // sparse blocks: at most kBinHashPairs pairs
        bin_hash(b.bkeys, b.bvals, lo, hi, tk, tv, list, &s_nocc);
        bin_emit(b, tile_rank0, urow, out, dec, err, who, list, s_nocc, tk, tv, false, 0, &s_base);
      }
    } else {  // a window of small tiles: fewer than kBinWindow + small_max positions
      const u64 w = j - nbig;
      const u32 f0 = b.first[w], f1 = b.first[w + 1];
      const BinWho who{true, 0, b.srk[f0]};
      bin_hash(b.keys, b.vals, b.spp[f0], b.spp[f1], tk, tv, list, &s_nocc);
      bin_emit(b, tile_rank0, urow, out, dec, err, who, list, s_nocc, tk, tv, false, 0, &s_base);
    }
    if (threadIdx.x == 0) s_job = next;
    __syncthreads();
  }
}

// ------------------------------------------------------- host pipeline ----

namespace {

struct HostClass {
  bool hash;
  int threads;
  u32 slots;  // hash table slots
  u64 pmax;   // multiply-adds per work item
  bool enabled;
};

struct Side {
  int order = 0;
  i64 nnz = 0;
  LinSpec lin{};
  u64 span = 1;      // external index space
  u64 keyspace = 1;  // contraction key space
  const int32_t *coords = nullptr;
  i64 sn = 0, sm = 0;
  const double *vals = nullptr;
};

u64 mul_checked(u64 a, u64 b, const char *what) {
  unsigned __int128 p = (unsigned __int128)a * b;
  if (p > (unsigned __int128)(~0ull) - 1)
    throw Error{FCC_ERR_OVERFLOW, std::string(what) + " exceeds 64 bits"};
  return u64(p);
}

void check_tensor(const fcc_tensor *t, const char *name) {
  std::string n(name);
  if (!t) throw Error{FCC_ERR_ARG, n + " is NULL"};
  if (t->order < 0 || t->order > FCC_MAX_ORDER) throw Error{FCC_ERR_ARG, n + ": order must be in 0..8"};
  if (t->nnz < 0 || t->nnz > 0x7FFFFFFFll) throw Error{FCC_ERR_ARG, n + ": nnz must be in 0..2^31-1"};
  if (t->order > 0 && !t->max_index) throw Error{FCC_ERR_ARG, n + ": max_index is NULL"};
  for (int m = 0; m < t->order; m++)
    if (t->max_index[m] < 0) throw Error{FCC_ERR_ARG, n + ": negative max_index"};
  if (t->nnz > 0 && ((t->order > 0 && !t->coords) || !t->values))
    throw Error{FCC_ERR_ARG, n + ": coords or values is NULL"};
  if (t->location != FCC_HOST && t->location != FCC_DEVICE) throw Error{FCC_ERR_ARG, n + ": bad location"};
  if (t->nnz > 0 && t->order > 0 && (t->stride_nnz < 0 || t->stride_mode < 0))
    throw Error{FCC_ERR_ARG, n + ": negative stride"};
}

void check_ctr(const fcc_tensor *t, const int32_t *ctr, int k, const char *name) {
  if (k > 0 && !ctr) throw Error{FCC_ERR_ARG, std::string(name) + " is NULL"};
  for (int i = 0; i < k; i++) {
    if (ctr[i] < 0 || ctr[i] >= t->order)
      throw Error{FCC_ERR_ARG, std::string(name) + ": contracted mode out of range"};
    for (int j = 0; j < i; j++)
      if (ctr[j] == ctr[i]) throw Error{FCC_ERR_ARG, std::string(name) + ": repeated contracted mode"};
  }
}

void build_side(const fcc_tensor *t, const int32_t *ctr, const int32_t *other_max,
                const int32_t *other_ctr, int k, int radix_mode, Side &s) {
  s.order = t->order;
  s.nnz = t->nnz;
  LinSpec &l = s.lin;
  std::memset(&l, 0, sizeof(l));
  l.order = t->order;
  bool is_ctr[FCC_MAX_ORDER] = {};
  for (int i = 0; i < k; i++) is_ctr[ctr[i]] = true;
  for (int m = 0; m < t->order; m++) {
    l.max_index[m] = t->max_index[m];
    if (!is_ctr[m]) {
      l.ext_mode[l.n_ext] = m;
      l.ext_radix[l.n_ext] = u64(t->max_index[m]) + 1;
      s.span = mul_checked(s.span, l.ext_radix[l.n_ext], "external index space");
      l.n_ext++;
    }
  }
  l.n_ctr = k;
  for (int i = 0; i < k; i++) {
    u64 r = u64(t->max_index[ctr[i]]) + 1;
    if (radix_mode == FCC_RADIX_SHARED) r = std::max<u64>(r, u64(other_max[other_ctr[i]]) + 1);
    l.ctr_mode[i] = ctr[i];
    l.ctr_radix[i] = r;
    s.keyspace = mul_checked(s.keyspace, r, "contraction key space");
  }
}

const int32_t *upload_coords(Runtime *ctx, const fcc_tensor *t) {
  if (t->nnz == 0 || t->order == 0 || t->location == FCC_DEVICE) return t->coords;
  const i64 extent = (t->nnz - 1) * t->stride_nnz + i64(t->order - 1) * t->stride_mode + 1;
  int32_t *d = ctx->arena.get_n<int32_t>(size_t(extent));
  FCC_CUDA(cudaMemcpyAsync(d, t->coords, sizeof(int32_t) * size_t(extent), cudaMemcpyHostToDevice,
                           ctx->stream));
  return d;
}

const double *upload_values(Runtime *ctx, const fcc_tensor *t) {
  if (t->nnz == 0 || t->location == FCC_DEVICE) return t->values;
  double *d = ctx->arena.get_n<double>(size_t(t->nnz));
  FCC_CUDA(cudaMemcpyAsync(d, t->values, sizeof(double) * size_t(t->nnz), cudaMemcpyHostToDevice,
                           ctx->stream));
  return d;
}

// Device scalar block: slot numbers in a u64 array.
enum Scalar { S_NSEG = 0, S_NA2, S_NTILES, S_NITEMS, S_NSPLIT, S_CAP, S_HASH, S_CURSOR, S_COUNTER, S_NROWS,
              S_PTOTAL, S_ERR, S_TINY, S_HOT, S_NSPLIT_H, S_CLS0, S_CLS_END = S_CLS0 + FCC_NUM_CLASSES,
              S_PSUM0, S_PSUM_END = S_PSUM0 + FCC_NUM_CLASSES + 1, S_NESC, S_ESC_PAIRS, S_ESC_RUNS, S_ESC_BASE,
              S_COUNT };
static_assert(S_COUNT <= 32, "the pinned scalar block holds 32 entries");

// Copies the scalar block and the error word to pinned host memory, waits,
// and raises the error bits that are not recoverable.
void read_scalars(Runtime *ctx, u64 *d_sc) {
  FCC_CUDA(cudaMemcpyAsync(d_sc + S_ERR, ctx->d_err, sizeof(u32), cudaMemcpyDeviceToDevice, ctx->stream));
  FCC_CUDA(cudaMemcpyAsync(ctx->h_scalars, d_sc, sizeof(u64) * S_COUNT, cudaMemcpyDeviceToHost, ctx->stream));
  FCC_CUDA(cudaStreamSynchronize(ctx->stream));
  const u32 err = u32(ctx->h_scalars[S_ERR]);
  if (err & ERRB_COORD) throw Error{FCC_ERR_ARG, "a coordinate lies outside [0, max_index]"};
  if (err & ERRB_HASH) throw Error{FCC_ERR_HASH_FULL, "hash accumulator probe limit reached"};
  if (err & ERRB_TIMEOUT)
    throw Error{FCC_ERR_TIMEOUT, "a bounded device wait gave up (bulk-copy ring or injected wait); the kernels "
                                 "stopped after their copies in flight landed"};
  if (err & ERRB_INTERNAL) throw Error{FCC_ERR_CUDA, "internal plan invariant violated"};
}

u32 scalar32(Runtime *ctx, int s) { return u32(ctx->h_scalars[s] & 0xFFFFFFFFu); }

int grid_tiles(Runtime *ctx, const void *kernel, int threads, size_t smem, u32 nitems, int *ctas_per_sm) {
  int per_sm = 0;
  FCC_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, threads, smem));
  if (per_sm < 1) throw Error{FCC_ERR_CUDA, "tile kernel does not fit on an SM"};
  *ctas_per_sm = per_sm;
  i64 g = i64(per_sm) * ctx->num_sms;
  if (g > i64(nitems)) g = nitems;
  return int(std::max<i64>(g, 1));
}

void free_result_buffers(fcc_result *r, cudaStream_t s) {
  if (r->owned) {
    if (r->d_vals) cudaFreeAsync(r->d_vals, s);
    if (r->d_coords) cudaFreeAsync(r->d_coords, s);
  }
  r->d_vals = nullptr;
  r->d_coords = nullptr;
}

struct Timing {
  Runtime *ctx;
  bool on;
  int next = 0;
  void mark(int slot) {  // records every slot up to `slot`
    if (!on) return;
    while (next <= slot) FCC_CUDA(cudaEventRecord(ctx->ev[next++], ctx->stream));
  }
  void finish() {
    if (!on) return;
    mark(5);
    FCC_CUDA(cudaEventSynchronize(ctx->ev[5]));
    const int map[FCC_NUM_PHASES][2] = {{0, 1}, {1, 2}, {2, 3}, {3, 4}, {4, 5}, {0, 5}};
    for (int p = 0; p < FCC_NUM_PHASES; p++) {
      float ms = 0;
      FCC_CUDA(cudaEventElapsedTime(&ms, ctx->ev[map[p][0]], ctx->ev[map[p][1]]));
      ctx->phase_ms[p] = ms;
    }
  }
};

}  // namespace

// The whole contraction. count_only stops after the segment lookup and
// returns the multiply-add count in *products. res (NULL when count_only)
// receives the output; its buffers come from ctx->pool, or are the caller's
// buffers (ctx->out_*) when ctx->caller_out is set or there is no pool. group_lb (ngroups entries, may be
// NULL) makes A's leading external index a group index: rows of group g use
// B columns [0, group_lb[g]) only, and dense tiles are sized per group.
void contract(Runtime *ctx, const fcc_tensor *A, const fcc_tensor *B, const int32_t *ctrA,
              const int32_t *ctrB, int k, const fcc_options &opt, fcc_result *res, i64 *products,
              bool count_only, const u32 *group_lb, u32 ngroups) {
  check_tensor(A, "A");
  check_tensor(B, "B");
  if (k < 0 || k > A->order || k > B->order) throw Error{FCC_ERR_ARG, "bad number of contracted modes"};
  check_ctr(A, ctrA, k, "ctrA");
  check_ctr(B, ctrB, k, "ctrB");
  if (opt.radix_mode != FCC_RADIX_PER_OPERAND && opt.radix_mode != FCC_RADIX_SHARED)
    throw Error{FCC_ERR_ARG, "bad radix_mode"};
  if (opt.accumulator < FCC_ACC_AUTO || opt.accumulator > FCC_ACC_HASH) throw Error{FCC_ERR_ARG, "bad accumulator"};
  if (opt.rows_per_tile < 0 || opt.products_per_item < 0 || opt.dense_cap < 0 || opt.hash_slots < 0 ||
      opt.capacity_hint < 0)
    throw Error{FCC_ERR_ARG, "negative tuning option"};

  Side sa, sb;
  build_side(A, ctrA, B->max_index, ctrB, k, opt.radix_mode, sa);
  build_side(B, ctrB, A->max_index, ctrA, k, opt.radix_mode, sb);
  const int out_order = sa.lin.n_ext + sb.lin.n_ext;
  cudaStream_t st = ctx->stream;
  Timing tm{ctx, opt.timing != 0 && ctx->ev != nullptr};
  if (ctx->phase_ms)
    for (int i = 0; i < FCC_NUM_PHASES; i++) ctx->phase_ms[i] = 0;

  if (!count_only) {
    res->order = out_order;
    res->owned = !(ctx->caller_out || !ctx->pool);
  }
  struct Cleanup {
    fcc_result *r;
    cudaStream_t s;
    bool done = false;
    ~Cleanup() { if (r && !done) free_result_buffers(r, s); }
  } cleanup{count_only ? nullptr : res, st};

  ctx->arena.begin(st);
  tm.mark(0);
  if (A->nnz == 0 || B->nnz == 0) {
    if (products) *products = 0;
    tm.finish();
    cleanup.done = true;
    return;
  }

  // ---- upload (host operands) ----
  Arena &ar = ctx->arena;
  sa.coords = upload_coords(ctx, A);
  sa.sn = A->stride_nnz;
  sa.sm = A->stride_mode;
  sa.vals = upload_values(ctx, A);
  sb.coords = upload_coords(ctx, B);
  sb.sn = B->stride_nnz;
  sb.sm = B->stride_mode;
  sb.vals = upload_values(ctx, B);
  tm.mark(1);

  const i64 nA = sa.nnz, nB = sb.nnz;
  u64 *d_sc = ar.get_n<u64>(S_COUNT);
  FCC_CUDA(cudaMemsetAsync(d_sc, 0, sizeof(u64) * S_COUNT, st));
  FCC_CUDA(cudaMemsetAsync(ctx->d_err, 0, sizeof(u32), st));
  auto sc32 = [&](int s) { return reinterpret_cast<u32 *>(d_sc + s); };

  // ---- index: linearise, sort B by key, segments ----
  u64 *extA = ar.get_n<u64>(nA), *keyA = ar.get_n<u64>(nA);
  u32 *permA = ar.get_n<u32>(nA);
  u64 *extB = ar.get_n<u64>(nB), *keyB = ar.get_n<u64>(nB);
  u32 *permB = ar.get_n<u32>(nB);
  k_linearize<<<grid_for(nA, 256), 256, 0, st>>>(sa.coords, sa.sn, sa.sm, nA, sa.lin, extA, keyA, permA, ctx->d_err);
  FCC_LAUNCH_CHECK();
  k_linearize<<<grid_for(nB, 256), 256, 0, st>>>(sb.coords, sb.sn, sb.sm, nB, sb.lin, extB, keyB, permB, ctx->d_err);
  FCC_LAUNCH_CHECK();
  radix_sort_pairs(keyB, permB, nB, bits_for(sb.keyspace - 1), ar, st, ctx->d_err);

  const bool colb32 = sb.span <= 0xFFFFFFFFull;
  // padded: staged copies round their end up to 16 bytes
  double *valB = ar.get_n<double>(nB + 2);
  void *colB = colb32 ? static_cast<void *>(ar.get_n<u32>(nB + 4)) : static_cast<void *>(ar.get_n<u64>(nB));
  if (colb32)
    k_gather_b<u32><<<grid_for(nB, 256), 256, 0, st>>>(permB, extB, sb.vals, nB, static_cast<u32 *>(colB), valB,
                                                       sc32(S_TINY));
  else
    k_gather_b<u64><<<grid_for(nB, 256), 256, 0, st>>>(permB, extB, sb.vals, nB, static_cast<u64 *>(colB), valB,
                                                       sc32(S_TINY));
  FCC_LAUNCH_CHECK();
  u32 *flagB = ar.get_n<u32>(nB), *idxB = ar.get_n<u32>(nB);
  k_flag_change<<<grid_for(nB, 256), 256, 0, st>>>(keyB, nB, flagB);
  FCC_LAUNCH_CHECK();
  scan_exclusive(flagB, idxB, nB, sc32(S_NSEG), ar, st);
  u64 *ukey = ar.get_n<u64>(nB);
  u32 *segbeg = ar.get_n<u32>(nB + 1);
  k_seg_write<<<grid_for(nB, 256), 256, 0, st>>>(keyB, flagB, idxB, nB, ukey, segbeg);
  FCC_LAUNCH_CHECK();
  // about one bucket per B nonzero over the key space (keys < 2^kbits)
  const int kbits = bits_for(sb.keyspace - 1), bbits = std::min(kbits, std::max(1, bits_for(u64(nB))));
  const int bshift = kbits - bbits;
  const u64 nbuckets = u64(1) << bbits;
  u32 *bcount = ar.get_n<u32>(nbuckets + 1), *bstart = ar.get_n<u32>(nbuckets + 1);
  FCC_CUDA(cudaMemsetAsync(bcount, 0, sizeof(u32) * (nbuckets + 1), st));
  k_seg_buckets<<<grid_for(nB, 256), 256, 0, st>>>(ukey, sc32(S_NSEG), bshift, bcount);
  FCC_LAUNCH_CHECK();
  scan_exclusive(bcount, bstart, i64(nbuckets + 1), nullptr, ar, st);

  // ---- A: sort by row, look up segments, drop unmatched ----
  radix_sort_pairs(extA, permA, nA, bits_for(sa.span - 1), ar, st, ctx->d_err);
  u32 *segTmp = ar.get_n<u32>(nA), *flagA = ar.get_n<u32>(nA), *idxA = ar.get_n<u32>(nA);
  k_lookup<<<grid_for(nA, 256), 256, 0, st>>>(keyA, permA, nA, ukey, sc32(S_NSEG), bstart, bshift, nbuckets,
                                               segTmp, flagA);
  FCC_LAUNCH_CHECK();
  scan_exclusive(flagA, idxA, nA, sc32(S_NA2), ar, st);
  u64 *rowA = ar.get_n<u64>(nA);
  u32 *sbA = ar.get_n<u32>(nA), *lenA = ar.get_n<u32>(nA);
  double *valA = ar.get_n<double>(nA);
  FCC_CUDA(cudaMemsetAsync(lenA, 0, sizeof(u32) * nA, st));
  k_compact_a<<<grid_for(nA, 256), 256, 0, st>>>(flagA, idxA, nA, permA, extA, segTmp, sa.vals, segbeg, rowA,
                                                 sbA, valA, lenA, sc32(S_TINY));
  FCC_LAUNCH_CHECK();
  u64 *P = ar.get_n<u64>(nA + 1);
  scan_exclusive_wide(lenA, P, nA, P + nA, ar, st);
  FCC_CUDA(cudaMemcpyAsync(d_sc + S_PTOTAL, P + nA, sizeof(u64), cudaMemcpyDeviceToDevice, st));
  tm.mark(2);

  read_scalars(ctx, d_sc);
  const u32 nA2 = scalar32(ctx, S_NA2);
  const u64 ptotal = ctx->h_scalars[S_PTOTAL];
  if (products) *products = i64(ptotal);
  if (count_only) {
    tm.finish();
    return;
  }
  res->products = i64(ptotal);
  if (nA2 == 0 || ptotal == 0) {
    tm.finish();
    cleanup.done = true;
    return;
  }

  // ---- plan ----
  const u64 LB = sb.span;
  const size_t smem_cap = ctx->smem_optin - 1024;
  // the dense kernel's static shared memory (item plan, drain counts) comes first
  const size_t dense_dyn_cap = smem_cap - (sizeof(ItemPlan) + 4096 + 512);
  const u64 max_dense_area = std::min<u64>((u64(dense_dyn_cap) * 8) / 65, 32 * 1024);  // 8 B + 1 mask bit
  u64 dense_cap = opt.dense_cap > 0 ? std::min<u64>(u64(opt.dense_cap), max_dense_area) : max_dense_area;
  bool dense = LB <= dense_cap && opt.accumulator != FCC_ACC_HASH;
  if (opt.accumulator == FCC_ACC_DENSE && !dense)
    throw Error{FCC_ERR_ARG, "dense accumulator: B external span exceeds the shared-memory tile"};
  u64 TL = 1;
  if (opt.rows_per_tile > 0) TL = u64(opt.rows_per_tile);
  else if (dense) TL = std::max<u64>(1, dense_cap / LB);
  if (dense && TL * LB > dense_cap)
    throw Error{FCC_ERR_ARG, "rows_per_tile x B external span exceeds the dense tile capacity"};
  if (!dense && (unsigned __int128)TL * LB > (unsigned __int128)(~0ull) - 1)
    throw Error{FCC_ERR_OVERFLOW, "rows_per_tile x B external span exceeds 64 bits"};
  // ---- tile classes ----
  // Every output tile runs in one class: the shared-memory dense tile (640
  // threads by default), or an open-addressing hash table of 8192 slots (1024
  // threads, one CTA per SM), 4096 or 2048 slots (256 / 128 threads, several
  // CTAs per SM, so that small tiles overlap their barriers and memory
  // latency). The schedule picks a class per tile; the items of one class run
  // in one persistent launch. Hash-class tiles are expanded, sorted and
  // reduced instead unless a hash class is forced (below).
  const bool custom_hash = opt.hash_slots > 0 || (opt.tile_threads > 0 && opt.accumulator == FCC_ACC_HASH);
  HostClass hc[FCC_NUM_CLASSES];
  const int tt = opt.tile_threads;  // dense tiles: 512, 640, 768, 1024; large hash tables: 128 ... 1024
  const bool tt_dense = tt == 512 || tt == 640 || tt == 768 || tt == 1024;
  const bool tt_hash = tt == 128 || tt == 256 || tt == 512 || tt == 1024;
  if (tt < 0 || (tt > 0 && !tt_dense && !tt_hash))
    throw Error{FCC_ERR_ARG, "tile_threads must be 128, 256, 512, 640, 768 or 1024"};
  hc[FCC_CLASS_DENSE] = {false, tt > 0 ? tt : kTileThreads, 0u, 0, dense};
  hc[FCC_CLASS_HASH_L] = {true, tt > 0 && tt_hash ? tt : 1024, opt.hash_slots > 0 ? u32(opt.hash_slots) : 8192u, 0,
                          opt.accumulator != FCC_ACC_DENSE};
  hc[FCC_CLASS_HASH_M] = {true, 256, 4096u, 0, opt.accumulator != FCC_ACC_DENSE && !custom_hash};
  hc[FCC_CLASS_HASH_S] = {true, 128, 2048u, 0, opt.accumulator != FCC_ACC_DENSE && !custom_hash};
  if (opt.accumulator == FCC_ACC_HASH) hc[FCC_CLASS_DENSE].enabled = false;
  if (tt > 0 && !tt_dense) {  // 128 or 256: hash tables only
    if (opt.accumulator == FCC_ACC_DENSE) throw Error{FCC_ERR_ARG, "tile_threads 128 and 256 are for the hash accumulator"};
    hc[FCC_CLASS_DENSE].enabled = false;
    hc[FCC_CLASS_DENSE].threads = kTileThreads;
  }
  hc[FCC_CLASS_DENSE_FLAT] = hc[FCC_CLASS_DENSE];  // the same tile, flat items
  {
    const u32 hs = hc[FCC_CLASS_HASH_L].slots;
    if (hs & (hs - 1)) throw Error{FCC_ERR_ARG, "hash_slots must be a power of two"};
    if (size_t(hs) * 16 > smem_cap || hs < 64) throw Error{FCC_ERR_ARG, "hash_slots out of range"};
  }
  {
    u64 pd = opt.products_per_item > 0 ? u64(opt.products_per_item) : (u64(1) << 20);
    hc[FCC_CLASS_DENSE].pmax = std::min<u64>(pd, u64(kListMax) * kCtaRun);
    hc[FCC_CLASS_DENSE_FLAT].pmax = hc[FCC_CLASS_DENSE].pmax;
    // an item's distinct outputs never exceed its multiply-adds, and the probe
    // loop covers the whole table: 3/4 of the slots bounds the load at 0.75
    for (int c = FCC_CLASS_HASH_L; c <= FCC_CLASS_HASH_S; c++) {
      const u64 cap = hc[c].slots / 4 * 3;
      hc[c].pmax = opt.products_per_item > 0 ? std::min<u64>(u64(opt.products_per_item), cap) : cap;
    }
  }
  int forced = -1;
  if (opt.accumulator == FCC_ACC_DENSE) forced = FCC_CLASS_DENSE;
  else if (opt.accumulator == FCC_ACC_AUTO && opt.schedule >= FCC_SCHED_FORCE) forced = opt.schedule - FCC_SCHED_FORCE;
  if (opt.schedule < 0 || opt.schedule >= FCC_SCHED_FORCE + FCC_NUM_CLASSES)
    throw Error{FCC_ERR_ARG, "bad schedule"};
  if (forced >= 0 && !hc[forced].enabled)
    throw Error{FCC_ERR_ARG, (forced == FCC_CLASS_DENSE || forced == FCC_CLASS_DENSE_FLAT)
                                 ? "dense accumulator: B external span exceeds the shared-memory tile"
                                 : "the forced hash class is disabled by hash_slots or tile_threads"};
  if (custom_hash && forced < 0 && opt.accumulator == FCC_ACC_HASH) forced = FCC_CLASS_HASH_L;
  if (opt.dense_fill_log2 < -1 || opt.dense_fill_log2 > 40) throw Error{FCC_ERR_ARG, "dense_fill_log2 out of range"};
  if (opt.dense_staging < -1 || opt.dense_staging > 0) throw Error{FCC_ERR_ARG, "dense_staging must be -1 or 0"};
  if (opt.sched_mix_margin < 0 || opt.sched_mix_margin > 1000) throw Error{FCC_ERR_ARG, "bad sched_mix_margin"};
  if (opt.hash_esc < -1 || opt.hash_esc > 2) throw Error{FCC_ERR_ARG, "hash_esc must be -1, 0, 1 or 2"};
  if (opt.out_waves < 0 || opt.out_waves > kMaxWaves) throw Error{FCC_ERR_ARG, "out_waves must be in 0..16"};
  if (opt.wait_polls < 0) throw Error{FCC_ERR_ARG, "wait_polls must be >= 0"};
  if (opt.fault_wait != 0 && opt.fault_wait != 1) throw Error{FCC_ERR_ARG, "fault_wait must be 0 or 1"};
  if (opt.dense_kernel < 0 || opt.dense_kernel > 3) throw Error{FCC_ERR_ARG, "dense_kernel must be 0, 1, 2 or 3"};
  if (opt.esc_group < 0) throw Error{FCC_ERR_ARG, "esc_group must be >= 0"};
  if (opt.esc_reduce < 0 || opt.esc_reduce > 2) throw Error{FCC_ERR_ARG, "esc_reduce must be 0, 1 or 2"};
  if (opt.esc_small < 0 || opt.esc_small > int(kBinSmallMax))
    throw Error{FCC_ERR_ARG, "esc_small must be in [0, " + std::to_string(kBinSmallMax) + "]"};
  bool learned = forced < 0 && opt.schedule == FCC_SCHED_LEARNED && ctx->sched && ctx->sched->model;
  const bool want_record = opt.timing == 2 && ctx->sched;
  // Row groups (batched contractions): dense tiles hold rows of one group,
  // group_tl rows of the group's own column span each.
  const bool grouped = dense && group_lb && ngroups > 0;
  u64 area = TL * LB;
  if (grouped) {
    area = 0;
    for (u32 g = 0; g < ngroups; g++) {
      const u64 lb = std::max<u32>(group_lb[g], 1u);
      if (lb > LB) throw Error{FCC_ERR_CUDA, "group column span exceeds the B span"};
      const u64 tl = opt.rows_per_tile > 0 ? TL : std::max<u64>(1, dense_cap / lb);
      area = std::max(area, tl * lb);
    }
  }
  if (opt.hot_columns < -1 || (opt.hot_columns > 0 && opt.hot_columns % 32))
    throw Error{FCC_ERR_ARG, "hot_columns must be -1, 0 or a positive multiple of 32"};

  // Hot columns (row tiles only): frequency of each B column, most frequent first.
  const u32 hot_want = opt.hot_columns > 0 ? u32(opt.hot_columns) : 128u;
  const bool hot_try = !grouped && TL == 1 && opt.hot_columns > 0 && LB <= (u64(1) << 26) && LB >= 2 * u64(hot_want);
  u32 *colmap = nullptr, *inv_col = nullptr;
  if (hot_try) {
    const int lbits = bits_for(LB - 1);
    u32 *count = ar.get_n<u32>(LB);
    u64 *ckey = ar.get_n<u64>(LB);
    u32 *cidx = ar.get_n<u32>(LB);
    colmap = ar.get_n<u32>(LB);
    inv_col = ar.get_n<u32>(LB);
    FCC_CUDA(cudaMemsetAsync(count, 0, sizeof(u32) * LB, st));
    if (colb32) k_col_hist<u32><<<grid_for(nB, 256), 256, 0, st>>>(static_cast<const u32 *>(colB), nB, count);
    else k_col_hist<u64><<<grid_for(nB, 256), 256, 0, st>>>(static_cast<const u64 *>(colB), nB, count);
    FCC_LAUNCH_CHECK();
    k_col_sortkeys<<<grid_for(i64(LB), 256), 256, 0, st>>>(count, LB, lbits, ckey, cidx);
    FCC_LAUNCH_CHECK();
    radix_sort_pairs(ckey, cidx, i64(LB), 32 + lbits, ar, st, ctx->d_err);
    k_col_tables<<<grid_for(i64(LB), 256), 256, 0, st>>>(ckey, LB, lbits, hot_want, colmap, inv_col,
                                                        reinterpret_cast<unsigned long long *>(d_sc + S_HOT));
    FCC_LAUNCH_CHECK();
  }

  // ---- tiles over the rows that occur ----
  RowGroups rg{};
  rg.LB = LB;
  rg.area = dense_cap;
  rg.TL = (grouped && opt.rows_per_tile <= 0) ? 0 : TL;
  const u32 ng = grouped ? ngroups : 1u;
  if (grouped) {
    rg.gdiv = sa.span / sa.lin.ext_radix[0];
    u32 *d_lb = ar.get_n<u32>(ng);
    FCC_CUDA(cudaMemcpyAsync(d_lb, group_lb, sizeof(u32) * ng, cudaMemcpyHostToDevice, st));
    rg.lb = d_lb;
  }
  u32 *rflag = ar.get_n<u32>(nA2), *rexcl = ar.get_n<u32>(nA2), *rank = ar.get_n<u32>(nA2);
  u64 *urow = ar.get_n<u64>(nA2);
  u32 *gfirst = ar.get_n<u32>(ng);
  k_flag_change<<<grid_for(nA2, 256), 256, 0, st>>>(rowA, nA2, rflag);
  FCC_LAUNCH_CHECK();
  scan_exclusive(rflag, rexcl, nA2, sc32(S_NROWS), ar, st);
  k_row_rank<<<grid_for(nA2, 256), 256, 0, st>>>(rowA, rflag, rexcl, nA2, rg, rank, urow, gfirst);
  FCC_LAUNCH_CHECK();
  u32 *slotA = ar.get_n<u32>(nA2), *tflag = ar.get_n<u32>(nA2), *tidx = ar.get_n<u32>(nA2);
  k_row_tiles<<<grid_for(nA2, 256), 256, 0, st>>>(rowA, rflag, rank, nA2, rg, gfirst, slotA, tflag);
  FCC_LAUNCH_CHECK();
  scan_exclusive(tflag, tidx, nA2, sc32(S_NTILES), ar, st);
  // The tile count sizes every per-tile array, scan and launch below (tiles
  // are far fewer than A entries: 20,000 against 10M on zipf3).
  read_scalars(ctx, d_sc);
  const u32 NT = std::max<u32>(scalar32(ctx, S_NTILES), 1);
  u32 *tile_abeg = ar.get_n<u32>(NT + 1), *tile_rank0 = ar.get_n<u32>(NT);
  u32 *tile_lb = ar.get_n<u32>(NT), *tile_nrows = ar.get_n<u32>(NT);
  k_tile_write<<<grid_for(nA2, 256), 256, 0, st>>>(rowA, tflag, tidx, rank, nA2, rg, tile_abeg, tile_rank0,
                                                   tile_lb);
  FCC_LAUNCH_CHECK();
  k_tile_nrows<<<grid_for(NT, 256), 256, 0, st>>>(sc32(S_NTILES), tile_abeg, rank, tile_rank0, tile_nrows);
  FCC_LAUNCH_CHECK();

  // Hash tiles expanded, sorted and reduced instead of accumulated in tables
  // (esc_mode 2: every hash tile; 1: tiles too big for their table, which
  // otherwise split into items merged through a global hash table), when the
  // pairs fit (at most 56 bytes of temporaries per multiply-add, within half
  // of the free device memory) and the key space fits 64 bits. By default
  // every hash tile, unless the caller forced a hash class (then its tables
  // run and only the oversized tiles expand); a fixed workspace (the
  // allocation-free call) expands only on request, since the pairs may not fit
  // where the hash tables do.
  const u64 esc_rows = grouped ? dense_cap : TL;
  bool esc = false;
  int esc_mode = opt.hash_esc;
  if (esc_mode == 0)
    esc_mode = ar.is_fixed()                                                                  ? -1
               : (forced >= 0 && forced != FCC_CLASS_DENSE && forced != FCC_CLASS_DENSE_FLAT) ? 1
                                                                                                : 2;
  const bool esc_wanted = esc_mode > 0;
  // (not while recording per-tile costs: expanded tiles have no work items to time)
  if (esc_wanted && !want_record) {
    const size_t fb = ar.available();
    const unsigned __int128 keyspace = (unsigned __int128)NT * esc_rows * LB;
    esc = ptotal <= 0xFFFFFFFFull && (unsigned __int128)ptotal * 56 <= fb / 2 && keyspace < ((unsigned __int128)1 << 64);
  }

  // ---- class per tile ----
  ClassTable ctab{};
  for (int c = 0; c < FCC_NUM_CLASSES; c++) {
    ctab.enabled[c] = hc[c].enabled ? 1u : 0u;
    ctab.pmax[c] = hc[c].pmax;
    ctab.hash[c] = hc[c].hash ? 1u : 0u;
  }
  ctab.forced = forced;
  // dense_fill_log2 = 0: tiles under a quarter full leave the dense class
  // when hash tiles are expanded (expansion beats a sparse dense tile), else
  // every tile that fits stays dense
  ctab.fill_log2 = opt.dense_fill_log2 > 0 ? opt.dense_fill_log2 : (opt.dense_fill_log2 == 0 && esc && esc_mode == 2) ? 2 : 0;
  ctab.override_log2 = 0.32f;     // the model must predict at least 25% cheaper to leave the rule
  ctab.dense_switch_log2 = 0.074f;  // ... or 5% cheaper for the other dense class
  // Without a dense class and with every hash tile expanded, the class of a
  // tile changes nothing: the rule runs alone (no features, no predictions).
  if (learned && !hc[FCC_CLASS_DENSE].enabled && esc && esc_mode == 2) learned = false;
  const u32 *lb_or_null = dense ? tile_lb : nullptr;
  float *feat = nullptr, *pred = nullptr;
  if (learned || want_record) {
    feat = ar.get_n<float>(size_t(NT) * FCC_SCHED_FEATURES);
    tile_features(st, sc32(S_NTILES), u32(NT), tile_abeg, P, tile_nrows, lb_or_null, LB, feat, ctx->num_sms);
  }
  if (learned) {
    pred = ar.get_n<float>(size_t(NT) * FCC_NUM_CLASSES);
    predict_costs(st, sc32(S_NTILES), u32(NT), feat, ctx->sched->model, pred);
    // With sched_mix_margin > 0, a launch-level decision: predicted totals of
    // every class run on all tiles, and of the per-tile best; classes are mixed
    // only when the mix is predicted to win by that margin, otherwise every
    // tile takes the class of the lowest predicted total.
    if (opt.sched_mix_margin > 0) {
    FCC_CUDA(cudaMemsetAsync(d_sc + S_PSUM0, 0, sizeof(u64) * (FCC_NUM_CLASSES + 1), st));
    k_pred_sums<<<grid_for(NT, 256), 256, 0, st>>>(sc32(S_NTILES), NT, pred, ctab,
                                                    reinterpret_cast<double *>(d_sc + S_PSUM0));
    FCC_LAUNCH_CHECK();
    read_scalars(ctx, d_sc);
    double best = 1e300, mix = 0;
    int best_c = -1;
    for (int c = 0; c < FCC_NUM_CLASSES; c++) {
      if (!hc[c].enabled) continue;
      double v;
      std::memcpy(&v, &ctx->h_scalars[S_PSUM0 + c], sizeof(v));
      if (v < best) { best = v; best_c = c; }
    }
    std::memcpy(&mix, &ctx->h_scalars[S_PSUM0 + FCC_NUM_CLASSES], sizeof(mix));
    if (best_c >= 0 && !(mix * (1.0 + opt.sched_mix_margin / 100.0) < best)) {
      ctab.forced = best_c;
      pred = nullptr;
    }
    }
  }
  u32 *cls = ar.get_n<u32>(NT);
  u64 *ckey = ar.get_n<u64>(NT);
  u32 *corder = ar.get_n<u32>(NT);
  k_tile_class<<<grid_for(NT, 256), 256, 0, st>>>(sc32(S_NTILES), NT, tile_abeg, P, tile_nrows, lb_or_null, LB,
                                                   ctab, pred, cls, ckey, corder);
  FCC_LAUNCH_CHECK();
  // tiles in class order (stable), so that each class's items are contiguous
  radix_sort_pairs(ckey, corder, NT, 3, ar, st, ctx->d_err);

  u32 *t_items = ar.get_n<u32>(NT), *t_split_d = ar.get_n<u32>(NT), *t_split_h = ar.get_n<u32>(NT);
  u64 *t_cap = ar.get_n<u64>(NT), *t_hsz = ar.get_n<u64>(NT);
  u32 *esc_flag = ar.get_n<u32>(NT), *esc_idx = ar.get_n<u32>(NT);
  u64 *esc_cnt = ar.get_n<u64>(NT), *esc_off = ar.get_n<u64>(NT);
  k_tile_items<<<grid_for(NT, 256), 256, 0, st>>>(sc32(S_NTILES), NT, corder, cls, tile_abeg, P, tile_nrows,
                                                   lb_or_null, LB, ctab, esc ? esc_mode : 0, t_items, t_split_d, t_split_h,
                                                   t_cap, t_hsz, esc_flag, esc_cnt);
  FCC_LAUNCH_CHECK();
  scan_exclusive(esc_flag, esc_idx, NT, sc32(S_NESC), ar, st);
  scan_exclusive(esc_cnt, esc_off, NT, d_sc + S_ESC_PAIRS, ar, st);
  u32 *item_off = ar.get_n<u32>(NT), *split_d_idx = ar.get_n<u32>(NT), *split_h_idx = ar.get_n<u32>(NT);
  u64 *t_hoff = ar.get_n<u64>(NT);
  scan_exclusive(t_items, item_off, NT, sc32(S_NITEMS), ar, st);
  scan_exclusive(t_split_d, split_d_idx, NT, sc32(S_NSPLIT), ar, st);
  scan_exclusive(t_split_h, split_h_idx, NT, sc32(S_NSPLIT_H), ar, st);
  scan_exclusive(t_cap, t_cap, NT, d_sc + S_CAP, ar, st);
  scan_exclusive(t_hsz, t_hoff, NT, d_sc + S_HASH, ar, st);
  FCC_CUDA(cudaMemsetAsync(d_sc + S_CLS0, 0xFF, sizeof(u64) * FCC_NUM_CLASSES, st));  // ~0: class unused
  k_class_bounds<<<grid_for(NT, 256), 256, 0, st>>>(sc32(S_NTILES), ckey, item_off, d_sc + S_CLS0);
  FCC_LAUNCH_CHECK();
  read_scalars(ctx, d_sc);
  const u32 nitems = scalar32(ctx, S_NITEMS);
  const u32 nsplit_d = scalar32(ctx, S_NSPLIT);
  const u32 nsplit_h = scalar32(ctx, S_NSPLIT_H);
  const u64 cap_total = ctx->h_scalars[S_CAP];
  const u64 hash_total = ctx->h_scalars[S_HASH];
  const u32 nesc = scalar32(ctx, S_NESC);
  const u64 esc_pairs = ctx->h_scalars[S_ESC_PAIRS];
  u32 cbeg[FCC_NUM_CLASSES + 1], ccount[FCC_NUM_CLASSES];
  {
    u32 next = nitems;
    for (int c = FCC_NUM_CLASSES - 1; c >= 0; c--) {
      const u64 b = ctx->h_scalars[S_CLS0 + c];
      if (b == ~0ull) { cbeg[c] = next; ccount[c] = 0; continue; }
      cbeg[c] = u32(b);
      ccount[c] = next - u32(b);
      next = u32(b);
    }
  }

  Item *items = ar.get_n<Item>(std::max<u32>(nitems, 1));
  int *split_of_tile = ar.get_n<int>(NT);
  u32 *split_tiles_d = ar.get_n<u32>(std::max<u32>(nsplit_d, 1));
  u32 *split_tiles_h = ar.get_n<u32>(std::max<u32>(nsplit_h, 1));
  u64 *hoff_t = ar.get_n<u64>(NT), *hsz_t = ar.get_n<u64>(NT);
  u32 *esc_tiles = ar.get_n<u32>(std::max<u32>(nesc, 1));
  u64 *esc_base = ar.get_n<u64>(std::max<u32>(nesc, 1));
  k_item_write<<<grid_for(NT, 256), 256, 0, st>>>(sc32(S_NTILES), corder, cls, tile_abeg, P, item_off, ctab, items,
                                                   t_split_d, t_split_h, split_d_idx, split_h_idx, split_of_tile,
                                                   split_tiles_d, split_tiles_h, t_hoff, t_hsz, hoff_t, hsz_t,
                                                   esc_flag, esc_idx, esc_off, esc_tiles, esc_base);
  FCC_LAUNCH_CHECK();
  // Expanded tiles run in groups of at most G tiles, so that the keys (local
  // tile index x span + slot x LB + column) fit 32 bits, a quarter less
  // traffic per sort pass than 64-bit keys; a span over 32 bits takes one
  // group with 64-bit keys. Each group is expanded, sorted and reduced on
  // its own buffers.
  struct EscGroup {
    EscArgs a;
    u32 *heads, *offc;  // per chunk: run heads, runs before it
    u64 chunks;
    int grid, bits;
  };
  std::vector<EscGroup> escg;
  const u64 esc_span = esc_rows * LB;
  const bool esc_k32 = esc_span <= 0xFFFFFFFFull;
  // Expanded tiles are reduced in shared memory (one set of launches, keys
  // local to a window or a tile) when a tile spans at most kBinMaxBlocks key
  // blocks and the padded pairs count in 32 bits; otherwise they are sorted
  // in groups whose keys fit 32 bits.
  const u32 bin_nb = u32((esc_span + kBinWidth - 1) / kBinWidth);
  const u32 bin_small = opt.esc_small > 0 ? u32(opt.esc_small) : kBinSmallMax;
  const bool binned = nesc > 0 && opt.esc_reduce != 2 && esc_span <= u64(kBinMaxBlocks) * kBinWidth &&
                      esc_pairs + u64(kBinPer) * nesc < 0xFFFFFFFFull;
  BinArgs bins{};
  u32 *bin_bsum = nullptr;
  u32 bin_nblk = 0;
  if (binned) {
    const u64 cap = esc_pairs + u64(kBinPer) * nesc;  // with every tile's padding
    const u64 maxch = esc_pairs / kBinChunk + esc_pairs / (u64(bin_small) + 1) + 1;  // a large tile has > small_max pairs
    bins.n = nesc;
    bins.small_max = bin_small;
    bins.nb = bin_nb;
    bins.span = u32(esc_span);
    bins.LB = u32(LB);
    bins.rows = u32(esc_rows);
    bins.spanm = magic_for(esc_span);
    bins.lbm = magic_for(LB);
    bins.tiles = esc_tiles;
    bins.base = esc_base;
    bins.total = esc_pairs;
    bins.keys = ar.get_n<u32>(cap);
    bins.vals = ar.get_n<u64>(cap);
    u32 *per = ar.get_n<u32>(2 * u64(nesc));
    bins.nch = per;
    bins.small_list = per + nesc;
    u32 *pre = ar.get_n<u32>(3 * (u64(nesc) + 1));
    bins.spp = pre;
    bins.chpre = pre + (u64(nesc) + 1);
    bins.srk = pre + 2 * (u64(nesc) + 1);
    bin_nblk = (nesc + kPrepThreads - 1) / kPrepThreads;
    bin_bsum = ar.get_n<u32>(u64(kPrepVals) * bin_nblk);
    bins.chunk_tile = ar.get_n<u32>(maxch);
    bins.max_windows = cap / kBinWindow + 2;
    bins.first = ar.get_n<u32>(bins.max_windows);
    bins.hist_len = u64(bin_nb) * maxch;
    bins.hist = ar.get_n<u32>(bins.hist_len);
    bins.hpre = ar.get_n<u32>(bins.hist_len + 1);
    bins.bkeys = ar.get_n<u32>(esc_pairs);
    bins.bvals = ar.get_n<u64>(esc_pairs);
    bins.jobs = ar.get_n<BinJob>(u64(bin_nb) * std::min<u64>(nesc, esc_pairs / (u64(bin_small) + 1) + 1));
    bins.njobs = ar.get_n<u32>(2);
    bins.work = bins.njobs + 1;
  }
  if (nesc > 0 && !binned) {
    u64 G = esc_k32 ? std::max<u64>(1, 0xFFFFFFFFull / esc_span) : u64(nesc);
    if (opt.esc_group > 0) G = std::min<u64>(G, u64(opt.esc_group));
    const u32 ng = u32((u64(nesc) + G - 1) / G);
    std::vector<u64> start(ng + 1, 0);
    if (ng > 1) {
      u64 *d_start = ar.get_n<u64>(ng);
      k_esc_group_starts<<<1, 256, 0, st>>>(esc_base, u32(G), ng, d_start);
      FCC_LAUNCH_CHECK();
      FCC_CUDA(cudaMemcpyAsync(start.data(), d_start, sizeof(u64) * ng, cudaMemcpyDeviceToHost, st));
      FCC_CUDA(cudaStreamSynchronize(st));
    }
    start[ng] = esc_pairs;
    for (u32 g = 0; g < ng; g++) {
      const u32 s0 = u32(u64(g) * G), n = u32(std::min<u64>(G, u64(nesc) - s0));
      const u64 pairs = start[g + 1] - start[g];
      EscGroup e{EscArgs{esc_tiles + s0, esc_base + s0, n, esc_span, LB, esc_rows, magic_for(LB), magic_for(esc_rows),
                         start[g], nullptr, nullptr, pairs},
                 nullptr, nullptr, 0, 1, 0};
      e.a.keys = esc_k32 ? static_cast<void *>(ar.get_n<u32>(pairs)) : static_cast<void *>(ar.get_n<u64>(pairs));
      e.a.vals = ar.get_n<u64>(pairs);
      e.chunks = (pairs + kEscChunk - 1) / kEscChunk;
      e.heads = ar.get_n<u32>(e.chunks);
      e.offc = ar.get_n<u32>(e.chunks);
      e.grid = int(std::max<u64>(1, std::min<u64>((e.chunks + 7) / 8, u64(ctx->num_sms) * 8)));
      e.bits = bits_for(u64(n) * esc_span - 1);
      escg.push_back(e);
    }
  }
  const u64 words = dense ? (area + 31) / 32 : 0;
  double *gacc = nullptr;
  u32 *gmask = nullptr;
  u64 *gkeys = nullptr;
  double *gvals = nullptr;
  if (nsplit_d > 0) {
    gacc = ar.get_n<double>(size_t(nsplit_d) * area);
    gmask = ar.get_n<u32>(size_t(nsplit_d) * words);
  }
  if (nsplit_h > 0) {
    gkeys = ar.get_n<u64>(hash_total);
    gvals = ar.get_n<double>(hash_total);
  }
  u64 *item_cyc = want_record ? ar.get_n<u64>(std::max<u32>(nitems, 1)) : nullptr;
  u64 *merge_cyc = want_record ? ar.get_n<u64>(NT) : nullptr;
  if (merge_cyc) FCC_CUDA(cudaMemsetAsync(merge_cyc, 0, sizeof(u64) * NT, st));
  u32 *counters = ar.get_n<u32>(FCC_NUM_CLASSES * kMaxWaves);  // item counters per wave and class
  tm.mark(3);

  // ---- contract + drain ----
  // Dense tiles that the multiply-adds fill well keep -0.0 at untouched
  // positions instead of a touched bitmask (one shared atomic per multiply-add
  // instead of two); it needs inputs without zero or tiny values, which could
  // make a product round to -0.0.
  const bool tiny = (ctx->h_scalars[S_TINY] & 1) != 0;
  const u32 ntiles = scalar32(ctx, S_NTILES);
  const bool sentinel = dense && !tiny && opt.dense_mode != FCC_DENSE_BITMASK &&
                        (opt.dense_mode == FCC_DENSE_SENTINEL || ptotal >= u64(ntiles) * area / 4);
  auto class_smem = [&](int c, u32 hot_n) -> size_t {
    const size_t nw = size_t(hc[c].threads / 32);
    const size_t base = hc[c].hash ? size_t(hc[c].slots) * 16
                                   : ((size_t(area) * 8 + (sentinel ? 0 : size_t(words) * 4) + 15) & ~size_t(15));
    return base + nw * hot_n * 8 + nw * (hot_n / 32) * 4;
  };
  // Per-warp hot columns on request (hot_columns > 0) when the private copies
  // fit next to every tile class in use. Not automatic: measured on the
  // 10M-nonzero Zipf(1.2) benchmark tensor they cost more than the contention
  // they remove, because its heavy segments spread over all columns.
  u32 hot = 0;
  if (hot_try && opt.hot_columns > 0) {
    bool fits = true;
    for (int c = 0; c < FCC_NUM_CLASSES; c++)
      if (ccount[c] && class_smem(c, hot_want) > (hc[c].hash ? smem_cap : dense_dyn_cap)) fits = false;
    if (fits) {
      hot = hot_want;
      if (colb32) k_apply_colmap<u32><<<grid_for(nB, 256), 256, 0, st>>>(static_cast<u32 *>(colB), nB, colmap);
      else k_apply_colmap<u64><<<grid_for(nB, 256), 256, 0, st>>>(static_cast<u64 *>(colB), nB, colmap);
      FCC_LAUNCH_CHECK();
    }
  }
  const ProdSrc src{P, slotA, sbA, valA, valB};
  Decode dec{};
  dec.inv_col = hot ? inv_col : nullptr;
  dec.na = sa.lin.n_ext;
  dec.nb = sb.lin.n_ext;
  for (int e = 0; e < dec.na; e++) dec.ra[e] = sa.lin.ext_radix[e], dec.ma[e] = magic_for(dec.ra[e]);
  for (int e = 0; e < dec.nb; e++) dec.rb[e] = sb.lin.ext_radix[e], dec.mb[e] = magic_for(dec.rb[e]);
  dec.narrow = (sa.span <= 0xFFFFFFFFull && sb.span <= 0xFFFFFFFFull) ? 1 : 0;

  // Output capacity: the planner's upper bound, limited to half of the free
  // device memory (the pool's unused memory included); an overflow is
  // detected on the device and retried once with the exact count (the cursor
  // counts every reservation).
  const size_t free_b = ctx->arena.available();
  const u64 per_out = 8 + 4 * u64(out_order);
  const u64 budget = std::max<u64>(u64(free_b / 2) / per_out, 1 << 20);
  u64 cap = std::max<u64>(std::min(cap_total, budget), 1);
  if (opt.capacity_hint > 0) cap = std::min<u64>(cap, u64(opt.capacity_hint));

  int ctas_per_sm[FCC_NUM_CLASSES] = {};
  const bool caller_out = ctx->caller_out || !ctx->pool;
  if (caller_out) {  // caller buffers: their capacity, no retry
    cap = ctx->out_cap;
    if (cap > 0 && (!ctx->out_vals || (out_order > 0 && (!ctx->out_coords || ctx->out_stride < i64(cap)))))
      throw Error{FCC_ERR_ARG, "output buffers missing or mode stride below the capacity"};
  }
  // A caller output in pinned host memory is produced in device memory and
  // copied out in waves of tiles: the outputs of a wave (a range of the output
  // cursor) cross the host link while the next wave computes, instead of the
  // tile kernels storing across the link themselves (about 0.5 GB per wave).
  bool stream_out = false;
  if (caller_out && ctx->pool && ctx->copy_stream && ctx->wave_ev && ctx->h_cursors && cap > 0) {
    auto pinned_host = [](const void *p) {
      cudaPointerAttributes pa{};
      const bool h = cudaPointerGetAttributes(&pa, p) == cudaSuccess && pa.type == cudaMemoryTypeHost;
      cudaGetLastError();
      return h;
    };
    stream_out = pinned_host(ctx->out_vals) && (out_order == 0 || pinned_host(ctx->out_coords));
  }
  struct StageBufs {  // device copy of a streamed output, freed after its copies
    cudaStream_t st = nullptr, cs = nullptr;
    void *p[2] = {nullptr, nullptr};
    ~StageBufs() {
      if (cs) cudaStreamSynchronize(cs);
      for (void *q : p)
        if (q) cudaFreeAsync(q, st);
    }
  } stage_bufs;
  stage_bufs.st = st;
  if (stream_out) {  // without room for the device copy, the tile kernels store to the host themselves
    try {
      stage_bufs.p[0] = pool_alloc(ctx->pool, sizeof(double) * cap, st);
      if (out_order > 0) stage_bufs.p[1] = pool_alloc(ctx->pool, sizeof(u32) * cap * out_order, st);
      stage_bufs.cs = ctx->copy_stream;
    } catch (const Error &e) {
      if (e.status != FCC_ERR_OOM) throw;
      stream_out = false;
    }
  }
  // One wave (compute, then one copy) unless more are asked for, or, for a
  // large output with out_waves 0, unless the context measured waves faster
  // (WaveTune): the copies of a wave slow the tile kernels running beside
  // them, by a factor that differs from box to box (measured 1.9x to 6x on
  // the contract phase).
  int waves = !stream_out || opt.out_waves <= 0 ? 1 : opt.out_waves;
  const u64 out_bytes = cap * (8 + 4 * u64(out_order));
  WaveTune *wt = stream_out && opt.out_waves == 0 && out_bytes >= kAutoWaveBytes ? ctx->wave_tune : nullptr;
  const int wt_trial = wt && wt->trials < 2 ? wt->trials : -1;
  if (wt) waves = wt_trial == 0 ? 1 : wt_trial == 1 ? kAutoWaves : wt->pick;
  const auto wt_t0 = std::chrono::steady_clock::now();
  for (int attempt = 0;; attempt++) {
    i64 stride = i64(cap);
    if (!caller_out) {
      res->d_vals = static_cast<double *>(pool_alloc(ctx->pool, sizeof(double) * cap, st));
      if (out_order > 0) res->d_coords = static_cast<u32 *>(pool_alloc(ctx->pool, sizeof(u32) * cap * out_order, st));
    } else if (stream_out) {
      res->d_vals = static_cast<double *>(stage_bufs.p[0]);
      res->d_coords = static_cast<u32 *>(stage_bufs.p[1]);
    } else {
      res->d_vals = ctx->out_vals;
      res->d_coords = ctx->out_coords;
      stride = ctx->out_stride;
    }
    res->cap = stride;
    Out o{res->d_coords, stride, res->d_vals, cap, d_sc + S_CURSOR};
    FCC_CUDA(cudaMemsetAsync(d_sc + S_CURSOR, 0, sizeof(u64), st));
    FCC_CUDA(cudaMemsetAsync(counters, 0, sizeof(u32) * FCC_NUM_CLASSES * kMaxWaves, st));
    FCC_CUDA(cudaMemsetAsync(ctx->d_err, 0, sizeof(u32), st));
    if (nsplit_d > 0) {
      FCC_CUDA(cudaMemsetAsync(gacc, 0, sizeof(double) * nsplit_d * area, st));
      FCC_CUDA(cudaMemsetAsync(gmask, 0, sizeof(u32) * nsplit_d * words, st));
    }
    if (nsplit_h > 0) {
      FCC_CUDA(cudaMemsetAsync(gkeys, 0xFF, sizeof(u64) * hash_total, st));
      FCC_CUDA(cudaMemsetAsync(gvals, 0, sizeof(double) * hash_total, st));
    }
    DenseArgs da{items + cbeg[FCC_CLASS_DENSE], ccount[FCC_CLASS_DENSE], counters + FCC_CLASS_DENSE, tile_abeg,
                 tile_rank0, tile_lb, tile_nrows, urow, split_of_tile, split_tiles_d, nsplit_d, src,
                 static_cast<const u32 *>(colB), u32(area), u32(words), hot, gacc, gmask, o, dec, ctx->d_err,
                 item_cyc ? item_cyc + cbeg[FCC_CLASS_DENSE] : nullptr, 0u, merge_cyc};
    if (opt.wait_polls > 0) da.wait_polls = opt.wait_polls;
    da.fault_wait = opt.fault_wait ? 1u : 0u;
    // The rule's dense tiles run one kernel for every tile: dense_kernel, by
    // default the two-phase items with a flat second phase. The learned
    // schedule instead picks per tile between the two pure kernels, two-phase
    // items (FCC_CLASS_DENSE) and flat items (FCC_CLASS_DENSE_FLAT).
    const int dmode = opt.dense_kernel != 0 ? opt.dense_kernel : learned ? 1 : kDefaultDenseMode;
    // Items of class c in wave w: a contiguous slice of the class's items.
    auto wave_items = [&](int c, int w, u32 &lo, u32 &n) {
      lo = u32(u64(ccount[c]) * u64(w) / u64(waves));
      n = u32(u64(ccount[c]) * u64(w + 1) / u64(waves)) - lo;
    };
    // The items of dense class c (FCC_CLASS_DENSE: dense_kernel's items;
    // FCC_CLASS_DENSE_FLAT: flat items) in wave w.
    auto run_dense = [&](int c, int w) {
      u32 lo = 0, n = 0;
      wave_items(c, w, lo, n);
      if (!n) return;
      const int mode = c == FCC_CLASS_DENSE_FLAT ? 2 : dmode;
      da.items = items + cbeg[c] + lo;
      da.nitems = n;
      da.counter = counters + w * FCC_NUM_CLASSES + c;
      da.item_cyc = item_cyc ? item_cyc + cbeg[c] + lo : nullptr;
      da.stage_off = 0;
      const int threads = hc[c].threads;
      size_t smem = class_smem(c, hot);
      // phase 1's staging ring, when it fits beside the tile
      const size_t soff = (smem + 15) & ~size_t(15);
      if (mode != 2 && opt.dense_staging >= 0 && soff + kStageBytes <= dense_dyn_cap) {
        da.stage_off = u32(soff);
        smem = soff + kStageBytes;
      }
      const DenseKernel kern = mode == 2   ? dense_kernel_for<2>(sentinel, threads)
                               : mode == 3 ? dense_kernel_for<3>(sentinel, threads)
                                           : dense_kernel_for<1>(sentinel, threads);
      FCC_CUDA(cudaFuncSetAttribute(reinterpret_cast<const void *>(kern), cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    int(smem)));
      const int grid = grid_tiles(ctx, reinterpret_cast<const void *>(kern), threads, smem, da.nitems,
                                  &ctas_per_sm[c]);
      kern<<<grid, threads, smem, st>>>(da);
      FCC_LAUNCH_CHECK();
    };
    // w >= 0: the hash classes' items of wave w; w < 0: the merges of split
    // tiles and the expanded tiles, after every wave.
    auto run_hash = [&](auto colptr, int w) {
      using ColT = std::remove_const_t<std::remove_pointer_t<decltype(colptr)>>;
      HashArgs<ColT> ha{nullptr, 0, nullptr, tile_rank0, urow, tile_nrows, tile_abeg, split_of_tile, split_tiles_h,
                        nsplit_h, src, colptr, LB, u32(grouped ? std::max<u64>(TL, 2) : TL), 0u, hot, hoff_t,
                        hsz_t, gkeys, gvals, o, dec,
                        ctx->d_err, nullptr, merge_cyc};
      for (int c = FCC_CLASS_HASH_L; c <= FCC_CLASS_HASH_S && w >= 0; c++) {
        u32 lo = 0, n = 0;
        wave_items(c, w, lo, n);
        if (!n) continue;
        ha.items = items + cbeg[c] + lo;
        ha.nitems = n;
        ha.counter = counters + w * FCC_NUM_CLASSES + c;
        ha.slots = hc[c].slots;
        ha.item_cyc = item_cyc ? item_cyc + cbeg[c] + lo : nullptr;
        const int threads = hc[c].threads;
        const size_t smem = class_smem(c, hot);
        const void *kern = threads == 128   ? reinterpret_cast<const void *>(k_contract_hash<ColT, 128>)
                           : threads == 256 ? reinterpret_cast<const void *>(k_contract_hash<ColT, 256>)
                           : threads == 512 ? reinterpret_cast<const void *>(k_contract_hash<ColT, 512>)
                                            : reinterpret_cast<const void *>(k_contract_hash<ColT, 1024>);
        FCC_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem)));
        const int grid = grid_tiles(ctx, kern, threads, smem, ha.nitems, &ctas_per_sm[c]);
        if (threads == 128) k_contract_hash<ColT, 128><<<grid, 128, smem, st>>>(ha);
        else if (threads == 256) k_contract_hash<ColT, 256><<<grid, 256, smem, st>>>(ha);
        else if (threads == 512) k_contract_hash<ColT, 512><<<grid, 512, smem, st>>>(ha);
        else k_contract_hash<ColT, 1024><<<grid, 1024, smem, st>>>(ha);
        FCC_LAUNCH_CHECK();
      }
      if (w >= 0) return;
      if (nsplit_d > 0) {
        k_merge_dense<<<std::min<u32>(nsplit_d, u32(ctx->num_sms) * 2), kMergeThreads, 0, st>>>(da);
        FCC_LAUNCH_CHECK();
      }
      if (nsplit_h > 0) {
        k_merge_hash<ColT><<<std::min<u32>(nsplit_h, u32(ctx->num_sms) * 2), kMergeThreads, 0, st>>>(ha);
        FCC_LAUNCH_CHECK();
      }
      if (binned) {  // expand (the pairs stay for a retry), partition the large tiles, reduce
        if (attempt == 0) {
          const u32 pgrid = bin_nblk;
          k_bin_prep<<<pgrid, kPrepThreads, 0, st>>>(bins, bin_bsum);
          FCC_LAUNCH_CHECK();
          k_bin_prep_totals<<<1, kPrepThreads, 0, st>>>(bins, bin_bsum, pgrid);
          FCC_LAUNCH_CHECK();
          k_bin_prep_add<<<pgrid, kPrepThreads, 0, st>>>(bins, bin_bsum);
          FCC_LAUNCH_CHECK();
          k_bin_index<<<grid_for(i64(std::max<u64>(nesc, bins.max_windows)), 256), 256, 0, st>>>(bins);
          FCC_LAUNCH_CHECK();
          const u64 cap = esc_pairs + u64(kBinPer) * nesc;
          const u32 xgrid = u32(std::max<u64>(1, std::min<u64>((cap + 2047) / 2048, u64(ctx->num_sms) * 16)));
          k_bin_expand<ColT><<<xgrid, 256, 0, st>>>(bins, src, colptr, tile_abeg);
          FCC_LAUNCH_CHECK();
          FCC_CUDA(cudaMemsetAsync(bins.hist, 0, sizeof(u32) * bins.hist_len, st));
          const int cgrid = ctx->num_sms * 8;
          k_bin_count<ColT><<<cgrid, 256, 0, st>>>(bins, src, colptr, tile_abeg);
          FCC_LAUNCH_CHECK();
          scan_exclusive(bins.hist, bins.hpre, i64(bins.hist_len), bins.hpre + bins.hist_len, ar, st);
          k_bin_place<ColT><<<cgrid, 256, 0, st>>>(bins, src, colptr, tile_abeg);
          FCC_LAUNCH_CHECK();
          FCC_CUDA(cudaMemsetAsync(bins.njobs, 0, sizeof(u32), st));
          k_bin_jobs<<<grid_for(nesc, 256), 256, 0, st>>>(bins);
          FCC_LAUNCH_CHECK();
        }
        FCC_CUDA(cudaMemsetAsync(bins.work, 0, sizeof(u32), st));  // (a retry runs the reduction again)
        FCC_CUDA(cudaFuncSetAttribute(k_bin_reduce, cudaFuncAttributeMaxDynamicSharedMemorySize, int(kBinSmem)));
        k_bin_reduce<<<ctx->num_sms * 2, kBinThreads, kBinSmem, st>>>(bins, tile_rank0, urow, o, dec, ctx->d_err);
        FCC_LAUNCH_CHECK();
      }
      for (const EscGroup &e : escg) {  // expanded tiles: expand, sort, reduce, group by group
        const EscArgs &ea = e.a;
        if (attempt == 0) {  // the sorted pairs stay for a retry
          const u32 xgrid = u32(std::max<u64>(1, std::min<u64>((ea.total + 2047) / 2048, u64(ctx->num_sms) * 8)));
          if (esc_k32) {
            k_esc_expand<ColT, u32><<<xgrid, 256, 0, st>>>(ea, src, colptr, tile_abeg);
            FCC_LAUNCH_CHECK();
            radix_sort_pairs64(static_cast<u32 *>(ea.keys), ea.vals, i64(ea.total), e.bits, ar, st, ctx->d_err);
          } else {
            k_esc_expand<ColT, u64><<<xgrid, 256, 0, st>>>(ea, src, colptr, tile_abeg);
            FCC_LAUNCH_CHECK();
            radix_sort_pairs64(static_cast<u64 *>(ea.keys), ea.vals, i64(ea.total), e.bits, ar, st, ctx->d_err);
          }
        }
        if (esc_k32) k_esc_count<u32><<<e.grid, 256, 0, st>>>(ea, e.heads);
        else k_esc_count<u64><<<e.grid, 256, 0, st>>>(ea, e.heads);
        FCC_LAUNCH_CHECK();
        scan_exclusive(e.heads, e.offc, i64(e.chunks), sc32(S_ESC_RUNS), ar, st);
        k_esc_reserve<<<1, 32, 0, st>>>(o, sc32(S_ESC_RUNS), d_sc + S_ESC_BASE, ctx->d_err);
        FCC_LAUNCH_CHECK();
        if (esc_k32) k_esc_reduce<u32><<<e.grid, 256, 0, st>>>(ea, e.offc, d_sc + S_ESC_BASE, tile_rank0, urow, o, dec);
        else k_esc_reduce<u64><<<e.grid, 256, 0, st>>>(ea, e.offc, d_sc + S_ESC_BASE, tile_rank0, urow, o, dec);
        FCC_LAUNCH_CHECK();
      }
    };
    auto snapshot = [&](int w) {  // the output cursor after wave w, for the host's copies
      FCC_CUDA(cudaMemcpyAsync(ctx->h_cursors + w, d_sc + S_CURSOR, sizeof(u64), cudaMemcpyDeviceToHost, st));
      FCC_CUDA(cudaEventRecord(ctx->wave_ev[w], st));
    };
    for (int w = 0; w < waves; w++) {
      run_dense(FCC_CLASS_DENSE, w);
      run_dense(FCC_CLASS_DENSE_FLAT, w);
      if (colb32) run_hash(static_cast<const u32 *>(colB), w);
      else run_hash(static_cast<const u64 *>(colB), w);
      if (stream_out) snapshot(w);
    }
    tm.mark(4);
    if (colb32) run_hash(static_cast<const u32 *>(colB), -1);
    else run_hash(static_cast<const u64 *>(colB), -1);
    if (stream_out) snapshot(waves);
    tm.mark(5);
    if (stream_out) {  // copy each finished range while later waves run
      u64 prev = 0;
      for (int w = 0; w <= waves; w++) {
        FCC_CUDA(cudaEventSynchronize(ctx->wave_ev[w]));
        const u64 cur = std::min<u64>(ctx->h_cursors[w], cap);
        if (cur <= prev) continue;
        const size_t n = size_t(cur - prev);
        for (int m = 0; m < out_order; m++)
          FCC_CUDA(cudaMemcpyAsync(ctx->out_coords + i64(m) * ctx->out_stride + prev, res->d_coords + i64(m) * stride + prev,
                                   sizeof(u32) * n, cudaMemcpyDeviceToHost, ctx->copy_stream));
        FCC_CUDA(cudaMemcpyAsync(ctx->out_vals + prev, res->d_vals + prev, sizeof(double) * n, cudaMemcpyDeviceToHost,
                                 ctx->copy_stream));
        prev = cur;
      }
      FCC_CUDA(cudaStreamSynchronize(ctx->copy_stream));
      res->d_vals = ctx->out_vals;
      res->d_coords = ctx->out_coords;
      res->cap = ctx->out_stride;
    }
    read_scalars(ctx, d_sc);
    const u64 produced = ctx->h_scalars[S_CURSOR];
    const bool overflow = (u32(ctx->h_scalars[S_ERR]) & ERRB_OVERFLOW) != 0 || produced > cap;
    if (!overflow) {
      res->nnz = i64(produced);
      if (wt_trial >= 0) {  // a measured trial of the wave choice
        wt->ms[wt_trial] = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - wt_t0).count();
        if (++wt->trials == 2) wt->pick = wt->ms[1] < wt->ms[0] ? kAutoWaves : 1;
      }
      break;
    }
    if (caller_out) {
      res->nnz = i64(produced);  // tells the caller the capacity it needs
      throw Error{FCC_ERR_CAPACITY, "the output needs " + std::to_string(produced) + " entries, the buffers hold " +
                                        std::to_string(cap)};
    }
    if (attempt >= 1) throw Error{FCC_ERR_CUDA, "output count changed between attempts"};
    free_result_buffers(res, st);
    cap = produced;
    tm.next = 4;  // re-time the contraction
  }
  if (ctx->sched) {  // per-tile record for fcc_sched_last_tiles
    SchedIo &io = *ctx->sched;
    io.ntiles = ntiles;
    io.features = feat;
    io.cls = cls;
    io.cost = nullptr;
    if (want_record && ntiles > 0) {
      double *cost = ar.get_n<double>(ntiles);
      double occ[FCC_NUM_CLASSES];
      for (int c = 0; c < FCC_NUM_CLASSES; c++) occ[c] = ctas_per_sm[c] > 0 ? double(ctas_per_sm[c]) : 1.0;
      // merges run up to two CTAs per SM (grid <= 2 x SMs)
      tile_costs(st, ntiles, corder, cls, item_off, t_items, item_cyc, occ, merge_cyc, 2.0, cost);
      FCC_CUDA(cudaStreamSynchronize(st));
      io.cost = cost;
    }
  }
  tm.finish();
  cleanup.done = true;
}

}  // namespace fcc
