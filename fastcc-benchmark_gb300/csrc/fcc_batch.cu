// fcc_contract_batch (include/fastcc_gpu.h): many independent contractions of
// one mode pattern, A[t] x B[t], run as ONE contraction of the concatenated
// operands with an instance key.
//
//   A_cat mode order: [t, A modes..., t]   (t first: an external mode, so it
//                                            leads the output coordinates;
//                                            t last: contracted)
//   B_cat mode order: [B modes..., t]      (t contracted)
//   ctrA_cat = [dA+1, ctrA+1...], ctrB_cat = [dB, ctrB...]
//
// The contraction key then starts with the instance, so A[t] only meets
// B[t], and output rows (t, A external) of different instances never mix.
// Every instance's index build, tiles and drain run in the one pipeline of
// fcc_contract: one set of launches and host read-backs for the batch, and
// one persistent tile-kernel launch whose work queue holds the output tiles
// of all instances. Per-mode radices are the maxima over the batch, shared by
// both operands (FCC_RADIX_SHARED semantics).

#include <algorithm>
#include <vector>

#include "fcc_internal.cuh"

namespace fcc {

void contract(Runtime *ctx, const fcc_tensor *A, const fcc_tensor *B, const int32_t *ctrA,
              const int32_t *ctrB, int k, const fcc_options &opt, fcc_result *res, i64 *products,
              bool count_only, const u32 *group_lb, u32 ngroups);

namespace {

struct PackSrc {  // one instance of one operand
  const int32_t *coords;
  const double *values;  // NULL: already copied into place
  i64 sn, sm;
  i64 nnz, offset;  // rows [offset, offset + nnz) of the concatenation
  int32_t max_index[FCC_MAX_ORDER];
};

// SoA concatenation: out[m * total + row]. Instance columns are written at
// `inst_first` (mode 0, or -1 for none) and `inst_last` (the last mode).
__global__ void k_batch_pack(const PackSrc *__restrict__ src, int n, int order, i64 total, int shift,
                             int inst_first, int inst_last, int32_t *__restrict__ out,
                             double *__restrict__ vals) {
  for (i64 r = i64(blockIdx.x) * blockDim.x + threadIdx.x; r < total; r += i64(gridDim.x) * blockDim.x) {
    int lo = 0, hi = n;  // instance: last with offset <= r
    while (hi - lo > 1) {
      const int mid = (lo + hi) >> 1;
      if (src[mid].offset <= r) lo = mid; else hi = mid;
    }
    const PackSrc &s = src[lo];
    const i64 i = r - s.offset;
    for (int m = 0; m < order; m++) {
      const int32_t v = s.coords[i * s.sn + m * s.sm];
      // outside the instance's own bounds: -1, which the contraction's
      // coordinate check reports (its error word is reset after this kernel)
      out[i64(m + shift) * total + r] = (v < 0 || v > s.max_index[m]) ? -1 : v;
    }
    if (s.values) vals[r] = s.values[i];
    if (inst_first >= 0) out[i64(inst_first) * total + r] = lo;
    out[i64(inst_last) * total + r] = lo;
  }
}

// Entries per instance (mode 0 of the batched result). Warps take contiguous
// runs of entries: the tile kernels write each tile's entries together and a
// tile belongs to one instance, so a run usually holds one instance, counted
// in a register and added once when the run ends (one atomic per warp and
// instance instead of one per 32 entries on a few hot counters).
__global__ void k_instance_counts(const u32 *__restrict__ inst, i64 n, unsigned long long *counts) {
  const u32 lane = threadIdx.x & 31;
  const i64 nw = (i64(gridDim.x) * blockDim.x) >> 5, w = (i64(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
  const i64 per = (n + nw - 1) / nw, lo = w * per, hi = min(n, lo + per);
  u32 cur = 0xFFFFFFFFu;       // the run's instance (warp-uniform)
  unsigned long long cnt = 0;  // its entries so far (lane 0)
  for (i64 base = lo; base < hi; base += 32) {
    const i64 i = base + lane;
    const bool in = i < hi;
    const u32 t = in ? inst[i] : 0xFFFFFFFEu;  // lanes past the run match no instance
    const u32 valid = __ballot_sync(kFull, in);  // every lane takes part in the vote
    if (__all_sync(kFull, !in || t == cur)) {
      if (lane == 0) cnt += __popc(valid);
      continue;
    }
    if (lane == 0 && cnt) atomicAdd(&counts[cur], cnt);
    cnt = 0;
    // the last valid lane's instance continues as the run; other groups are added now
    const u32 last = 31 - __clz(valid);
    const u32 tl = __shfl_sync(kFull, t, last);
    const u32 peers = __match_any_sync(kFull, t);
    const bool leader = in && lane == u32(__ffs(peers) - 1);
    if (leader && t != tl) atomicAdd(&counts[t], (unsigned long long)__popc(peers));
    const u32 run = __shfl_sync(kFull, __popc(peers), last);
    cur = tl;
    if (lane == 0) cnt = run;
  }
  if (lane == 0 && cnt) atomicAdd(&counts[cur], cnt);
}

struct Concat {
  int32_t *coords = nullptr;
  double *values = nullptr;
  std::vector<int32_t> max_index;
  i64 total = 0;
};

void concat_operand(Runtime *ctx, int n, const fcc_tensor *T, int shift, int inst_first, int inst_last,
                    int order_out, Concat &c, std::vector<void *> &frees) {
  cudaStream_t st = ctx->stream;
  const int order = T[0].order;
  std::vector<PackSrc> src(static_cast<size_t>(n));
  c.max_index.assign(size_t(order_out), 0);
  i64 total = 0;
  for (int t = 0; t < n; t++) {
    const fcc_tensor &x = T[t];
    if (x.order != order) throw Error{FCC_ERR_ARG, "batch operands differ in order"};
    if (x.nnz < 0 || (x.nnz > 0 && (!x.coords || !x.values || !x.max_index)))
      throw Error{FCC_ERR_ARG, "batch operand without coords, values or max_index"};
    if (x.location != FCC_HOST && x.location != FCC_DEVICE) throw Error{FCC_ERR_ARG, "bad location"};
    PackSrc &s = src[size_t(t)];
    s.sn = x.stride_nnz;
    s.sm = x.stride_mode;
    s.nnz = x.nnz;
    s.offset = total;
    for (int m = 0; m < order; m++) {  // an empty instance may leave max_index NULL
      s.max_index[m] = x.max_index ? x.max_index[m] : 0;
      c.max_index[size_t(m + shift)] = std::max(c.max_index[size_t(m + shift)], s.max_index[m]);
    }
    total += x.nnz;
  }
  if (total > 0x7FFFFFFFll) throw Error{FCC_ERR_ARG, "batch holds more than 2^31-1 nonzeros per operand"};
  c.total = total;
  if (inst_first >= 0) c.max_index[size_t(inst_first)] = n - 1;
  c.max_index[size_t(inst_last)] = n - 1;
  if (total == 0) return;
  void *p = nullptr;
  p = pool_alloc(ctx->pool, sizeof(int32_t) * size_t(total) * order_out, st);
  frees.push_back(p);
  c.coords = static_cast<int32_t *>(p);
  p = pool_alloc(ctx->pool, sizeof(double) * size_t(total), st);
  frees.push_back(p);
  c.values = static_cast<double *>(p);
  // host instances: coordinates staged in one pooled buffer, values copied
  // straight into place; device instances are read by the pack kernel
  i64 host_elems = 0;
  for (int t = 0; t < n; t++)
    if (T[t].location == FCC_HOST && T[t].nnz > 0)
      host_elems += (T[t].nnz - 1) * T[t].stride_nnz + i64(order - 1) * T[t].stride_mode + 1;
  int32_t *stage = nullptr;
  if (host_elems > 0) {
    p = pool_alloc(ctx->pool, sizeof(int32_t) * size_t(host_elems), st);
    frees.push_back(p);
    stage = static_cast<int32_t *>(p);
  }
  i64 so = 0;
  for (int t = 0; t < n; t++) {
    const fcc_tensor &x = T[t];
    PackSrc &s = src[size_t(t)];
    s.coords = x.coords;
    s.values = x.values;
    if (x.nnz == 0 || x.location != FCC_HOST) continue;
    FCC_CUDA(cudaMemcpyAsync(c.values + s.offset, x.values, sizeof(double) * size_t(x.nnz),
                             cudaMemcpyHostToDevice, st));
    s.values = nullptr;
    {
      const i64 ext = (x.nnz - 1) * x.stride_nnz + i64(order - 1) * x.stride_mode + 1;
      FCC_CUDA(cudaMemcpyAsync(stage + so, x.coords, sizeof(int32_t) * size_t(ext), cudaMemcpyHostToDevice, st));
      s.coords = stage + so;
      so += ext;
    }
  }
  p = pool_alloc(ctx->pool, sizeof(PackSrc) * size_t(n), st);
  frees.push_back(p);
  PackSrc *dsrc = static_cast<PackSrc *>(p);
  FCC_CUDA(cudaMemcpyAsync(dsrc, src.data(), sizeof(PackSrc) * size_t(n), cudaMemcpyHostToDevice, st));
  k_batch_pack<<<grid_for(total, 256), 256, 0, st>>>(dsrc, n, order, total, shift, inst_first, inst_last,
                                                     c.coords, c.values);
  FCC_LAUNCH_CHECK();
  // the staging buffer and the table are freed behind the pack kernel on the
  // same stream; the pageable copy of `src` has been staged on return
}

}  // namespace

void contract_batch(Runtime *ctx, int n, const fcc_tensor *A, const fcc_tensor *B, const int32_t *ctrA,
                    const int32_t *ctrB, int k, const fcc_options &opt, fcc_result *res, i64 *counts) {
  if (n < 1 || !A || !B) throw Error{FCC_ERR_ARG, "empty batch"};
  if (!ctx->pool) throw Error{FCC_ERR_ARG, "batched contraction needs a context"};
  const int dA = A[0].order, dB = B[0].order;
  if (dA < 0 || dB < 0 || dA + 2 > FCC_MAX_ORDER || dB + 1 > FCC_MAX_ORDER)
    throw Error{FCC_ERR_ARG, "batch operands need order(A) <= 6 and order(B) <= 7"};
  if (k < 0 || k > dA || k > dB || (k > 0 && (!ctrA || !ctrB))) throw Error{FCC_ERR_ARG, "bad contracted modes"};
  std::vector<void *> frees;
  struct FreeAll {
    std::vector<void *> &f;
    cudaStream_t s;
    ~FreeAll() {
      for (void *p : f) cudaFreeAsync(p, s);
    }
  } free_all{frees, ctx->stream};
  Concat ca, cb;
  concat_operand(ctx, n, A, 1, 0, dA + 1, dA + 2, ca, frees);
  concat_operand(ctx, n, B, 0, -1, dB, dB + 1, cb, frees);
  std::vector<int32_t> cA(size_t(k) + 1), cB(size_t(k) + 1);
  cA[0] = dA + 1;
  cB[0] = dB;
  for (int i = 0; i < k; i++) {
    if (ctrA[i] < 0 || ctrA[i] >= dA || ctrB[i] < 0 || ctrB[i] >= dB)
      throw Error{FCC_ERR_ARG, "contracted mode out of range"};
    cA[size_t(i) + 1] = ctrA[i] + 1;
    cB[size_t(i) + 1] = ctrB[i];
  }
  fcc_tensor TA{dA + 2, ca.total, ca.max_index.data(), ca.coords, 1, ca.total, ca.values, FCC_DEVICE};
  fcc_tensor TB{dB + 1, cb.total, cb.max_index.data(), cb.coords, 1, cb.total, cb.values, FCC_DEVICE};
  // Instance t's column span: its largest B external column (linearised with
  // the batch's radices) + 1. Dense tiles of t are that wide, not as wide as
  // the widest instance.
  std::vector<u32> glb(static_cast<size_t>(n));
  std::vector<char> bctr(static_cast<size_t>(dB), 0);
  for (int i = 0; i < k; i++) bctr[size_t(ctrB[i])] = 1;
  for (int t = 0; t < n; t++) {
    unsigned __int128 col = 0;
    for (int m = 0; m < dB; m++)
      if (!bctr[size_t(m)]) col = col * (u64(cb.max_index[size_t(m)]) + 1) + u64(B[t].max_index ? std::max(B[t].max_index[m], 0) : 0);
    glb[size_t(t)] = u32(std::min<unsigned __int128>(col + 1, 0xFFFFFFFFu));
  }
  fcc_options o = opt;
  o.radix_mode = FCC_RADIX_SHARED;
  contract(ctx, &TA, &TB, cA.data(), cB.data(), k + 1, o, res, nullptr, false, glb.data(), u32(n));
  if (counts) {
    unsigned long long *dc = nullptr;
    void *p = nullptr;
    p = pool_alloc(ctx->pool, sizeof(unsigned long long) * size_t(n), ctx->stream);
    frees.push_back(p);
    dc = static_cast<unsigned long long *>(p);
    FCC_CUDA(cudaMemsetAsync(dc, 0, sizeof(unsigned long long) * size_t(n), ctx->stream));
    if (res->nnz > 0) {
      k_instance_counts<<<std::max(ctx->num_sms, 1) * 8, 256, 0, ctx->stream>>>(res->d_coords, res->nnz, dc);
      FCC_LAUNCH_CHECK();
    }
    FCC_CUDA(cudaMemcpyAsync(counts, dc, sizeof(unsigned long long) * size_t(n), cudaMemcpyDeviceToHost,
                             ctx->stream));
    FCC_CUDA(cudaStreamSynchronize(ctx->stream));
  }
}

}  // namespace fcc

// ---- batch modes inside one contraction ----
//
// fcc_contract_modes: modes shared by A and B that stay in the output, as in
// the reference's Tensor<DT>::multiply(other, left_contr, left_batch,
// right_contr, right_batch) (contract.hpp:284-367), whose output coordinate is
// (batch coordinates in left_batch order, A's external modes, B's external
// modes). Run as one contraction of
//   A' = [A's batch modes in batchA order, A's modes...]
// with ctrA' = [nb + batchA..., nb + ctrA...] and ctrB' = [batchB..., ctrB...]:
// A' has the batch copies as its leading external modes, and the batch modes
// join the contraction key so only equal batch coordinates meet.

namespace fcc {
namespace {

struct ModeSrc {
  int m[FCC_MAX_ORDER];
};
__global__ void k_gather_modes_v(const int32_t *__restrict__ coords, i64 sn, i64 sm, i64 nnz, int order_out,
                                 ModeSrc src, int32_t *__restrict__ out) {
  for (i64 r = i64(blockIdx.x) * blockDim.x + threadIdx.x; r < nnz; r += i64(gridDim.x) * blockDim.x)
    for (int m = 0; m < order_out; m++) out[i64(m) * nnz + r] = coords[r * sn + i64(src.m[m]) * sm];
}

}  // namespace

void contract_modes(Runtime *ctx, const fcc_tensor *A, const fcc_tensor *B, const int32_t *ctrA,
                    const int32_t *ctrB, int k, const int32_t *batchA, const int32_t *batchB, int nb,
                    const fcc_options &opt, fcc_result *res) {
  if (!A || !B) throw Error{FCC_ERR_ARG, "null operand"};
  if (nb < 0 || (nb > 0 && (!batchA || !batchB))) throw Error{FCC_ERR_ARG, "bad batch modes"};
  if (k < 0 || (k > 0 && (!ctrA || !ctrB))) throw Error{FCC_ERR_ARG, "bad contracted modes"};
  const int dA = A->order, dB = B->order;
  if (dA + nb > FCC_MAX_ORDER) throw Error{FCC_ERR_ARG, "order(A) + batch modes exceeds FCC_MAX_ORDER"};
  if (A->nnz < 0 || (A->nnz > 0 && (!A->coords || !A->values)) || !A->max_index)
    throw Error{FCC_ERR_ARG, "A without coords, values or max_index"};
  for (int i = 0; i < nb; i++) {
    if (batchA[i] < 0 || batchA[i] >= dA || batchB[i] < 0 || batchB[i] >= dB)
      throw Error{FCC_ERR_ARG, "batch mode out of range"};
    for (int j = 0; j < k; j++)
      if (ctrA[j] == batchA[i] || ctrB[j] == batchB[i])
        throw Error{FCC_ERR_ARG, "a mode is both contracted and batch"};
  }
  std::vector<void *> frees;
  struct FreeAll {
    std::vector<void *> &f;
    cudaStream_t s;
    ~FreeAll() {
      for (void *p : f) cudaFreeAsync(p, s);
    }
  } free_all{frees, ctx->stream};
  cudaStream_t st = ctx->stream;
  const int dA2 = dA + nb;
  ModeSrc src{};
  std::vector<int32_t> mx(static_cast<size_t>(dA2));
  for (int i = 0; i < nb; i++) src.m[i] = batchA[i];
  for (int m = 0; m < dA; m++) src.m[nb + m] = m;
  for (int m = 0; m < dA2; m++) mx[size_t(m)] = A->max_index[src.m[m]];
  const i64 n = A->nnz;
  int32_t *coords = nullptr;
  const double *vals = A->values;
  if (n > 0) {
    const int32_t *cin = A->coords;
    if (A->location == FCC_HOST) {  // stage host operands on the device
      const i64 ext = (n - 1) * A->stride_nnz + i64(dA - 1) * A->stride_mode + 1;
      void *p = pool_alloc(ctx->pool, sizeof(int32_t) * size_t(ext), st);
      frees.push_back(p);
      FCC_CUDA(cudaMemcpyAsync(p, A->coords, sizeof(int32_t) * size_t(ext), cudaMemcpyHostToDevice, st));
      cin = static_cast<const int32_t *>(p);
      p = pool_alloc(ctx->pool, sizeof(double) * size_t(n), st);
      frees.push_back(p);
      FCC_CUDA(cudaMemcpyAsync(p, A->values, sizeof(double) * size_t(n), cudaMemcpyHostToDevice, st));
      vals = static_cast<const double *>(p);
    }
    void *p = pool_alloc(ctx->pool, sizeof(int32_t) * size_t(n) * dA2, st);
    frees.push_back(p);
    coords = static_cast<int32_t *>(p);
    k_gather_modes_v<<<grid_for(n, 256), 256, 0, st>>>(cin, A->stride_nnz, A->stride_mode, n, dA2, src, coords);
    FCC_LAUNCH_CHECK();
  }
  fcc_tensor TA{dA2, n, mx.data(), coords, 1, n, vals, FCC_DEVICE};
  std::vector<int32_t> cA(size_t(nb + k)), cB(size_t(nb + k));
  for (int i = 0; i < nb; i++) cA[size_t(i)] = nb + batchA[i], cB[size_t(i)] = batchB[i];
  for (int i = 0; i < k; i++) cA[size_t(nb + i)] = nb + ctrA[i], cB[size_t(nb + i)] = ctrB[i];
  contract(ctx, &TA, B, cA.data(), cB.data(), nb + k, opt, res, nullptr, false, nullptr, 0);
}

}  // namespace fcc
