// Tile scheduling: per-tile features, the cost model's inference inside the
// planner, measured per-tile costs, and the FP32 MLP's training kernels
// (forward, backward, weight gradients, Adam). Nothing here touches the
// contraction's values: the schedule only picks which tile kernel runs a
// tile, and every class computes the same sums.
//
// Model layout (include/fastcc_gpu.h): mean[12] scale[12] W1[12][64] b1[64]
// W2[64][64] b2[64] W3[64][FCC_NUM_CLASSES] b3[FCC_NUM_CLASSES], row-major
// (input index first).

#include <algorithm>
#include <cmath>
#include <numeric>
#include <random>
#include <vector>

#include "fcc_internal.cuh"

namespace fcc {
namespace {

constexpr int kF = FCC_SCHED_FEATURES;  // 12
constexpr int kH = FCC_SCHED_HIDDEN;    // 64
constexpr int kO = FCC_NUM_CLASSES;
constexpr int kMean = 0, kScale = kF, kW1 = 2 * kF, kB1 = kW1 + kF * kH, kW2 = kB1 + kH, kB2 = kW2 + kH * kH,
              kW3 = kB2 + kH, kB3 = kW3 + kH * kO, kTotal = kB3 + kO;
static_assert(kTotal == FCC_SCHED_MODEL_FLOATS, "model layout");
constexpr int kTrain0 = kW1;  // trainable parameters start after mean and scale

// ---- per-tile features ----
//
// Two passes. k_tile_sums: warps take contiguous runs of A entries (tiles are
// contiguous runs of entries, so a warp sees few tiles), sum per tile the
// multiply-adds of entries whose B segment is short (< 64), medium or long
// (>= 1024) and the longest segment, in registers while the tile lasts, and
// add them into the tile's row of `feat` (its first 32 bytes, as four u64)
// with one set of atomics per tile and warp. A tile of a million entries is
// shared by many warps instead of one. k_tile_features then turns each row
// into the 12 FP32 features in place. Integer sums and FP32 logarithms: FP64
// issues at 1/64 of FP32 on this GPU.
constexpr int kRowU64 = kF / 2;  // a feature row holds 12 floats = 6 u64

__device__ __forceinline__ u32 tile_of(const u32 *__restrict__ abeg, u32 ntiles, u32 e) {
  u32 lo = 0, hi = ntiles;  // last tile t with abeg[t] <= e
  while (hi - lo > 1) {
    const u32 mid = (lo + hi) >> 1;
    if (abeg[mid] <= e) lo = mid; else hi = mid;
  }
  return lo;
}

__global__ void k_tile_sums(const u32 *__restrict__ ntiles_p, u32 nmax, const u32 *__restrict__ abeg,
                            const u64 *__restrict__ P, unsigned long long *__restrict__ acc) {
  const u32 ntiles = min(*ntiles_p, nmax);
  if (ntiles == 0) return;
  const u32 lane = threadIdx.x & 31;
  const u64 nw = (u64(gridDim.x) * blockDim.x) >> 5, w = (u64(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
  const u32 e_first = abeg[0], e_last = abeg[ntiles];
  const u64 per = (u64(e_last - e_first) + nw - 1) / nw;
  const u64 lo64 = u64(e_first) + w * per;
  if (lo64 >= e_last) return;
  const u32 lo = u32(lo64), hi = u32(lo64 + per < u64(e_last) ? lo64 + per : u64(e_last));
  u32 t = tile_of(abeg, ntiles, lo), tend = abeg[t + 1];
  u64 sl = 0, sw = 0, sc = 0, mx = 0;  // this lane's part of tile t
  auto flush = [&]() {
    for (int o = 16; o; o >>= 1) {
      sl += __shfl_xor_sync(kFull, (unsigned long long)sl, o);
      sw += __shfl_xor_sync(kFull, (unsigned long long)sw, o);
      sc += __shfl_xor_sync(kFull, (unsigned long long)sc, o);
      mx = max(mx, (u64)__shfl_xor_sync(kFull, (unsigned long long)mx, o));
    }
    if (lane == 0 && (sl | sw | sc | mx)) {
      unsigned long long *a = acc + size_t(t) * kRowU64;
      if (sl) atomicAdd(&a[0], (unsigned long long)sl);
      if (sw) atomicAdd(&a[1], (unsigned long long)sw);
      if (sc) atomicAdd(&a[2], (unsigned long long)sc);
      atomicMax(&a[3], (unsigned long long)mx);
    }
    sl = sw = sc = mx = 0;
  };
  for (u32 base = lo; base < hi; base += 32) {
    const u32 e = base + lane;
    const bool in = e < hi;
    const u64 len = in ? P[e + 1] - P[e] : 0;
    bool left = in;  // not yet added to a tile
    for (;;) {
      if (left && e < tend) {
        if (len < 64) sl += len;
        else if (len < 1024) sw += len;
        else sc += len;
        mx = max(mx, len);
        left = false;
      }
      const u32 rest = __ballot_sync(kFull, left);
      if (!rest) break;
      flush();  // tile t ends inside this round: move on to the next lane's tile
      const u32 enext = __shfl_sync(kFull, e, __ffs(rest) - 1);
      t = tile_of(abeg, ntiles, enext);
      tend = abeg[t + 1];
    }
  }
  flush();
}

__global__ void k_tile_features(const u32 *__restrict__ ntiles_p, u32 nmax, const u32 *__restrict__ abeg,
                                const u64 *__restrict__ P, const u32 *__restrict__ nrows, const u32 *__restrict__ lb,
                                u64 LB, float *__restrict__ feat) {
  const u32 ntiles = min(*ntiles_p, nmax);
  for (u32 t = blockIdx.x * blockDim.x + threadIdx.x; t < ntiles; t += gridDim.x * blockDim.x) {
    float *f = feat + size_t(t) * kF;
    const unsigned long long *a = reinterpret_cast<const unsigned long long *>(f);
    const u64 sl = a[0], sw = a[1], sc = a[2], mx = a[3];
    const u32 e0 = abeg[t], e1 = abeg[t + 1];
    const u64 prodi = P[e1] - P[e0];
    const float prod = float(prodi), nent = float(e1 - e0), rows = float(nrows[t]);
    const float span = float(lb ? u64(lb[t]) : LB), area = rows * span;
    const float pd = prodi > 0 ? prod : 1.f;
    f[0] = log2f(1.f + prod);
    f[1] = log2f(1.f + nent);
    f[2] = log2f(rows);
    f[3] = log2f(span);
    f[4] = log2f(area);
    f[5] = fminf(prod, area) / area;
    f[6] = float(sl) / pd;
    f[7] = float(sw) / pd;
    f[8] = float(sc) / pd;
    f[9] = log2f(1.f + prod / fmaxf(nent, 1.f));
    f[10] = log2f(1.f + float(mx));
    f[11] = log2f(1.f + prod / rows);
  }
}

// ---- MLP ----
__device__ __forceinline__ void load_model(const float *__restrict__ model, float *s) {
  for (int i = threadIdx.x; i < kTotal; i += blockDim.x) s[i] = model[i];
  __syncthreads();
}

// y = MLP(x) for one row; optionally keeps the standardised input and both
// hidden activations (after ReLU).
__device__ __forceinline__ void mlp_row(const float *s, const float *x_raw, float *y, float *xs_out, float *a1_out,
                                        float *a2_out) {
  float x[kF];
#pragma unroll
  for (int i = 0; i < kF; i++) {
    x[i] = (x_raw[i] - s[kMean + i]) * s[kScale + i];
    if (xs_out) xs_out[i] = x[i];
  }
  float h1[kH];
#pragma unroll
  for (int j = 0; j < kH; j++) {
    float z = s[kB1 + j];
#pragma unroll
    for (int i = 0; i < kF; i++) z = fmaf(x[i], s[kW1 + i * kH + j], z);
    h1[j] = fmaxf(z, 0.f);
    if (a1_out) a1_out[j] = h1[j];
  }
  float out[kO];
#pragma unroll
  for (int k = 0; k < kO; k++) out[k] = s[kB3 + k];
  for (int j = 0; j < kH; j++) {
    float z = s[kB2 + j];
#pragma unroll
    for (int i = 0; i < kH; i++) z = fmaf(h1[i], s[kW2 + i * kH + j], z);
    const float a = fmaxf(z, 0.f);
    if (a2_out) a2_out[j] = a;
#pragma unroll
    for (int k = 0; k < kO; k++) out[k] = fmaf(a, s[kW3 + j * kO + k], out[k]);
  }
#pragma unroll
  for (int k = 0; k < kO; k++) y[k] = out[k];
}

// Rows [0, n) (n read from n_dev when given): Y = MLP(X).
__global__ void __launch_bounds__(128) k_mlp_predict(const u32 *__restrict__ n_dev, u32 n_max,
                                                     const float *__restrict__ X, const float *__restrict__ model,
                                                     float *__restrict__ Y) {
  __shared__ float s[kTotal];
  load_model(model, s);
  const u32 n = n_dev ? min(*n_dev, n_max) : n_max;
  for (u32 r = blockIdx.x * blockDim.x + threadIdx.x; r < n; r += gridDim.x * blockDim.x)
    mlp_row(s, X + size_t(r) * kF, Y + size_t(r) * kO, nullptr, nullptr, nullptr);
}

// Training forward: keeps Xs (standardised input), A1, A2 and the outputs.
__global__ void __launch_bounds__(128) k_mlp_forward(u32 n, const float *__restrict__ X,
                                                     const float *__restrict__ model, float *__restrict__ Xs,
                                                     float *__restrict__ A1, float *__restrict__ A2,
                                                     float *__restrict__ Yp) {
  __shared__ float s[kTotal];
  load_model(model, s);
  for (u32 r = blockIdx.x * blockDim.x + threadIdx.x; r < n; r += gridDim.x * blockDim.x)
    mlp_row(s, X + size_t(r) * kF, Yp + size_t(r) * kO, Xs + size_t(r) * kF, A1 + size_t(r) * kH,
            A2 + size_t(r) * kH);
}

// Backward through the rows: G3 = dL/dy, D2 = dL/dz2, D1 = dL/dz1 (z: before
// ReLU). L = sum M (y' - y)^2 * inv_msum. loss_acc += this batch's loss.
__global__ void __launch_bounds__(128) k_mlp_backward(u32 n, const float *__restrict__ Y, const float *__restrict__ M,
                                                      float inv_msum, const float *__restrict__ model,
                                                      const float *__restrict__ A1, const float *__restrict__ A2,
                                                      const float *__restrict__ Yp, float *__restrict__ G3,
                                                      float *__restrict__ D2, float *__restrict__ D1,
                                                      float *__restrict__ loss_acc) {
  __shared__ float s[kTotal];
  load_model(model, s);
  float part = 0.f;
  for (u32 r = blockIdx.x * blockDim.x + threadIdx.x; r < n; r += gridDim.x * blockDim.x) {
    float g[kO];
#pragma unroll
    for (int k = 0; k < kO; k++) {
      const float m = M[size_t(r) * kO + k], d = Yp[size_t(r) * kO + k] - Y[size_t(r) * kO + k];
      part += m * d * d * inv_msum;
      g[k] = 2.f * m * d * inv_msum;
      G3[size_t(r) * kO + k] = g[k];
    }
    float d2[kH];
#pragma unroll
    for (int j = 0; j < kH; j++) {
      float v = 0.f;
#pragma unroll
      for (int k = 0; k < kO; k++) v = fmaf(g[k], s[kW3 + j * kO + k], v);
      d2[j] = A2[size_t(r) * kH + j] > 0.f ? v : 0.f;
      D2[size_t(r) * kH + j] = d2[j];
    }
    for (int i = 0; i < kH; i++) {
      float v = 0.f;
#pragma unroll
      for (int j = 0; j < kH; j++) v = fmaf(d2[j], s[kW2 + i * kH + j], v);
      D1[size_t(r) * kH + i] = A1[size_t(r) * kH + i] > 0.f ? v : 0.f;
    }
  }
  for (int o = 16; o; o >>= 1) part += __shfl_xor_sync(kFull, part, o);
  if ((threadIdx.x & 31) == 0 && part != 0.f) atomicAdd(loss_acc, part);
}

// One thread per trainable parameter; sums over the n rows in order (no
// atomics: the gradient is deterministic).
__global__ void k_mlp_wgrad(u32 n, const float *__restrict__ Xs, const float *__restrict__ A1,
                            const float *__restrict__ A2, const float *__restrict__ G3, const float *__restrict__ D1,
                            const float *__restrict__ D2, float *__restrict__ grad) {
  const int p = kTrain0 + int(blockIdx.x * blockDim.x + threadIdx.x);
  if (p >= kTotal) return;
  const float *L = nullptr;  // left factor column (nullptr: bias)
  const float *R;
  int ls = 0, rs, li = 0, ri;
  if (p < kB1) { const int q = p - kW1; L = Xs; ls = kF; li = q / kH; R = D1; rs = kH; ri = q % kH; }
  else if (p < kW2) { R = D1; rs = kH; ri = p - kB1; }
  else if (p < kB2) { const int q = p - kW2; L = A1; ls = kH; li = q / kH; R = D2; rs = kH; ri = q % kH; }
  else if (p < kW3) { R = D2; rs = kH; ri = p - kB2; }
  else if (p < kB3) { const int q = p - kW3; L = A2; ls = kH; li = q / kO; R = G3; rs = kO; ri = q % kO; }
  else { R = G3; rs = kO; ri = p - kB3; }
  float acc = 0.f;
  if (L) {
    for (u32 r = 0; r < n; r++) acc = fmaf(L[size_t(r) * ls + li], R[size_t(r) * rs + ri], acc);
  } else {
    for (u32 r = 0; r < n; r++) acc += R[size_t(r) * rs + ri];
  }
  grad[p] = acc;
}

__global__ void k_adam(float *__restrict__ w, const float *__restrict__ g, float *__restrict__ m,
                       float *__restrict__ v, float lr, float c1, float c2) {
  const int p = kTrain0 + int(blockIdx.x * blockDim.x + threadIdx.x);
  if (p >= kTotal) return;
  const float gi = g[p];
  const float mi = 0.9f * m[p] + 0.1f * gi, vi = 0.999f * v[p] + 0.001f * gi * gi;
  m[p] = mi;
  v[p] = vi;
  w[p] -= lr * (mi * c1) / (sqrtf(vi * c2) + 1e-8f);
}

__global__ void k_gather_rows(const u32 *__restrict__ idx, u32 n, const float *__restrict__ X,
                              const float *__restrict__ Y, const float *__restrict__ M, float *__restrict__ Xb,
                              float *__restrict__ Yb, float *__restrict__ Mb) {
  for (u32 r = blockIdx.x * blockDim.x + threadIdx.x; r < n; r += gridDim.x * blockDim.x) {
    const size_t s = idx[r];
    for (int i = 0; i < kF; i++) Xb[size_t(r) * kF + i] = X[s * kF + i];
    for (int k = 0; k < kO; k++) {
      Yb[size_t(r) * kO + k] = Y[s * kO + k];
      Mb[size_t(r) * kO + k] = M[s * kO + k];
    }
  }
}

// cost[t] = sum of tile t's item cycles / CTAs per SM of its class, plus its
// split-tile merge cycles / merge CTAs per SM.
struct Occ {
  double v[FCC_NUM_CLASSES];
};
__global__ void k_tile_costs(u32 ntiles, const u32 *__restrict__ corder, const u32 *__restrict__ cls,
                             const u32 *__restrict__ item_off, const u32 *__restrict__ t_items,
                             const u64 *__restrict__ item_cyc, Occ occ, const u64 *__restrict__ merge_cyc,
                             double merge_occ, double *__restrict__ cost) {
  for (u32 i = blockIdx.x * blockDim.x + threadIdx.x; i < ntiles; i += gridDim.x * blockDim.x) {
    const u32 t = corder[i];
    double s = 0;
    for (u32 k = 0; k < t_items[i]; k++) s += double(item_cyc[item_off[i] + k]);
    cost[t] = s / occ.v[cls[t]] + (merge_cyc ? double(merge_cyc[t]) / merge_occ : 0.0);
  }
}

int grid_rows(u32 n, int threads) { return int(std::max<u32>(1, std::min<u32>((n + threads - 1) / threads, 4096))); }

// Device buffers of one training or gradient run.
struct MlpBufs {
  cudaStream_t st;
  std::vector<void *> owned;
  ~MlpBufs() {
    for (void *p : owned) cudaFreeAsync(p, st);
    cudaStreamSynchronize(st);
  }
  template <class T>
  T *get(size_t n) {
    void *p = nullptr;
    FCC_CUDA(cudaMallocAsync(&p, sizeof(T) * std::max<size_t>(n, 1), st));
    owned.push_back(p);
    return static_cast<T *>(p);
  }
};

struct MlpPass {  // activations of up to `cap` rows
  float *Xs, *A1, *A2, *Yp, *G3, *D1, *D2;
  MlpPass(MlpBufs &b, size_t cap)
      : Xs(b.get<float>(cap * kF)), A1(b.get<float>(cap * kH)), A2(b.get<float>(cap * kH)),
        Yp(b.get<float>(cap * kO)), G3(b.get<float>(cap * kO)), D1(b.get<float>(cap * kH)),
        D2(b.get<float>(cap * kH)) {}
};

// One forward + backward + weight-gradient pass over n rows on the device.
void mlp_pass(cudaStream_t st, u32 n, const float *X, const float *Y, const float *M, float inv_msum,
              const float *model, MlpPass &p, float *grad, float *loss_acc) {
  k_mlp_forward<<<grid_rows(n, 128), 128, 0, st>>>(n, X, model, p.Xs, p.A1, p.A2, p.Yp);
  FCC_LAUNCH_CHECK();
  k_mlp_backward<<<grid_rows(n, 128), 128, 0, st>>>(n, Y, M, inv_msum, model, p.A1, p.A2, p.Yp, p.G3, p.D2, p.D1,
                                                    loss_acc);
  FCC_LAUNCH_CHECK();
  const int np = kTotal - kTrain0;
  k_mlp_wgrad<<<(np + 127) / 128, 128, 0, st>>>(n, p.Xs, p.A1, p.A2, p.G3, p.D1, p.D2, grad);
  FCC_LAUNCH_CHECK();
}

void check_rows(const void *X, int64_t n) {
  if (!X || n < 1 || n > (int64_t(1) << 28)) throw Error{FCC_ERR_ARG, "bad MLP rows"};
}

}  // namespace

void tile_features(cudaStream_t st, const u32 *ntiles_p, u32 nmax, const u32 *abeg, const u64 *P, const u32 *nrows,
                   const u32 *lb, u64 LB, float *feat, int num_sms) {
  if (nmax == 0) return;
  FCC_CUDA(cudaMemsetAsync(feat, 0, sizeof(float) * size_t(nmax) * kF, st));
  k_tile_sums<<<std::max(num_sms, 1) * 8, 256, 0, st>>>(ntiles_p, nmax, abeg, P,
                                                         reinterpret_cast<unsigned long long *>(feat));
  FCC_LAUNCH_CHECK();
  k_tile_features<<<grid_rows(nmax, 256), 256, 0, st>>>(ntiles_p, nmax, abeg, P, nrows, lb, LB, feat);
  FCC_LAUNCH_CHECK();
}

void predict_costs(cudaStream_t st, const u32 *ntiles_p, u32 nmax, const float *feat, const float *model,
                   float *pred) {
  if (nmax == 0) return;
  k_mlp_predict<<<grid_rows(nmax, 128), 128, 0, st>>>(ntiles_p, nmax, feat, model, pred);
  FCC_LAUNCH_CHECK();
}

void tile_costs(cudaStream_t st, u32 ntiles, const u32 *corder, const u32 *cls, const u32 *item_off,
                const u32 *t_items, const u64 *item_cyc, const double *occ, const u64 *merge_cyc,
                double merge_occ, double *cost) {
  Occ o;
  for (int c = 0; c < FCC_NUM_CLASSES; c++) o.v[c] = occ[c];
  k_tile_costs<<<grid_rows(ntiles, 256), 256, 0, st>>>(ntiles, corder, cls, item_off, t_items, item_cyc, o,
                                                       merge_cyc, merge_occ, cost);
  FCC_LAUNCH_CHECK();
}

}  // namespace fcc

namespace {
template <class F>
int sched_guard(fcc_ctx *ctx, F &&f) {
  try {
    FCC_CUDA(cudaSetDevice(ctx->device));
    f();
    return FCC_OK;
  } catch (const fcc::Error &e) {
    ctx->last_error = e.msg;
    return e.status;
  } catch (const std::bad_alloc &) {
    ctx->last_error = "host allocation failed";
    return FCC_ERR_OOM;
  }
}
}  // namespace

extern "C" {

int fcc_sched_set_model(fcc_ctx *ctx, const float *model, int64_t n) {
  if (!ctx) return FCC_ERR_ARG;
  return sched_guard(ctx, [&] {
    if (!model) {
      if (ctx->sched.model) {
        FCC_CUDA(cudaStreamSynchronize(ctx->stream));
        FCC_CUDA(cudaFree(ctx->sched.model));
      }
      ctx->sched.model = nullptr;
      return;
    }
    if (n != FCC_SCHED_MODEL_FLOATS) throw fcc::Error{FCC_ERR_ARG, "model must hold FCC_SCHED_MODEL_FLOATS floats"};
    for (int64_t i = 0; i < n; i++)
      if (!std::isfinite(model[i])) throw fcc::Error{FCC_ERR_ARG, "model holds a non-finite value"};
    if (!ctx->sched.model)
      FCC_CUDA(cudaMalloc(reinterpret_cast<void **>(&ctx->sched.model), sizeof(float) * FCC_SCHED_MODEL_FLOATS));
    FCC_CUDA(cudaMemcpyAsync(ctx->sched.model, model, sizeof(float) * FCC_SCHED_MODEL_FLOATS,
                             cudaMemcpyHostToDevice, ctx->stream));
    FCC_CUDA(cudaStreamSynchronize(ctx->stream));
  });
}

int fcc_sched_last_tiles(fcc_ctx *ctx, float *features, int32_t *cls, double *cost, int64_t cap, int64_t *ntiles) {
  if (!ctx) return FCC_ERR_ARG;
  return sched_guard(ctx, [&] {
    const fcc::SchedIo &io = ctx->sched;
    if (ntiles) *ntiles = io.ntiles;
    const size_t n = size_t(std::max<int64_t>(0, std::min<int64_t>(cap, io.ntiles)));
    if (n == 0) return;
    cudaStream_t st = ctx->stream;
    if (features) {
      if (!io.features) throw fcc::Error{FCC_ERR_ARG, "no features recorded (run with timing = 2)"};
      FCC_CUDA(cudaMemcpyAsync(features, io.features, sizeof(float) * FCC_SCHED_FEATURES * n,
                               cudaMemcpyDeviceToHost, st));
    }
    if (cls) FCC_CUDA(cudaMemcpyAsync(cls, io.cls, sizeof(int32_t) * n, cudaMemcpyDeviceToHost, st));
    if (cost) {
      if (!io.cost) throw fcc::Error{FCC_ERR_ARG, "no tile costs recorded (run with timing = 2)"};
      FCC_CUDA(cudaMemcpyAsync(cost, io.cost, sizeof(double) * n, cudaMemcpyDeviceToHost, st));
    }
    FCC_CUDA(cudaStreamSynchronize(st));
  });
}

int fcc_mlp_predict(fcc_ctx *ctx, const float *X, int64_t n, const float *model, float *Y) {
  if (!ctx || !model || !Y) return FCC_ERR_ARG;
  return sched_guard(ctx, [&] {
    fcc::check_rows(X, n);
    cudaStream_t st = ctx->stream;
    fcc::MlpBufs b{st, {}};
    float *dX = b.get<float>(size_t(n) * fcc::kF), *dY = b.get<float>(size_t(n) * fcc::kO);
    float *dm = b.get<float>(fcc::kTotal);
    FCC_CUDA(cudaMemcpyAsync(dX, X, sizeof(float) * n * fcc::kF, cudaMemcpyHostToDevice, st));
    FCC_CUDA(cudaMemcpyAsync(dm, model, sizeof(float) * fcc::kTotal, cudaMemcpyHostToDevice, st));
    fcc::k_mlp_predict<<<fcc::grid_rows(fcc::u32(n), 128), 128, 0, st>>>(nullptr, fcc::u32(n), dX, dm, dY);
    FCC_LAUNCH_CHECK();
    FCC_CUDA(cudaMemcpyAsync(Y, dY, sizeof(float) * n * fcc::kO, cudaMemcpyDeviceToHost, st));
    FCC_CUDA(cudaStreamSynchronize(st));
  });
}

int fcc_mlp_grad(fcc_ctx *ctx, const float *X, const float *Y, const float *M, int64_t n, const float *model,
                 float *grad, float *loss) {
  if (!ctx || !Y || !M || !model || !grad) return FCC_ERR_ARG;
  return sched_guard(ctx, [&] {
    fcc::check_rows(X, n);
    double msum = 0;
    for (int64_t i = 0; i < n * fcc::kO; i++) msum += M[i];
    cudaStream_t st = ctx->stream;
    fcc::MlpBufs b{st, {}};
    float *dX = b.get<float>(size_t(n) * fcc::kF), *dY = b.get<float>(size_t(n) * fcc::kO);
    float *dM = b.get<float>(size_t(n) * fcc::kO), *dm = b.get<float>(fcc::kTotal);
    float *dg = b.get<float>(fcc::kTotal), *dl = b.get<float>(1);
    fcc::MlpPass pass(b, size_t(n));
    FCC_CUDA(cudaMemcpyAsync(dX, X, sizeof(float) * n * fcc::kF, cudaMemcpyHostToDevice, st));
    FCC_CUDA(cudaMemcpyAsync(dY, Y, sizeof(float) * n * fcc::kO, cudaMemcpyHostToDevice, st));
    FCC_CUDA(cudaMemcpyAsync(dM, M, sizeof(float) * n * fcc::kO, cudaMemcpyHostToDevice, st));
    FCC_CUDA(cudaMemcpyAsync(dm, model, sizeof(float) * fcc::kTotal, cudaMemcpyHostToDevice, st));
    FCC_CUDA(cudaMemsetAsync(dg, 0, sizeof(float) * fcc::kTotal, st));
    FCC_CUDA(cudaMemsetAsync(dl, 0, sizeof(float), st));
    fcc::mlp_pass(st, fcc::u32(n), dX, dY, dM, float(msum > 0 ? 1.0 / msum : 0.0), dm, pass, dg, dl);
    FCC_CUDA(cudaMemcpyAsync(grad, dg, sizeof(float) * fcc::kTotal, cudaMemcpyDeviceToHost, st));
    float l = 0;
    FCC_CUDA(cudaMemcpyAsync(&l, dl, sizeof(float), cudaMemcpyDeviceToHost, st));
    FCC_CUDA(cudaStreamSynchronize(st));
    if (loss) *loss = l;
  });
}

int fcc_mlp_train(fcc_ctx *ctx, const float *X, const float *Y, const float *M, int64_t n, int32_t epochs,
                  int32_t batch, float lr, uint64_t seed, float *model, float *loss) {
  if (!ctx || !Y || !M || !model || epochs < 0 || batch < 1 || !(lr > 0)) return FCC_ERR_ARG;
  return sched_guard(ctx, [&] {
    fcc::check_rows(X, n);
    cudaStream_t st = ctx->stream;
    const size_t nb = size_t(std::min<int64_t>(batch, n));
    fcc::MlpBufs b{st, {}};
    float *dX = b.get<float>(size_t(n) * fcc::kF), *dY = b.get<float>(size_t(n) * fcc::kO);
    float *dM = b.get<float>(size_t(n) * fcc::kO), *dm = b.get<float>(fcc::kTotal);
    float *dg = b.get<float>(fcc::kTotal), *dmo = b.get<float>(fcc::kTotal), *dv = b.get<float>(fcc::kTotal);
    float *dl = b.get<float>(1);
    float *bX = b.get<float>(nb * fcc::kF), *bY = b.get<float>(nb * fcc::kO), *bM = b.get<float>(nb * fcc::kO);
    fcc::u32 *didx = b.get<fcc::u32>(size_t(n));
    fcc::MlpPass pass(b, std::max<size_t>(nb, size_t(n)));
    FCC_CUDA(cudaMemcpyAsync(dX, X, sizeof(float) * n * fcc::kF, cudaMemcpyHostToDevice, st));
    FCC_CUDA(cudaMemcpyAsync(dY, Y, sizeof(float) * n * fcc::kO, cudaMemcpyHostToDevice, st));
    FCC_CUDA(cudaMemcpyAsync(dM, M, sizeof(float) * n * fcc::kO, cudaMemcpyHostToDevice, st));
    FCC_CUDA(cudaMemcpyAsync(dm, model, sizeof(float) * fcc::kTotal, cudaMemcpyHostToDevice, st));
    FCC_CUDA(cudaMemsetAsync(dmo, 0, sizeof(float) * fcc::kTotal, st));
    FCC_CUDA(cudaMemsetAsync(dv, 0, sizeof(float) * fcc::kTotal, st));
    std::vector<fcc::u32> perm(static_cast<size_t>(n));
    std::iota(perm.begin(), perm.end(), 0u);
    std::mt19937_64 rng(seed);
    const int np = fcc::kTotal - fcc::kTrain0;
    long step = 0;
    for (int ep = 0; ep < epochs; ep++) {
      for (size_t i = perm.size(); i > 1; i--) std::swap(perm[i - 1], perm[size_t(rng() % i)]);
      FCC_CUDA(cudaMemcpyAsync(didx, perm.data(), sizeof(fcc::u32) * n, cudaMemcpyHostToDevice, st));
      FCC_CUDA(cudaStreamSynchronize(st));  // perm is rewritten next epoch
      for (size_t s0 = 0; s0 < size_t(n); s0 += nb) {
        const fcc::u32 cnt = fcc::u32(std::min(nb, size_t(n) - s0));
        double msum = 0;
        for (fcc::u32 r = 0; r < cnt; r++)
          for (int k = 0; k < fcc::kO; k++) msum += M[size_t(perm[s0 + r]) * fcc::kO + k];
        if (msum <= 0) continue;
        fcc::k_gather_rows<<<fcc::grid_rows(cnt, 256), 256, 0, st>>>(didx + s0, cnt, dX, dY, dM, bX, bY, bM);
        FCC_LAUNCH_CHECK();
        fcc::mlp_pass(st, cnt, bX, bY, bM, float(1.0 / msum), dm, pass, dg, dl);
        step++;
        const float c1 = float(1.0 / (1.0 - std::pow(0.9, double(step))));
        const float c2 = float(1.0 / (1.0 - std::pow(0.999, double(step))));
        fcc::k_adam<<<(np + 127) / 128, 128, 0, st>>>(dm, dg, dmo, dv, lr, c1, c2);
        FCC_LAUNCH_CHECK();
      }
    }
    // final loss over all rows
    double msum = 0;
    for (int64_t i = 0; i < n * fcc::kO; i++) msum += M[i];
    FCC_CUDA(cudaMemsetAsync(dl, 0, sizeof(float), st));
    fcc::mlp_pass(st, fcc::u32(n), dX, dY, dM, float(msum > 0 ? 1.0 / msum : 0.0), dm, pass, dg, dl);
    float l = 0;
    FCC_CUDA(cudaMemcpyAsync(model, dm, sizeof(float) * fcc::kTotal, cudaMemcpyDeviceToHost, st));
    FCC_CUDA(cudaMemcpyAsync(&l, dl, sizeof(float), cudaMemcpyDeviceToHost, st));
    FCC_CUDA(cudaStreamSynchronize(st));
    if (loss) *loss = l;
  });
}

}  // extern "C"
