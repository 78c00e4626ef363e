// C ABI of libfastcc_gpu.so (include/fastcc_gpu.h): contexts, the contraction
// entry point and result access. Exceptions never cross this boundary; each
// entry point returns an fcc_status and keeps the message for fcc_last_error.

#include <cstdlib>
#include <cstring>
#include <memory>
#include <new>
#include <vector>

#include "fcc_internal.cuh"

namespace fcc {
void contract(Runtime *ctx, const fcc_tensor *A, const fcc_tensor *B, const int32_t *ctrA,
              const int32_t *ctrB, int k, const fcc_options &opt, fcc_result *res, i64 *products,
              bool count_only, const u32 *group_lb, u32 ngroups);
void contract_batch(Runtime *ctx, int n, const fcc_tensor *A, const fcc_tensor *B, const int32_t *ctrA,
                    const int32_t *ctrB, int k, const fcc_options &opt, fcc_result *res, i64 *counts);
void contract_modes(Runtime *ctx, const fcc_tensor *A, const fcc_tensor *B, const int32_t *ctrA,
                    const int32_t *ctrB, int k, const int32_t *batchA, const int32_t *batchB, int nb,
                    const fcc_options &opt, fcc_result *res);
}

namespace {

thread_local std::string g_last_error;  // errors without a context

// SoA result coordinates (mode m at in[m * cap + i]) -> row-major out[i * order + m].
__global__ void k_interleave(const uint32_t *__restrict__ in, int64_t cap, int order, int64_t n,
                             uint32_t *__restrict__ out) {
  for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x)
    for (int m = 0; m < order; m++) out[i * order + m] = in[int64_t(m) * cap + i];
}

fcc::Runtime runtime_of(fcc_ctx *ctx) {
  fcc::Runtime rt(ctx->arena);
  rt.stream = ctx->stream;
  rt.d_err = ctx->d_err;
  rt.h_scalars = ctx->h_scalars;
  rt.num_sms = ctx->num_sms;
  rt.smem_optin = ctx->smem_optin;
  rt.ev = ctx->ev;
  rt.phase_ms = ctx->phase_ms;
  rt.pool = ctx->pool;
  rt.sched = &ctx->sched;
  rt.copy_stream = ctx->copy_stream;
  rt.wave_ev = ctx->wave_ev;
  rt.h_cursors = ctx->h_cursors;
  rt.wave_tune = &ctx->wave_tune;
  return rt;
}

template <class F>
int guarded(fcc_ctx *ctx, F &&f) {
  try {
    if (ctx) FCC_CUDA(cudaSetDevice(ctx->device));
    f();
    return FCC_OK;
  } catch (const fcc::Error &e) {
    (ctx ? ctx->last_error : g_last_error) = e.msg;
    return e.status;
  } catch (const std::bad_alloc &) {
    (ctx ? ctx->last_error : g_last_error) = "host allocation failed";
    return FCC_ERR_OOM;
  } catch (...) {
    (ctx ? ctx->last_error : g_last_error) = "unexpected exception";
    return FCC_ERR_CUDA;
  }
}

}  // namespace

namespace fcc {
void set_thread_error(const std::string &msg) { g_last_error = msg; }
}  // namespace fcc

extern "C" {

static_assert(sizeof(fcc_options) == 104, "fcc_options layout is part of the ABI");

int fcc_abi_version(void) { return FCC_ABI_VERSION; }

int64_t fcc_launch_count(void) { return fcc::g_launches.load(); }

const char *fcc_status_string(int32_t s) {
  switch (s) {
    case FCC_OK: return "ok";
    case FCC_ERR_ARG: return "invalid argument";
    case FCC_ERR_OOM: return "out of memory";
    case FCC_ERR_HASH_FULL: return "hash accumulator full";
    case FCC_ERR_TIMEOUT: return "bounded device wait timed out";
    case FCC_ERR_CUDA: return "CUDA error";
    case FCC_ERR_OVERFLOW: return "index space exceeds 64 bits";
    case FCC_ERR_NO_DEVICE: return "no usable sm_103 device";
    case FCC_ERR_CAPACITY: return "output buffer too small";
    default: return "unknown status";
  }
}

int fcc_options_default(fcc_options *o) {
  if (!o) return FCC_ERR_ARG;
  std::memset(o, 0, sizeof(*o));
  o->tile_size = 100;
  return FCC_OK;
}

const char *fcc_last_error(const fcc_ctx *ctx) {
  return ctx ? ctx->last_error.c_str() : g_last_error.c_str();
}

int fcc_ctx_create(int32_t device, fcc_ctx **out) {
  if (!out) return FCC_ERR_ARG;
  *out = nullptr;
  fcc_ctx *ctx = nullptr;
  int st = guarded(nullptr, [&] {
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0) {
      cudaGetLastError();
      throw fcc::Error{FCC_ERR_NO_DEVICE, "no CUDA device"};
    }
    int dev = device;
    if (dev < 0) FCC_CUDA(cudaGetDevice(&dev));
    if (dev >= n) throw fcc::Error{FCC_ERR_ARG, "device index out of range"};
    FCC_CUDA(cudaSetDevice(dev));
    cudaDeviceProp p{};
    FCC_CUDA(cudaGetDeviceProperties(&p, dev));
    if (!(p.major == 10 && p.minor == 3))
      throw fcc::Error{FCC_ERR_NO_DEVICE, "this library is built for sm_103a (GB300) only"};
    ctx = new fcc_ctx();
    ctx->device = dev;
    ctx->num_sms = p.multiProcessorCount;
    int optin = 0;
    FCC_CUDA(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
    ctx->smem_optin = size_t(optin);
    FCC_CUDA(cudaStreamCreateWithFlags(&ctx->own_stream, cudaStreamNonBlocking));
    ctx->stream = ctx->own_stream;
    cudaMemPoolProps props{};
    props.allocType = cudaMemAllocationTypePinned;
    props.location.type = cudaMemLocationTypeDevice;
    props.location.id = dev;
    FCC_CUDA(cudaMemPoolCreate(&ctx->pool, &props));
    uint64_t keep = ~0ull;
    FCC_CUDA(cudaMemPoolSetAttribute(ctx->pool, cudaMemPoolAttrReleaseThreshold, &keep));
    ctx->arena.init(ctx->pool);
    FCC_CUDA(cudaMalloc(reinterpret_cast<void **>(&ctx->d_err), sizeof(fcc::u32)));
    FCC_CUDA(cudaMallocHost(reinterpret_cast<void **>(&ctx->h_scalars), sizeof(fcc::u64) * 32));
    for (auto &e : ctx->ev) FCC_CUDA(cudaEventCreate(&e));
    FCC_CUDA(cudaStreamCreateWithFlags(&ctx->copy_stream, cudaStreamNonBlocking));
    for (auto &e : ctx->wave_ev) FCC_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    FCC_CUDA(cudaMallocHost(reinterpret_cast<void **>(&ctx->h_cursors), sizeof(fcc::u64) * (fcc::kMaxWaves + 1)));
  });
  if (st != FCC_OK) {
    if (ctx) fcc_ctx_destroy(ctx);
    return st;
  }
  *out = ctx;
  return FCC_OK;
}

int fcc_ctx_destroy(fcc_ctx *ctx) {
  if (!ctx) return FCC_ERR_ARG;
  cudaSetDevice(ctx->device);
  if (ctx->stream) cudaStreamSynchronize(ctx->stream);
  if (ctx->stream) ctx->arena.release_all(ctx->stream);
  if (ctx->stream) cudaStreamSynchronize(ctx->stream);
  for (auto &e : ctx->ev)
    if (e) cudaEventDestroy(e);
  if (ctx->copy_stream) cudaStreamSynchronize(ctx->copy_stream);
  for (auto &e : ctx->wave_ev)
    if (e) cudaEventDestroy(e);
  if (ctx->h_cursors) cudaFreeHost(ctx->h_cursors);
  if (ctx->copy_stream) cudaStreamDestroy(ctx->copy_stream);
  if (ctx->d_err) cudaFree(ctx->d_err);
  if (ctx->sched.model) cudaFree(ctx->sched.model);
  if (ctx->h_scalars) cudaFreeHost(ctx->h_scalars);
  if (ctx->pool) cudaMemPoolDestroy(ctx->pool);
  if (ctx->own_stream) cudaStreamDestroy(ctx->own_stream);
  delete ctx;
  return FCC_OK;
}

int fcc_ctx_set_stream(fcc_ctx *ctx, void *stream) {
  if (!ctx) return FCC_ERR_ARG;
  return guarded(ctx, [&] {
    // workspace frees are ordered on the previous stream: drain it first
    FCC_CUDA(cudaStreamSynchronize(ctx->stream));
    ctx->stream = stream ? static_cast<cudaStream_t>(stream) : ctx->own_stream;
  });
}

int fcc_contract(fcc_ctx *ctx, const fcc_tensor *A, const fcc_tensor *B, const int32_t *ctrA,
                 const int32_t *ctrB, int32_t k, const fcc_options *opts, fcc_result **out) {
  if (!ctx || !out) return FCC_ERR_ARG;
  *out = nullptr;
  fcc_options o;
  if (opts) o = *opts; else fcc_options_default(&o);
  return guarded(ctx, [&] {
    fcc::Runtime rt = runtime_of(ctx);
    std::unique_ptr<fcc_result> r(new fcc_result());
    r->ctx = ctx;
    fcc::contract(&rt, A, B, ctrA, ctrB, k, o, r.get(), nullptr, false, nullptr, 0);
    *out = r.release();
  });
}

int fcc_contract_into(fcc_ctx *ctx, const fcc_tensor *A, const fcc_tensor *B, const int32_t *ctrA,
                      const int32_t *ctrB, int32_t k, const fcc_options *opts, uint32_t *out_coords,
                      int64_t out_mode_stride, double *out_values, int64_t out_capacity, int64_t *out_nnz,
                      int64_t *out_products) {
  if (!ctx || !out_nnz) return FCC_ERR_ARG;
  *out_nnz = 0;
  if (out_products) *out_products = 0;
  if (out_capacity < 0 || (out_capacity > 0 && (!out_values || out_mode_stride < out_capacity)))
    return FCC_ERR_ARG;
  fcc_options o;
  if (opts) o = *opts; else fcc_options_default(&o);
  o.capacity_hint = 0;
  fcc_result res;
  res.ctx = ctx;
  const int st = guarded(ctx, [&] {
    fcc::Runtime rt = runtime_of(ctx);
    rt.out_coords = out_coords;
    rt.out_stride = out_mode_stride;
    rt.out_vals = out_values;
    rt.out_cap = fcc::u64(out_capacity);
    rt.caller_out = true;
    fcc::i64 products = 0;
    fcc::contract(&rt, A, B, ctrA, ctrB, k, o, &res, &products, false, nullptr, 0);
    if (out_products) *out_products = products;
  });
  *out_nnz = res.nnz;  // on FCC_ERR_CAPACITY: the entries the output needs
  return st;
}

int fcc_contract_modes(fcc_ctx *ctx, const fcc_tensor *A, const fcc_tensor *B, const int32_t *ctrA,
                       const int32_t *ctrB, int32_t k, const int32_t *batchA, const int32_t *batchB, int32_t nb,
                       const fcc_options *opts, fcc_result **out) {
  if (!ctx || !out) return FCC_ERR_ARG;
  *out = nullptr;
  fcc_options o;
  if (opts) o = *opts; else fcc_options_default(&o);
  return guarded(ctx, [&] {
    fcc::Runtime rt = runtime_of(ctx);
    std::unique_ptr<fcc_result> r(new fcc_result());
    r->ctx = ctx;
    fcc::contract_modes(&rt, A, B, ctrA, ctrB, k, batchA, batchB, nb, o, r.get());
    *out = r.release();
  });
}

int fcc_contract_batch(fcc_ctx *ctx, int32_t n, const fcc_tensor *A, const fcc_tensor *B, const int32_t *ctrA,
                       const int32_t *ctrB, int32_t k, const fcc_options *opts, fcc_result **out,
                       int64_t *counts) {
  if (!ctx || !out) return FCC_ERR_ARG;
  *out = nullptr;
  fcc_options o;
  if (opts) o = *opts; else fcc_options_default(&o);
  return guarded(ctx, [&] {
    fcc::Runtime rt = runtime_of(ctx);
    std::unique_ptr<fcc_result> r(new fcc_result());
    r->ctx = ctx;
    fcc::contract_batch(&rt, n, A, B, ctrA, ctrB, k, o, r.get(), counts);
    *out = r.release();
  });
}

}  // extern "C"

namespace {

// Shape signature of a problem for the autotuner's cache: orders, contracted
// modes, and log2 buckets of the nonzero counts and mode extents.
std::string tune_signature(int n, const fcc_tensor *A, const fcc_tensor *B, const int32_t *ctrA,
                           const int32_t *ctrB, int32_t k) {
  auto lg = [](int64_t v) { int b = 0; while (v > 1) { v >>= 1; b++; } return b; };
  std::string s = "n" + std::to_string(n) + ":";
  for (int side = 0; side < 2; side++) {
    const fcc_tensor *T = side ? B : A;
    int64_t nnz = 0;
    std::vector<int32_t> mx(size_t(std::max(T[0].order, 0)), 0);
    for (int t = 0; t < n; t++) {
      nnz += T[t].nnz;
      for (int m = 0; m < T[0].order && T[t].max_index; m++) mx[size_t(m)] = std::max(mx[size_t(m)], T[t].max_index[m]);
    }
    s += "o" + std::to_string(T[0].order) + "z" + std::to_string(lg(nnz));
    for (int32_t v : mx) s += "e" + std::to_string(lg(int64_t(v) + 1));
    s += "|";
  }
  for (int i = 0; i < k; i++) s += std::to_string(ctrA[i]) + "-" + std::to_string(ctrB[i]) + ",";
  return s;
}

// Times each candidate schedule with `run` (a full contraction with
// opts.timing = 1) and keeps the fastest.
template <class Run>
void autotune(fcc_ctx *ctx, const std::string &sig, const fcc_options &base, int reps, Run &&run,
              fcc_options *best, double *best_ms) {
  auto hit = ctx->tuned.find(sig);
  if (hit != ctx->tuned.end()) {
    *best = hit->second.first;
    if (best_ms) *best_ms = hit->second.second;
    return;
  }
  std::vector<fcc_options> cand;
  auto add = [&](int schedule, int threads, int fill) {
    fcc_options o = base;
    o.accumulator = FCC_ACC_AUTO;
    o.hash_slots = 0;
    o.schedule = schedule;
    o.tile_threads = threads;
    o.dense_fill_log2 = fill;
    cand.push_back(o);
  };
  for (int threads : {640, 512, 1024}) {
    add(FCC_SCHED_RULE, threads, 0);
    add(FCC_SCHED_RULE, threads, -1);
    add(FCC_SCHED_RULE, threads, 6);
    add(FCC_SCHED_FORCE + FCC_CLASS_DENSE, threads, 0);
  }
  for (int c = FCC_CLASS_HASH_L; c < FCC_NUM_CLASSES; c++) add(FCC_SCHED_FORCE + c, 0, 0);
  double best_t = 1e300;
  fcc_options best_o = base;
  for (fcc_options o : cand) {
    o.timing = 1;
    double t = 0;
    bool ok = true;
    for (int r = 0; r <= reps && ok; r++) {  // the first run warms up
      try {
        run(o);
      } catch (const fcc::Error &e) {
        // a class this problem cannot use, or whose split buffers do not fit
        if (e.status != FCC_ERR_ARG && e.status != FCC_ERR_OOM) throw;
        ok = false;
        break;
      }
      if (r > 0) t += ctx->phase_ms[FCC_PHASE_TOTAL];
    }
    if (!ok) continue;
    t /= std::max(reps, 1);
    if (t < best_t) {
      best_t = t;
      best_o = o;
    }
  }
  // the trials' workspace (the largest of every candidate's) stays out of later calls
  ctx->arena.shrink(ctx->stream);
  if (best_t == 1e300) throw fcc::Error{FCC_ERR_ARG, "no schedule can run this problem"};
  best_o.timing = base.timing;
  ctx->tuned[sig] = {best_o, best_t};
  *best = best_o;
  if (best_ms) *best_ms = best_t;
}

}  // namespace

extern "C" {

int fcc_autotune(fcc_ctx *ctx, const fcc_tensor *A, const fcc_tensor *B, const int32_t *ctrA, const int32_t *ctrB,
                 int32_t k, const fcc_options *base, int32_t reps, fcc_options *best, double *best_ms) {
  if (!ctx || !A || !B || !best || k < 0 || (k > 0 && (!ctrA || !ctrB))) return FCC_ERR_ARG;
  fcc_options o;
  if (base) o = *base; else fcc_options_default(&o);
  return guarded(ctx, [&] {
    const std::string sig = tune_signature(1, A, B, ctrA, ctrB, k);
    autotune(ctx, sig, o, std::max(reps, 1), [&](const fcc_options &c) {
      fcc::Runtime rt = runtime_of(ctx);
      std::unique_ptr<fcc_result> r(new fcc_result());
      r->ctx = ctx;
      fcc::contract(&rt, A, B, ctrA, ctrB, k, c, r.get(), nullptr, false, nullptr, 0);
      fcc_result_free(r.release());
    }, best, best_ms);
  });
}

int fcc_autotune_batch(fcc_ctx *ctx, int32_t n, const fcc_tensor *A, const fcc_tensor *B, const int32_t *ctrA,
                       const int32_t *ctrB, int32_t k, const fcc_options *base, int32_t reps, fcc_options *best,
                       double *best_ms) {
  if (!ctx || n < 1 || !A || !B || !best || k < 0 || (k > 0 && (!ctrA || !ctrB))) return FCC_ERR_ARG;
  fcc_options o;
  if (base) o = *base; else fcc_options_default(&o);
  return guarded(ctx, [&] {
    const std::string sig = tune_signature(n, A, B, ctrA, ctrB, k);
    autotune(ctx, sig, o, std::max(reps, 1), [&](const fcc_options &c) {
      fcc::Runtime rt = runtime_of(ctx);
      std::unique_ptr<fcc_result> r(new fcc_result());
      r->ctx = ctx;
      fcc::contract_batch(&rt, n, A, B, ctrA, ctrB, k, c, r.get(), nullptr);
      fcc_result_free(r.release());
    }, best, best_ms);
  });
}

int fcc_count_products(fcc_ctx *ctx, const fcc_tensor *A, const fcc_tensor *B, const int32_t *ctrA,
                       const int32_t *ctrB, int32_t k, const fcc_options *opts, int64_t *products) {
  if (!ctx || !products) return FCC_ERR_ARG;
  fcc_options o;
  if (opts) o = *opts; else fcc_options_default(&o);
  return guarded(ctx, [&] {
    fcc::Runtime rt = runtime_of(ctx);
    fcc::contract(&rt, A, B, ctrA, ctrB, k, o, nullptr, products, true, nullptr, 0);
  });
}

int fcc_result_info(const fcc_result *r, int32_t *order, int64_t *nnz, int64_t *products) {
  if (!r) return FCC_ERR_ARG;
  if (order) *order = r->order;
  if (nnz) *nnz = r->nnz;
  if (products) *products = r->products;
  return FCC_OK;
}

int fcc_result_device(const fcc_result *r, const uint32_t **coords, int64_t *mode_stride,
                      const double **values) {
  if (!r) return FCC_ERR_ARG;
  if (coords) *coords = r->d_coords;
  if (mode_stride) *mode_stride = r->cap;
  if (values) *values = r->d_vals;
  return FCC_OK;
}

int fcc_result_copy_to_host(const fcc_result *r, int32_t *coords, int64_t stride_nnz,
                            int64_t stride_mode, double *values) {
  if (!r || !r->ctx) return FCC_ERR_ARG;
  fcc_ctx *ctx = r->ctx;
  return guarded(ctx, [&] {
    const int64_t n = r->nnz;
    if (n == 0) return;
    cudaStream_t s = ctx->stream;
    if (values) FCC_CUDA(cudaMemcpyAsync(values, r->d_vals, sizeof(double) * n, cudaMemcpyDeviceToHost, s));
    if (coords && r->order > 0) {
      if (stride_nnz == 1) {
        for (int m = 0; m < r->order; m++)
          FCC_CUDA(cudaMemcpyAsync(coords + m * stride_mode, r->d_coords + m * r->cap, sizeof(uint32_t) * n,
                                   cudaMemcpyDeviceToHost, s));
        FCC_CUDA(cudaStreamSynchronize(s));
      } else if (stride_mode == 1 && stride_nnz == r->order) {
        // row-major (the drop-in's ListTensor): interleave on the device, one copy out
        void *p = fcc::pool_alloc(ctx->pool, sizeof(uint32_t) * size_t(n) * r->order, s);
        k_interleave<<<fcc::grid_for(n, 256), 256, 0, s>>>(r->d_coords, r->cap, r->order, n,
                                                           static_cast<uint32_t *>(p));
        FCC_LAUNCH_CHECK();
        FCC_CUDA(cudaMemcpyAsync(coords, p, sizeof(uint32_t) * size_t(n) * r->order, cudaMemcpyDeviceToHost, s));
        FCC_CUDA(cudaFreeAsync(p, s));
      } else {
        std::vector<uint32_t> tmp(size_t(n) * r->order);
        for (int m = 0; m < r->order; m++)
          FCC_CUDA(cudaMemcpyAsync(tmp.data() + size_t(m) * n, r->d_coords + m * r->cap, sizeof(uint32_t) * n,
                                   cudaMemcpyDeviceToHost, s));
        FCC_CUDA(cudaStreamSynchronize(s));
        for (int m = 0; m < r->order; m++) {
          const uint32_t *src = tmp.data() + size_t(m) * n;
          int32_t *dst = coords + m * stride_mode;
          for (int64_t i = 0; i < n; i++) dst[i * stride_nnz] = int32_t(src[i]);
        }
      }
    }
    FCC_CUDA(cudaStreamSynchronize(s));
  });
}

int fcc_result_free(fcc_result *r) {
  if (!r) return FCC_ERR_ARG;
  if (r->ctx && r->owned) {
    cudaSetDevice(r->ctx->device);
    if (r->d_vals) cudaFreeAsync(r->d_vals, r->ctx->stream);
    if (r->d_coords) cudaFreeAsync(r->d_coords, r->ctx->stream);
  }
  delete r;
  return FCC_OK;
}

int fcc_last_timings(const fcc_ctx *ctx, double *ms, int32_t n) {
  if (!ctx || !ms || n < 0) return FCC_ERR_ARG;
  for (int i = 0; i < n && i < FCC_NUM_PHASES; i++) ms[i] = ctx->phase_ms[i];
  return FCC_OK;
}

}  // extern "C"
