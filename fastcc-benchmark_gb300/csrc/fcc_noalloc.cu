// fcc_contract_noalloc (include/fastcc_gpu.h): the contraction for callers
// that cannot allocate device memory. Every temporary of the pipeline comes
// from one file-scope device array; inputs and outputs are the caller's.

#include <mutex>

#include "fcc_internal.cuh"

namespace fcc {
void contract(Runtime *ctx, const fcc_tensor *A, const fcc_tensor *B, const int32_t *ctrA,
              const int32_t *ctrB, int k, const fcc_options &opt, fcc_result *res, i64 *products,
              bool count_only, const u32 *group_lb, u32 ngroups);
}

namespace {

using fcc::Error;

// The scratch. Host code must not take g_scratch's address as a device
// pointer: here it names a host-side stand-in. The device address comes from
// cudaGetSymbolAddress, looked up once per device (setup_device).
__device__ __align__(256) unsigned char g_scratch[FCC_NOALLOC_SCRATCH_BYTES];

// The first 256 bytes hold the device error word; the arena gets the rest.
constexpr size_t kReserved = 256;
constexpr int kMaxDevices = 64;

struct DeviceSetup {
  bool ready = false;
  unsigned char *scratch = nullptr;  // device address of g_scratch on this device
  int num_sms = 0;
  size_t smem_optin = 0;
};

DeviceSetup g_devices[kMaxDevices];
std::mutex g_mutex;

// With device `dev` current: its scratch address and the attributes the
// planner needs. Runs once per device.
const DeviceSetup &setup_device(int dev) {
  std::lock_guard<std::mutex> lock(g_mutex);
  DeviceSetup &d = g_devices[dev];
  if (!d.ready) {
    int major = 0, minor = 0, sms = 0, optin = 0;
    FCC_CUDA(cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, dev));
    FCC_CUDA(cudaDeviceGetAttribute(&minor, cudaDevAttrComputeCapabilityMinor, dev));
    if (!(major == 10 && minor == 3))
      throw Error{FCC_ERR_NO_DEVICE, "this library is built for sm_103a (GB300) only"};
    FCC_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    FCC_CUDA(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
    void *ptr = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&ptr, g_scratch);
    if (e != cudaSuccess || !ptr)
      throw Error{FCC_ERR_CUDA, std::string("cudaGetSymbolAddress(scratch): ") + cudaGetErrorString(e)};
    d.scratch = static_cast<unsigned char *>(ptr);
    d.num_sms = sms;
    d.smem_optin = size_t(optin);
    d.ready = true;
  }
  return d;
}

}  // namespace

extern "C" int fcc_contract_noalloc(const fcc_tensor *A, const fcc_tensor *B, const int32_t *ctrA,
                                    const int32_t *ctrB, int32_t k, const fcc_options *opts,
                                    void *cuda_stream, uint32_t *out_coords, int64_t out_mode_stride,
                                    double *out_values, int64_t out_capacity, int64_t *out_nnz,
                                    int64_t *out_products) {
  if (!out_nnz) return FCC_ERR_ARG;
  *out_nnz = 0;
  if (out_products) *out_products = 0;
  fcc_result res;
  cudaStream_t stream = static_cast<cudaStream_t>(cuda_stream);
  bool launched = false;  // work of this call may be queued on `stream`
  // An error return also means that no work of this call still runs: wait
  // for what was queued before the error (its own error, if any, is dropped).
  auto drain = [&] {
    if (launched) {
      cudaStreamSynchronize(stream);
      cudaGetLastError();
    }
  };
  try {
    if (!A || !B) throw Error{FCC_ERR_ARG, "A or B is NULL"};
    if (A->nnz < 0 || B->nnz < 0 || A->nnz + B->nnz > FCC_NOALLOC_MAX_NNZ)
      throw Error{FCC_ERR_CAPACITY, "nnz(A) + nnz(B) exceeds FCC_NOALLOC_MAX_NNZ (131072)"};
    if (out_capacity < 0 || (out_capacity > 0 && !out_values)) throw Error{FCC_ERR_ARG, "bad output buffers"};
    int dev = 0;
    FCC_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= kMaxDevices) throw Error{FCC_ERR_ARG, "device index out of range"};
    const DeviceSetup &d = setup_device(dev);

    fcc::Arena arena;
    arena.init_fixed(d.scratch + kReserved, FCC_NOALLOC_SCRATCH_BYTES - kReserved);
    fcc::u64 host_scalars[32] = {};
    fcc::Runtime rt(arena);
    rt.stream = stream;
    rt.d_err = reinterpret_cast<fcc::u32 *>(d.scratch);
    rt.h_scalars = host_scalars;
    rt.num_sms = d.num_sms;
    rt.smem_optin = d.smem_optin;
    rt.out_coords = out_coords;
    rt.out_stride = out_mode_stride;
    rt.out_vals = out_values;
    rt.out_cap = fcc::u64(out_capacity);
    rt.caller_out = true;
    fcc_options o;
    if (opts) {
      o = *opts;
    } else {
      fcc_options_default(&o);
    }
    o.timing = 0;
    o.capacity_hint = 0;
    fcc::i64 products = 0;
    launched = true;
    fcc::contract(&rt, A, B, ctrA, ctrB, k, o, &res, &products, false, nullptr, 0);
    *out_nnz = res.nnz;
    if (out_products) *out_products = products;
    return FCC_OK;
  } catch (const Error &e) {
    drain();
    fcc::set_thread_error(e.msg);
    *out_nnz = res.nnz;
    return e.status;
  } catch (...) {
    drain();
    fcc::set_thread_error("unexpected exception");
    return FCC_ERR_CUDA;
  }
}
