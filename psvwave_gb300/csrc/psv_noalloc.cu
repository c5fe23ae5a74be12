// L2 misfit for callers that must not allocate device memory.
//
// Some callers run this library inside another system's execution step, where
// device memory belongs to that system and allocating is not allowed: a
// TensorRT plugin's enqueue(), an XLA/JAX custom call, an inference server's
// pre-planned memory arena, or a region being captured into a CUDA graph.
// cudaMalloc there either synchronises the whole device, breaks the capture,
// or is forbidden outright. psv_l2_misfit_noalloc computes the same misfit as
// psv_calculate_l2_misfit (src/fdModel.cpp:1128-1145) from device arrays the
// caller owns, and keeps its partial sums in the fixed array below instead of
// in allocated scratch.
//
// The scratch holds one FP64 partial sum per 2048 samples, at most
// kMaxPartials of them: up to kMaxPartials * 2048 = 16,777,216 samples per
// component (n_shots * nr * nt). The array is a file-scope __device__ object,
// so every GPU that loads this library holds its 64 KiB until the process
// exits, and every call on a device shares it.
#include <cuda_runtime.h>

#include <mutex>
#include <string>

#include "../../include/psvwave.h"
#include "psv_solver.hpp"

namespace psv {
void set_last_error(const std::string &msg);  // psv_capi.cpp; read by psv_last_error()
}

namespace {
constexpr int kMaxPartials = 8192;
constexpr size_t kSamplesPerPartial = 2048;
constexpr int kMaxDevices = 64;
}  // namespace

// The fixed scratch: one partial sum per 2048 samples. In host code the name
// g_partials is only a host-side stand-in for the symbol, never a device
// address; the address comes from cudaGetSymbolAddress below.
static __device__ __align__(256) double g_partials[kMaxPartials];

namespace {

// Device address of g_partials, looked up once per device ordinal and kept
// for the life of the process. It is the address in the device's primary
// context; cudaDeviceReset unloads the module and makes it stale.
double *g_partials_addr[kMaxDevices] = {};
std::mutex g_setup_mutex;

int fail(int code, const std::string &msg) {
  psv::set_last_error(msg);
  return code;
}

}  // namespace

extern "C" {

int psv_l2_misfit_noalloc(const double *obs_ux, const double *syn_ux, const double *obs_uz,
                          const double *syn_uz, size_t n, double dt, double *misfit,
                          void *stream) {
  if (!obs_ux || !syn_ux || !obs_uz || !syn_uz || !misfit)
    return fail(PSV_ERR_INVALID_ARGUMENT, "psv_l2_misfit_noalloc: NULL array");
  const size_t max_n = static_cast<size_t>(kMaxPartials) * kSamplesPerPartial;
  if (n > max_n)
    return fail(PSV_ERR_INVALID_ARGUMENT,
                "psv_l2_misfit_noalloc: " + std::to_string(n) +
                    " samples per component exceed the fixed-scratch maximum of " +
                    std::to_string(max_n));
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess)
    return fail(PSV_ERR_CUDA, std::string("cudaGetDevice: ") + cudaGetErrorString(e));
  if (dev < 0 || dev >= kMaxDevices)
    return fail(PSV_ERR_CUDA, "psv_l2_misfit_noalloc: device index beyond 63");
  double *scratch = nullptr;
  {
    // First call on this device (which is current): resolve the array's
    // device address. This touches no stream, but should still come before
    // any stream capture that contains the call.
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    if (!g_partials_addr[dev]) {
      void *addr = nullptr;
      e = cudaGetSymbolAddress(&addr, g_partials);
      if (e != cudaSuccess)
        return fail(PSV_ERR_CUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
      g_partials_addr[dev] = static_cast<double *>(addr);
    }
    scratch = g_partials_addr[dev];
  }
  // Every partial that the final sum reads is written by this launch, so the
  // scratch needs no clearing.
  size_t parts = (n + kSamplesPerPartial - 1) / kSamplesPerPartial;
  if (parts == 0) parts = 1;
  e = psv::misfit_l2(n, dt, obs_ux, syn_ux, obs_uz, syn_uz, scratch, static_cast<int>(parts),
                     misfit, static_cast<cudaStream_t>(stream));
  if (e != cudaSuccess)
    return fail(PSV_ERR_CUDA, std::string("psv_l2_misfit_noalloc: ") + cudaGetErrorString(e));
  return PSV_OK;
}

}  // extern "C"
