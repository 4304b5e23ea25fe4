// Allocation-free inner product for callers that cannot call cudaMalloc.
//
// lpg_dot_f64 keeps its partial sums in a buffer the library allocates with cudaMalloc
// on first use. Some callers cannot let a library allocate: host frameworks that own
// all device memory through their own pool (a cudaMalloc behind their back can fail or
// fragment what they reserved), and latency-sensitive loops where cudaMalloc/cudaFree
// would synchronise the device and stall other streams. For them this file keeps the
// partial sums in a fixed device array that is part of the loaded module, so no call
// allocates anything.
//
// Scratch: kNoAllocPartials = 1024 doubles (8 KB) on every GPU that loads the library,
// held until the process exits. The first stage of the reduction launches at most 1024
// CTAs (one partial each), so the array serves any accepted N; N is limited to
// 0 <= N <= 2^40 (8.8 TB of FP64 data, more than one GPU holds). Every stage-1 CTA
// overwrites its slot before stage 2 reads it, so nothing needs clearing between calls.
// All calls on a device share the array: calls that overlap on the GPU race.
#include <mutex>

#include "lpg_common.cuh"
#include "lpg_internal.hpp"

namespace {

constexpr int kNoAllocPartials = 1024;
constexpr int64_t kNoAllocMaxN = int64_t(1) << 40;

static __device__ __align__(256) double g_noalloc_partials[kNoAllocPartials];

std::mutex g_mu;
double* g_partials_addr[64] = {nullptr};

// Device address of g_noalloc_partials on the current device, resolved once per device
// with that device current. The symbol's name in host code is only a host-side stand-in.
int partials_address(double** out) {
  int dev = 0;
  LPG_CUDA_TRY(cudaGetDevice(&dev));
  if (dev < 0 || dev >= 64) return lpg::set_error(LPG_ERR_INVALID, "device index out of range");
  std::lock_guard<std::mutex> lk(g_mu);
  if (!g_partials_addr[dev]) {
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_partials);
    if (e != cudaSuccess)
      return lpg::set_error(LPG_ERR_CUDA, std::string("cudaGetSymbolAddress(g_noalloc_partials): ") +
                                              cudaGetErrorString(e));
    g_partials_addr[dev] = static_cast<double*>(p);
  }
  *out = g_partials_addr[dev];
  return LPG_OK;
}

}  // namespace

extern "C" int lpg_dot_f64_noalloc(int64_t N, const double* x, const double* y, double* result_dev,
                                   void* stream) {
  if (N < 0 || N > kNoAllocMaxN)
    return lpg::set_error(LPG_ERR_INVALID, "lpg_dot_f64_noalloc: N must be between 0 and 2^40 (got " +
                                               std::to_string(N) + ")");
  if (!result_dev || (N > 0 && (!x || !y))) return lpg::set_error(LPG_ERR_INVALID, "lpg_dot_f64_noalloc: null pointer");
  if (lpg::reduction_blocks(N) > kNoAllocPartials)
    return lpg::set_error(LPG_ERR_INVALID, "lpg_dot_f64_noalloc: more partial sums than the 1024-entry scratch");
  double* partials = nullptr;
  const int rc = partials_address(&partials);
  if (rc) return rc;
  return lpg::dot(N, x, y, result_dev, partials, (cudaStream_t)stream);
}
