// Shared device-side definitions of the GB300 (sm_103a) elliptic library:
// launch helpers and geometric-factor load conversions.
#pragma once

#include <cuda_runtime.h>
#include <cuda_bf16.h>
#include <cstdint>
#include <mutex>

#include "lpg_errors.hpp"

namespace lpg {

inline cudaStream_t as_stream(void* s) { return reinterpret_cast<cudaStream_t>(s); }

// Geometric-factor storage types: FP64, FP32, or BF16 (FP32 accumulation).
template <typename T, typename G> __device__ __forceinline__ T load_geo(const G* p) { return (T)(*p); }
template <> __device__ __forceinline__ float load_geo<float, __nv_bfloat16>(const __nv_bfloat16* p) {
  return __bfloat162float(__ldg(p));
}
template <> __device__ __forceinline__ double load_geo<double, double>(const double* p) { return __ldg(p); }
template <> __device__ __forceinline__ float load_geo<float, float>(const float* p) { return __ldg(p); }

constexpr int kMaxNq = 9;   // polynomial degree N <= 8 in the device kernels

#define LPG_PI 3.14159265358979323846

// Launch configuration of one kernel on one device: SM count and resident CTAs per SM.
struct KernelConfig {
  int numSMs = 0;
  int ctasPerSM = 1;
};

// One-time set-up of a kernel per device. Function attributes (the dynamic shared-memory
// opt-in) and occupancy belong to the device a kernel launches on, so the set-up runs once
// for every device index the calling thread has current, under a mutex (concurrent first
// calls from several host threads are ordered). `setup(dev, cfg)` fills cfg and returns a
// status; a failed set-up is retried on the next call.
constexpr int kMaxDevices = 64;
class PerDeviceConfig {
 public:
  template <typename F>
  int get(F setup, KernelConfig* out) {
    int dev = 0;
    LPG_CUDA_TRY(cudaGetDevice(&dev));
    if (dev < 0 || dev >= kMaxDevices) return set_error(LPG_ERR_UNSUPPORTED, "device index beyond 64");
    std::lock_guard<std::mutex> lk(mu_);
    if (!done_[dev]) {
      KernelConfig c;
      LPG_CUDA_TRY(cudaDeviceGetAttribute(&c.numSMs, cudaDevAttrMultiProcessorCount, dev));
      const int rc = setup(dev, c);
      if (rc) return rc;
      cfg_[dev] = c;
      done_[dev] = true;
    }
    *out = cfg_[dev];
    return LPG_OK;
  }

 private:
  std::mutex mu_;
  bool done_[kMaxDevices] = {};
  KernelConfig cfg_[kMaxDevices];
};

}  // namespace lpg
