// Shared device-side definitions of the GB300 (sm_103a) elliptic library:
// launch helpers and geometric-factor load conversions.
#pragma once

#include <cuda_runtime.h>
#include <cuda_bf16.h>
#include <cstdint>

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

}  // namespace lpg
