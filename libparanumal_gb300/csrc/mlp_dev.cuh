// Device helpers shared by the MLP kernels: GELU in its tanh form and its derivative
// (the activation the learned smoother is trained and run with).
#pragma once

#include <cuda_runtime.h>

namespace lpg {

__device__ __forceinline__ float gelu_f(float z) {
  const float c = 0.7978845608028654f;  // sqrt(2/pi)
  const float u = c * (z + 0.044715f * z * z * z);
  return 0.5f * z * (1.0f + tanhf(u));
}
__device__ __forceinline__ float gelu_grad_f(float z) {
  const float c = 0.7978845608028654f;
  const float u = c * (z + 0.044715f * z * z * z);
  const float t = tanhf(u);
  const float du = c * (1.0f + 3.0f * 0.044715f * z * z);
  return 0.5f * (1.0f + t) + 0.5f * z * (1.0f - t * t) * du;
}

}  // namespace lpg
