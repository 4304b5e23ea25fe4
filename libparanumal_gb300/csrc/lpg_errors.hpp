// Status codes, error recording and CUDA-call checking usable from host (.cpp)
// and device (.cu) translation units.
#pragma once

#include <cuda_runtime_api.h>
#include <string>

#include "../../include/lpg.h"

namespace lpg {

// Records a message for lpg_last_error() and returns the status.
int set_error(int status, const std::string& msg);

inline int cuda_status(cudaError_t e, const char* what) {
  if (e == cudaSuccess) return LPG_OK;
  return set_error(LPG_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

}  // namespace lpg

#define LPG_CUDA_TRY(call)                                       \
  do {                                                           \
    cudaError_t _e = (call);                                     \
    if (_e != cudaSuccess) return ::lpg::cuda_status(_e, #call); \
  } while (0)

#define LPG_LAUNCH_CHECK(name)                                   \
  do {                                                           \
    cudaError_t _e = cudaGetLastError();                         \
    if (_e != cudaSuccess) return ::lpg::cuda_status(_e, name);  \
  } while (0)
