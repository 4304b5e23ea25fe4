// Element-local MLP of the learned fine-level smoother: sizes, parameter layout and
// kernel entry points (mlp.cu).
#pragma once

#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <cstdint>

#include "lpg_internal.hpp"

namespace lpg {

constexpr int kMlpIn = 896;      // 512 element residual values + 6 x 64 face traces (N = 7)
constexpr int kMlpHidden = 256;
constexpr int kMlpOut = 512;
constexpr int kMlpNq = 8;        // the network is defined for N = 7 (8 x 8 x 8 nodes)
// parameter vector: W0 (896x256), b0, W1 (256x256), b1, W2 (256x256), b2, W3 (256x512), b3
constexpr int64_t kMlpParams = (int64_t)kMlpIn * kMlpHidden + kMlpHidden + 2 * ((int64_t)kMlpHidden * kMlpHidden + kMlpHidden) +
                               (int64_t)kMlpHidden * kMlpOut + kMlpOut;

struct MLPParams {
  float* W[4];
  float* b[4];
  static MLPParams view(float* base) {
    MLPParams p;
    const int dims[5] = {kMlpIn, kMlpHidden, kMlpHidden, kMlpHidden, kMlpOut};
    int64_t off = 0;
    for (int l = 0; l < 4; ++l) {
      p.W[l] = base + off;
      off += (int64_t)dims[l] * dims[l + 1];
      p.b[l] = base + off;
      off += dims[l + 1];
    }
    return p;
  }
};

// Activations of a batch of B rows: A[l] = layer outputs (B x 256, last B x 512), Z[l] =
// pre-activations of the hidden layers. Workspace floats: B * (3*256*2 + 512).
struct MLPActs {
  float* A[4];
  float* Z[3];
  static int64_t floats(int64_t B) { return B * (6 * (int64_t)kMlpHidden + kMlpOut); }
  static MLPActs view(float* base, int64_t B) {
    MLPActs a;
    int64_t off = 0;
    for (int l = 0; l < 3; ++l) { a.A[l] = base + off; off += B * kMlpHidden; }
    a.A[3] = base + off;
    off += B * kMlpOut;
    for (int l = 0; l < 3; ++l) { a.Z[l] = base + off; off += B * kMlpHidden; }
    return a;
  }
};

int sgemm(bool ta, bool tb, int M, int N, int K, const float* A, int lda, const float* B, int ldb, float* C,
          int ldc, const float* bias, bool gelu, float* Z, float beta, cudaStream_t s);
int mlp_forward_f32(const MLPParams& P, int B, const float* X, MLPActs& act, cudaStream_t s);
// gradients into G (same layout as P); work0/work1 hold B x 256 floats each
int mlp_backward_f32(const MLPParams& P, int B, const float* X, const MLPActs& act, const float* dY, MLPParams& G,
                     float* work0, float* work1, cudaStream_t s);
int mse_loss(int64_t n, int B, const float* y, const float* t, float* dy, float* loss, cudaStream_t s);
int adam_step(int64_t n, float* w, const float* g, float* m, float* v, float lr, int step, cudaStream_t s);

int bf16_linear(int M, int N, int K, const __nv_bfloat16* X, const __nv_bfloat16* Wt, const float* bias, bool gelu,
                bool outBf16, void* Y, cudaStream_t s);
int transpose_to_bf16(int K, int N, const float* W, __nv_bfloat16* Wt, cudaStream_t s);
// Fused inference Y (B x 512, FP32) = MLP(X (B x 896, BF16)) on the tcgen05 tensor cores
// (all four layers per 128-row tile on one SM). Wt[l]: BF16 weights stored N x K (K
// contiguous), bias[l] FP32. errFlag (device int) is set to a nonzero code if a CTA's
// pipeline timed out and is never cleared here: the caller clears it, runs any number of
// launches and reads it once after the stream has run.
int mlp_forward_tc(int64_t B, const __nv_bfloat16* X, const __nv_bfloat16* const Wt[4], const float* const bias[4],
                   float* Y, int* errFlag, cudaStream_t s);
// Diagnostics: every following mlp_forward_tc launch first waits up to ns nanoseconds on a
// barrier that nothing signals, then records a pipeline timeout (code 8) before issuing any
// copy or MMA; 0 turns this off.
void mlp_tc_set_hold(unsigned long long ns);

template <typename TIN, typename TOUT>
// scale_e = max(RMS of the element's residual, sfloor); features = values / scale_e
int element_features(const BoxNumbering& b, int64_t E, int64_t e0, int64_t count, const int32_t* g2l, const TIN* r,
                     TOUT* X, float* scale, float sfloor, cudaStream_t s);
// z[g] += coef[g] * scale[e] * out[e][n] over the local nodes (coef = weight / diag)
template <typename TV>
int apply_correction(int Np, int64_t count, int64_t e0, const int32_t* g2l, const float* out, const float* scale,
                     const TV* coef, TV* z, cudaStream_t s);
// The same correction summed per global lattice node, one thread per node of the lattice
// planes Zbegin <= Z < Zend: z[g] += coef[g] * sum over the copies (e, n) of the node of
// scale[e] * out[e][n] (out and scale indexed by global element; the elements touching
// those planes must be filled). No atomics: each dof is written by one thread.
template <typename TV>
int lattice_correction(const BoxNumbering& b, const int32_t* g2l, const float* out, const float* scale,
                       const TV* coef, TV* z, int Zbegin, int Zend, cudaStream_t s);
int training_targets(int Np, int64_t count, const int32_t* elems, const int32_t* g2l, const double* e,
                     const double* invDiag, const float* scale, float* T, cudaStream_t s);
int gather_rows(int64_t count, const int32_t* elems, const float* Xall, float* X, cudaStream_t s);
// dst[i][:] = src[idx[i]][:], rows of `width` floats
int gather_rows_w(int64_t count, int width, const int32_t* idx, const float* src, float* dst, cudaStream_t s);
// T[i][n] -= w X[i][n], n < kMlpOut (targets of a damped-Jacobi + network smoother)
int subtract_inputs(int64_t count, float w, const float* X, float* T, cudaStream_t s);
// T (E x 512) = (e - F e) / (invDiag s_e) per element, F the 1D modal low-pass (Nq x Nq)
int highpass_targets(int Nq, int64_t E, const int32_t* g2l, const double* e, const double* invDiag, const float* scale,
                     const double* F, float* T, cudaStream_t s);

}  // namespace lpg
