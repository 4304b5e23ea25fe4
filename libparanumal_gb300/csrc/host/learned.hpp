// Learned fine-level smoother: inference object and training driver.
#pragma once

#include <vector>

#include "objects.hpp"

namespace lpg {

struct LearnedSmoother {
  static constexpr int64_t kChunk = 65536;  // elements per inference pass
  // element scales are floored at this fraction of the global residual RMS, so elements
  // with (near-)zero residual get small inputs instead of amplified noise
  static constexpr double kScaleFloor = 1e-3;
  bool ready = false;
  DevBuf<double> red, partials;
  DevBuf<float> params;                     // FP32 master weights (MLPParams layout)
  DevBuf<__nv_bfloat16> Wt[4];              // BF16 transposed weights for inference
  DevBuf<__nv_bfloat16> X, H0, H1;
  DevBuf<float> out, scale;
  // outputs and scales of all E elements, for the one-pass lattice correction
  DevBuf<float> outAll, scaleAll;
  DevBuf<int> tcErr;                        // timeout flag of the tensor-core kernel
  int64_t chunk = 0, allRows = 0;
  int load(const float* hostParams, cudaStream_t s);
  int ensure_chunk(int64_t rows);
  int forward_bf16(int64_t rows, float* dst, cudaStream_t s);   // dst = MLP(X) for `rows` rows
  int check_tc(cudaStream_t s);            // waits for the stream; LPG_ERR_TIMEOUT if set
  int clear_tc(cudaStream_t s);            // clears the timeout flag (stream-ordered)
  // z (assembled) += sum over copies of coef .* s_e MLP(features(r)), coef = weight / diag
  // (the average over copies of s_e invDiag .* output). Element scales s_e are floored at
  // sfloor (the caller's kScaleFloor x residual RMS). The network runs in chunks of kChunk
  // elements and each chunk's copies are added with atomics. LPG_LEARNED_CORRECTION=lattice (a tuning override, measured 3-7 % slower per
  // solve at 64^3 and 112^3) keeps all outputs and sums each dof's copies in one thread per
  // lattice node instead, in whole element layers as each chunk completes them. The
  // tensor-core timeout flag accumulates: clear_tc before, check_tc after a batch of calls.
  template <typename T>
  int apply(const BoxNumbering& b, int64_t E, const int32_t* g2l, const T* r, const T* coef, T* z, int64_t Nglobal,
            float sfloor, cudaStream_t s);
};

struct TrainOptions {
  int nsolves = 4;
  int samplesPerSolve = 5000;
  int epochs = 30;
  int batch = 250;
  float lr = 1e-3f;
  int bumps = 8;
  double solveTol = 1e-10;
  uint64_t seed = 7;
  double targetCap = 4.0;   // keep samples whose RMS normalised target is at most this
  // odd-numbered sample sets are synthetic: e = random lattice noise smoothed by 0, 2 or
  // 6 damped-Jacobi sweeps, r = A e (no solve), instead of a solver-trajectory pair
  bool synthetic = true;
};

// fraction of elements that passed the sample filter in the last training run
extern double lastKeptFraction;

// Generates (residual, exact error) samples with the plain solver `plainMG` on `el` and
// trains the network; returns FP32 weights and the per-epoch mean training loss.
int train_smoother(Platform* plat, Elliptic* el, Precon* plainMG, const BoxNumbering& b, const TrainOptions& o,
                   std::vector<float>& weights, std::vector<float>& lossHistory);

}  // namespace lpg
