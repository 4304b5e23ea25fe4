// Plot-node interpolation for VTU output (mesh_t::PlotInterpHex3D,
// meshPlotInterpHex3D.cpp:30-100; plot nodes from meshReferenceNodesHex3D.cpp:53-63):
// per element, a degree-N nodal field is evaluated at the (N+4)^3 equispaced plot nodes
// by three 1D contractions (r, then s, then t), and the plot-node coordinates are the
// trilinear image of the element's 8 vertices.
#include <cuda_runtime.h>

#include <cstdint>

#include "lpg_errors.hpp"
#include "lpg_internal.hpp"

namespace lpg {

namespace {

constexpr int kMaxNq = 9;        // N <= 8
constexpr int kMaxPlotNq = 12;   // N + 4

__global__ void __launch_bounds__(256)
plot_interp_kernel(int Nq, int pNq, const double* __restrict__ I, const double* __restrict__ q,
                   const double* __restrict__ EX, const double* __restrict__ EY, const double* __restrict__ EZ,
                   const double* __restrict__ pr, double* __restrict__ out) {
  __shared__ double s_q[kMaxNq * kMaxNq * kMaxNq];
  __shared__ double s_a[kMaxPlotNq * kMaxNq * kMaxNq];
  __shared__ double s_b[kMaxPlotNq * kMaxPlotNq * kMaxNq];
  __shared__ double s_I[kMaxPlotNq * kMaxNq];
  const int64_t e = blockIdx.x;
  const int Np = Nq * Nq * Nq, pNp = pNq * pNq * pNq;
  for (int n = threadIdx.x; n < Np; n += blockDim.x) s_q[n] = q[e * Np + n];
  for (int n = threadIdx.x; n < pNq * Nq; n += blockDim.x) s_I[n] = I[n];
  __syncthreads();
  // r: a[k][j][i'] = sum_m I[i'][m] q[k][j][m]
  for (int n = threadIdx.x; n < pNq * Nq * Nq; n += blockDim.x) {
    const int i = n % pNq, j = (n / pNq) % Nq, k = n / (pNq * Nq);
    double acc = 0;
    for (int m = 0; m < Nq; ++m) acc += s_I[i * Nq + m] * s_q[m + j * Nq + k * Nq * Nq];
    s_a[n] = acc;
  }
  __syncthreads();
  // s: b[k][j'][i'] = sum_m I[j'][m] a[k][m][i']
  for (int n = threadIdx.x; n < pNq * pNq * Nq; n += blockDim.x) {
    const int i = n % pNq, j = (n / pNq) % pNq, k = n / (pNq * pNq);
    double acc = 0;
    for (int m = 0; m < Nq; ++m) acc += s_I[j * Nq + m] * s_a[i + m * pNq + k * pNq * Nq];
    s_b[n] = acc;
  }
  __syncthreads();
  // t, and the plot-node coordinates; out = [e][4][pNp]: x, y, z, field
  double vx[8], vy[8], vz[8];
#pragma unroll
  for (int v = 0; v < 8; ++v) { vx[v] = EX[e * 8 + v]; vy[v] = EY[e * 8 + v]; vz[v] = EZ[e * 8 + v]; }
  double* o = out + e * 4 * (int64_t)pNp;
  for (int n = threadIdx.x; n < pNp; n += blockDim.x) {
    const int i = n % pNq, j = (n / pNq) % pNq, k = n / (pNq * pNq);
    double acc = 0;
    for (int m = 0; m < Nq; ++m) acc += s_I[k * Nq + m] * s_b[i + j * pNq + m * pNq * pNq];
    const double r = pr[i], s = pr[j], t = pr[k];
    const double w[8] = {(1 - r) * (1 - s) * (1 - t), (1 + r) * (1 - s) * (1 - t), (1 + r) * (1 + s) * (1 - t),
                         (1 - r) * (1 + s) * (1 - t), (1 - r) * (1 - s) * (1 + t), (1 + r) * (1 - s) * (1 + t),
                         (1 + r) * (1 + s) * (1 + t), (1 - r) * (1 + s) * (1 + t)};
    double x = 0, y = 0, z = 0;
#pragma unroll
    for (int v = 0; v < 8; ++v) { x += 0.125 * w[v] * vx[v]; y += 0.125 * w[v] * vy[v]; z += 0.125 * w[v] * vz[v]; }
    o[n] = x;
    o[pNp + n] = y;
    o[2 * pNp + n] = z;
    o[3 * pNp + n] = acc;
  }
}

}  // namespace

int plot_interp(int N, int64_t E, const double* I, const double* pr, const double* qL, const double* EX,
                const double* EY, const double* EZ, double* out, cudaStream_t s) {
  if (N < 1 || N + 1 > kMaxNq) return set_error(LPG_ERR_UNSUPPORTED, "plot: POLYNOMIAL DEGREE must be 1..8");
  if (E <= 0) return LPG_OK;
  plot_interp_kernel<<<(unsigned)E, 256, 0, s>>>(N + 1, N + 4, I, qL, EX, EY, EZ, pr, out);
  LPG_LAUNCH_CHECK("plot_interp_kernel");
  return LPG_OK;
}

}  // namespace lpg
