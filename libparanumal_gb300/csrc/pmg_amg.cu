// p-multigrid transfers (tensor-product restriction / prolongation between GLL degrees)
// and the sparse / dense kernels of the algebraic coarse levels.
//
// Restriction follows ellipticPartialPreconCoarsenHex3D
// (solvers/elliptic/okl/ellipticPreconCoarsenHex3D.okl:209-294) with the inverse-degree
// weighting (ellipticPreconMultiGridLevel.cpp:41-82) folded into the load and the coarse
// ogs Gather(Add, Trans) folded into the store (atomics). Prolongation follows
// ellipticPartialPreconProlongateHex3D (ellipticPreconProlongateHex3D.okl:216-301) with the
// Gather(NoTrans) + axpy folded into the store: the owning copy of each fine dof adds
// its value.
#include "lpg_common.cuh"
#include "lpg_internal.hpp"

namespace lpg {

template <typename T>
__global__ void __launch_bounds__(256)
pmg_coarsen_kernel(const int NqF, const int NqC, const int32_t* __restrict__ g2lF,
                   const T* __restrict__ wF, const T* __restrict__ xF, const T* __restrict__ Pg,
                   const int32_t* __restrict__ g2lC, T* __restrict__ xC) {
  __shared__ T s_f[kMaxNq * kMaxNq * kMaxNq];
  __shared__ T s_cff[kMaxNq * kMaxNq * kMaxNq];
  __shared__ T s_ccf[kMaxNq * kMaxNq * kMaxNq];
  __shared__ T s_P[kMaxNq * kMaxNq];
  const int64_t e = blockIdx.x;
  const int NpF = NqF * NqF * NqF, NpC = NqC * NqC * NqC;
  for (int t = threadIdx.x; t < NqF * NqC; t += blockDim.x) s_P[t] = Pg[t];
  for (int t = threadIdx.x; t < NpF; t += blockDim.x) {
    const int32_t g = g2lF[e * NpF + t];
    s_f[t] = (g >= 0) ? wF[g] * xF[g] : T(0);
  }
  __syncthreads();
  // k: s_cff[k][j][i] = sum_m P[m][k] f[m][j][i]
  for (int t = threadIdx.x; t < NqC * NqF * NqF; t += blockDim.x) {
    const int i = t % NqF, j = (t / NqF) % NqF, k = t / (NqF * NqF);
    T r = 0;
    for (int m = 0; m < NqF; ++m) r += s_P[m * NqC + k] * s_f[m * NqF * NqF + j * NqF + i];
    s_cff[t] = r;
  }
  __syncthreads();
  // j: s_ccf[k][j][i] = sum_m P[m][j] cff[k][m][i]
  for (int t = threadIdx.x; t < NqC * NqC * NqF; t += blockDim.x) {
    const int i = t % NqF, j = (t / NqF) % NqC, k = t / (NqF * NqC);
    T r = 0;
    for (int m = 0; m < NqF; ++m) r += s_P[m * NqC + j] * s_cff[k * NqF * NqF + m * NqF + i];
    s_ccf[t] = r;
  }
  __syncthreads();
  // i: qc[k][j][i] = sum_m P[m][i] ccf[k][j][m]
  for (int t = threadIdx.x; t < NpC; t += blockDim.x) {
    const int i = t % NqC, j = (t / NqC) % NqC, k = t / (NqC * NqC);
    T r = 0;
    for (int m = 0; m < NqF; ++m) r += s_P[m * NqC + i] * s_ccf[k * NqC * NqF + j * NqF + m];
    const int32_t g = g2lC[e * NpC + t];
    if (g >= 0) atomicAdd(xC + g, r);
  }
}

// Tensor-product transfers for fixed (fine, coarse) node counts per direction: several
// elements per CTA, Nq_f x Nq_f threads per element holding a fine k-pencil in
// registers, the other two directions through shared memory. Same arithmetic as the
// generic kernels above (ellipticPreconCoarsenHex3D.okl:209-294,
// ellipticPreconProlongateHex3D.okl:216-301).
template <int NQF, int NQC>
constexpr int tp_elems() { return 256 / (NQF * NQF); }

template <int NQF, int NQC, typename T>
__global__ void __launch_bounds__(256)
pmg_coarsen_tp_kernel(const int64_t E, const int32_t* __restrict__ g2lF, const T* __restrict__ wF,
                      const T* __restrict__ xF, const T* __restrict__ Pg, const int32_t* __restrict__ g2lC,
                      T* __restrict__ xC) {
  constexpr int EPB = tp_elems<NQF, NQC>(), NPF = NQF * NQF * NQF, NPC = NQC * NQC * NQC;
  __shared__ T s_P[NQF][NQC];                  // P[m][c] = l_c(x_m)
  __shared__ T s_u[EPB][NQC][NQF][NQF];        // [kc][j][i]
  __shared__ T s_v[EPB][NQC][NQC][NQF];        // [kc][jc][i]
  const int i = threadIdx.x, j = threadIdx.y, el = threadIdx.z;
  const int lt = i + NQF * j, tid = lt + NQF * NQF * el;
  for (int t = tid; t < NQF * NQC; t += 256) s_P[t / NQC][t % NQC] = Pg[t];
  const int64_t e = (int64_t)blockIdx.x * EPB + el;
  const bool active = e < E;
  T wx[NQF];
#pragma unroll
  for (int k = 0; k < NQF; ++k) {
    const int32_t g = active ? g2lF[e * NPF + k * NQF * NQF + lt] : -1;
    wx[k] = (g >= 0) ? wF[g] * xF[g] : T(0);
  }
  __syncthreads();
#pragma unroll
  for (int kc = 0; kc < NQC; ++kc) {
    T u = 0;
#pragma unroll
    for (int k = 0; k < NQF; ++k) u += s_P[k][kc] * wx[k];
    s_u[el][kc][j][i] = u;
  }
  __syncthreads();
  for (int p = j; p < NQC * NQC; p += NQF) {
    const int kc = p / NQC, jc = p % NQC;
    T v = 0;
#pragma unroll
    for (int m = 0; m < NQF; ++m) v += s_P[m][jc] * s_u[el][kc][m][i];
    s_v[el][kc][jc][i] = v;
  }
  __syncthreads();
  if (!active) return;
  for (int p = lt; p < NPC; p += NQF * NQF) {
    const int kc = p / (NQC * NQC), jc = (p / NQC) % NQC, ic = p % NQC;
    T c = 0;
#pragma unroll
    for (int m = 0; m < NQF; ++m) c += s_P[m][ic] * s_v[el][kc][jc][m];
    const int32_t g = g2lC[e * NPC + p];
    if (g >= 0) atomicAdd(xC + g, c);
  }
}

template <int NQF, int NQC, typename T>
__global__ void __launch_bounds__(256)
pmg_prolong_tp_kernel(const int64_t E, const int32_t* __restrict__ g2lC, const T* __restrict__ xC,
                      const T* __restrict__ Pg, const int32_t* __restrict__ g2lF, const int32_t* __restrict__ ownerF,
                      T* __restrict__ xF) {
  constexpr int EPB = tp_elems<NQF, NQC>(), NPF = NQF * NQF * NQF, NPC = NQC * NQC * NQC;
  __shared__ T s_P[NQF][NQC];
  __shared__ T s_c[EPB][NQC][NQC][NQC];        // coarse values [kc][jc][ic]
  __shared__ T s_cf[EPB][NQC][NQC][NQF];       // [kc][jc][i]
  const int i = threadIdx.x, j = threadIdx.y, el = threadIdx.z;
  const int lt = i + NQF * j, tid = lt + NQF * NQF * el;
  for (int t = tid; t < NQF * NQC; t += 256) s_P[t / NQC][t % NQC] = Pg[t];
  const int64_t e = (int64_t)blockIdx.x * EPB + el;
  const bool active = e < E;
  for (int p = lt; p < NPC; p += NQF * NQF) {
    const int32_t g = active ? g2lC[e * NPC + p] : -1;
    s_c[el][p / (NQC * NQC)][(p / NQC) % NQC][p % NQC] = (g >= 0) ? xC[g] : T(0);
  }
  __syncthreads();
  for (int p = j; p < NQC * NQC; p += NQF) {
    const int kc = p / NQC, jc = p % NQC;
    T v = 0;
#pragma unroll
    for (int m = 0; m < NQC; ++m) v += s_P[i][m] * s_c[el][kc][jc][m];
    s_cf[el][kc][jc][i] = v;
  }
  __syncthreads();
  if (!active) return;
  T u[NQC];
#pragma unroll
  for (int kc = 0; kc < NQC; ++kc) {
    T v = 0;
#pragma unroll
    for (int m = 0; m < NQC; ++m) v += s_P[j][m] * s_cf[el][kc][m][i];
    u[kc] = v;
  }
  // the owning copy of each fine dof adds the value; nodes strictly inside the element
  // (no other copy) are their own owners
  const bool inner_ij = i > 0 && i < NQF - 1 && j > 0 && j < NQF - 1;
#pragma unroll
  for (int k = 0; k < NQF; ++k) {
    T f = 0;
#pragma unroll
    for (int m = 0; m < NQC; ++m) f += s_P[k][m] * u[m];
    const int64_t id = e * NPF + k * NQF * NQF + lt;
    const int32_t g = g2lF[id];
    if (g < 0) continue;
    if ((inner_ij && k > 0 && k < NQF - 1) || ownerF[g] == (int32_t)id) xF[g] += f;
  }
}

template <int NQF, int NQC>
static bool tp_pair(int Nf, int Nc) { return Nf + 1 == NQF && Nc + 1 == NQC; }

template <typename T>
int pmg_coarsen(int Nf, int Nc, int64_t E, const int32_t* g2lF, const T* weightF, const T* xF,
                const T* P, const int32_t* g2lC, T* xC, int64_t NglobalC, cudaStream_t s) {
  if (Nf + 1 > kMaxNq || Nc < 1 || Nc > Nf) return set_error(LPG_ERR_UNSUPPORTED, "pmg_coarsen: bad degrees");
  LPG_CUDA_TRY(cudaMemsetAsync(xC, 0, sizeof(T) * NglobalC, s));
  if (E <= 0) return LPG_OK;
  if (tp_pair<8, 4>(Nf, Nc) || tp_pair<4, 2>(Nf, Nc)) {
    if (Nf == 7) {
      pmg_coarsen_tp_kernel<8, 4, T><<<(unsigned)((E + 3) / 4), dim3(8, 8, 4), 0, s>>>(E, g2lF, weightF, xF, P, g2lC, xC);
    } else {
      pmg_coarsen_tp_kernel<4, 2, T><<<(unsigned)((E + 15) / 16), dim3(4, 4, 16), 0, s>>>(E, g2lF, weightF, xF, P, g2lC,
                                                                                           xC);
    }
    LPG_LAUNCH_CHECK("pmg_coarsen_tp_kernel");
    return LPG_OK;
  }
  pmg_coarsen_kernel<T><<<(unsigned)E, 256, 0, s>>>(Nf + 1, Nc + 1, g2lF, weightF, xF, P, g2lC, xC);
  LPG_LAUNCH_CHECK("pmg_coarsen_kernel");
  return LPG_OK;
}

template <typename T>
__global__ void __launch_bounds__(256)
pmg_prolong_kernel(const int NqF, const int NqC, const int32_t* __restrict__ g2lC,
                   const T* __restrict__ xC, const T* __restrict__ Pg, const int32_t* __restrict__ g2lF,
                   const int32_t* __restrict__ ownerF, T* __restrict__ xF) {
  __shared__ T s_ccc[kMaxNq * kMaxNq * kMaxNq];
  __shared__ T s_ccf[kMaxNq * kMaxNq * kMaxNq];
  __shared__ T s_cff[kMaxNq * kMaxNq * kMaxNq];
  __shared__ T s_P[kMaxNq * kMaxNq];
  const int64_t e = blockIdx.x;
  const int NpF = NqF * NqF * NqF, NpC = NqC * NqC * NqC;
  for (int t = threadIdx.x; t < NqF * NqC; t += blockDim.x) s_P[t] = Pg[t];
  for (int t = threadIdx.x; t < NpC; t += blockDim.x) {
    const int32_t g = g2lC[e * NpC + t];
    s_ccc[t] = (g >= 0) ? xC[g] : T(0);
  }
  __syncthreads();
  // i: ccf[k][j][i] = sum_m P[i][m] ccc[k][j][m]
  for (int t = threadIdx.x; t < NqC * NqC * NqF; t += blockDim.x) {
    const int i = t % NqF, j = (t / NqF) % NqC, k = t / (NqF * NqC);
    T r = 0;
    for (int m = 0; m < NqC; ++m) r += s_P[i * NqC + m] * s_ccc[k * NqC * NqC + j * NqC + m];
    s_ccf[t] = r;
  }
  __syncthreads();
  // j: cff[k][j][i] = sum_m P[j][m] ccf[k][m][i]
  for (int t = threadIdx.x; t < NqC * NqF * NqF; t += blockDim.x) {
    const int i = t % NqF, j = (t / NqF) % NqF, k = t / (NqF * NqF);
    T r = 0;
    for (int m = 0; m < NqC; ++m) r += s_P[j * NqC + m] * s_ccf[k * NqC * NqF + m * NqF + i];
    s_cff[t] = r;
  }
  __syncthreads();
  // k: f[k][j][i] = sum_m P[k][m] cff[m][j][i]; the owning copy adds it to xF
  for (int t = threadIdx.x; t < NpF; t += blockDim.x) {
    const int i = t % NqF, j = (t / NqF) % NqF, k = t / (NqF * NqF);
    T r = 0;
    for (int m = 0; m < NqC; ++m) r += s_P[k * NqC + m] * s_cff[m * NqF * NqF + j * NqF + i];
    const int64_t id = e * NpF + t;
    const int32_t g = g2lF[id];
    if (g >= 0 && ownerF[g] == (int32_t)id) xF[g] += r;
  }
}

template <typename T>
int pmg_prolongate_map(int Nf, int Nc, int64_t E, const int32_t* g2lC, const T* xC, const T* P,
                       const int32_t* g2lF, const int32_t* ownerF, T* xF, cudaStream_t s) {
  if (Nf + 1 > kMaxNq || Nc < 1 || Nc > Nf) return set_error(LPG_ERR_UNSUPPORTED, "pmg_prolongate: bad degrees");
  if (E <= 0) return LPG_OK;
  if (tp_pair<8, 4>(Nf, Nc) || tp_pair<4, 2>(Nf, Nc)) {
    if (Nf == 7) {
      pmg_prolong_tp_kernel<8, 4, T><<<(unsigned)((E + 3) / 4), dim3(8, 8, 4), 0, s>>>(E, g2lC, xC, P, g2lF, ownerF, xF);
    } else {
      pmg_prolong_tp_kernel<4, 2, T><<<(unsigned)((E + 15) / 16), dim3(4, 4, 16), 0, s>>>(E, g2lC, xC, P, g2lF, ownerF,
                                                                                           xF);
    }
    LPG_LAUNCH_CHECK("pmg_prolong_tp_kernel");
    return LPG_OK;
  }
  pmg_prolong_kernel<T><<<(unsigned)E, 256, 0, s>>>(Nf + 1, Nc + 1, g2lC, xC, P, g2lF, ownerF, xF);
  LPG_LAUNCH_CHECK("pmg_prolong_kernel");
  return LPG_OK;
}

template int pmg_coarsen<double>(int, int, int64_t, const int32_t*, const double*, const double*, const double*,
                                 const int32_t*, double*, int64_t, cudaStream_t);
template int pmg_coarsen<float>(int, int, int64_t, const int32_t*, const float*, const float*, const float*,
                                const int32_t*, float*, int64_t, cudaStream_t);
template int pmg_prolongate_map<double>(int, int, int64_t, const int32_t*, const double*, const double*,
                                        const int32_t*, const int32_t*, double*, cudaStream_t);
template int pmg_prolongate_map<float>(int, int, int64_t, const int32_t*, const float*, const float*,
                                       const int32_t*, const int32_t*, float*, cudaStream_t);

// ---------------------------------------------------------------- CSR (AMG levels)
// Eight lanes per row: AMG rows of the N=1 hierarchy hold ~7-30 nonzeros.
constexpr int kLanesPerRow = 8;

__global__ void __launch_bounds__(256)
csr_spmv_kernel(const int64_t Nrows, const int64_t* __restrict__ rs, const int32_t* __restrict__ cols,
                const double* __restrict__ vals, const double alpha, const double* __restrict__ x,
                const double beta, double* __restrict__ y) {
  const int64_t row = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) / kLanesPerRow;
  const int lane = threadIdx.x % kLanesPerRow;
  double acc = 0;
  if (row < Nrows)
    for (int64_t jj = rs[row] + lane; jj < rs[row + 1]; jj += kLanesPerRow) acc += vals[jj] * x[cols[jj]];
  for (int o = kLanesPerRow / 2; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o, kLanesPerRow);
  if (row < Nrows && lane == 0) y[row] = (beta != 0.0) ? alpha * acc + beta * y[row] : alpha * acc;
}

int csr_spmv(int64_t Nrows, const int64_t* rowStarts, const int32_t* cols, const double* vals, double alpha,
             const double* x, double beta, double* y, cudaStream_t s) {
  if (Nrows <= 0) return LPG_OK;
  const int64_t threads = Nrows * kLanesPerRow;
  csr_spmv_kernel<<<(unsigned)((threads + 255) / 256), 256, 0, s>>>(Nrows, rowStarts, cols, vals, alpha, x,
                                                                    beta, y);
  LPG_LAUNCH_CHECK("csr_spmv_kernel");
  return LPG_OK;
}

__global__ void csr_cheb_start_kernel(const int64_t N, const double invTheta, const double* __restrict__ diagInv,
                                      const double* __restrict__ b, double* __restrict__ r,
                                      double* __restrict__ d, double* __restrict__ x) {
  for (int64_t n = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; n < N; n += (int64_t)gridDim.x * blockDim.x) {
    const double rr = diagInv[n] * b[n];
    r[n] = rr;
    d[n] = invTheta * rr;
    x[n] = invTheta * rr;
  }
}
int csr_cheb_start(int64_t N, double invTheta, const double* diagInv, const double* b, double* r, double* d,
                   double* x, cudaStream_t s) {
  if (N <= 0) return LPG_OK;
  csr_cheb_start_kernel<<<(unsigned)std::min<int64_t>((N + 255) / 256, 4096), 256, 0, s>>>(N, invTheta, diagInv, b,
                                                                                          r, d, x);
  LPG_LAUNCH_CHECK("csr_cheb_start_kernel");
  return LPG_OK;
}

// r = alpha r + D^{-1} (beta b - A x)
__global__ void __launch_bounds__(256)
csr_cheb_residual_kernel(const int64_t Nrows, const int64_t* __restrict__ rs, const int32_t* __restrict__ cols,
                         const double* __restrict__ vals, const double alpha, const double beta,
                         const double* __restrict__ diagInv, const double* __restrict__ b,
                         const double* __restrict__ x, double* __restrict__ r) {
  const int64_t row = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) / kLanesPerRow;
  const int lane = threadIdx.x % kLanesPerRow;
  double acc = 0;
  if (row < Nrows)
    for (int64_t jj = rs[row] + lane; jj < rs[row + 1]; jj += kLanesPerRow) acc += vals[jj] * x[cols[jj]];
  for (int o = kLanesPerRow / 2; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o, kLanesPerRow);
  if (row < Nrows && lane == 0) {
    const double res = ((beta != 0.0) ? beta * b[row] : 0.0) - acc;
    const double rk = (alpha != 0.0) ? alpha * r[row] : 0.0;
    r[row] = rk + diagInv[row] * res;
  }
}
int csr_cheb_residual(int64_t N, const int64_t* rowStarts, const int32_t* cols, const double* vals, double alpha,
                      double beta, const double* diagInv, const double* b, const double* x, double* r,
                      cudaStream_t s) {
  if (N <= 0) return LPG_OK;
  const int64_t threads = N * kLanesPerRow;
  csr_cheb_residual_kernel<<<(unsigned)((threads + 255) / 256), 256, 0, s>>>(N, rowStarts, cols, vals, alpha,
                                                                             beta, diagInv, b, x, r);
  LPG_LAUNCH_CHECK("csr_cheb_residual_kernel");
  return LPG_OK;
}

// d = a d + b r ; x += d   (SmoothChebyshevUpdate)
__global__ void csr_cheb_update_kernel(const int64_t N, const double a, const double b, const int lastIt,
                                       const double* __restrict__ r, double* __restrict__ d,
                                       double* __restrict__ x) {
  for (int64_t n = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; n < N; n += (int64_t)gridDim.x * blockDim.x) {
    const double dk = (a != 0.0) ? d[n] : 0.0;
    const double dn = a * dk + b * r[n];
    if (!lastIt) d[n] = dn;
    x[n] += dn;
  }
}
int csr_cheb_update(int64_t N, double a, double b, int lastIt, const double* r, double* d, double* x,
                    cudaStream_t s) {
  if (N <= 0) return LPG_OK;
  csr_cheb_update_kernel<<<(unsigned)std::min<int64_t>((N + 255) / 256, 4096), 256, 0, s>>>(N, a, b, lastIt, r,
                                                                                           d, x);
  LPG_LAUNCH_CHECK("csr_cheb_update_kernel");
  return LPG_OK;
}

// ---------------------------------------------------------------- dense coarse solve
// One warp per row of the dense inverse (parAlmond okl/dGEMV.okl).
__global__ void __launch_bounds__(256)
gemv_kernel(const int64_t n, const double* __restrict__ A, const double* __restrict__ x, double* __restrict__ y) {
  const int64_t row = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (row >= n) return;
  double acc = 0;
  for (int64_t j = lane; j < n; j += 32) acc += A[row * n + j] * x[j];
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
  if (lane == 0) y[row] = acc;
}
int gemv(int64_t n, const double* A, const double* x, double* y, cudaStream_t s) {
  if (n <= 0) return LPG_OK;
  gemv_kernel<<<(unsigned)((n * 32 + 255) / 256), 256, 0, s>>>(n, A, x, y);
  LPG_LAUNCH_CHECK("gemv_kernel");
  return LPG_OK;
}

}  // namespace lpg
