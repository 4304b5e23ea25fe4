// Element-local MLP of the learned fine-level smoother (no reference counterpart).
//
// Network: 896 -> 256 -> 256 -> 256 -> 512, GELU (tanh form) after the hidden layers.
// Input per element: its 512 residual values and the 6 x 64 residual values of the first
// interior node layer of each face neighbour (zero on boundary faces), all divided by the
// element's residual RMS s_e. Output: 512 values; the smoother's correction at the
// element's nodes is s_e * invDiag * output, averaged over shared nodes.
//
// Training runs in FP32 (tiled SIMT GEMMs with fused bias/GELU epilogues, backward,
// Adam); inference uses BF16 tensor-core tiles (mma.sync m16n8k16, FP32 accumulate)
// with BF16 activations between layers and an FP32 output layer.
#include "lpg_common.cuh"
#include "lpg_internal.hpp"
#include "mlp.hpp"
#include "mlp_dev.cuh"

namespace lpg {

// ---------------------------------------------------------------- FP32 tiled GEMM
// C[M x N] (+)= op(A)[M x K] * op(B)[K x N] (+ bias[N]); optional GELU with the
// pre-activation stored in Z. Row-major; TA: A is stored K x M; TB: B is stored N x K.
constexpr int SG_BM = 64, SG_BN = 64, SG_BK = 16;

template <bool TA, bool TB>
__global__ void __launch_bounds__(256)
sgemm_kernel(const int M, const int N, const int K, const float* __restrict__ A, const int lda,
             const float* __restrict__ B, const int ldb, float* __restrict__ C, const int ldc,
             const float* __restrict__ bias, const int act, float* __restrict__ Z, const float beta) {
  __shared__ float sA[SG_BK][SG_BM + 4];
  __shared__ float sB[SG_BK][SG_BN + 4];
  const int tx = threadIdx.x % 16, ty = threadIdx.x / 16;
  const int m0 = blockIdx.y * SG_BM, n0 = blockIdx.x * SG_BN;
  float acc[4][4] = {};
  for (int k0 = 0; k0 < K; k0 += SG_BK) {
    for (int t = threadIdx.x; t < SG_BK * SG_BM; t += 256) {
      const int kk = t / SG_BM, mm = t % SG_BM;
      const int gm = m0 + mm, gk = k0 + kk;
      float v = 0.f;
      if (gm < M && gk < K) v = TA ? A[(int64_t)gk * lda + gm] : A[(int64_t)gm * lda + gk];
      sA[kk][mm] = v;
    }
    for (int t = threadIdx.x; t < SG_BK * SG_BN; t += 256) {
      const int kk = t / SG_BN, nn = t % SG_BN;
      const int gn = n0 + nn, gk = k0 + kk;
      float v = 0.f;
      if (gn < N && gk < K) v = TB ? B[(int64_t)gn * ldb + gk] : B[(int64_t)gk * ldb + gn];
      sB[kk][nn] = v;
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < SG_BK; ++kk) {
      float a[4], b[4];
#pragma unroll
      for (int r = 0; r < 4; ++r) a[r] = sA[kk][ty * 4 + r];
#pragma unroll
      for (int c = 0; c < 4; ++c) b[c] = sB[kk][tx * 4 + c];
#pragma unroll
      for (int r = 0; r < 4; ++r)
#pragma unroll
        for (int c = 0; c < 4; ++c) acc[r][c] += a[r] * b[c];
    }
    __syncthreads();
  }
#pragma unroll
  for (int r = 0; r < 4; ++r) {
    const int gm = m0 + ty * 4 + r;
    if (gm >= M) continue;
#pragma unroll
    for (int c = 0; c < 4; ++c) {
      const int gn = n0 + tx * 4 + c;
      if (gn >= N) continue;
      float v = acc[r][c];
      if (bias) v += bias[gn];
      const int64_t idx = (int64_t)gm * ldc + gn;
      if (beta != 0.f) v += beta * C[idx];
      if (act) {
        if (Z) Z[idx] = v;
        v = gelu_f(v);
      }
      C[idx] = v;
    }
  }
}

int sgemm(bool ta, bool tb, int M, int N, int K, const float* A, int lda, const float* B, int ldb, float* C,
          int ldc, const float* bias, bool gelu, float* Z, float beta, cudaStream_t s) {
  if (M <= 0 || N <= 0) return LPG_OK;
  dim3 grid((N + SG_BN - 1) / SG_BN, (M + SG_BM - 1) / SG_BM);
  if (!ta && !tb) sgemm_kernel<false, false><<<grid, 256, 0, s>>>(M, N, K, A, lda, B, ldb, C, ldc, bias, gelu, Z, beta);
  else if (!ta && tb) sgemm_kernel<false, true><<<grid, 256, 0, s>>>(M, N, K, A, lda, B, ldb, C, ldc, bias, gelu, Z, beta);
  else if (ta && !tb) sgemm_kernel<true, false><<<grid, 256, 0, s>>>(M, N, K, A, lda, B, ldb, C, ldc, bias, gelu, Z, beta);
  else sgemm_kernel<true, true><<<grid, 256, 0, s>>>(M, N, K, A, lda, B, ldb, C, ldc, bias, gelu, Z, beta);
  LPG_LAUNCH_CHECK("sgemm_kernel");
  return LPG_OK;
}

// dZ = dA .* gelu'(Z) (in place on dA)
__global__ void gelu_backward_kernel(const int64_t n, const float* __restrict__ Z, float* __restrict__ dA) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    dA[i] *= gelu_grad_f(Z[i]);
}
// db[c] = sum_r dZ[r][c]
__global__ void bias_grad_kernel(const int rows, const int cols, const float* __restrict__ dZ, float* __restrict__ db) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= cols) return;
  float s = 0.f;
  for (int r = 0; r < rows; ++r) s += dZ[(int64_t)r * cols + c];
  db[c] = s;
}
// MSE loss 0.5/B * sum (y - t)^2 ; dY = (y - t)/B ; loss accumulated into *loss
__global__ void mse_kernel(const int64_t n, const float invB, const float* __restrict__ y, const float* __restrict__ t,
                           float* __restrict__ dy, float* __restrict__ loss) {
  float acc = 0.f;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const float d = y[i] - t[i];
    dy[i] = d * invB;
    acc += 0.5f * d * d * invB;
  }
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
  if ((threadIdx.x & 31) == 0) atomicAdd(loss, acc);
}
// Adam (Kingma & Ba): m = b1 m + (1-b1) g; v = b2 v + (1-b2) g^2; w -= lr mhat / (sqrt(vhat) + eps)
__global__ void adam_kernel(const int64_t n, float* __restrict__ w, const float* __restrict__ g, float* __restrict__ m,
                            float* __restrict__ v, const float lr, const float b1, const float b2, const float eps,
                            const float c1, const float c2) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.f - b1) * gi;
    const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    w[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
  }
}

static unsigned grid_n(int64_t n) { return (unsigned)std::max<int64_t>(1, std::min<int64_t>((n + 255) / 256, 4096)); }

int mlp_forward_f32(const MLPParams& P, int B, const float* X, MLPActs& act, cudaStream_t s) {
  const int dims[5] = {kMlpIn, kMlpHidden, kMlpHidden, kMlpHidden, kMlpOut};
  const float* in = X;
  int rc;
  for (int l = 0; l < 4; ++l) {
    const bool last = (l == 3);
    if ((rc = sgemm(false, false, B, dims[l + 1], dims[l], in, dims[l], P.W[l], dims[l + 1], act.A[l], dims[l + 1],
                    P.b[l], !last, last ? nullptr : act.Z[l], 0.f, s)))
      return rc;
    in = act.A[l];
  }
  return LPG_OK;
}

int mlp_backward_f32(const MLPParams& P, int B, const float* X, const MLPActs& act, const float* dY, MLPParams& G,
                     float* work0, float* work1, cudaStream_t s) {
  const int dims[5] = {kMlpIn, kMlpHidden, kMlpHidden, kMlpHidden, kMlpOut};
  // dcur holds dL/d(pre-activation) of layer l
  const float* dcur = dY;
  int rc;
  for (int l = 3; l >= 0; --l) {
    const float* in = (l == 0) ? X : act.A[l - 1];
    // dW[l] = in^T dcur ; db[l] = colsum(dcur)
    if ((rc = sgemm(true, false, dims[l], dims[l + 1], B, in, dims[l], dcur, dims[l + 1], G.W[l], dims[l + 1], nullptr,
                    false, nullptr, 0.f, s)))
      return rc;
    bias_grad_kernel<<<(dims[l + 1] + 127) / 128, 128, 0, s>>>(B, dims[l + 1], dcur, G.b[l]);
    LPG_LAUNCH_CHECK("bias_grad_kernel");
    if (l == 0) break;
    float* dprev = (l % 2) ? work0 : work1;
    // dA[l-1] = dcur W[l]^T, then times gelu'(Z[l-1])
    if ((rc = sgemm(false, true, B, dims[l], dims[l + 1], dcur, dims[l + 1], P.W[l], dims[l + 1], dprev, dims[l],
                    nullptr, false, nullptr, 0.f, s)))
      return rc;
    gelu_backward_kernel<<<grid_n((int64_t)B * dims[l]), 256, 0, s>>>((int64_t)B * dims[l], act.Z[l - 1], dprev);
    LPG_LAUNCH_CHECK("gelu_backward_kernel");
    dcur = dprev;
  }
  return LPG_OK;
}

int mse_loss(int64_t n, int B, const float* y, const float* t, float* dy, float* loss, cudaStream_t s) {
  LPG_CUDA_TRY(cudaMemsetAsync(loss, 0, sizeof(float), s));
  mse_kernel<<<grid_n(n), 256, 0, s>>>(n, 1.0f / (float)B, y, t, dy, loss);
  LPG_LAUNCH_CHECK("mse_kernel");
  return LPG_OK;
}

int adam_step(int64_t n, float* w, const float* g, float* m, float* v, float lr, int step, cudaStream_t s) {
  const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
  const float c1 = 1.f - powf(b1, (float)step), c2 = 1.f - powf(b2, (float)step);
  adam_kernel<<<grid_n(n), 256, 0, s>>>(n, w, g, m, v, lr, b1, b2, eps, c1, c2);
  LPG_LAUNCH_CHECK("adam_kernel");
  return LPG_OK;
}

// ---------------------------------------------------------------- BF16 tensor-core inference
// Y[M x N] = act(X[M x K] W + b): X bf16 row-major (lda = K), Wt bf16 stored N x K
// (k contiguous), FP32 accumulate in mma.sync.m16n8k16 tiles. CTA tile 128 x 64, BK 32,
// 8 warps as 4 (M) x 2 (N), each warp 32 x 32 = 2 x 4 mma tiles. K and N are multiples of
// 32 and 64 for every layer of this network; M is guarded.
constexpr int TB_M = 128, TB_N = 64, TB_K = 32, TB_PAD = 8;

__device__ __forceinline__ void mma_bf16_16816(float* c, const uint32_t* a, const uint32_t* b) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};\n"
      : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

template <int OUT_BF16>
__global__ void __launch_bounds__(256)
bf16_linear_kernel(const int M, const int N, const int K, const __nv_bfloat16* __restrict__ X,
                   const __nv_bfloat16* __restrict__ Wt, const float* __restrict__ bias, const int act,
                   void* __restrict__ Yv) {
  __shared__ __align__(16) __nv_bfloat16 sA[TB_M][TB_K + TB_PAD];
  __shared__ __align__(16) __nv_bfloat16 sB[TB_N][TB_K + TB_PAD];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int wm = warp % 4, wn = warp / 4;
  const int g = lane >> 2, t = lane & 3;
  const int m0 = blockIdx.y * TB_M, n0 = blockIdx.x * TB_N;
  float acc[2][4][4] = {};
  for (int k0 = 0; k0 < K; k0 += TB_K) {
    // A tile: 128 x 32 bf16 = 512 x 16 B chunks, 2 per thread
    for (int c = threadIdx.x; c < TB_M * TB_K / 8; c += 256) {
      const int row = c / (TB_K / 8), col = (c % (TB_K / 8)) * 8;
      const int gm = m0 + row;
      uint4 v = make_uint4(0, 0, 0, 0);
      if (gm < M) v = *reinterpret_cast<const uint4*>(X + (int64_t)gm * K + k0 + col);
      *reinterpret_cast<uint4*>(&sA[row][col]) = v;
    }
    // B tile: 64 x 32 bf16 = 256 chunks, 1 per thread
    for (int c = threadIdx.x; c < TB_N * TB_K / 8; c += 256) {
      const int row = c / (TB_K / 8), col = (c % (TB_K / 8)) * 8;
      *reinterpret_cast<uint4*>(&sB[row][col]) = *reinterpret_cast<const uint4*>(Wt + (int64_t)(n0 + row) * K + k0 + col);
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < TB_K; kk += 16) {
      uint32_t a[2][4], b[4][2];
#pragma unroll
      for (int im = 0; im < 2; ++im) {
        const int r = wm * 32 + im * 16;
        a[im][0] = *reinterpret_cast<const uint32_t*>(&sA[r + g][kk + t * 2]);
        a[im][1] = *reinterpret_cast<const uint32_t*>(&sA[r + g + 8][kk + t * 2]);
        a[im][2] = *reinterpret_cast<const uint32_t*>(&sA[r + g][kk + t * 2 + 8]);
        a[im][3] = *reinterpret_cast<const uint32_t*>(&sA[r + g + 8][kk + t * 2 + 8]);
      }
#pragma unroll
      for (int in = 0; in < 4; ++in) {
        const int cidx = wn * 32 + in * 8 + g;
        b[in][0] = *reinterpret_cast<const uint32_t*>(&sB[cidx][kk + t * 2]);
        b[in][1] = *reinterpret_cast<const uint32_t*>(&sB[cidx][kk + t * 2 + 8]);
      }
#pragma unroll
      for (int im = 0; im < 2; ++im)
#pragma unroll
        for (int in = 0; in < 4; ++in) mma_bf16_16816(acc[im][in], a[im], b[in]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int im = 0; im < 2; ++im)
#pragma unroll
    for (int in = 0; in < 4; ++in)
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        const int row = m0 + wm * 32 + im * 16 + g + h * 8;
        const int col = n0 + wn * 32 + in * 8 + t * 2;
        if (row >= M) continue;
        float v0 = acc[im][in][h * 2 + 0] + bias[col];
        float v1 = acc[im][in][h * 2 + 1] + bias[col + 1];
        if (act) { v0 = gelu_f(v0); v1 = gelu_f(v1); }
        if (OUT_BF16) {
          __nv_bfloat162 p = __floats2bfloat162_rn(v0, v1);
          *reinterpret_cast<__nv_bfloat162*>(reinterpret_cast<__nv_bfloat16*>(Yv) + (int64_t)row * N + col) = p;
        } else {
          float2 p = make_float2(v0, v1);
          *reinterpret_cast<float2*>(reinterpret_cast<float*>(Yv) + (int64_t)row * N + col) = p;
        }
      }
}

int bf16_linear(int M, int N, int K, const __nv_bfloat16* X, const __nv_bfloat16* Wt, const float* bias, bool gelu,
                bool outBf16, void* Y, cudaStream_t s) {
  if (M <= 0) return LPG_OK;
  if (N % TB_N || K % TB_K) return set_error(LPG_ERR_INVALID, "bf16_linear: N must be a multiple of 64 and K of 32");
  dim3 grid(N / TB_N, (M + TB_M - 1) / TB_M);
  if (outBf16) bf16_linear_kernel<1><<<grid, 256, 0, s>>>(M, N, K, X, Wt, bias, gelu, Y);
  else bf16_linear_kernel<0><<<grid, 256, 0, s>>>(M, N, K, X, Wt, bias, gelu, Y);
  LPG_LAUNCH_CHECK("bf16_linear_kernel");
  return LPG_OK;
}

// W (K x N fp32 row-major) -> Wt (N x K bf16)
__global__ void transpose_to_bf16_kernel(const int K, const int N, const float* __restrict__ W,
                                         __nv_bfloat16* __restrict__ Wt) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < (int64_t)K * N; i += (int64_t)gridDim.x * blockDim.x) {
    const int k = (int)(i / N), n = (int)(i % N);
    Wt[(int64_t)n * K + k] = __float2bfloat16(W[i]);
  }
}
int transpose_to_bf16(int K, int N, const float* W, __nv_bfloat16* Wt, cudaStream_t s) {
  transpose_to_bf16_kernel<<<grid_n((int64_t)K * N), 256, 0, s>>>(K, N, W, Wt);
  LPG_LAUNCH_CHECK("transpose_to_bf16_kernel");
  return LPG_OK;
}

// ---------------------------------------------------------------- element features
// Face f of element (ex,ey,ez) in the reference's numbering (meshBasisHex3D.cpp:60-90):
// 0: k=0, 1: j=0, 2: i=N, 3: j=N, 4: i=0, 5: k=N. The trace of face f is the neighbour's
// node layer next to the shared face (i=1 / i=N-1 ...), listed in face-node order.
template <typename TIN, typename TOUT>
__global__ void __launch_bounds__(256)
features_kernel(const BoxNumbering b, const int64_t e0, const int64_t count, const int32_t* __restrict__ g2l,
                const TIN* __restrict__ r, TOUT* __restrict__ X, float* __restrict__ scale, const float sfloor) {
  // one warp per element (Nq = 8): lane l holds inputs l, l + 32, ... (28 per lane); the
  // element's own 512 nodes are the first 16, the 6 x 64 face values the other 12
  constexpr int Nq = 8, N = Nq - 1, Np = Nq * Nq * Nq, Nfp = Nq * Nq, PER = kMlpIn / 32;
  static_assert(Np + 6 * Nfp == kMlpIn, "896 inputs");
  const int lane = threadIdx.x & 31;
  const int64_t w = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (w >= count) return;   // uniform per warp
  const int64_t eb = e0 + w;
  const int ex = (int)(eb % b.nx), ey = (int)((eb / b.nx) % b.ny), ez = (int)(eb / ((int64_t)b.nx * b.ny));
  float v[PER];
  float ss = 0.f;
#pragma unroll
  for (int k = 0; k < Np / 32; ++k) {
    const int32_t g = g2l[eb * Np + lane + 32 * k];
    v[k] = (g >= 0) ? (float)r[g] : 0.f;
    ss += v[k] * v[k];
  }
#pragma unroll
  for (int k = Np / 32; k < PER; ++k) {
    const int t = lane + 32 * k - Np;
    const int f = t / Nfp, m = t % Nfp;   // f is the same for the whole warp
    const int p = m % Nq, q = m / Nq;      // face-local coordinates in node order
    int nx = ex, ny = ey, nz = ez, i = 0, j = 0, kk = 0;
    switch (f) {
      case 0: nz = ez - 1; i = p; j = q; kk = N - 1; break;
      case 1: ny = ey - 1; i = p; kk = q; j = N - 1; break;
      case 2: nx = ex + 1; j = p; kk = q; i = 1; break;
      case 3: ny = ey + 1; i = p; kk = q; j = 1; break;
      case 4: nx = ex - 1; j = p; kk = q; i = N - 1; break;
      default: nz = ez + 1; i = p; j = q; kk = 1; break;
    }
    if (b.periodic) { nx = (nx + b.nx) % b.nx; ny = (ny + b.ny) % b.ny; nz = (nz + b.nz) % b.nz; }
    float val = 0.f;
    if (nx >= 0 && nx < b.nx && ny >= 0 && ny < b.ny && nz >= 0 && nz < b.nz) {
      const int64_t en = nx + (int64_t)ny * b.nx + (int64_t)nz * b.nx * b.ny;
      const int32_t g = g2l[en * Np + i + j * Nq + kk * Nfp];
      val = (g >= 0) ? (float)r[g] : 0.f;
    }
    v[k] = val;
  }
  for (int o = 16; o > 0; o >>= 1) ss += __shfl_xor_sync(0xffffffffu, ss, o);
  const float sc = fmaxf(sqrtf(ss / (float)Np), sfloor) + 1e-30f;
  if (lane == 0) scale[w] = sc;
  const float inv = 1.f / sc;
#pragma unroll
  for (int k = 0; k < PER; ++k) X[w * (int64_t)kMlpIn + lane + 32 * k] = (TOUT)(v[k] * inv);
}

template <typename TIN, typename TOUT>
int element_features(const BoxNumbering& b, int64_t E, int64_t e0, int64_t count, const int32_t* g2l, const TIN* r,
                     TOUT* X, float* scale, float sfloor, cudaStream_t s) {
  if ((b.N + 1) * (b.N + 1) * (b.N + 1) + 6 * (b.N + 1) * (b.N + 1) != kMlpIn)
    return set_error(LPG_ERR_UNSUPPORTED, "learned smoother needs N = 7 (896 inputs per element)");
  if (count <= 0) return LPG_OK;
  if (e0 < 0 || e0 + count > E) return set_error(LPG_ERR_INVALID, "element_features: chunk outside the mesh");
  features_kernel<TIN, TOUT><<<(unsigned)((count * 32 + 255) / 256), 256, 0, s>>>(b, e0, count, g2l, r, X, scale, sfloor);
  LPG_LAUNCH_CHECK("features_kernel");
  return LPG_OK;
}
template int element_features<double, float>(const BoxNumbering&, int64_t, int64_t, int64_t, const int32_t*,
                                             const double*, float*, float*, float, cudaStream_t);
template int element_features<double, __nv_bfloat16>(const BoxNumbering&, int64_t, int64_t, int64_t, const int32_t*,
                                                     const double*, __nv_bfloat16*, float*, float, cudaStream_t);
template int element_features<float, __nv_bfloat16>(const BoxNumbering&, int64_t, int64_t, int64_t, const int32_t*,
                                                    const float*, __nv_bfloat16*, float*, float, cudaStream_t);

// z[g] += coef[g] * s_e * out (coef = weight / diag: the correction s_e invDiag out
// averaged over the copies of g), in the vector's precision; z holds the caller's
// starting value (zero, or the damped-Jacobi part of the smoother)
template <typename TV>
__global__ void apply_correction_kernel(const int Np, const int64_t count, const int64_t e0,
                                        const int32_t* __restrict__ g2l, const float* __restrict__ out,
                                        const float* __restrict__ scale, const TV* __restrict__ coef,
                                        TV* __restrict__ z) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < count * Np; i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t el = i / Np;
    const int n = (int)(i % Np);
    const int32_t g = g2l[(e0 + el) * Np + n];
    if (g < 0) continue;
    // every copy as a fire-and-forget atomic add, the nodes strictly inside the element
    // too: a plain read-modify-write there waits for its load and splits each warp between
    // the two paths (64^3 learned solve: 0.2531 against 0.2580 s)
    atomicAdd(z + g, coef[g] * (TV)(scale[el] * out[el * kMlpOut + n]));
  }
}
template <typename TV>
int apply_correction(int Np, int64_t count, int64_t e0, const int32_t* g2l, const float* out, const float* scale,
                     const TV* coef, TV* z, cudaStream_t s) {
  if (count <= 0) return LPG_OK;
  apply_correction_kernel<TV><<<grid_n(count * Np), 256, 0, s>>>(Np, count, e0, g2l, out, scale, coef, z);
  LPG_LAUNCH_CHECK("apply_correction_kernel");
  return LPG_OK;
}
template int apply_correction<double>(int, int64_t, int64_t, const int32_t*, const float*, const float*, const double*,
                                      double*, cudaStream_t);
template int apply_correction<float>(int, int64_t, int64_t, const int32_t*, const float*, const float*, const float*,
                                     float*, cudaStream_t);

// copies of lattice coordinate X along one axis of n elements (degree kMlpNq - 1): the
// element index and local index of each, one copy inside an element, two on an element face
__device__ __forceinline__ int axis_copies(const int X, const int n, const int periodic, int* e, int* a) {
  constexpr int N = kMlpNq - 1;
  const int k = X / N, r = X - k * N;
  if (r != 0) {
    e[0] = k;
    a[0] = r;
    return 1;
  }
  if (periodic) {
    e[0] = (k - 1 + n) % n;
    a[0] = N;
    e[1] = k % n;
    a[1] = 0;
    return 2;
  }
  int c = 0;
  if (k - 1 >= 0) { e[c] = k - 1; a[c] = N; ++c; }
  if (k < n) { e[c] = k; a[c] = 0; ++c; }
  return c;
}

// block (x-run of a lattice row, Y = blockIdx.y, Z = Z0 + blockIdx.z); one thread per node
template <typename TV>
__global__ void lattice_correction_kernel(const BoxNumbering b, const int NX, const int Z0,
                                          const int32_t* __restrict__ g2l, const float* __restrict__ out,
                                          const float* __restrict__ scale, const TV* __restrict__ coef,
                                          TV* __restrict__ z) {
  constexpr int Nq = kMlpNq, Np = Nq * Nq * Nq;
  const int X = blockIdx.x * blockDim.x + threadIdx.x;
  if (X >= NX) return;
  int ex[2], ax[2], ey[2], ay[2], ez[2], az[2];
  const int cx = axis_copies(X, b.nx, b.periodic, ex, ax);
  const int cy = axis_copies((int)blockIdx.y, b.ny, b.periodic, ey, ay);
  const int cz = axis_copies(Z0 + (int)blockIdx.z, b.nz, b.periodic, ez, az);
  const int64_t nxy = (int64_t)b.nx * b.ny;
  const int64_t e0 = ex[0] + (int64_t)b.nx * ey[0] + nxy * ez[0];
  const int32_t g = g2l[e0 * Np + ax[0] + Nq * (ay[0] + Nq * az[0])];
  if (g < 0) return;
  TV sum = 0;
  for (int k = 0; k < cz; ++k)
    for (int j = 0; j < cy; ++j)
      for (int i = 0; i < cx; ++i) {
        const int64_t e = ex[i] + (int64_t)b.nx * ey[j] + nxy * ez[k];
        sum += (TV)(scale[e] * out[e * kMlpOut + ax[i] + Nq * (ay[j] + Nq * az[k])]);
      }
  z[g] += coef[g] * sum;
}
template <typename TV>
int lattice_correction(const BoxNumbering& b, const int32_t* g2l, const float* out, const float* scale,
                       const TV* coef, TV* z, int Zbegin, int Zend, cudaStream_t s) {
  if (b.N != kMlpNq - 1) return set_error(LPG_ERR_UNSUPPORTED, "lattice correction: N = 7 only");
  const int64_t NX = (int64_t)b.nx * b.N + (b.periodic ? 0 : 1);
  const int64_t NY = (int64_t)b.ny * b.N + (b.periodic ? 0 : 1);
  const int64_t NZ = (int64_t)b.nz * b.N + (b.periodic ? 0 : 1);
  if (NX > INT32_MAX / 2 || NY > 65535 || Zbegin < 0 || Zend > NZ || Zend - Zbegin > 65535)
    return set_error(LPG_ERR_UNSUPPORTED, "lattice correction: lattice too large for the launch grid");
  if (Zend <= Zbegin) return LPG_OK;
  constexpr int T = 128;
  const dim3 grid((unsigned)((NX + T - 1) / T), (unsigned)NY, (unsigned)(Zend - Zbegin));
  lattice_correction_kernel<TV><<<grid, T, 0, s>>>(b, (int)NX, Zbegin, g2l, out, scale, coef, z);
  LPG_LAUNCH_CHECK("lattice_correction_kernel");
  return LPG_OK;
}
template int lattice_correction<double>(const BoxNumbering&, const int32_t*, const float*, const float*, const double*,
                                        double*, int, int, cudaStream_t);
template int lattice_correction<float>(const BoxNumbering&, const int32_t*, const float*, const float*, const float*,
                                       float*, int, int, cudaStream_t);

// training target: t = D .* e_local / s (network output units), e gathered from the dofs
__global__ void target_kernel(const int Np, const int64_t count, const int32_t* __restrict__ elems,
                              const int32_t* __restrict__ g2l, const double* __restrict__ e, const double* __restrict__ invDiag,
                              const float* __restrict__ scale, float* __restrict__ T) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < count * Np; i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t el = i / Np;
    const int n = (int)(i % Np);
    const int32_t g = g2l[(int64_t)elems[el] * Np + n];
    T[el * kMlpOut + n] = (g >= 0) ? (float)(e[g] / invDiag[g] / (double)scale[el]) : 0.f;
  }
}
int training_targets(int Np, int64_t count, const int32_t* elems, const int32_t* g2l, const double* e,
                     const double* invDiag, const float* scale, float* T, cudaStream_t s) {
  if (count <= 0) return LPG_OK;
  target_kernel<<<grid_n(count * Np), 256, 0, s>>>(Np, count, elems, g2l, e, invDiag, scale, T);
  LPG_LAUNCH_CHECK("target_kernel");
  return LPG_OK;
}

// High-pass training target: the exact error on each element minus its modal projection
// onto Legendre degrees <= Nc per direction (F = V diag(mask) V^{-1}, applied as three
// 1D contractions), in network output units: T = (e - F e) / (invDiag s_e).
__global__ void __launch_bounds__(256)
highpass_target_kernel(const int Nq, const int32_t* __restrict__ g2l, const double* __restrict__ e,
                       const double* __restrict__ invDiag, const float* __restrict__ scale,
                       const double* __restrict__ Fg, float* __restrict__ T) {
  __shared__ double s_e[kMaxNq * kMaxNq * kMaxNq], s_a[kMaxNq * kMaxNq * kMaxNq], s_b[kMaxNq * kMaxNq * kMaxNq];
  __shared__ double s_F[kMaxNq * kMaxNq];
  __shared__ double s_d[kMaxNq * kMaxNq * kMaxNq];
  const int64_t el = blockIdx.x;
  const int Np = Nq * Nq * Nq;
  for (int t = threadIdx.x; t < Nq * Nq; t += blockDim.x) s_F[t] = Fg[t];
  for (int t = threadIdx.x; t < Np; t += blockDim.x) {
    const int32_t g = g2l[el * Np + t];
    s_e[t] = (g >= 0) ? e[g] : 0.0;
    s_d[t] = (g >= 0) ? 1.0 / invDiag[g] : 0.0;
  }
  __syncthreads();
  for (int t = threadIdx.x; t < Np; t += blockDim.x) {  // i direction
    const int i = t % Nq, jk = t / Nq;
    double r = 0;
    for (int m = 0; m < Nq; ++m) r += s_F[i * Nq + m] * s_e[jk * Nq + m];
    s_a[t] = r;
  }
  __syncthreads();
  for (int t = threadIdx.x; t < Np; t += blockDim.x) {  // j direction
    const int i = t % Nq, j = (t / Nq) % Nq, k = t / (Nq * Nq);
    double r = 0;
    for (int m = 0; m < Nq; ++m) r += s_F[j * Nq + m] * s_a[k * Nq * Nq + m * Nq + i];
    s_b[t] = r;
  }
  __syncthreads();
  const double inv = 1.0 / (double)scale[el];
  for (int t = threadIdx.x; t < Np; t += blockDim.x) {  // k direction
    const int ij = t % (Nq * Nq), k = t / (Nq * Nq);
    double r = 0;
    for (int m = 0; m < Nq; ++m) r += s_F[k * Nq + m] * s_b[m * Nq * Nq + ij];
    T[el * kMlpOut + t] = (float)((s_e[t] - r) * s_d[t] * inv);
  }
}
int highpass_targets(int Nq, int64_t E, const int32_t* g2l, const double* e, const double* invDiag, const float* scale,
                     const double* F, float* T, cudaStream_t s) {
  if (E <= 0) return LPG_OK;
  if (Nq * Nq * Nq != kMlpOut) return set_error(LPG_ERR_UNSUPPORTED, "highpass targets need N = 7");
  highpass_target_kernel<<<(unsigned)E, 256, 0, s>>>(Nq, g2l, e, invDiag, scale, F, T);
  LPG_LAUNCH_CHECK("highpass_target_kernel");
  return LPG_OK;
}

// features of a list of elements (training samples)
template <typename TOUT>
__global__ void gather_rows_kernel(const int64_t count, const int32_t* __restrict__ elems, const TOUT* __restrict__ Xall,
                                   TOUT* __restrict__ X) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < count * kMlpIn; i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t el = i / kMlpIn;
    X[i] = Xall[(int64_t)elems[el] * kMlpIn + (i % kMlpIn)];
  }
}
int gather_rows(int64_t count, const int32_t* elems, const float* Xall, float* X, cudaStream_t s) {
  if (count <= 0) return LPG_OK;
  gather_rows_kernel<float><<<grid_n(count * kMlpIn), 256, 0, s>>>(count, elems, Xall, X);
  LPG_LAUNCH_CHECK("gather_rows_kernel");
  return LPG_OK;
}

// dst[i][:] = src[idx[i]][:] for rows of `width` floats (minibatch assembly)
__global__ void gather_rows_w_kernel(const int64_t count, const int width, const int32_t* __restrict__ idx,
                                     const float* __restrict__ src, float* __restrict__ dst) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < count * width; i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t row = i / width;
    dst[i] = src[(int64_t)idx[row] * width + (i % width)];
  }
}
int gather_rows_w(int64_t count, int width, const int32_t* idx, const float* src, float* dst, cudaStream_t s) {
  if (count <= 0) return LPG_OK;
  gather_rows_w_kernel<<<grid_n(count * width), 256, 0, s>>>(count, width, idx, src, dst);
  LPG_LAUNCH_CHECK("gather_rows_w_kernel");
  return LPG_OK;
}

// T[i][n] -= w * X[i][n] for the first kMlpOut inputs (the element's normalised
// residual): targets of the network part of a damped-Jacobi + network smoother
__global__ void subtract_inputs_kernel(const int64_t count, const float w, const float* __restrict__ X,
                                       float* __restrict__ T) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < count * kMlpOut; i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t row = i / kMlpOut;
    T[i] -= w * X[row * kMlpIn + (i % kMlpOut)];
  }
}
int subtract_inputs(int64_t count, float w, const float* X, float* T, cudaStream_t s) {
  if (count <= 0 || w == 0.f) return LPG_OK;
  subtract_inputs_kernel<<<grid_n(count * kMlpOut), 256, 0, s>>>(count, w, X, T);
  LPG_LAUNCH_CHECK("subtract_inputs_kernel");
  return LPG_OK;
}

}  // namespace lpg
