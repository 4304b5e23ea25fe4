// Matrix-free screened-Poisson operator on hexahedra (sum-factorised, GLL collocation)
// with the gather-scatter assembly fused into the kernel.
//
// Same arithmetic as ellipticPartialAxHex3D (solvers/elliptic/okl/ellipticAxHex3D.okl:156-295):
// per element, pencils q(i,j,0:N) live in registers, one k-layer at a time is shared,
// r/s derivatives come from shared memory, the metric product G*grad is formed per node,
// and the transposed derivatives accumulate back into the register pencil.
// Differences for GB300:
//   * several elements per CTA (NQ*NQ threads each) so a CTA has ~256 threads;
//   * the assembled result is accumulated straight into Aq with atomics (the reference
//     writes AqL, then an ogs Gather kernel re-reads it);
//   * geometric-factor offsets are 64-bit (the reference's int offsets overflow at 112^3, N=7);
//   * per-element lambda; FP64, FP32 and BF16-storage variants from one template.
#include "lpg_common.cuh"
#include "lpg_internal.hpp"

namespace lpg {

enum { IN_GATHER = 0, IN_LOCAL = 1 };
enum { OUT_ASSEMBLE = 0, OUT_LOCAL = 1, OUT_LOCAL_SUB = 2 };

template <int NQ>
constexpr int elems_per_block() {
  return (256 / (NQ * NQ)) > 0 ? (256 / (NQ * NQ)) : 1;
}

template <int NQ, typename T, typename G, int INMODE, int OUTMODE>
__global__ void __launch_bounds__(NQ * NQ * elems_per_block<NQ>())
ax_hex_kernel(const int64_t Nelements, const int32_t* __restrict__ elementList,
              const int32_t* __restrict__ g2l, const G* __restrict__ ggeo, const int64_t geoStride,
              const G* __restrict__ wJ, const int64_t wJStride, const T* __restrict__ Dg,
              const T lambda, const T* __restrict__ lambdaE, const T* __restrict__ q,
              T* __restrict__ out) {
  constexpr int NP = NQ * NQ * NQ;
  constexpr int EPB = elems_per_block<NQ>();
  __shared__ T s_D[NQ][NQ];
  __shared__ T s_q[EPB][NQ][NQ];
  __shared__ T s_Gqr[EPB][NQ][NQ];
  __shared__ T s_Gqs[EPB][NQ][NQ];

  const int i = threadIdx.x, j = threadIdx.y, el = threadIdx.z;
  const int tid = i + NQ * (j + NQ * el);
  for (int t = tid; t < NQ * NQ; t += NQ * NQ * EPB) s_D[t / NQ][t % NQ] = Dg[t];

  int64_t e = (int64_t)blockIdx.x * EPB + el;
  const bool active = e < Nelements;
  if (active && elementList) e = elementList[e];
  if (!active) e = 0;

  T r_q[NQ], r_Aq[NQ];
  int32_t r_id[NQ];
  const int64_t nodeBase = e * NP + j * NQ + i;
#pragma unroll
  for (int k = 0; k < NQ; ++k) {
    r_Aq[k] = 0;
    if (INMODE == IN_GATHER) {
      const int32_t id = active ? __ldg(g2l + nodeBase + k * NQ * NQ) : -1;
      r_id[k] = id;
      r_q[k] = (id >= 0) ? q[id] : T(0);
    } else {
      r_id[k] = 0;
      r_q[k] = active ? q[nodeBase + k * NQ * NQ] : T(0);
    }
  }
  if (OUTMODE == OUT_ASSEMBLE && INMODE != IN_GATHER) {
#pragma unroll
    for (int k = 0; k < NQ; ++k) r_id[k] = active ? __ldg(g2l + nodeBase + k * NQ * NQ) : -1;
  }
  const T lam = (lambdaE && active) ? lambdaE[e] : lambda;
  const G* gp = ggeo + e * geoStride + j * NQ + i;
  const G* wp = wJ + e * wJStride + j * NQ + i;
  __syncthreads();

#pragma unroll
  for (int k = 0; k < NQ; ++k) {
    T G00 = 0, G01 = 0, G02 = 0, G11 = 0, G12 = 0, G22 = 0, GwJ = 0;
    if (active) {
      const int off = k * NQ * NQ;
      G00 = load_geo<T, G>(gp + 0 * NP + off);
      G01 = load_geo<T, G>(gp + 1 * NP + off);
      G02 = load_geo<T, G>(gp + 2 * NP + off);
      G11 = load_geo<T, G>(gp + 3 * NP + off);
      G12 = load_geo<T, G>(gp + 4 * NP + off);
      G22 = load_geo<T, G>(gp + 5 * NP + off);
      GwJ = load_geo<T, G>(wp + off);
    }
    s_q[el][j][i] = r_q[k];
    T qt = 0;
#pragma unroll
    for (int m = 0; m < NQ; ++m) qt += s_D[k][m] * r_q[m];
    __syncthreads();

    T qr = 0, qs = 0;
#pragma unroll
    for (int m = 0; m < NQ; ++m) {
      qr += s_D[i][m] * s_q[el][j][m];
      qs += s_D[j][m] * s_q[el][m][i];
    }
    s_Gqs[el][j][i] = (G01 * qr + G11 * qs + G12 * qt);
    s_Gqr[el][j][i] = (G00 * qr + G01 * qs + G02 * qt);
    const T Gqt = (G02 * qr + G12 * qs + G22 * qt);
    T Auk = GwJ * lam * r_q[k];
    __syncthreads();

#pragma unroll
    for (int m = 0; m < NQ; ++m) {
      Auk += s_D[m][j] * s_Gqs[el][m][i];
      r_Aq[m] += s_D[k][m] * Gqt;
      Auk += s_D[m][i] * s_Gqr[el][j][m];
    }
    r_Aq[k] += Auk;
    __syncthreads();
  }

  if (!active) return;
#pragma unroll
  for (int k = 0; k < NQ; ++k) {
    if (OUTMODE == OUT_ASSEMBLE) {
      if (r_id[k] >= 0) atomicAdd(out + r_id[k], r_Aq[k]);
    } else if (OUTMODE == OUT_LOCAL) {
      out[nodeBase + k * NQ * NQ] = r_Aq[k];
    } else {
      out[nodeBase + k * NQ * NQ] -= r_Aq[k];
    }
  }
}

template <int NQ, typename T, typename G, int INMODE, int OUTMODE>
static int launch_ax(const AxArgs<T, G>& a, cudaStream_t s) {
  constexpr int EPB = elems_per_block<NQ>();
  if (a.Nelements <= 0) return LPG_OK;
  const int64_t blocks = (a.Nelements + EPB - 1) / EPB;
  if (blocks > 0x7fffffffLL) return set_error(LPG_ERR_INVALID, "ax: too many elements");
  dim3 block(NQ, NQ, EPB);
  ax_hex_kernel<NQ, T, G, INMODE, OUTMODE><<<(unsigned)blocks, block, 0, s>>>(
      a.Nelements, a.elementList, a.g2l, a.ggeo, a.geoStride, a.wJ, a.wJStride, a.D, a.lambda,
      a.lambdaE, a.q, a.out);
  LPG_LAUNCH_CHECK("ax_hex_kernel");
  return LPG_OK;
}

template <typename T, typename G, int INMODE, int OUTMODE>
static int dispatch_ax(const AxArgs<T, G>& a, cudaStream_t s) {
  switch (a.N) {
    case 1: return launch_ax<2, T, G, INMODE, OUTMODE>(a, s);
    case 2: return launch_ax<3, T, G, INMODE, OUTMODE>(a, s);
    case 3: return launch_ax<4, T, G, INMODE, OUTMODE>(a, s);
    case 4: return launch_ax<5, T, G, INMODE, OUTMODE>(a, s);
    case 5: return launch_ax<6, T, G, INMODE, OUTMODE>(a, s);
    case 6: return launch_ax<7, T, G, INMODE, OUTMODE>(a, s);
    case 7: return launch_ax<8, T, G, INMODE, OUTMODE>(a, s);
    case 8: return launch_ax<9, T, G, INMODE, OUTMODE>(a, s);
    default: return set_error(LPG_ERR_UNSUPPORTED, "ax: polynomial degree must be 1..8");
  }
}

template <typename T, typename G>
int ax_hex(const AxArgs<T, G>& a, AxMode mode, cudaStream_t s) {
  switch (mode) {
    case AxMode::Assemble: {
      if (a.Nglobal > 0) LPG_CUDA_TRY(cudaMemsetAsync(a.out, 0, sizeof(T) * a.Nglobal, s));
      return dispatch_ax<T, G, IN_GATHER, OUT_ASSEMBLE>(a, s);
    }
    case AxMode::AccumulateAssembled:
      return dispatch_ax<T, G, IN_GATHER, OUT_ASSEMBLE>(a, s);
    case AxMode::PartialLocal:
      return dispatch_ax<T, G, IN_GATHER, OUT_LOCAL>(a, s);
    case AxMode::LocalInSubtract:
      return dispatch_ax<T, G, IN_LOCAL, OUT_LOCAL_SUB>(a, s);
  }
  return set_error(LPG_ERR_INVALID, "ax: bad mode");
}

template int ax_hex<double, double>(const AxArgs<double, double>&, AxMode, cudaStream_t);
template int ax_hex<float, float>(const AxArgs<float, float>&, AxMode, cudaStream_t);
template int ax_hex<float, __nv_bfloat16>(const AxArgs<float, __nv_bfloat16>&, AxMode, cudaStream_t);

}  // namespace lpg

using namespace lpg;

template <typename T, typename G>
static int ax_entry(int N, int64_t Nelements, const int32_t* elementList, const int32_t* g2l,
                    const G* ggeo, int64_t geoStride, const G* wJ, int64_t wJStride, const T* D,
                    T lambda, const T* lambdaE, const T* q, T* out, int64_t Nglobal, AxMode mode,
                    void* stream) {
  if (N < 1 || N > 8) return set_error(LPG_ERR_UNSUPPORTED, "polynomial degree must be 1..8");
  if (Nelements < 0 || !g2l || !ggeo || !wJ || !D || !q || !out)
    return set_error(LPG_ERR_INVALID, "ax: null pointer or negative size");
  const int64_t Np = (int64_t)(N + 1) * (N + 1) * (N + 1);
  if (geoStride < 6 * Np || wJStride < Np) return set_error(LPG_ERR_INVALID, "ax: stride too small");
  AxArgs<T, G> a;
  a.N = N; a.Nelements = Nelements; a.elementList = elementList; a.g2l = g2l;
  a.ggeo = ggeo; a.geoStride = geoStride; a.wJ = wJ; a.wJStride = wJStride; a.D = D;
  a.lambda = lambda; a.lambdaE = lambdaE; a.q = q; a.out = out; a.Nglobal = Nglobal;
  return ax_hex<T, G>(a, mode, as_stream(stream));
}

extern "C" int lpg_ax_hex_f64(int N, int64_t Nelements, const int32_t* elementList,
                              const int32_t* GlobalToLocal, const double* ggeo, int64_t geoStride,
                              const double* wJ, int64_t wJStride, const double* D, double lambda,
                              const double* lambdaE, const double* q, double* Aq, int64_t Nglobal,
                              void* stream) {
  return ax_entry<double, double>(N, Nelements, elementList, GlobalToLocal, ggeo, geoStride, wJ,
                                  wJStride, D, lambda, lambdaE, q, Aq, Nglobal, AxMode::Assemble,
                                  stream);
}

extern "C" int lpg_ax_hex_f32(int N, int64_t Nelements, const int32_t* elementList,
                              const int32_t* GlobalToLocal, const float* ggeo, int64_t geoStride,
                              const float* wJ, int64_t wJStride, const float* D, float lambda,
                              const float* lambdaE, const float* q, float* Aq, int64_t Nglobal,
                              void* stream) {
  return ax_entry<float, float>(N, Nelements, elementList, GlobalToLocal, ggeo, geoStride, wJ,
                                wJStride, D, lambda, lambdaE, q, Aq, Nglobal, AxMode::Assemble,
                                stream);
}

extern "C" int lpg_ax_hex_bf16g(int N, int64_t Nelements, const int32_t* elementList,
                                const int32_t* GlobalToLocal, const void* ggeo_bf16,
                                int64_t geoStride, const void* wJ_bf16, int64_t wJStride,
                                const float* D, float lambda, const float* lambdaE, const float* q,
                                float* Aq, int64_t Nglobal, void* stream) {
  return ax_entry<float, __nv_bfloat16>(
      N, Nelements, elementList, GlobalToLocal, (const __nv_bfloat16*)ggeo_bf16, geoStride,
      (const __nv_bfloat16*)wJ_bf16, wJStride, D, lambda, lambdaE, q, Aq, Nglobal,
      AxMode::Assemble, stream);
}

extern "C" int lpg_partial_ax_hex_f64(int N, int64_t Nelements, const int32_t* elementList,
                                      const int32_t* GlobalToLocal, const double* ggeo,
                                      int64_t geoStride, const double* wJ, int64_t wJStride,
                                      const double* D, double lambda, const double* lambdaE,
                                      const double* q, double* AqL, void* stream) {
  return ax_entry<double, double>(N, Nelements, elementList, GlobalToLocal, ggeo, geoStride, wJ,
                                  wJStride, D, lambda, lambdaE, q, AqL, 0, AxMode::PartialLocal,
                                  stream);
}
