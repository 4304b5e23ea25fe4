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
#include <cstdlib>
#include <cstring>
#include <type_traits>

#include "df64.cuh"
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
              T* __restrict__ out, const T outScale) {
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
      // FP32: the scaled assembly of the fused residual; FP64 always adds A q itself
      if constexpr (std::is_same<T, float>::value) {
        if (r_id[k] >= 0) atomicAdd(out + r_id[k], outScale * r_Aq[k]);
      } else {
        if (r_id[k] >= 0) atomicAdd(out + r_id[k], r_Aq[k]);
      }
    } else if (OUTMODE == OUT_LOCAL) {
      out[nodeBase + k * NQ * NQ] = r_Aq[k];
    } else {
      out[nodeBase + k * NQ * NQ] -= r_Aq[k];
    }
  }
}

// ---------------------------------------------------------------- staged variant
// Persistent CTAs walk groups of EPB elements. Each element's geometric factors (7 x Np)
// and GlobalToLocal block (Np int32) are copied into a STAGES-deep shared-memory ring
// with 16-byte cp.async, STAGES-1 groups ahead of the one being computed, so DRAM traffic
// overlaps the contractions. D's rows and columns needed by a thread live in registers;
// the t-direction contractions of the whole pencil run once per element (64 FMA each way).
__device__ __forceinline__ void cp_async16(void* smem, const void* gmem) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(s), "l"(gmem) : "memory");
}
// L2 prefetch of `bytes` (a multiple of 16) from global memory; skipped unless the address
// is 16-byte aligned, as the bulk prefetch requires
__device__ __forceinline__ void prefetch_l2_bulk(const void* gmem, unsigned bytes) {
  if (((uintptr_t)gmem & 15u) == 0 && (bytes & 15u) == 0)
    asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;\n" ::"l"(gmem), "r"(bytes) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory"); }

// Barrier over the NQ*NQ threads of one element (named barrier 1 + el) when that is a
// whole number of warps, else over the CTA.
template <int NQ>
__device__ __forceinline__ void elem_sync(const int el) {
  if constexpr ((NQ * NQ) % 32 == 0) {
    asm volatile("bar.sync %0, %1;\n" ::"r"(1 + el), "r"(NQ * NQ) : "memory");
  } else {
    __syncthreads();
  }
}

template <typename G> __device__ __forceinline__ float geo_to_float(G v);
template <> __device__ __forceinline__ float geo_to_float<float>(float v) { return v; }
template <> __device__ __forceinline__ float geo_to_float<__nv_bfloat16>(__nv_bfloat16 v) { return __bfloat162float(v); }

template <int NQ, typename G>
struct StagedLayout {
  static constexpr int NP = NQ * NQ * NQ;
  static constexpr int ROW_BYTES = NP * (int)sizeof(G);
  static constexpr int GEO_BYTES = 7 * ROW_BYTES;
  static constexpr int IDX_BYTES = NP * 4;
  static constexpr int ELEM_BYTES = GEO_BYTES + IDX_BYTES;
  static constexpr bool ok = (ROW_BYTES % 16 == 0) && (IDX_BYTES % 16 == 0);
};

// Dot product of NQ coefficients with a shared-memory row: 128-bit loads when the row is
// 16-byte aligned and NQ is a multiple of 4.
template <int NQ, bool VEC>
__device__ __forceinline__ float row_dot(const float* __restrict__ row, const float* c) {
  float acc = 0.f;
  if constexpr (VEC) {
    // two partial sums halve the dependent FMA chain
    float acc1 = 0.f;
#pragma unroll
    for (int m = 0; m < NQ; m += 4) {
      const float4 v = *reinterpret_cast<const float4*>(row + m);
      acc += c[m] * v.x;
      acc1 += c[m + 1] * v.y;
      acc += c[m + 2] * v.z;
      acc1 += c[m + 3] * v.w;
    }
    acc += acc1;
  } else {
#pragma unroll
    for (int m = 0; m < NQ; ++m) acc += c[m] * row[m];
  }
  return acc;
}

// MASS = false: lambda == 0 and no lambda field, the wJ row is neither copied nor used
template <int NQ, typename T, typename G, int EPB, int STAGES, bool PF = false, bool MASS = true>
__global__ void __launch_bounds__(NQ * NQ * EPB)
ax_hex_staged_kernel(const int64_t Nelements, const int32_t* __restrict__ elementList,
                     const int32_t* __restrict__ g2l, const G* __restrict__ ggeo, const int64_t geoStride,
                     const G* __restrict__ wJ, const int64_t wJStride, const T* __restrict__ Dg, const T lambda,
                     const T* __restrict__ lambdaE, const T* __restrict__ q, T* __restrict__ out,
                     const T outScale) {
  static_assert(std::is_same<T, float>::value, "staged kernel is FP32");
  using L = StagedLayout<NQ, G>;
  constexpr int NP = L::NP, NT = NQ * NQ * EPB;
  constexpr int CHUNKS = L::ELEM_BYTES / 16;
  constexpr int STAGE_BYTES = EPB * L::ELEM_BYTES;
  constexpr bool VEC = (NQ % 4 == 0);
  constexpr int RS = VEC ? NQ : NQ;          // row stride of s_q / s_Gqr
  constexpr int TS = VEC ? NQ + 4 : NQ + 1;  // row stride of the transposed copies (bank-conflict padding)
  extern __shared__ __align__(16) unsigned char smem[];
  __shared__ __align__(16) float s_D[NQ][NQ];
  // layer slabs, double-buffered by layer parity so one barrier per layer suffices
  // between reading a slab and overwriting it two layers later
  __shared__ __align__(16) float s_q[2][EPB][NQ][RS];     // s_q[j][i]   = q(i,j,k)
  __shared__ __align__(16) float s_qT[2][EPB][NQ][TS];    // s_qT[i][j]  = q(i,j,k)
  __shared__ __align__(16) float s_Gqr[2][EPB][NQ][RS];   // s_Gqr[j][i]
  __shared__ __align__(16) float s_GqsT[2][EPB][NQ][TS];  // s_GqsT[i][j]

  const int i = threadIdx.x, j = threadIdx.y, el = threadIdx.z;
  const int tid = i + NQ * (j + NQ * el);
  for (int t = tid; t < NQ * NQ; t += NT) s_D[t / NQ][t % NQ] = Dg[t];
  const int64_t ngroups = (Nelements + EPB - 1) / EPB;

  // copy of one element group: 7 geometric-factor rows and the index row per element,
  // each a contiguous run of 16-byte chunks (compile-time trip counts)
  constexpr int ROW_CHUNKS = L::ROW_BYTES / 16, IDX_CHUNKS = L::IDX_BYTES / 16;
  auto issue = [&](const int64_t grp, const int stage) {
    if (grp < ngroups) {
      unsigned char* base = smem + stage * STAGE_BYTES;
#pragma unroll
      for (int le = 0; le < EPB; ++le) {
        const int64_t ei = grp * EPB + le;
        if (ei < Nelements) {
          const int64_t e = elementList ? (int64_t)elementList[ei] : ei;
          unsigned char* dst = base + le * L::ELEM_BYTES;
#pragma unroll
          for (int comp = 0; comp < (MASS ? 7 : 6); ++comp) {
            const unsigned char* src =
                (comp < 6) ? reinterpret_cast<const unsigned char*>(ggeo + e * geoStride + (int64_t)comp * NP)
                           : reinterpret_cast<const unsigned char*>(wJ + e * wJStride);
            for (int c = tid; c < ROW_CHUNKS; c += NT) cp_async16(dst + comp * L::ROW_BYTES + c * 16, src + c * 16);
          }
          const unsigned char* srci = reinterpret_cast<const unsigned char*>(g2l + e * NP);
          for (int c = tid; c < IDX_CHUNKS; c += NT) cp_async16(dst + L::GEO_BYTES + c * 16, srci + c * 16);
        }
      }
    }
    cp_async_commit();
  };

#pragma unroll
  for (int st = 0; st < STAGES - 1; ++st) issue(blockIdx.x + (int64_t)st * gridDim.x, st);
  __syncthreads();
  float Dr[NQ], Ds[NQ], DTi[NQ], DTj[NQ];
#pragma unroll
  for (int m = 0; m < NQ; ++m) {
    Dr[m] = s_D[i][m];
    Ds[m] = s_D[j][m];
    DTi[m] = s_D[m][i];
    DTj[m] = s_D[m][j];
  }

  const int node = j * NQ + i;
  // PF: the gather of the next group's q through its staged index row is issued half-way
  // through this group's layers (after a wait for that group's copy, which was issued at
  // the start of this group), so its L2 latency overlaps the remaining layers
  float n_q[PF ? NQ : 1];
  int32_t n_id[PF ? NQ : 1];
  auto gather_next = [&](const int64_t g, const int stage) {
    if constexpr (PF) {
      const int32_t* nidx = reinterpret_cast<const int32_t*>(smem + stage * STAGE_BYTES + el * L::ELEM_BYTES +
                                                            L::GEO_BYTES);
      const bool act = (g < ngroups) && (g * EPB + el < Nelements);
#pragma unroll
      for (int k = 0; k < NQ; ++k) {
        const int32_t id = act ? nidx[k * NQ * NQ + node] : -1;
        n_id[k] = id;
        n_q[k] = (id >= 0) ? q[id] : 0.f;
      }
    }
  };
  if constexpr (PF) {
    static_assert(STAGES == 2, "prefetching variant uses two stages");
    cp_async_wait<0>();
    __syncthreads();
    gather_next(blockIdx.x, 0);
  }

  for (int64_t it = 0;; ++it) {
    const int64_t grp = blockIdx.x + it * gridDim.x;
    if (grp >= ngroups) break;
    // this group's copies are complete, and after the barrier no thread still reads the
    // stage of the previous group, which the next copy then refills
    if constexpr (!PF) cp_async_wait<STAGES - 2>();
    __syncthreads();
    issue(grp + (int64_t)(STAGES - 1) * gridDim.x, (int)((it + STAGES - 1) % STAGES));
    const unsigned char* base = smem + (it % STAGES) * STAGE_BYTES + el * L::ELEM_BYTES;
    const G* sg = reinterpret_cast<const G*>(base);
    const int32_t* sidx = reinterpret_cast<const int32_t*>(base + L::GEO_BYTES);
    const int64_t ei = grp * EPB + el;
    const bool active = ei < Nelements;
    const int64_t e = active ? (elementList ? (int64_t)elementList[ei] : ei) : 0;

    float r_q[NQ], r_Aq[NQ], qt[NQ], Gqt[NQ];
    int32_t r_id[NQ];
#pragma unroll
    for (int k = 0; k < NQ; ++k) {
      if constexpr (PF) {
        r_id[k] = n_id[k];
        r_q[k] = n_q[k];
      } else {
        const int32_t id = active ? sidx[k * NQ * NQ + node] : -1;
        r_id[k] = id;
        r_q[k] = (id >= 0) ? q[id] : 0.f;
      }
    }
    (void)sidx;
    const float lam = (lambdaE && active) ? lambdaE[e] : lambda;
    // t-direction of the pencil: qt = D r_q (rows of D are broadcast reads)
#pragma unroll
    for (int k = 0; k < NQ; ++k) qt[k] = row_dot<NQ, VEC>(&s_D[k][0], r_q);
#pragma unroll
    for (int k = 0; k < NQ; ++k) {
      const int off = k * NQ * NQ + node;
      const float G00 = geo_to_float(sg[0 * NP + off]), G01 = geo_to_float(sg[1 * NP + off]);
      const float G02 = geo_to_float(sg[2 * NP + off]), G11 = geo_to_float(sg[3 * NP + off]);
      const float G12 = geo_to_float(sg[4 * NP + off]), G22 = geo_to_float(sg[5 * NP + off]);
      float GwJ = 0.f;
      if constexpr (MASS) GwJ = geo_to_float(sg[6 * NP + off]);
      const int b = k & 1;
      s_q[b][el][j][i] = r_q[k];
      s_qT[b][el][i][j] = r_q[k];
      elem_sync<NQ>(el);
      const float qr = row_dot<NQ, VEC>(&s_q[b][el][j][0], Dr);    // sum_m D[i][m] q(m,j)
      const float qs = row_dot<NQ, VEC>(&s_qT[b][el][i][0], Ds);   // sum_m D[j][m] q(i,m)
      s_GqsT[b][el][i][j] = G01 * qr + G11 * qs + G12 * qt[k];
      s_Gqr[b][el][j][i] = G00 * qr + G01 * qs + G02 * qt[k];
      Gqt[k] = G02 * qr + G12 * qs + G22 * qt[k];
      float Auk = 0.f;
      if constexpr (MASS) Auk = GwJ * lam * r_q[k];
      elem_sync<NQ>(el);
      Auk += row_dot<NQ, VEC>(&s_GqsT[b][el][i][0], DTj);       // sum_m D[m][j] Gqs(i,m)
      Auk += row_dot<NQ, VEC>(&s_Gqr[b][el][j][0], DTi);        // sum_m D[m][i] Gqr(m,j)
      r_Aq[k] = Auk;
      if constexpr (PF) {
        if (k == NQ / 2) {
          cp_async_wait<0>();
          __syncthreads();   // the next group's copy (both elements of the CTA) is visible
          gather_next(grp + gridDim.x, (int)((it + 1) % STAGES));
        }
      }
    }
    // transposed t-direction: r_Aq[m] += sum_k D[k][m] Gqt[k]
#pragma unroll
    for (int k = 0; k < NQ; ++k) {
#pragma unroll
      for (int m = 0; m < NQ; m += (VEC ? 4 : 1)) {
        if constexpr (VEC) {
          const float4 d = *reinterpret_cast<const float4*>(&s_D[k][m]);
          r_Aq[m] += d.x * Gqt[k];
          r_Aq[m + 1] += d.y * Gqt[k];
          r_Aq[m + 2] += d.z * Gqt[k];
          r_Aq[m + 3] += d.w * Gqt[k];
        } else {
          r_Aq[m] += s_D[k][m] * Gqt[k];
        }
      }
    }
    if (active) {
#pragma unroll
      for (int k = 0; k < NQ; ++k)
        if (r_id[k] >= 0) atomicAdd(out + r_id[k], outScale * r_Aq[k]);
    }
  }
  cp_async_wait<0>();
}

// ---------------------------------------------------------------- FP64 even-odd variant
// GLL derivative matrices satisfy D[N-i][N-m] = -D[i][m], and so does D^T. Splitting a
// line q_0..q_N into e_m = q_m + q_{N-m} and o_m = q_m - q_{N-m} (m < H = Nq/2), the two
// outputs t and N-t of D q are A + B and B - A with A = sum_m Dp[t][m] e_m,
// B = sum_m Dm[t][m] o_m, Dp/Dm[t][m] = (D[t][m] +- D[t][N-m]) / 2: Nq FMA for two
// outputs instead of 2 Nq. GB300's FP64 operator is bound by the FP64 pipe, so the
// operation count is the lever: 49 instead of 59 FP64 operations per node at N = 7.
//
// Per layer k of an element, thread (i, j) forms one even/odd value of its row (partner
// (N-i, j) is lane ^ (Nq-1)) and one of its column (partner (i, N-j) is lane ^ 2Nq: the
// row map eo_row puts rows j and N-j in the same warp); then threads with i < H take
// the r-derivative pair (i, N-i) of row j and threads with i >= H the s-derivative pair
// (i-H, N-i+H) of column j. The t-direction works on the register pencil. The
// transposed derivatives repeat the pattern with D^T. Nq = 4 or 8 (N = 3, 7).
template <int NQ>
__device__ __forceinline__ int eo_row(const int jj) {
  const int lo = 2 * (jj >> 2) + (jj & 1);
  return (jj & 2) ? (NQ - 1 - lo) : lo;
}

template <int NQ>
__device__ __forceinline__ void eo_sync(const int el) {
  if constexpr ((NQ * NQ) % 32 == 0) elem_sync<NQ>(el);  // Nq = 8: the element's two warps
  else __syncwarp();                                    // Nq = 4: an element is half a warp
}

// MASS = false: lambda == 0 and no lambda field, the mass term and its wJ reads are left out
// UNIT: lambda == 1 without a lambda field, the mass term is wJ q (one FP64 multiply fewer
// per node, the same result: wJ * 1.0 is exact)
template <int NQ, bool MASS = true, bool UNIT = false>
__global__ void __launch_bounds__(NQ * NQ * elems_per_block<NQ>(), 3)
ax_hex_eo_kernel(const int64_t Nelements, const int32_t* __restrict__ elementList,
                 const int32_t* __restrict__ g2l, const double* __restrict__ ggeo, const int64_t geoStride,
                 const double* __restrict__ wJ, const int64_t wJStride, const double* __restrict__ Dg,
                 const double lambda, const double* __restrict__ lambdaE, const double* __restrict__ q,
                 double* __restrict__ out) {
  static_assert(NQ == 4 || NQ == 8, "even-odd kernel: Nq = 4 or 8");
  constexpr int NP = NQ * NQ * NQ, H = NQ / 2, N = NQ - 1;
  constexpr int EPB = elems_per_block<NQ>();
  constexpr unsigned FULL = 0xffffffffu;
  __shared__ double s_Dp[H][H], s_Dm[H][H];   // even/odd tables of D
  __shared__ double s_Tp[H][H], s_Tm[H][H];   // and of D^T
  __shared__ double s_R[EPB][NQ][NQ];         // row j: e_0..e_{H-1}, o_0..o_{H-1} along i
  __shared__ double s_S[EPB][NQ][NQ];         // column i: the same along j
  __shared__ double s_dr[EPB][NQ][NQ];        // [j][i] r-derivative, then r-transposed term
  __shared__ double s_ds[EPB][NQ][NQ];        // [j][i] s-derivative, then s-transposed term
  // per-thread pencils of D_t q and of G_t . grad q, [k][thread] (kept out of registers so
  // that three CTAs fit on an SM: the FP64 pipe needs the warps)
  __shared__ double s_qt[NQ][NQ * NQ * EPB];
  __shared__ double s_gt[NQ][NQ * NQ * EPB];

  const int i = threadIdx.x, jj = threadIdx.y, el = threadIdx.z;
  const int j = eo_row<NQ>(jj);
  const int tid = i + NQ * (jj + NQ * el);
  for (int t = tid; t < H * H; t += NQ * NQ * EPB) {
    const int a = t / H, m = t % H;
    const double d0 = Dg[a * NQ + m], d1 = Dg[a * NQ + N - m];     // D[a][m], D[a][N-m]
    const double t0 = Dg[m * NQ + a], t1 = Dg[(N - m) * NQ + a];   // D^T[a][m], D^T[a][N-m]
    s_Dp[a][m] = 0.5 * (d0 + d1);
    s_Dm[a][m] = 0.5 * (d0 - d1);
    s_Tp[a][m] = 0.5 * (t0 + t1);
    s_Tm[a][m] = 0.5 * (t0 - t1);
  }

  int64_t e = (int64_t)blockIdx.x * EPB + el;
  const bool active = e < Nelements;
  if (active && elementList) e = elementList[e];
  if (!active) e = 0;

  double r_q[NQ], r_Aq[NQ];
  int32_t r_id[NQ];
  const int64_t nodeBase = e * NP + j * NQ + i;
#pragma unroll
  for (int k = 0; k < NQ; ++k) {
    const int32_t id = active ? __ldg(g2l + nodeBase + k * NQ * NQ) : -1;
    r_id[k] = id;
    r_q[k] = (id >= 0) ? q[id] : 0.0;
  }
  const double lam = (lambdaE && active) ? lambdaE[e] : lambda;
  const double* gp = ggeo + e * geoStride + j * NQ + i;
  const double* wp = wJ + e * wJStride + j * NQ + i;
  __syncthreads();

  // t-direction of the pencil, even/odd
  {
    double E[H], O[H];
#pragma unroll
    for (int m = 0; m < H; ++m) {
      E[m] = r_q[m] + r_q[N - m];
      O[m] = r_q[m] - r_q[N - m];
    }
#pragma unroll
    for (int t = 0; t < H; ++t) {
      double A = 0, B = 0;
#pragma unroll
      for (int m = 0; m < H; ++m) {
        A += s_Dp[t][m] * E[m];
        B += s_Dm[t][m] * O[m];
      }
      s_qt[t][tid] = A + B;
      s_qt[N - t][tid] = B - A;
    }
  }

  // the pair task of this thread: r-pair of row j (i < H) or s-pair of column j (i >= H)
  const bool rtask = i < H;
  const int pt = rtask ? i : i - H;
  double* dst0 = rtask ? &s_dr[el][j][pt] : &s_ds[el][pt][j];
  double* dst1 = rtask ? &s_dr[el][j][N - pt] : &s_ds[el][N - pt][j];
  const double* line = rtask ? &s_R[el][j][0] : &s_S[el][j][0];
  // even/odd slot of this thread's node in its row (along i) and column (along j): the
  // value is partner + sign * own (e for the first half, o for the second), written
  // without branches so that no FP64 instruction issues twice in a diverged warp
  const int slotR = (i < H) ? i : H + N - i, slotS = (j < H) ? j : H + N - j;
  const double sgnR = (i < H) ? 1.0 : -1.0, sgnS = (j < H) ? 1.0 : -1.0;

#pragma unroll
  for (int k = 0; k < NQ; ++k) {
    const int off = k * NQ * NQ;
    double G00 = 0, G01 = 0, G02 = 0, G11 = 0, G12 = 0, G22 = 0, GwJ = 0;
    if (active) {
      G00 = gp[0 * NP + off]; G01 = gp[1 * NP + off]; G02 = gp[2 * NP + off];
      G11 = gp[3 * NP + off]; G12 = gp[4 * NP + off]; G22 = gp[5 * NP + off];
      if constexpr (MASS) GwJ = wp[off];
    }
    // even/odd values of q along i (row j) and along j (column i)
    const double v = r_q[k];
    const double pr = __shfl_xor_sync(FULL, v, NQ - 1);
    const double ps = __shfl_xor_sync(FULL, v, 2 * NQ);
    s_R[el][j][slotR] = fma(sgnR, v, pr);
    s_S[el][i][slotS] = fma(sgnS, v, ps);
    eo_sync<NQ>(el);
    {
      double A = 0, B = 0;
#pragma unroll
      for (int m = 0; m < H; ++m) {
        A += s_Dp[pt][m] * line[m];
        B += s_Dm[pt][m] * line[H + m];
      }
      *dst0 = A + B;
      *dst1 = B - A;
    }
    eo_sync<NQ>(el);
    const double qr = s_dr[el][j][i], qs = s_ds[el][j][i], qtk = s_qt[k][tid];
    const double Gqr = G00 * qr + G01 * qs + G02 * qtk;
    const double Gqs = G01 * qr + G11 * qs + G12 * qtk;
    s_gt[k][tid] = G02 * qr + G12 * qs + G22 * qtk;
    // even/odd values of Gqr along i and of Gqs along j for the transposed derivatives
    const double pr2 = __shfl_xor_sync(FULL, Gqr, NQ - 1);
    const double ps2 = __shfl_xor_sync(FULL, Gqs, 2 * NQ);
    s_R[el][j][slotR] = fma(sgnR, Gqr, pr2);
    s_S[el][i][slotS] = fma(sgnS, Gqs, ps2);
    eo_sync<NQ>(el);
    {
      double A = 0, B = 0;
#pragma unroll
      for (int m = 0; m < H; ++m) {
        A += s_Tp[pt][m] * line[m];
        B += s_Tm[pt][m] * line[H + m];
      }
      *dst0 = A + B;
      *dst1 = B - A;
    }
    eo_sync<NQ>(el);
    // the mass term lambda wJ q folded into the sum as one FMA
    const double sum = s_dr[el][j][i] + s_ds[el][j][i];
    if constexpr (MASS && UNIT) r_Aq[k] = fma(GwJ, v, sum);
    else if constexpr (MASS) r_Aq[k] = fma(GwJ * lam, v, sum);
    else r_Aq[k] = sum;
  }

  // transposed t-direction: r_Aq[t] += sum_m D[m][t] Gqt[m], even/odd
  {
    double E[H], O[H];
#pragma unroll
    for (int m = 0; m < H; ++m) {
      const double g0 = s_gt[m][tid], g1 = s_gt[N - m][tid];
      E[m] = g0 + g1;
      O[m] = g0 - g1;
    }
#pragma unroll
    for (int t = 0; t < H; ++t) {
      double A = 0, B = 0;
#pragma unroll
      for (int m = 0; m < H; ++m) {
        A += s_Tp[t][m] * E[m];
        B += s_Tm[t][m] * O[m];
      }
      r_Aq[t] += A + B;
      r_Aq[N - t] += B - A;
    }
  }

  if (!active) return;
#pragma unroll
  for (int k = 0; k < NQ; ++k)
    if (r_id[k] >= 0) atomicAdd(out + r_id[k], r_Aq[k]);
}

// ---------------------------------------------------------------- double-word variant
// The even-odd kernel above with every FP64 value held as a double-FP32 word (df64.cuh):
// FP64-accurate (48-bit significands, sums with absolute error of order 2^-48 times the
// magnitudes summed) on GB300's FP32 pipe, which runs ~64x the FP64 rate. q is read as
// FP64 and split with integer operations; the geometric factors come pre-split
// ([e][7][Np] hi/lo pairs, the same 8 bytes per value as FP64); each local result is
// rebuilt exactly as FP64 hi + lo (one FP64 add) and assembled with FP64 atomics.
// PFG: the geometric factors of layer k+1 are loaded into registers while layer k is
// computed, so their DRAM latency overlaps a whole layer's arithmetic
template <int NQ, bool PFG = false>
__global__ void __launch_bounds__(NQ * NQ * elems_per_block<NQ>(), (NQ == 4 ? 3 : 2))
ax_hex_dw_kernel(const int64_t Nelements, const int32_t* __restrict__ elementList,
                 const int32_t* __restrict__ g2l, const dw* __restrict__ ggeo, const int64_t geoStride,
                 const dw* __restrict__ wJ, const int64_t wJStride, const double* __restrict__ Dg,
                 const double lambda, const double* __restrict__ lambdaE, const double* __restrict__ q,
                 double* __restrict__ out) {
  static_assert(NQ == 4 || NQ == 8, "double-word kernel: Nq = 4 or 8");
  constexpr int NP = NQ * NQ * NQ, H = NQ / 2, N = NQ - 1;
  constexpr int EPB = elems_per_block<NQ>();
  __shared__ dw s_Dp[H][H], s_Dm[H][H], s_Tp[H][H], s_Tm[H][H];
  __shared__ dw s_R[EPB][NQ][NQ], s_S[EPB][NQ][NQ], s_dr[EPB][NQ][NQ], s_ds[EPB][NQ][NQ];
  __shared__ dw s_qt[NQ][NQ * NQ * EPB], s_gt[NQ][NQ * NQ * EPB];

  const int i = threadIdx.x, jj = threadIdx.y, el = threadIdx.z;
  const int j = eo_row<NQ>(jj);
  const int tid = i + NQ * (jj + NQ * el);
  for (int t = tid; t < H * H; t += NQ * NQ * EPB) {
    const int a = t / H, m = t % H;
    const double d0 = Dg[a * NQ + m], d1 = Dg[a * NQ + N - m];
    const double t0 = Dg[m * NQ + a], t1 = Dg[(N - m) * NQ + a];
    s_Dp[a][m] = dw_from_double(0.5 * (d0 + d1));
    s_Dm[a][m] = dw_from_double(0.5 * (d0 - d1));
    s_Tp[a][m] = dw_from_double(0.5 * (t0 + t1));
    s_Tm[a][m] = dw_from_double(0.5 * (t0 - t1));
  }

  int64_t e = (int64_t)blockIdx.x * EPB + el;
  const bool active = e < Nelements;
  if (active && elementList) e = elementList[e];
  if (!active) e = 0;

  dw r_q[NQ], r_Aq[NQ];
  int32_t r_id[NQ];
  const int64_t nodeBase = e * NP + j * NQ + i;
#pragma unroll
  for (int k = 0; k < NQ; ++k) {
    const int32_t id = active ? __ldg(g2l + nodeBase + k * NQ * NQ) : -1;
    r_id[k] = id;
    r_q[k] = dw_from_double((id >= 0) ? q[id] : 0.0);
  }
  const dw lam = dw_from_double((lambdaE && active) ? lambdaE[e] : lambda);
  const dw* gp = ggeo + e * geoStride + j * NQ + i;
  const dw* wp = wJ + e * wJStride + j * NQ + i;
  __syncthreads();

  {
    dw E[H], O[H];
#pragma unroll
    for (int m = 0; m < H; ++m) {
      E[m] = dw_add(r_q[m], r_q[N - m]);
      O[m] = dw_sub(r_q[m], r_q[N - m]);
    }
#pragma unroll
    for (int t = 0; t < H; ++t) {
      dw_acc A, B;
#pragma unroll
      for (int m = 0; m < H; ++m) {
        A.mac(s_Dp[t][m], E[m]);
        B.mac(s_Dm[t][m], O[m]);
      }
      const dw a = A.get(), b = B.get();
      s_qt[t][tid] = dw_add(a, b);
      s_qt[N - t][tid] = dw_sub(b, a);
    }
  }

  const bool rtask = i < H;
  const int pt = rtask ? i : i - H;
  dw* dst0 = rtask ? &s_dr[el][j][pt] : &s_ds[el][pt][j];
  dw* dst1 = rtask ? &s_dr[el][j][N - pt] : &s_ds[el][N - pt][j];
  const dw* line = rtask ? &s_R[el][j][0] : &s_S[el][j][0];
  const int slotR = (i < H) ? i : H + N - i, slotS = (j < H) ? j : H + N - j;
  const float sgnR = (i < H) ? 1.f : -1.f, sgnS = (j < H) ? 1.f : -1.f;

  const dw zero{0.f, 0.f};
  dw nG[7];   // next layer's factors (PFG)
  if constexpr (PFG) {
#pragma unroll
    for (int c = 0; c < 6; ++c) nG[c] = active ? gp[c * NP] : zero;
    nG[6] = active ? wp[0] : zero;
  }
#pragma unroll
  for (int k = 0; k < NQ; ++k) {
    const int off = k * NQ * NQ;
    dw G00, G01, G02, G11, G12, G22, GwJ;
    if constexpr (PFG) {
      G00 = nG[0]; G01 = nG[1]; G02 = nG[2]; G11 = nG[3]; G12 = nG[4]; G22 = nG[5]; GwJ = nG[6];
      if (k + 1 < NQ) {
        const int noff = off + NQ * NQ;
#pragma unroll
        for (int c = 0; c < 6; ++c) nG[c] = active ? gp[c * NP + noff] : zero;
        nG[6] = active ? wp[noff] : zero;
      }
    } else {
      G00 = active ? gp[0 * NP + off] : zero; G01 = active ? gp[1 * NP + off] : zero;
      G02 = active ? gp[2 * NP + off] : zero; G11 = active ? gp[3 * NP + off] : zero;
      G12 = active ? gp[4 * NP + off] : zero; G22 = active ? gp[5 * NP + off] : zero;
      GwJ = active ? wp[off] : zero;
    }
    const dw v = r_q[k];
    const dw pr = dw_shfl_xor(v, NQ - 1), ps = dw_shfl_xor(v, 2 * NQ);
    s_R[el][j][slotR] = dw_add(pr, dw_scale_sign(sgnR, v));
    s_S[el][i][slotS] = dw_add(ps, dw_scale_sign(sgnS, v));
    eo_sync<NQ>(el);
    {
      dw_acc A, B;
#pragma unroll
      for (int m = 0; m < H; ++m) {
        A.mac(s_Dp[pt][m], line[m]);
        B.mac(s_Dm[pt][m], line[H + m]);
      }
      const dw a = A.get(), b = B.get();
      *dst0 = dw_add(a, b);
      *dst1 = dw_sub(b, a);
    }
    eo_sync<NQ>(el);
    const dw qr = s_dr[el][j][i], qs = s_ds[el][j][i], qtk = s_qt[k][tid];
    dw_acc ar, as, at;
    ar.mac(G00, qr); ar.mac(G01, qs); ar.mac(G02, qtk);
    as.mac(G01, qr); as.mac(G11, qs); as.mac(G12, qtk);
    at.mac(G02, qr); at.mac(G12, qs); at.mac(G22, qtk);
    const dw Gqr = ar.get(), Gqs = as.get();
    s_gt[k][tid] = at.get();
    const dw mass = dw_mul(dw_mul(GwJ, lam), v);
    const dw pr2 = dw_shfl_xor(Gqr, NQ - 1), ps2 = dw_shfl_xor(Gqs, 2 * NQ);
    s_R[el][j][slotR] = dw_add(pr2, dw_scale_sign(sgnR, Gqr));
    s_S[el][i][slotS] = dw_add(ps2, dw_scale_sign(sgnS, Gqs));
    eo_sync<NQ>(el);
    {
      dw_acc A, B;
#pragma unroll
      for (int m = 0; m < H; ++m) {
        A.mac(s_Tp[pt][m], line[m]);
        B.mac(s_Tm[pt][m], line[H + m]);
      }
      const dw a = A.get(), b = B.get();
      *dst0 = dw_add(a, b);
      *dst1 = dw_sub(b, a);
    }
    eo_sync<NQ>(el);
    r_Aq[k] = dw_add(dw_add(mass, s_dr[el][j][i]), s_ds[el][j][i]);
  }

  {
    dw E[H], O[H];
#pragma unroll
    for (int m = 0; m < H; ++m) {
      const dw g0 = s_gt[m][tid], g1 = s_gt[N - m][tid];
      E[m] = dw_add(g0, g1);
      O[m] = dw_sub(g0, g1);
    }
#pragma unroll
    for (int t = 0; t < H; ++t) {
      dw_acc A, B;
#pragma unroll
      for (int m = 0; m < H; ++m) {
        A.mac(s_Tp[t][m], E[m]);
        B.mac(s_Tm[t][m], O[m]);
      }
      const dw a = A.get(), b = B.get();
      r_Aq[t] = dw_add(r_Aq[t], dw_add(a, b));
      r_Aq[N - t] = dw_add(r_Aq[N - t], dw_sub(b, a));
    }
  }

  if (!active) return;
#pragma unroll
  for (int k = 0; k < NQ; ++k)
    if (r_id[k] >= 0) atomicAdd(out + r_id[k], dw_to_double(r_Aq[k]));
}

// n double words from 16-byte aligned shared memory, two per 128-bit load
template <int n>
__device__ __forceinline__ void ld_dw4x2(const dw* src, dw* v) {
  const float4* p = reinterpret_cast<const float4*>(src);
#pragma unroll
  for (int t = 0; t < n / 2; ++t) {
    const float4 x = p[t];
    v[2 * t] = {x.x, x.y};
    v[2 * t + 1] = {x.z, x.w};
  }
}

// The N = 7 double-word kernel for four CTAs (32 warps) per SM, against two for the
// kernel above (64^3: 3.09 ms against 4.36 ms per application):
// - each thread's q pencil lives in shared memory (only the same thread reads it back),
//   and layer k's local result replaces its consumed t-derivative slot, so the thread
//   holds no pencils in registers (64 registers); dof indices are re-read at the end;
// - intermediate sums skip the renormalisation their consumers do not need (dw_add_u,
//   dw_acc::raw), sums start from their first product, and the +-1 of the even/odd line
//   values is folded into FMAs (~660 instructions per node against ~790);
// - line values and D rows are read from shared memory two double words per 128-bit load;
// - the layer loop is rolled (8x less code: instruction-cache misses were a stall with
//   four CTAs in different phases);
// - one thread per element asks L2 for the element's geometric factors (and wJ) in one
//   bulk prefetch each, so the per-layer loads of layers 1..N hit L2.
// Measured and not kept: the next layer's factors staged through shared memory with
// cp.async (more shared-memory traffic; slower at three CTAs per SM), a register prefetch
// (does not fit 64 registers). MASS = false: lambda == 0 and no lambda field, the mass term
// and its wJ reads are left out.
template <int NQ, bool MASS, bool UNIT = false>
__global__ void __launch_bounds__(NQ * NQ * elems_per_block<NQ>(), 4)
ax_hex_dw_lean_kernel(const int64_t Nelements, const int32_t* __restrict__ elementList,
                      const int32_t* __restrict__ g2l, const dw* __restrict__ ggeo, const int64_t geoStride,
                      const dw* __restrict__ wJ, const int64_t wJStride, const double* __restrict__ Dg,
                      const double lambda, const double* __restrict__ lambdaE, const double* __restrict__ q,
                      double* __restrict__ out) {
  static_assert(NQ == 8, "lean double-word kernel: Nq = 8");
  constexpr int NP = NQ * NQ * NQ, H = NQ / 2, N = NQ - 1;
  constexpr int EPB = elems_per_block<NQ>();
  constexpr int NT = NQ * NQ * EPB;
  __shared__ __align__(16) dw s_Dp[H][H], s_Dm[H][H], s_Tp[H][H], s_Tm[H][H];
  __shared__ __align__(16) dw s_R[EPB][NQ][NQ], s_S[EPB][NQ][NQ];
  __shared__ dw s_dr[EPB][NQ][NQ], s_ds[EPB][NQ][NQ];
  // s_q: layer k of the thread's q pencil until layer k reads it, then that layer's
  // t-contraction input G_t . grad q (the same thread writes and reads each slot)
  __shared__ dw s_q[NQ][NT], s_qt[NQ][NT];

  const int i = threadIdx.x, jj = threadIdx.y, el = threadIdx.z;
  const int j = eo_row<NQ>(jj);
  const int tid = i + NQ * (jj + NQ * el);
  for (int t = tid; t < H * H; t += NT) {
    const int a = t / H, m = t % H;
    const double d0 = Dg[a * NQ + m], d1 = Dg[a * NQ + N - m];
    const double t0 = Dg[m * NQ + a], t1 = Dg[(N - m) * NQ + a];
    s_Dp[a][m] = dw_from_double(0.5 * (d0 + d1));
    s_Dm[a][m] = dw_from_double(0.5 * (d0 - d1));
    s_Tp[a][m] = dw_from_double(0.5 * (t0 + t1));
    s_Tm[a][m] = dw_from_double(0.5 * (t0 - t1));
  }

  int64_t e = (int64_t)blockIdx.x * EPB + el;
  const bool active = e < Nelements;
  if (active && elementList) e = elementList[e];
  if (!active) e = 0;

  const int64_t nodeBase = e * NP + j * NQ + i;
  if (active && i == 0 && jj == 0) {
    prefetch_l2_bulk(ggeo + e * geoStride, 6 * NP * sizeof(dw));
    if constexpr (MASS) prefetch_l2_bulk(wJ + e * wJStride, NP * sizeof(dw));
  }
  {
    int32_t id[NQ];
#pragma unroll
    for (int k = 0; k < NQ; ++k) id[k] = active ? __ldg(g2l + nodeBase + k * NQ * NQ) : -1;
    double qv[NQ];
#pragma unroll
    for (int k = 0; k < NQ; ++k) qv[k] = (id[k] >= 0) ? q[id[k]] : 0.0;
#pragma unroll
    for (int k = 0; k < NQ; ++k) s_q[k][tid] = dw_from_double(qv[k]);
  }
  const dw lam = MASS ? dw_from_double((lambdaE && active) ? lambdaE[e] : lambda) : dw{0.f, 0.f};
  const dw* gp = ggeo + e * geoStride + j * NQ + i;
  const dw* wp = wJ + e * wJStride + j * NQ + i;
  __syncthreads();

  {
    dw E[H], O[H];
#pragma unroll
    for (int m = 0; m < H; ++m) {
      const dw q0 = s_q[m][tid], q1 = s_q[N - m][tid];
      E[m] = dw_add_u(q0, q1);
      O[m] = dw_add_u(q0, dw_neg(q1));
    }
#pragma unroll
    for (int t = 0; t < H; ++t) {
      dw_acc A(s_Dp[t][0], E[0]), B(s_Dm[t][0], O[0]);
#pragma unroll
      for (int m = 1; m < H; ++m) {
        A.mac(s_Dp[t][m], E[m]);
        B.mac(s_Dm[t][m], O[m]);
      }
      const dw a = A.raw(), b = B.raw();
      s_qt[t][tid] = dw_add_u(a, b);
      s_qt[N - t][tid] = dw_add_u(b, dw_neg(a));
    }
  }

  const bool rtask = i < H;
  const int pt = rtask ? i : i - H;
  dw* dst0 = rtask ? &s_dr[el][j][pt] : &s_ds[el][pt][j];
  dw* dst1 = rtask ? &s_dr[el][j][N - pt] : &s_ds[el][N - pt][j];
  const dw* line = rtask ? &s_R[el][j][0] : &s_S[el][j][0];
  const int slotR = (i < H) ? i : H + N - i, slotS = (j < H) ? j : H + N - j;
  const float sgnR = (i < H) ? 1.f : -1.f, sgnS = (j < H) ? 1.f : -1.f;

  const dw zero{0.f, 0.f};
  // the local result of layer k goes to s_qt[k] once layer k has read its t-derivative
#pragma unroll 1
  for (int k = 0; k < NQ; ++k) {
    const int off = k * NQ * NQ;
    const dw G00 = active ? gp[0 * NP + off] : zero, G01 = active ? gp[1 * NP + off] : zero;
    const dw G02 = active ? gp[2 * NP + off] : zero, G11 = active ? gp[3 * NP + off] : zero;
    const dw G12 = active ? gp[4 * NP + off] : zero, G22 = active ? gp[5 * NP + off] : zero;
    dw GwJ = zero;
    if constexpr (MASS) GwJ = active ? wp[off] : zero;
    const dw v = s_q[k][tid];
    const dw pr = dw_shfl_xor(v, NQ - 1), ps = dw_shfl_xor(v, 2 * NQ);
    s_R[el][j][slotR] = dw_add_sign_u(pr, sgnR, v);
    s_S[el][i][slotS] = dw_add_sign_u(ps, sgnS, v);
    eo_sync<NQ>(el);
    {
      dw L[NQ], Dp[H], Dm[H];
      ld_dw4x2<NQ>(line, L);
      ld_dw4x2<H>(&s_Dp[pt][0], Dp);
      ld_dw4x2<H>(&s_Dm[pt][0], Dm);
      dw_acc A(Dp[0], L[0]), B(Dm[0], L[H]);
#pragma unroll
      for (int m = 1; m < H; ++m) {
        A.mac(Dp[m], L[m]);
        B.mac(Dm[m], L[H + m]);
      }
      const dw a = A.raw(), b = B.raw();
      *dst0 = dw_add_u(a, b);
      *dst1 = dw_add_u(b, dw_neg(a));
    }
    eo_sync<NQ>(el);
    const dw qr = s_dr[el][j][i], qs = s_ds[el][j][i], qtk = s_qt[k][tid];
    dw_acc ar(G00, qr), as(G01, qr), at(G02, qr);
    ar.mac(G01, qs); ar.mac(G02, qtk);
    as.mac(G11, qs); as.mac(G12, qtk);
    at.mac(G12, qs); at.mac(G22, qtk);
    const dw Gqr = ar.raw(), Gqs = as.raw();
    s_q[k][tid] = at.raw();
    dw mass{0.f, 0.f};
    if constexpr (MASS && UNIT) mass = dw_mul(GwJ, v);   // lambda == 1: wJ q
    else if constexpr (MASS) mass = dw_mul(dw_mul(GwJ, lam), v);
    const dw pr2 = dw_shfl_xor(Gqr, NQ - 1), ps2 = dw_shfl_xor(Gqs, 2 * NQ);
    s_R[el][j][slotR] = dw_add_sign_u(pr2, sgnR, Gqr);
    s_S[el][i][slotS] = dw_add_sign_u(ps2, sgnS, Gqs);
    eo_sync<NQ>(el);
    {
      dw L[NQ], Tp[H], Tm[H];
      ld_dw4x2<NQ>(line, L);
      ld_dw4x2<H>(&s_Tp[pt][0], Tp);
      ld_dw4x2<H>(&s_Tm[pt][0], Tm);
      dw_acc A(Tp[0], L[0]), B(Tm[0], L[H]);
#pragma unroll
      for (int m = 1; m < H; ++m) {
        A.mac(Tp[m], L[m]);
        B.mac(Tm[m], L[H + m]);
      }
      const dw a = A.raw(), b = B.raw();
      *dst0 = dw_add_u(a, b);
      *dst1 = dw_add_u(b, dw_neg(a));
    }
    eo_sync<NQ>(el);
    if constexpr (MASS) s_qt[k][tid] = dw_add_u(dw_add_u(mass, s_dr[el][j][i]), s_ds[el][j][i]);
    else s_qt[k][tid] = dw_add_u(s_dr[el][j][i], s_ds[el][j][i]);
  }

  {
    dw E[H], O[H];
#pragma unroll
    for (int m = 0; m < H; ++m) {
      const dw g0 = s_q[m][tid], g1 = s_q[N - m][tid];
      E[m] = dw_add_u(g0, g1);
      O[m] = dw_add_u(g0, dw_neg(g1));
    }
#pragma unroll
    for (int t = 0; t < H; ++t) {
      dw_acc A(s_Tp[t][0], E[0]), B(s_Tm[t][0], O[0]);
#pragma unroll
      for (int m = 1; m < H; ++m) {
        A.mac(s_Tp[t][m], E[m]);
        B.mac(s_Tm[t][m], O[m]);
      }
      const dw a = A.raw(), b = B.raw();
      s_qt[t][tid] = dw_add_u(s_qt[t][tid], dw_add_u(a, b));
      s_qt[N - t][tid] = dw_add_u(s_qt[N - t][tid], dw_add_u(b, dw_neg(a)));
    }
  }

  if (!active) return;
#pragma unroll
  for (int k = 0; k < NQ; ++k) {
    const int32_t id = __ldg(g2l + nodeBase + k * NQ * NQ);
    if (id >= 0) atomicAdd(out + id, dw_to_double(s_qt[k][tid]));
  }
}

// Double-word operator for the degrees without an even-odd kernel (N = 1, 2, 4, 5, 6, 8):
// one thread per node, EPB elements per CTA (at least 128 threads), direct Nq-term
// contractions through shared memory, the same df64 building blocks and FP64 assembly.
template <int NQ>
constexpr int dw_generic_epb() {
  return (NQ * NQ * NQ >= 128) ? 1 : 128 / (NQ * NQ * NQ);
}

template <int NQ>
__global__ void __launch_bounds__(NQ * NQ * NQ * dw_generic_epb<NQ>())
ax_hex_dw_generic_kernel(const int64_t Nelements, const int32_t* __restrict__ elementList,
                         const int32_t* __restrict__ g2l, const dw* __restrict__ ggeo, const int64_t geoStride,
                         const dw* __restrict__ wJ, const int64_t wJStride, const double* __restrict__ Dg,
                         const double lambda, const double* __restrict__ lambdaE, const double* __restrict__ q,
                         double* __restrict__ out) {
  constexpr int NP = NQ * NQ * NQ, NFP = NQ * NQ, EPB = dw_generic_epb<NQ>();
  __shared__ dw s_D[NQ * NQ];
  __shared__ dw s_q[EPB][NP], s_r[EPB][NP], s_s[EPB][NP], s_t[EPB][NP];
  const int el = threadIdx.x / NP, n = threadIdx.x % NP;
  for (int t = threadIdx.x; t < NQ * NQ; t += blockDim.x) s_D[t] = dw_from_double(Dg[t]);
  int64_t e = (int64_t)blockIdx.x * EPB + el;
  const bool active = e < Nelements;
  if (active && elementList) e = elementList[e];
  if (!active) e = 0;
  const int32_t id = active ? g2l[e * NP + n] : -1;
  const dw qn = dw_from_double(id >= 0 ? q[id] : 0.0);
  s_q[el][n] = qn;
  __syncthreads();
  const int i = n % NQ, j = (n / NQ) % NQ, k = n / NFP;
  dw_acc ar, as, at;
#pragma unroll
  for (int m = 0; m < NQ; ++m) {
    ar.mac(s_D[i * NQ + m], s_q[el][m + j * NQ + k * NFP]);
    as.mac(s_D[j * NQ + m], s_q[el][i + m * NQ + k * NFP]);
    at.mac(s_D[k * NQ + m], s_q[el][i + j * NQ + m * NFP]);
  }
  const dw qr = ar.get(), qs = as.get(), qt = at.get();
  const dw* gp = ggeo + e * geoStride + n;
  const dw G00 = gp[0 * NP], G01 = gp[1 * NP], G02 = gp[2 * NP], G11 = gp[3 * NP], G12 = gp[4 * NP],
           G22 = gp[5 * NP];
  const dw GwJ = wJ[e * wJStride + n];
  const dw lam = dw_from_double((lambdaE && active) ? lambdaE[e] : lambda);
  {
    dw_acc gr, gs, gt;
    gr.mac(G00, qr); gr.mac(G01, qs); gr.mac(G02, qt);
    gs.mac(G01, qr); gs.mac(G11, qs); gs.mac(G12, qt);
    gt.mac(G02, qr); gt.mac(G12, qs); gt.mac(G22, qt);
    s_r[el][n] = gr.get();
    s_s[el][n] = gs.get();
    s_t[el][n] = gt.get();
  }
  const dw mass = dw_mul(dw_mul(GwJ, lam), qn);
  __syncthreads();
  dw_acc v;
  v.h = mass.h;
  v.l = mass.l;
#pragma unroll
  for (int p = 0; p < NQ; ++p) {
    v.mac(s_D[p * NQ + i], s_r[el][p + j * NQ + k * NFP]);
    v.mac(s_D[p * NQ + j], s_s[el][i + p * NQ + k * NFP]);
    v.mac(s_D[p * NQ + k], s_t[el][i + j * NQ + p * NFP]);
  }
  if (id >= 0) atomicAdd(out + id, dw_to_double(v.get()));
}

template <int NQ>
static int launch_dw_generic(const AxArgs<double, float2>& a, cudaStream_t s) {
  constexpr int EPB = dw_generic_epb<NQ>();
  const int64_t blocks = (a.Nelements + EPB - 1) / EPB;
  ax_hex_dw_generic_kernel<NQ><<<(unsigned)blocks, NQ * NQ * NQ * EPB, 0, s>>>(
      a.Nelements, a.elementList, a.g2l, reinterpret_cast<const dw*>(a.ggeo), a.geoStride,
      reinterpret_cast<const dw*>(a.wJ), a.wJStride, a.D, a.lambda, a.lambdaE, a.q, a.out);
  LPG_LAUNCH_CHECK("ax_hex_dw_generic_kernel");
  return LPG_OK;
}

// N = 7 double-word kernel: the four-CTA kernel (ax_hex_dw_lean_kernel). LPG_AX_DW =
// classic is a tuning override back to the two-CTA kernel with the register prefetch.
static bool dw7_classic() {
  static const bool v = [] {
    const char* ev = std::getenv("LPG_AX_DW");
    return ev && !std::strcmp(ev, "classic");
  }();
  return v;
}

int ax_hex_dw(const AxArgs<double, float2>& a, cudaStream_t s) {
  if (a.Nelements <= 0) return LPG_OK;
  if (a.N < 1 || a.N > 8) return set_error(LPG_ERR_UNSUPPORTED, "double-word operator: N must be 1..8");
  if (a.Nglobal > 0) LPG_CUDA_TRY(cudaMemsetAsync(a.out, 0, sizeof(double) * a.Nglobal, s));
  switch (a.N) {
    case 1: return launch_dw_generic<2>(a, s);
    case 2: return launch_dw_generic<3>(a, s);
    case 4: return launch_dw_generic<5>(a, s);
    case 5: return launch_dw_generic<6>(a, s);
    case 6: return launch_dw_generic<7>(a, s);
    case 8: return launch_dw_generic<9>(a, s);
    default: break;
  }
  if (a.N == 7) {
    const int64_t blocks = (a.Nelements + 3) / 4;
    const bool mass = a.lambdaE || a.lambda != 0.0;
#define LPG_DW_ARGS                                                                                   \
  a.Nelements, a.elementList, a.g2l, reinterpret_cast<const dw*>(a.ggeo), a.geoStride,               \
      reinterpret_cast<const dw*>(a.wJ), a.wJStride, a.D, a.lambda, a.lambdaE, a.q, a.out
    if (dw7_classic())
      ax_hex_dw_kernel<8, true><<<(unsigned)blocks, dim3(8, 8, 4), 0, s>>>(LPG_DW_ARGS);
    else if (mass && a.lambda == 1.0 && !a.lambdaE)
      ax_hex_dw_lean_kernel<8, true, true><<<(unsigned)blocks, dim3(8, 8, 4), 0, s>>>(LPG_DW_ARGS);
    else if (mass)
      ax_hex_dw_lean_kernel<8, true><<<(unsigned)blocks, dim3(8, 8, 4), 0, s>>>(LPG_DW_ARGS);
    else
      ax_hex_dw_lean_kernel<8, false><<<(unsigned)blocks, dim3(8, 8, 4), 0, s>>>(LPG_DW_ARGS);
#undef LPG_DW_ARGS
  } else {
    const int64_t blocks = (a.Nelements + 15) / 16;
    ax_hex_dw_kernel<4><<<(unsigned)blocks, dim3(4, 4, 16), 0, s>>>(
        a.Nelements, a.elementList, a.g2l, reinterpret_cast<const dw*>(a.ggeo), a.geoStride,
        reinterpret_cast<const dw*>(a.wJ), a.wJStride, a.D, a.lambda, a.lambdaE, a.q, a.out);
  }
  LPG_LAUNCH_CHECK("ax_hex_dw_kernel");
  return LPG_OK;
}

template <int NQ, typename T, typename G, int EPB, int STAGES, bool PF = false, bool MASS = true>
static int launch_staged(const AxArgs<T, G>& a, cudaStream_t s) {
  using L = StagedLayout<NQ, G>;
  constexpr int smem = STAGES * EPB * L::ELEM_BYTES;
  static PerDeviceConfig perDevice;   // per instantiation: dynamic shared memory opt-in, occupancy
  auto kern = ax_hex_staged_kernel<NQ, T, G, EPB, STAGES, PF, MASS>;
  KernelConfig cfg;
  const int rc = perDevice.get(
      [&](int, KernelConfig& c) {
        LPG_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
        LPG_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&c.ctasPerSM, kern, NQ * NQ * EPB, smem));
        if (c.ctasPerSM < 1) return set_error(LPG_ERR_UNSUPPORTED, "staged Ax: kernel does not fit on an SM");
        return (int)LPG_OK;
      },
      &cfg);
  if (rc) return rc;
  const int64_t groups = (a.Nelements + EPB - 1) / EPB;
  const int64_t grid = std::min<int64_t>(groups, (int64_t)cfg.numSMs * cfg.ctasPerSM);
  if (grid <= 0) return LPG_OK;
  kern<<<(unsigned)grid, dim3(NQ, NQ, EPB), smem, s>>>(a.Nelements, a.elementList, a.g2l, a.ggeo, a.geoStride, a.wJ,
                                                        a.wJStride, a.D, a.lambda, a.lambdaE, a.q, a.out,
                                                        a.outScale);
  LPG_LAUNCH_CHECK("ax_hex_staged_kernel");
  return LPG_OK;
}

static int staged_variant() {
  static int v = -2;
  if (v == -2) {
    const char* e = std::getenv("LPG_AX_STAGED");
    v = -1;
    if (e) {
      if (!std::strcmp(e, "off")) v = 0;
      else if (!std::strcmp(e, "2x2")) v = 22;
      else if (!std::strcmp(e, "2x3")) v = 23;
      else if (!std::strcmp(e, "4x2")) v = 42;
      else if (!std::strcmp(e, "4x3")) v = 43;
      else if (!std::strcmp(e, "2x2pf")) v = 122;
    }
  }
  return v;
}

// the staged kernel needs 16-byte aligned rows (even Nq) and aligned strides/pointers
template <int NQ, typename T, typename G>
static bool staged_ok(const AxArgs<T, G>& a) {
  using L = StagedLayout<NQ, G>;
  if (!L::ok) return false;
  auto al = [](const void* p) { return ((uintptr_t)p & 15) == 0; };
  return al(a.ggeo) && al(a.wJ) && al(a.g2l) && ((a.geoStride * (int64_t)sizeof(G)) % 16 == 0) &&
         ((a.wJStride * (int64_t)sizeof(G)) % 16 == 0);
}

// LPG_AX_FP64 = direct: tuning override back to the direct-contraction FP64 kernel
static bool fp64_direct_override() {
  static const bool direct = [] {
    const char* e = std::getenv("LPG_AX_FP64");
    return e && !std::strcmp(e, "direct");
  }();
  return direct;
}

template <int NQ, typename T, typename G, int INMODE, int OUTMODE>
static int launch_ax(const AxArgs<T, G>& a, cudaStream_t s) {
  if constexpr (std::is_same<T, float>::value && INMODE == IN_GATHER && OUTMODE == OUT_ASSEMBLE) {
    if (staged_ok<NQ, T, G>(a)) {
      // LPG_AX_STAGED = off | EPBxSTAGES (2x2, 2x3, 4x2, 4x3) | 2x2pf: tuning override
      const int v = staged_variant();
      if (v == 0) { /* fall through to the unstaged kernel */ }
      else if (v == 22) return launch_staged<NQ, T, G, 2, 2>(a, s);
      else if (v == 23) return launch_staged<NQ, T, G, 2, 3>(a, s);
      else if (v == 43) return launch_staged<NQ, T, G, 4, 3>(a, s);
      else if (v == 42) return launch_staged<NQ, T, G, 4, 2>(a, s);
      else if (v == 122) return launch_staged<NQ, T, G, 2, 2, true>(a, s);
      // measured best at N=7: FP32 geometry with the next group's q gathered half-way
      // through the current group (0.997 vs 1.112 ms at 64^3); BF16 geometry without it
      // (lambda = 0 without a lambda field: the instantiation without the mass term and wJ copy)
      const bool noMass = (a.lambda == 0 && !a.lambdaE);
      if constexpr (std::is_same<G, float>::value)
        return noMass ? launch_staged<NQ, T, G, 2, 2, true, false>(a, s) : launch_staged<NQ, T, G, 2, 2, true>(a, s);
      else
        return noMass ? launch_staged<NQ, T, G, 2, 2, false, false>(a, s) : launch_staged<NQ, T, G, 2, 2>(a, s);
    }
  }
  constexpr int EPB = elems_per_block<NQ>();
  if (a.Nelements <= 0) return LPG_OK;
  const int64_t blocks = (a.Nelements + EPB - 1) / EPB;
  if (blocks > 0x7fffffffLL) return set_error(LPG_ERR_INVALID, "ax: too many elements");
  dim3 block(NQ, NQ, EPB);
  if constexpr (std::is_same<T, double>::value && std::is_same<G, double>::value && INMODE == IN_GATHER &&
                OUTMODE == OUT_ASSEMBLE && (NQ == 4 || NQ == 8)) {
    if (!fp64_direct_override()) {
      if (a.lambda == 0.0 && !a.lambdaE)
        ax_hex_eo_kernel<NQ, false><<<(unsigned)blocks, block, 0, s>>>(a.Nelements, a.elementList, a.g2l, a.ggeo,
                                                                      a.geoStride, a.wJ, a.wJStride, a.D, a.lambda,
                                                                      a.lambdaE, a.q, a.out);
      else if (a.lambda == 1.0 && !a.lambdaE)
        ax_hex_eo_kernel<NQ, true, true><<<(unsigned)blocks, block, 0, s>>>(a.Nelements, a.elementList, a.g2l,
                                                                           a.ggeo, a.geoStride, a.wJ, a.wJStride,
                                                                           a.D, a.lambda, a.lambdaE, a.q, a.out);
      else
        ax_hex_eo_kernel<NQ, true><<<(unsigned)blocks, block, 0, s>>>(a.Nelements, a.elementList, a.g2l, a.ggeo,
                                                                     a.geoStride, a.wJ, a.wJStride, a.D, a.lambda,
                                                                     a.lambdaE, a.q, a.out);
      LPG_LAUNCH_CHECK("ax_hex_eo_kernel");
      return LPG_OK;
    }
  }
  ax_hex_kernel<NQ, T, G, INMODE, OUTMODE><<<(unsigned)blocks, block, 0, s>>>(
      a.Nelements, a.elementList, a.g2l, a.ggeo, a.geoStride, a.wJ, a.wJStride, a.D, a.lambda,
      a.lambdaE, a.q, a.out, a.outScale);
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
  if (!std::is_same<T, float>::value && a.outScale != T(1))
    return set_error(LPG_ERR_UNSUPPORTED, "ax: a scaled assembly is provided for FP32 only");
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

template <int NQ>
static cudaError_t fp64_occupancy(int* per, bool dw, bool mass, int epb) {
  if (dw) {
    if constexpr (NQ == 8) {
      return dw7_classic()
                 ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(per, ax_hex_dw_kernel<8, true>, NQ * NQ * epb, 0)
                 : cudaOccupancyMaxActiveBlocksPerMultiprocessor(per, ax_hex_dw_lean_kernel<8, true>, NQ * NQ * epb,
                                                                 0);
    } else {
      return cudaOccupancyMaxActiveBlocksPerMultiprocessor(per, ax_hex_dw_kernel<NQ>, NQ * NQ * epb, 0);
    }
  }
  if (fp64_direct_override())
    return cudaOccupancyMaxActiveBlocksPerMultiprocessor(
        per, ax_hex_kernel<NQ, double, double, IN_GATHER, OUT_ASSEMBLE>, NQ * NQ * epb, 0);
  return mass ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(per, ax_hex_eo_kernel<NQ, true>, NQ * NQ * epb, 0)
              : cudaOccupancyMaxActiveBlocksPerMultiprocessor(per, ax_hex_eo_kernel<NQ, false>, NQ * NQ * epb, 0);
}

int ax_wave_elements(int N, bool dw, bool mass) {
  int dev = 0, sms = 0, per = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
    return 1;
  cudaError_t e = cudaErrorInvalidValue;
  int epb = 1;
  if (N == 7) {
    epb = elems_per_block<8>();
    e = fp64_occupancy<8>(&per, dw, mass, epb);
  } else if (N == 3) {
    epb = elems_per_block<4>();
    e = fp64_occupancy<4>(&per, dw, mass, epb);
  }
  if (e != cudaSuccess || per < 1) {
    cudaGetLastError();
    return 1;
  }
  return sms * per * epb;
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
