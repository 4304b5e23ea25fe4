// Fused inference of the learned smoother's MLP (896 -> 256 -> 256 -> 256 -> 512, GELU)
// on the 5th-generation tensor cores: tcgen05.mma (kind::f16, BF16 operands, FP32
// accumulators in tensor memory), operands staged by TMA (cp.async.bulk.tensor) with
// 128-byte swizzle, one CTA per SM walking 128-row tiles.
//
// Per tile the four layers run back to back without leaving the SM: layer 0 streams the
// tile's input rows and W0 in 64-wide K blocks through a 3-stage ring; the hidden
// activations go TMEM -> registers (bias, GELU, BF16) -> shared memory, where they are
// the A operand of the next layer; the output layer's two 256-column halves fill all
// 512 TMEM columns and are written to global memory in FP32. The weights (985 KB in
// BF16) stay L2-resident across tiles.
//
// Warp roles (320 threads): warp 0 lane 0 issues TMA loads, warp 1 owns TMEM and its
// lane 0 issues the MMAs, warps 2-9 run the epilogue (warp w reads TMEM lanes
// 32 (w % 4) .. +31, one row per thread, and half of the columns: warps 2-5 the first,
// 6-9 the second). Stages are handed over with mbarriers;
// every wait is bounded by %globaltimer, and on a timeout the CTA records an error code,
// waits (bounded) for its own copies and MMAs in flight, frees TMEM and returns.
#include <cuda.h>
#include <cudaTypedefs.h>

#include <atomic>
#include <cstdlib>
#include <cstring>
#include <mutex>

#include "lpg_common.cuh"
#include "lpg_internal.hpp"
#include "mlp.hpp"

namespace lpg {
namespace {

constexpr int TM = 128;                         // rows per tile (MMA M)
constexpr int TK = 64;                          // K block: 64 BF16 = one 128-byte swizzle row
constexpr int NSTAGE = 3;
constexpr int A_BYTES = TM * TK * 2;            // 16 KB
constexpr int B_BYTES = 256 * TK * 2;           // 32 KB (N = 256 rows of W^T)
constexpr int STAGE_BYTES = A_BYTES + B_BYTES;
constexpr int H_BYTES = TM * kMlpHidden * 2;    // hidden activations, 4 K blocks of 16 KB
constexpr int NBIAS = 3 * kMlpHidden + kMlpOut;
constexpr int L0_STEPS = kMlpIn / TK;           // 14
constexpr int LH_STEPS = kMlpHidden / TK;       // 4
constexpr int TILE_STEPS = L0_STEPS + 2 * LH_STEPS + 2 * LH_STEPS;
constexpr int NBAR = 2 * NSTAGE + 5;            // full[], empty[], acc, hready, tfree, drain, hold
constexpr int SMEM_BYTES = 1024 + NSTAGE * STAGE_BYTES + H_BYTES + NBIAS * 4 + NBAR * 8 + 16;
constexpr unsigned long long kWaitNs = 2000000000ull;  // 2 s per wait
constexpr int EPI_WARPS = 8, THREADS = 32 * (2 + EPI_WARPS);
static_assert(kMlpIn % TK == 0 && kMlpHidden == 256 && kMlpOut == 512, "layer shapes");

// instruction descriptor of tcgen05.mma kind::f16: D FP32 (bits 4-5 = 1), A and B BF16
// (bits 7-9, 10-12 = 1), both K-major, N >> 3 at bits 17-22, M >> 4 at bits 24-28
constexpr uint32_t kIdesc = (1u << 4) | (1u << 7) | (1u << 10) | ((256u >> 3) << 17) | ((uint32_t)(TM >> 4) << 24);

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ unsigned long long gtimer() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint32_t bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(bar) : "memory");
}
// waits until the phase of the given parity has completed; false after limitNs
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity, unsigned long long limitNs = kWaitNs) {
  const unsigned long long t0 = gtimer();
  while (true) {
    uint32_t done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(bar), "r"(parity)
        : "memory");
    if (done) return true;
    if (gtimer() - t0 > limitNs) return false;
  }
}

__device__ __forceinline__ void tma_load_2d(uint32_t dst, const CUtensorMap* map, uint32_t bar, int x, int y) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%3, %4}], [%2];" ::"r"(dst),
      "l"((uint64_t)map), "r"(bar), "r"(x), "r"(y)
      : "memory");
}

// shared-memory matrix descriptor: K-major operand in 128-byte swizzled rows, 8-row
// groups 1024 bytes apart (stride byte offset), descriptor version 1 (bit 46)
__device__ __forceinline__ uint64_t sw128_desc(uint32_t saddr) {
  uint64_t d = (uint64_t)((saddr >> 4) & 0x3FFFu);
  d |= (uint64_t)1 << 16;               // leading byte offset (unused with 128-byte swizzle)
  d |= (uint64_t)(1024 >> 4) << 32;     // stride byte offset
  d |= (uint64_t)1 << 46;
  d |= (uint64_t)2 << 61;               // 128-byte swizzle
  return d;
}

__device__ __forceinline__ void umma_bf16(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc, uint32_t accumulate) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(
          tmem_d),
      "l"(adesc), "l"(bdesc), "r"(kIdesc), "r"(accumulate));
}
__device__ __forceinline__ void umma_commit(uint32_t bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar) : "memory");
}
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// 32 consecutive FP32 columns of this thread's TMEM lane
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float* v) {
  uint32_t r[32];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
      "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
        "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]),
        "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]),
        "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int c = 0; c < 32; ++c) v[c] = __uint_as_float(r[c]);
}

// GELU (tanh form) with the hardware tanh approximation (relative error ~2^-11, below
// the BF16 rounding of the activations it produces)
__device__ __forceinline__ float gelu_approx(float z) {
  const float u = 0.7978845608028654f * (z + 0.044715f * z * z * z);
  float t;
  asm("tanh.approx.f32 %0, %1;" : "=f"(t) : "f"(u));
  return 0.5f * z * (1.0f + t);
}

__device__ __forceinline__ uint32_t pack_bf16(float a, float b) {
  const __nv_bfloat162 p = __floats2bfloat162_rn(a, b);
  return *reinterpret_cast<const uint32_t*>(&p);
}

// 8 x 8 transpose of 16-byte chunks within each group of 8 lanes (b = lane & 7): on entry
// lane b holds chunks 0..7 of its row b, on exit chunk m of lane b is chunk b of row m.
// Three butterfly stages (lane distance 4, 2, 1); at each, the lanes of a pair swap the
// chunks whose index bit differs from their lane bit.
__device__ __forceinline__ void transpose8_chunks(float4* c, const int b) {
  constexpr unsigned FULL = 0xffffffffu;
#pragma unroll
  for (int d = 4; d >= 1; d >>= 1) {
    const bool hi = (b & d) != 0;
#pragma unroll
    for (int k = 0; k < 8; ++k) {
      if (k & d) continue;
      const int k2 = k | d;
      const float4 send = hi ? c[k] : c[k2];
      float4 recv;
      recv.x = __shfl_xor_sync(FULL, send.x, d);
      recv.y = __shfl_xor_sync(FULL, send.y, d);
      recv.z = __shfl_xor_sync(FULL, send.z, d);
      recv.w = __shfl_xor_sync(FULL, send.w, d);
      if (hi) c[k] = recv;
      else c[k2] = recv;
    }
  }
}

struct TcMaps {
  CUtensorMap x, w[4];
};

__global__ void __launch_bounds__(THREADS, 1)
mlp_tc_kernel(const __grid_constant__ TcMaps maps, const float* __restrict__ b0, const float* __restrict__ b1,
              const float* __restrict__ b2, const float* __restrict__ b3, float* __restrict__ Y, const int64_t rows,
              const int ntiles, int* __restrict__ err, const unsigned long long holdNs) {
  extern __shared__ unsigned char smem_raw[];
  // 128-byte swizzled operands need 1024-byte aligned shared-memory offsets
  unsigned char* smem = smem_raw + ((1024u - (smem_u32(smem_raw) & 1023u)) & 1023u);
  unsigned char* stage0 = smem;
  unsigned char* hbuf = smem + NSTAGE * STAGE_BYTES;
  float* s_bias = reinterpret_cast<float*>(hbuf + H_BYTES);
  uint64_t* bars = reinterpret_cast<uint64_t*>(s_bias + NBIAS);
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(bars + NBAR);
  __shared__ volatile int s_abort;

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  auto full = [&](int s) { return smem_u32(&bars[s]); };
  auto empty = [&](int s) { return smem_u32(&bars[NSTAGE + s]); };
  const uint32_t accBar = smem_u32(&bars[2 * NSTAGE]), hBar = smem_u32(&bars[2 * NSTAGE + 1]);
  const uint32_t freeBar = smem_u32(&bars[2 * NSTAGE + 2]), drainBar = smem_u32(&bars[2 * NSTAGE + 3]);
  const uint32_t holdBar = smem_u32(&bars[2 * NSTAGE + 4]);

  if (threadIdx.x == 0) {
    for (int s = 0; s < NSTAGE; ++s) {
      mbar_init(full(s), 1);
      mbar_init(empty(s), 1);
    }
    mbar_init(accBar, 1);
    mbar_init(hBar, 32 * EPI_WARPS);
    mbar_init(freeBar, 32 * EPI_WARPS);
    mbar_init(drainBar, 1);
    mbar_init(holdBar, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    s_abort = 0;
  }
  for (int t = threadIdx.x; t < NBIAS; t += blockDim.x)
    s_bias[t] = t < 256 ? b0[t] : t < 512 ? b1[t - 256] : t < 768 ? b2[t - 512] : b3[t - 768];
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                 "r"(512)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tmem_slot;

  auto fail = [&](int code) {
    s_abort = 1;
    atomicCAS(err, 0, code);
  };
  // diagnostics hook (holdNs > 0): before any copy or MMA is issued, thread 0 waits on a
  // barrier that nothing signals until the limit runs out, then records the timeout as a
  // pipeline wait would; every role sees the abort flag before its first step and the CTA
  // frees its tensor memory and returns
  if (holdNs) {
    if (threadIdx.x == 0 && !mbar_wait(holdBar, 0, holdNs)) fail(8);
    __syncthreads();
  }
  // control flow stays uniform in every warp: lane 0 waits (or reads the abort flag) and
  // broadcasts the outcome, so whole warps take the same branches and reach the final
  // barrier together
  constexpr unsigned FULLMASK = 0xffffffffu;
  auto wait0 = [&](uint32_t bar, uint32_t parity) {
    int ok = 1;
    if (lane == 0) ok = mbar_wait(bar, parity) ? 1 : 0;
    return __shfl_sync(FULLMASK, ok, 0) != 0;
  };
  auto aborted = [&]() { return __shfl_sync(FULLMASK, lane == 0 ? (int)s_abort : 0, 0) != 0; };
  // every lane observes the barrier itself (the epilogue lanes then read TMEM)
  auto waitAll = [&](uint32_t bar, uint32_t parity) { return __all_sync(FULLMASK, mbar_wait(bar, parity) ? 1 : 0) != 0; };

  if (warp == 0) {
    // ------------------------------------------------------------ TMA producer (lane 0 issues)
    int64_t step = 0;
    for (int tile = blockIdx.x; tile < ntiles && !aborted(); tile += gridDim.x) {
      const int row0 = tile * TM;
      bool stop = false;
      for (int st = 0; st < TILE_STEPS; ++st, ++step) {
        const int s = (int)(step % NSTAGE);
        if (!wait0(empty(s), (uint32_t)(((step / NSTAGE) & 1) ^ 1))) {
          if (lane == 0) fail(1);
          stop = true;
          break;
        }
        if (lane == 0) {
          const uint32_t a = smem_u32(stage0 + s * STAGE_BYTES), b = a + A_BYTES;
          if (st < L0_STEPS) {
            mbar_expect_tx(full(s), A_BYTES + B_BYTES);
            tma_load_2d(a, &maps.x, full(s), st * TK, row0);
            tma_load_2d(b, &maps.w[0], full(s), st * TK, 0);
          } else {
            const int r = st - L0_STEPS;            // W1 (4 blocks), W2 (4), W3 half 0 (4), half 1 (4)
            const int layer = 1 + (r < 8 ? r / 4 : 2);
            const int kb = r % 4, nh = (r >= 12) ? 1 : 0;
            mbar_expect_tx(full(s), B_BYTES);
            tma_load_2d(b, &maps.w[layer], full(s), kb * TK, nh * 256);
          }
        }
        __syncwarp();
      }
      if (stop) break;
    }
    // every issued copy has landed before the CTA can exit (bounded)
    for (int64_t k = (step > NSTAGE ? step - NSTAGE : 0); k < step; ++k)
      if (!wait0(full((int)(k % NSTAGE)), (uint32_t)((k / NSTAGE) & 1)) && lane == 0) fail(2);
  } else if (warp == 1) {
    // ------------------------------------------------------------ MMA issuer (lane 0 issues)
    int64_t step = 0;
    uint32_t hcount = 0, tiles = 0;
    bool stop = false;
    for (int tile = blockIdx.x; tile < ntiles && !stop && !aborted(); tile += gridDim.x) {
      for (int layer = 0; layer < 4 && !stop; ++layer) {
        if (layer == 0 && tiles > 0 && !wait0(freeBar, (tiles - 1) & 1)) { if (lane == 0) fail(3); stop = true; break; }
        if (layer > 0 && !wait0(hBar, hcount++ & 1)) { if (lane == 0) fail(4); stop = true; break; }
        if (aborted()) { stop = true; break; }
        tc_fence_after();
        const int nsteps = layer == 0 ? L0_STEPS : (layer == 3 ? 2 * LH_STEPS : LH_STEPS);
        for (int st = 0; st < nsteps; ++st, ++step) {
          const int s = (int)(step % NSTAGE);
          if (!wait0(full(s), (uint32_t)((step / NSTAGE) & 1))) { if (lane == 0) fail(5); stop = true; break; }
          tc_fence_after();
          if (lane == 0) {
            const int kb = (layer == 3) ? (st % LH_STEPS) : st;
            const uint32_t bAddr = smem_u32(stage0 + s * STAGE_BYTES) + A_BYTES;
            const uint32_t aAddr =
                layer == 0 ? smem_u32(stage0 + s * STAGE_BYTES) : smem_u32(hbuf) + kb * (TM * TK * 2);
            const uint32_t dcol = layer == 1 ? 256u : (layer == 3 ? 256u * (uint32_t)(st / LH_STEPS) : 0u);
#pragma unroll
            for (int kk = 0; kk < TK / 16; ++kk)
              umma_bf16(tmem + dcol, sw128_desc(aAddr + kk * 32), sw128_desc(bAddr + kk * 32),
                        (kb > 0 || kk > 0) ? 1u : 0u);
            umma_commit(empty(s));   // the stage is free once these MMAs have read it
          }
          __syncwarp();
        }
        if (stop) break;
        if (lane == 0) umma_commit(accBar);   // this layer's accumulator is complete
        __syncwarp();
      }
      ++tiles;
    }
    // no MMA may still run when TMEM is released (bounded)
    if (lane == 0) umma_commit(drainBar);
    __syncwarp();
    if (!wait0(drainBar, 0) && lane == 0) fail(6);
  } else {
    // ------------------------------------------------------------ epilogue (warps 2-9)
    const int q = warp & 3;
    const int half = (warp - 2) / 4;  // which half of the columns this warp converts
    const int rloc = 32 * q + lane;   // the tile row this thread owns (TMEM lane)
    const uint32_t tlane = tmem + ((uint32_t)(32 * q) << 16);
    uint32_t lc = 0;
    bool stop = false;
    for (int tile = blockIdx.x; tile < ntiles && !stop && !aborted(); tile += gridDim.x) {
      const int64_t row = (int64_t)tile * TM + rloc;
      for (int layer = 0; layer < 4; ++layer) {
        if (!waitAll(accBar, lc++ & 1)) { if (lane == 0) fail(7); stop = true; break; }
        tc_fence_after();
        float v[32];
        if (layer < 3) {
          const uint32_t dcol = layer == 1 ? 256u : 0u;
          const float* bias = s_bias + layer * 256;
          for (int c0 = half * (kMlpHidden / 2); c0 < (half + 1) * (kMlpHidden / 2); c0 += 32) {
            tmem_ld32(tlane + dcol + c0, v);
            // columns c0..c0+31 -> K block c0/64, 16-byte chunks (c0%64)/8 .. +3 of row rloc,
            // placed with the 128-byte swizzle (chunk ^ (row & 7)) the MMA descriptor expects
            unsigned char* rowp = hbuf + (c0 / TK) * (TM * TK * 2) + rloc * 128;
#pragma unroll
            for (int t = 0; t < 4; ++t) {
              const int chunk = ((c0 % TK) / 8 + t) ^ (rloc & 7);
              const float* bb = bias + c0 + 8 * t;
              uint4 w;
              w.x = pack_bf16(gelu_approx(v[8 * t + 0] + bb[0]), gelu_approx(v[8 * t + 1] + bb[1]));
              w.y = pack_bf16(gelu_approx(v[8 * t + 2] + bb[2]), gelu_approx(v[8 * t + 3] + bb[3]));
              w.z = pack_bf16(gelu_approx(v[8 * t + 4] + bb[4]), gelu_approx(v[8 * t + 5] + bb[5]));
              w.w = pack_bf16(gelu_approx(v[8 * t + 6] + bb[6]), gelu_approx(v[8 * t + 7] + bb[7]));
              *reinterpret_cast<uint4*>(rowp + chunk * 16) = w;
            }
          }
          // the generic-proxy writes of H become visible to the tensor cores' async proxy
          asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
          tc_fence_before();
          mbar_arrive(hBar);
        } else {
          const float* bias = s_bias + 3 * 256;
          for (int c0 = half * (kMlpOut / 2); c0 < (half + 1) * (kMlpOut / 2); c0 += 32) {
            tmem_ld32(tlane + c0, v);
            if (row < rows) {
              float4* dst = reinterpret_cast<float4*>(Y + row * kMlpOut + c0);
#pragma unroll
              for (int t = 0; t < 8; ++t)
                dst[t] = make_float4(v[4 * t] + bias[c0 + 4 * t], v[4 * t + 1] + bias[c0 + 4 * t + 1],
                                     v[4 * t + 2] + bias[c0 + 4 * t + 2], v[4 * t + 3] + bias[c0 + 4 * t + 3]);
            }
          }
          tc_fence_before();
          mbar_arrive(freeBar);
        }
      }
    }
  }

  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  if (warp == 1)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(512) : "memory");
}

// ---------------------------------------------------------------- two tiles in flight
// The same network with two 128-row tiles per CTA in flight ("slots" 0 and 1, tiles
// alternating): slot s accumulates in TMEM columns [256 s, 256 s + 256) and keeps its
// hidden activations in its own shared-memory buffer, so one slot's epilogue (TMEM ->
// bias, GELU, BF16 -> shared memory, or the FP32 output) runs while the tensor cores work
// on the other slot. Work per tile is five jobs: layers 0, 1, 2 and the two 256-column
// halves of the output layer; the MMA warp issues them slot 0, slot 1, slot 0, ... per
// job kind, and each job waits until its slot's epilogue has drained the previous job
// (which also means that job's activations are in place). The TMA producer streams the
// K blocks of the same job sequence through a 2-stage ring (2 x 48 KB; the two 64 KB
// activation buffers take the rest of shared memory). Epilogue warps: 4 x EPI2_G per
// slot; warp w reads TMEM lanes 32 (w % 4) .. +31 and 256 / EPI2_G of the columns.
constexpr int NSTAGE2 = 2;
constexpr int EPI2_G = 2;
constexpr int EPI2_WARPS = 2 * 4 * EPI2_G;
constexpr int THREADS2 = 32 * (2 + EPI2_WARPS);
constexpr int NBAR2 = 2 * NSTAGE2 + 4 + 2;     // full[], empty[], accFull[2], epiDone[2], drain, hold
constexpr int SMEM2_BYTES = 1024 + NSTAGE2 * STAGE_BYTES + 2 * H_BYTES + NBAR2 * 8 + 16;
static_assert(SMEM2_BYTES <= 232448 - 64, "two-slot MLP kernel: shared memory");
constexpr int JOBS = 5;                        // L0, L1, L2, L3 columns 0-255, L3 columns 256-511

__global__ void __launch_bounds__(THREADS2, 1)
mlp_tc2_kernel(const __grid_constant__ TcMaps maps, const float* __restrict__ b0, const float* __restrict__ b1,
               const float* __restrict__ b2, const float* __restrict__ b3, float* __restrict__ Y, const int64_t rows,
               const int ntiles, int* __restrict__ err, const unsigned long long holdNs) {
  extern __shared__ unsigned char smem_raw[];
  unsigned char* smem = smem_raw + ((1024u - (smem_u32(smem_raw) & 1023u)) & 1023u);
  unsigned char* stage0 = smem;
  unsigned char* hbuf0 = smem + NSTAGE2 * STAGE_BYTES;             // slot 0 activations, slot 1 after
  uint64_t* bars = reinterpret_cast<uint64_t*>(hbuf0 + 2 * H_BYTES);
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(bars + NBAR2);
  __shared__ volatile int s_abort;

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  auto full = [&](int s) { return smem_u32(&bars[s]); };
  auto empty = [&](int s) { return smem_u32(&bars[NSTAGE2 + s]); };
  auto accFull = [&](int sl) { return smem_u32(&bars[2 * NSTAGE2 + sl]); };
  auto epiDone = [&](int sl) { return smem_u32(&bars[2 * NSTAGE2 + 2 + sl]); };
  const uint32_t drainBar = smem_u32(&bars[2 * NSTAGE2 + 4]), holdBar = smem_u32(&bars[2 * NSTAGE2 + 5]);

  if (threadIdx.x == 0) {
    for (int s = 0; s < NSTAGE2; ++s) {
      mbar_init(full(s), 1);
      mbar_init(empty(s), 1);
    }
    for (int sl = 0; sl < 2; ++sl) {
      mbar_init(accFull(sl), 1);
      mbar_init(epiDone(sl), 32 * 4 * EPI2_G);
    }
    mbar_init(drainBar, 1);
    mbar_init(holdBar, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    s_abort = 0;
  }
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                 "r"(512)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tmem_slot;

  auto fail = [&](int code) {
    s_abort = 1;
    atomicCAS(err, 0, code);
  };
  if (holdNs) {
    if (threadIdx.x == 0 && !mbar_wait(holdBar, 0, holdNs)) fail(8);
    __syncthreads();
  }
  constexpr unsigned FULLMASK = 0xffffffffu;
  auto wait0 = [&](uint32_t bar, uint32_t parity) {
    int ok = 1;
    if (lane == 0) ok = mbar_wait(bar, parity) ? 1 : 0;
    return __shfl_sync(FULLMASK, ok, 0) != 0;
  };
  auto aborted = [&]() { return __shfl_sync(FULLMASK, lane == 0 ? (int)s_abort : 0, 0) != 0; };
  auto waitAll = [&](uint32_t bar, uint32_t parity) { return __all_sync(FULLMASK, mbar_wait(bar, parity) ? 1 : 0) != 0; };
  // the CTA's tiles: j-th tile blockIdx.x + j gridDim.x, slot j & 1; pairs p = j / 2
  const int npairs = (ntiles - (int)blockIdx.x + 2 * (int)gridDim.x - 1) / (2 * (int)gridDim.x);
  auto tile_of = [&](int p, int sl) { return (int)blockIdx.x + (2 * p + sl) * (int)gridDim.x; };
  auto job_steps = [](int job) { return job == 0 ? L0_STEPS : LH_STEPS; };

  if (warp == 0) {
    // ------------------------------------------------------------ TMA producer (lane 0 issues)
    int64_t step = 0;
    bool stop = false;
    for (int p = 0; p < npairs && !stop && !aborted(); ++p)
      for (int job = 0; job < JOBS && !stop; ++job)
        for (int sl = 0; sl < 2 && !stop; ++sl) {
          const int tile = tile_of(p, sl);
          if (tile >= ntiles) continue;
          for (int st = 0; st < job_steps(job); ++st, ++step) {
            const int s = (int)(step % NSTAGE2);
            if (!wait0(empty(s), (uint32_t)(((step / NSTAGE2) & 1) ^ 1))) {
              if (lane == 0) fail(1);
              stop = true;
              break;
            }
            if (lane == 0) {
              const uint32_t a = smem_u32(stage0 + s * STAGE_BYTES), b = a + A_BYTES;
              if (job == 0) {
                mbar_expect_tx(full(s), A_BYTES + B_BYTES);
                tma_load_2d(a, &maps.x, full(s), st * TK, tile * TM);
                tma_load_2d(b, &maps.w[0], full(s), st * TK, 0);
              } else {
                const int layer = job < 3 ? job : 3, nh = job == 4 ? 1 : 0;
                mbar_expect_tx(full(s), B_BYTES);
                tma_load_2d(b, &maps.w[layer], full(s), st * TK, nh * 256);
              }
            }
            __syncwarp();
          }
        }
    for (int64_t k = (step > NSTAGE2 ? step - NSTAGE2 : 0); k < step; ++k)
      if (!wait0(full((int)(k % NSTAGE2)), (uint32_t)((k / NSTAGE2) & 1)) && lane == 0) fail(2);
  } else if (warp == 1) {
    // ------------------------------------------------------------ MMA issuer (lane 0 issues)
    int64_t step = 0;
    uint32_t njob[2] = {0u, 0u};
    bool stop = false;
    for (int p = 0; p < npairs && !stop && !aborted(); ++p)
      for (int job = 0; job < JOBS && !stop; ++job)
        for (int sl = 0; sl < 2 && !stop; ++sl) {
          if (tile_of(p, sl) >= ntiles) continue;
          // the slot's epilogue has drained its previous job (TMEM free, activations written)
          if (njob[sl] > 0 && !wait0(epiDone(sl), (njob[sl] - 1) & 1)) { if (lane == 0) fail(4); stop = true; break; }
          if (aborted()) { stop = true; break; }
          tc_fence_after();
          const uint32_t hAddr = smem_u32(hbuf0 + sl * H_BYTES);
          for (int st = 0; st < job_steps(job); ++st, ++step) {
            const int s = (int)(step % NSTAGE2);
            if (!wait0(full(s), (uint32_t)((step / NSTAGE2) & 1))) { if (lane == 0) fail(5); stop = true; break; }
            tc_fence_after();
            if (lane == 0) {
              const uint32_t bAddr = smem_u32(stage0 + s * STAGE_BYTES) + A_BYTES;
              const uint32_t aAddr = job == 0 ? smem_u32(stage0 + s * STAGE_BYTES) : hAddr + st * (TM * TK * 2);
#pragma unroll
              for (int kk = 0; kk < TK / 16; ++kk)
                umma_bf16(tmem + 256u * (uint32_t)sl, sw128_desc(aAddr + kk * 32), sw128_desc(bAddr + kk * 32),
                          (st > 0 || kk > 0) ? 1u : 0u);
              umma_commit(empty(s));
            }
            __syncwarp();
          }
          if (stop) break;
          if (lane == 0) umma_commit(accFull(sl));
          __syncwarp();
          ++njob[sl];
        }
    if (lane == 0) umma_commit(drainBar);
    __syncwarp();
    if (!wait0(drainBar, 0) && lane == 0) fail(6);
  } else {
    // ------------------------------------------------------------ epilogue (4 x EPI2_G warps per slot)
    const int u = warp - 2;
    const int sl = u / (4 * EPI2_G);
    const int g = (u % (4 * EPI2_G)) / 4;          // column group
    const int q = warp & 3;                         // TMEM lane quarter this warp may read
    const int rloc = 32 * q + lane;
    const uint32_t tlane = tmem + ((uint32_t)(32 * q) << 16) + 256u * (uint32_t)sl;
    unsigned char* hb = hbuf0 + sl * H_BYTES;
    constexpr int CW = 256 / EPI2_G;                // columns per warp
    uint32_t n = 0;
    bool stop = false;
    for (int p = 0; p < npairs && !stop && !aborted(); ++p) {
      const int tile = tile_of(p, sl);
      if (tile >= ntiles) break;
      const int64_t row = (int64_t)tile * TM + rloc;
      for (int job = 0; job < JOBS; ++job) {
        if (!waitAll(accFull(sl), n++ & 1)) { if (lane == 0) fail(7); stop = true; break; }
        tc_fence_after();
        float v[32];
        if (job < 3) {
          const float* bias = job == 0 ? b0 : job == 1 ? b1 : b2;
          for (int c0 = g * CW; c0 < (g + 1) * CW; c0 += 32) {
            tmem_ld32(tlane + c0, v);
            unsigned char* rowp = hb + (c0 / TK) * (TM * TK * 2) + rloc * 128;
#pragma unroll
            for (int t = 0; t < 4; ++t) {
              const int chunk = ((c0 % TK) / 8 + t) ^ (rloc & 7);
              const float4 bl = __ldg(reinterpret_cast<const float4*>(bias + c0 + 8 * t));
              const float4 bh = __ldg(reinterpret_cast<const float4*>(bias + c0 + 8 * t + 4));
              uint4 w;
              w.x = pack_bf16(gelu_approx(v[8 * t + 0] + bl.x), gelu_approx(v[8 * t + 1] + bl.y));
              w.y = pack_bf16(gelu_approx(v[8 * t + 2] + bl.z), gelu_approx(v[8 * t + 3] + bl.w));
              w.z = pack_bf16(gelu_approx(v[8 * t + 4] + bh.x), gelu_approx(v[8 * t + 5] + bh.y));
              w.w = pack_bf16(gelu_approx(v[8 * t + 6] + bh.z), gelu_approx(v[8 * t + 7] + bh.w));
              *reinterpret_cast<uint4*>(rowp + chunk * 16) = w;
            }
          }
          asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        } else {
          const int cbase = 256 * (job - 3);
          for (int c0 = g * CW; c0 < (g + 1) * CW; c0 += 32) {
            tmem_ld32(tlane + c0, v);
            float4 ch[8];
#pragma unroll
            for (int t = 0; t < 8; ++t) {
              const float4 bb = __ldg(reinterpret_cast<const float4*>(b3 + cbase + c0 + 4 * t));
              ch[t] = make_float4(v[4 * t] + bb.x, v[4 * t + 1] + bb.y, v[4 * t + 2] + bb.z, v[4 * t + 3] + bb.w);
            }
            // each lane holds 8 16-byte chunks of its own row; an 8 x 8 transpose within
            // groups of 8 lanes leaves lane b with chunk b of the group's 8 rows, so each
            // store below writes whole 128-byte row segments (4 per warp) instead of 32
            // separate 16-byte pieces
            transpose8_chunks(ch, lane & 7);
            const int64_t grow0 = (int64_t)tile * TM + 32 * q + 8 * (lane >> 3);
#pragma unroll
            for (int m = 0; m < 8; ++m)
              if (grow0 + m < rows)
                *reinterpret_cast<float4*>(Y + (grow0 + m) * kMlpOut + cbase + c0 + 4 * (lane & 7)) = ch[m];
          }
        }
        tc_fence_before();
        mbar_arrive(epiDone(sl));
      }
    }
  }

  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  if (warp == 1)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(512) : "memory");
}

PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
  });
  return fn;
}

// 2D BF16 map of a row-major [outer x inner] matrix, box [boxOuter x 64], 128-byte swizzle
int make_map(CUtensorMap* m, const void* base, uint64_t inner, uint64_t outer, uint32_t boxOuter) {
  auto fn = encode_fn();
  if (!fn) return set_error(LPG_ERR_CUDA, "cuTensorMapEncodeTiled is not available");
  const cuuint64_t dims[2] = {inner, outer};
  const cuuint64_t strides[1] = {inner * 2};
  const cuuint32_t box[2] = {(cuuint32_t)TK, boxOuter};
  const cuuint32_t estr[2] = {1, 1};
  const CUresult r = fn(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void*>(base), dims, strides, box, estr,
                        CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                        CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) return set_error(LPG_ERR_CUDA, "cuTensorMapEncodeTiled failed: " + std::to_string((int)r));
  return LPG_OK;
}

}  // namespace

std::atomic<unsigned long long> g_holdNs{0};

void mlp_tc_set_hold(unsigned long long ns) { g_holdNs.store(ns, std::memory_order_relaxed); }

int mlp_forward_tc(int64_t B, const __nv_bfloat16* X, const __nv_bfloat16* const Wt[4], const float* const bias[4],
                   float* Y, int* errFlag, cudaStream_t s) {
  if (B <= 0) return LPG_OK;
  if (B > (int64_t)INT32_MAX - TM) return set_error(LPG_ERR_INVALID, "mlp tc: too many rows");
  auto al16 = [](const void* p) { return ((uintptr_t)p & 15) == 0; };
  if (!al16(X) || !al16(Wt[0]) || !al16(Wt[1]) || !al16(Wt[2]) || !al16(Wt[3]) || !al16(Y))
    return set_error(LPG_ERR_INVALID, "mlp tc: operands must be 16-byte aligned");
  TcMaps maps;
  int rc;
  if ((rc = make_map(&maps.x, X, kMlpIn, (uint64_t)B, TM)) || (rc = make_map(&maps.w[0], Wt[0], kMlpIn, kMlpHidden, 256)) ||
      (rc = make_map(&maps.w[1], Wt[1], kMlpHidden, kMlpHidden, 256)) ||
      (rc = make_map(&maps.w[2], Wt[2], kMlpHidden, kMlpHidden, 256)) ||
      (rc = make_map(&maps.w[3], Wt[3], kMlpHidden, kMlpOut, 256)))
    return rc;
  if (!al16(bias[0]) || !al16(bias[1]) || !al16(bias[2]) || !al16(bias[3]))
    return set_error(LPG_ERR_INVALID, "mlp tc: biases must be 16-byte aligned");
  // LPG_MLP_TC=single (a tuning override): the one-tile-per-CTA kernel
  static const bool single = [] {
    const char* e = std::getenv("LPG_MLP_TC");
    return e && !std::strcmp(e, "single");
  }();
  static PerDeviceConfig perDevice;   // dynamic shared memory opt-in per device
  KernelConfig cfg;
  rc = perDevice.get(
      [&](int, KernelConfig&) {
        LPG_CUDA_TRY(cudaFuncSetAttribute(mlp_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM_BYTES));
        LPG_CUDA_TRY(cudaFuncSetAttribute(mlp_tc2_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM2_BYTES));
        return (int)LPG_OK;
      },
      &cfg);
  if (rc) return rc;
  const int ntiles = (int)((B + TM - 1) / TM);
  const int grid = ntiles < cfg.numSMs ? ntiles : cfg.numSMs;
  const unsigned long long hold = g_holdNs.load(std::memory_order_relaxed);
  if (single) {
    mlp_tc_kernel<<<grid, THREADS, SMEM_BYTES, s>>>(maps, bias[0], bias[1], bias[2], bias[3], Y, B, ntiles, errFlag,
                                                    hold);
    LPG_LAUNCH_CHECK("mlp_tc_kernel");
  } else {
    mlp_tc2_kernel<<<grid, THREADS2, SMEM2_BYTES, s>>>(maps, bias[0], bias[1], bias[2], bias[3], Y, B, ntiles, errFlag,
                                                       hold);
    LPG_LAUNCH_CHECK("mlp_tc2_kernel");
  }
  return LPG_OK;
}

}  // namespace lpg
