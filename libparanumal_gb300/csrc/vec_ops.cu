// Gather-scatter, streaming vector kernels and deterministic reductions.
//
// Reductions (linAlgInnerProd.okl / linAlgNorm2.okl / linAlgSum.okl and the fused
// linearSolverUpdatePCG.okl of the reference) run as two fixed-shape stages:
// a grid of at most kReducePartials CTAs writes one partial each, then one CTA
// sums the partials in a fixed tree. The result stays in device memory, so the
// caller decides when (and whether) to synchronise; the summation order depends
// only on N, which makes repeated runs bit-identical.
#include <algorithm>
#include <type_traits>

#include "lpg_common.cuh"
#include "lpg_internal.hpp"

namespace lpg {

static inline unsigned grid_for(int64_t n, int threads, int64_t cap) {
  int64_t b = (n + threads - 1) / threads;
  if (b > cap) b = cap;
  if (b < 1) b = 1;
  return (unsigned)b;
}
constexpr int64_t kStreamCap = 152 * 32;

// ---------------------------------------------------------------- ogs
template <typename T>
__global__ void gather_add_kernel(const int64_t Nlocal, const int32_t* __restrict__ g2l,
                                  const T* __restrict__ v, T* __restrict__ gv) {
  for (int64_t n = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; n < Nlocal;
       n += (int64_t)gridDim.x * blockDim.x) {
    const int32_t g = g2l[n];
    if (g >= 0) atomicAdd(gv + g, v[n]);
  }
}

template <typename T>
int gather_add(int64_t Nlocal, const int32_t* g2l, const T* v, T* gv, int64_t Nglobal, bool zero,
               cudaStream_t s) {
  if (zero && Nglobal > 0) LPG_CUDA_TRY(cudaMemsetAsync(gv, 0, sizeof(T) * Nglobal, s));
  if (Nlocal <= 0) return LPG_OK;
  gather_add_kernel<T><<<grid_for(Nlocal, 256, kStreamCap), 256, 0, s>>>(Nlocal, g2l, v, gv);
  LPG_LAUNCH_CHECK("gather_add_kernel");
  return LPG_OK;
}

template <typename T>
__global__ void gather_owner_kernel(const int64_t Ng, const int32_t* __restrict__ owner,
                                    const T* __restrict__ v, T* __restrict__ gv) {
  for (int64_t g = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; g < Ng;
       g += (int64_t)gridDim.x * blockDim.x)
    gv[g] = v[owner[g]];
}

template <typename T>
int gather_owner(int64_t Nglobal, const int32_t* owner, const T* v, T* gv, cudaStream_t s) {
  if (Nglobal <= 0) return LPG_OK;
  gather_owner_kernel<T><<<grid_for(Nglobal, 256, kStreamCap), 256, 0, s>>>(Nglobal, owner, v, gv);
  LPG_LAUNCH_CHECK("gather_owner_kernel");
  return LPG_OK;
}

template <typename T>
__global__ void scatter_kernel(const int64_t Nlocal, const int32_t* __restrict__ g2l,
                               const T* __restrict__ gv, T* __restrict__ v) {
  for (int64_t n = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; n < Nlocal;
       n += (int64_t)gridDim.x * blockDim.x) {
    const int32_t g = g2l[n];
    v[n] = (g >= 0) ? gv[g] : T(0);
  }
}

template <typename T>
int scatter(int64_t Nlocal, const int32_t* g2l, const T* gv, T* v, cudaStream_t s) {
  if (Nlocal <= 0) return LPG_OK;
  scatter_kernel<T><<<grid_for(Nlocal, 256, kStreamCap), 256, 0, s>>>(Nlocal, g2l, gv, v);
  LPG_LAUNCH_CHECK("scatter_kernel");
  return LPG_OK;
}

template int gather_add<double>(int64_t, const int32_t*, const double*, double*, int64_t, bool, cudaStream_t);
template int gather_add<float>(int64_t, const int32_t*, const float*, float*, int64_t, bool, cudaStream_t);
template int gather_owner<double>(int64_t, const int32_t*, const double*, double*, cudaStream_t);
template int gather_owner<float>(int64_t, const int32_t*, const float*, float*, cudaStream_t);
template int scatter<double>(int64_t, const int32_t*, const double*, double*, cudaStream_t);
template int scatter<float>(int64_t, const int32_t*, const float*, float*, cudaStream_t);

// ---------------------------------------------------------------- streaming
template <typename T>
__global__ void axpy_kernel(const int64_t N, const T a, const T* __restrict__ x, const T b,
                            T* __restrict__ y) {
  for (int64_t n = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; n < N; n += (int64_t)gridDim.x * blockDim.x)
    y[n] = (b != T(0)) ? a * x[n] + b * y[n] : a * x[n];
}
template <typename T>
int axpy(int64_t N, T a, const T* x, T b, T* y, cudaStream_t s) {
  if (N <= 0) return LPG_OK;
  axpy_kernel<T><<<grid_for(N, 256, kStreamCap), 256, 0, s>>>(N, a, x, b, y);
  LPG_LAUNCH_CHECK("axpy_kernel");
  return LPG_OK;
}

template <typename T>
__global__ void amxpy_kernel(const int64_t N, const T a, const T* __restrict__ x, const T* __restrict__ y,
                             const T b, T* __restrict__ z) {
  for (int64_t n = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; n < N; n += (int64_t)gridDim.x * blockDim.x)
    z[n] = (b != T(0)) ? a * x[n] * y[n] + b * z[n] : a * x[n] * y[n];
}
template <typename T>
int amxpy(int64_t N, T a, const T* x, const T* y, T b, T* z, cudaStream_t s) {
  if (N <= 0) return LPG_OK;
  amxpy_kernel<T><<<grid_for(N, 256, kStreamCap), 256, 0, s>>>(N, a, x, y, b, z);
  LPG_LAUNCH_CHECK("amxpy_kernel");
  return LPG_OK;
}

template <typename T>
__global__ void fill_kernel(const int64_t N, const T v, T* __restrict__ x) {
  for (int64_t n = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; n < N; n += (int64_t)gridDim.x * blockDim.x)
    x[n] = v;
}
template <typename T>
int fill(int64_t N, T v, T* x, cudaStream_t s) {
  if (N <= 0) return LPG_OK;
  fill_kernel<T><<<grid_for(N, 256, kStreamCap), 256, 0, s>>>(N, v, x);
  LPG_LAUNCH_CHECK("fill_kernel");
  return LPG_OK;
}

template <typename Tin, typename Tout>
__global__ void convert_kernel(const int64_t N, const Tin* __restrict__ x, Tout* __restrict__ y) {
  for (int64_t n = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; n < N; n += (int64_t)gridDim.x * blockDim.x)
    y[n] = (Tout)x[n];
}
template <>
__global__ void convert_kernel<double, __nv_bfloat16>(const int64_t N, const double* __restrict__ x,
                                                      __nv_bfloat16* __restrict__ y) {
  for (int64_t n = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; n < N; n += (int64_t)gridDim.x * blockDim.x)
    y[n] = __double2bfloat16(x[n]);
}
template <>
__global__ void convert_kernel<float, __nv_bfloat16>(const int64_t N, const float* __restrict__ x,
                                                     __nv_bfloat16* __restrict__ y) {
  for (int64_t n = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; n < N; n += (int64_t)gridDim.x * blockDim.x)
    y[n] = __float2bfloat16(x[n]);
}
template <typename Tin, typename Tout>
int convert(int64_t N, const Tin* x, Tout* y, cudaStream_t s) {
  if (N <= 0) return LPG_OK;
  convert_kernel<Tin, Tout><<<grid_for(N, 256, kStreamCap), 256, 0, s>>>(N, x, y);
  LPG_LAUNCH_CHECK("convert_kernel");
  return LPG_OK;
}

// x -> (hi, lo): hi = x rounded to FP32, lo = (x - hi) rounded to FP32 (setup-time split
// of FP64 data for the double-word operator)
__global__ void split_to_float2_kernel(const int64_t N, const double* __restrict__ x, float2* __restrict__ y) {
  for (int64_t n = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; n < N; n += (int64_t)gridDim.x * blockDim.x) {
    const double v = x[n];
    const float hi = __double2float_rn(v);
    y[n] = make_float2(hi, __double2float_rn(v - (double)hi));
  }
}
int split_to_float2(int64_t n, const double* x, float2* y, cudaStream_t s) {
  if (n <= 0) return LPG_OK;
  split_to_float2_kernel<<<grid_for(n, 256, kStreamCap), 256, 0, s>>>(n, x, y);
  LPG_LAUNCH_CHECK("split_to_float2_kernel");
  return LPG_OK;
}

__global__ void inverse_kernel(const int64_t N, const double* __restrict__ x, double* __restrict__ y,
                               const int guard) {
  for (int64_t n = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; n < N; n += (int64_t)gridDim.x * blockDim.x) {
    const double v = x[n];
    y[n] = guard ? ((v > 0.0) ? 1.0 / v : 0.0) : 1.0 / v;
  }
}
int inverse_in_place(int64_t N, double* x, cudaStream_t s) {
  if (N <= 0) return LPG_OK;
  inverse_kernel<<<grid_for(N, 256, kStreamCap), 256, 0, s>>>(N, x, x, 1);
  LPG_LAUNCH_CHECK("inverse_kernel");
  return LPG_OK;
}
int inverse_f64(int64_t N, const double* x, double* y, cudaStream_t s) {
  if (N <= 0) return LPG_OK;
  inverse_kernel<<<grid_for(N, 256, kStreamCap), 256, 0, s>>>(N, x, y, 0);
  LPG_LAUNCH_CHECK("inverse_kernel");
  return LPG_OK;
}

__global__ void mult_to_weight_kernel(const int64_t n, const int32_t* __restrict__ m, double* __restrict__ w) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    w[i] = (m[i] > 0) ? 1.0 / (double)m[i] : 0.0;
}
int multiplicity_to_weight(int64_t N, const int32_t* mult, double* w, cudaStream_t s) {
  if (N <= 0) return LPG_OK;
  mult_to_weight_kernel<<<grid_for(N, 256, kStreamCap), 256, 0, s>>>(N, mult, w);
  LPG_LAUNCH_CHECK("mult_to_weight_kernel");
  return LPG_OK;
}

template int axpy<double>(int64_t, double, const double*, double, double*, cudaStream_t);
template int axpy<float>(int64_t, float, const float*, float, float*, cudaStream_t);
template int amxpy<double>(int64_t, double, const double*, const double*, double, double*, cudaStream_t);
template int amxpy<float>(int64_t, float, const float*, const float*, float, float*, cudaStream_t);
template int fill<double>(int64_t, double, double*, cudaStream_t);
template int fill<float>(int64_t, float, float*, cudaStream_t);
template int convert<double, float>(int64_t, const double*, float*, cudaStream_t);
template int convert<float, double>(int64_t, const float*, double*, cudaStream_t);
template int convert<double, __nv_bfloat16>(int64_t, const double*, __nv_bfloat16*, cudaStream_t);
template int convert<float, __nv_bfloat16>(int64_t, const float*, __nv_bfloat16*, cudaStream_t);

// ---------------------------------------------------------------- reductions
constexpr int kRedThreads = 512;

__device__ __forceinline__ double block_sum(double v) {
  __shared__ double s_w[32];
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  __syncthreads();
  if (lane == 0) s_w[warp] = v;
  __syncthreads();
  v = (threadIdx.x < (blockDim.x >> 5)) ? s_w[lane] : 0.0;
  if (warp == 0)
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  return v;
}

// Stage 1 variants
enum { RED_DOT = 0, RED_SUM = 1, RED_DOT32 = 2 };

template <int KIND>
__global__ void __launch_bounds__(kRedThreads)
reduce_stage1(const int64_t N, const void* __restrict__ xv, const void* __restrict__ yv,
              double* __restrict__ partials) {
  double acc = 0;
  if (KIND == RED_DOT32) {
    // FP32 products summed per thread with Kahan compensation on the FP32 pipe (GB300's
    // FP64 pipe would bound this loop); one conversion per thread, then FP64 across threads
    float s = 0.f, c = 0.f;
    for (int64_t n = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; n < N; n += (int64_t)gridDim.x * blockDim.x) {
      const float y = ((const float*)xv)[n] * ((const float*)yv)[n] - c;
      const float t = s + y;
      c = (t - s) - y;
      s = t;
    }
    acc = (double)s - (double)c;
  } else {
    for (int64_t n = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; n < N; n += (int64_t)gridDim.x * blockDim.x) {
      if (KIND == RED_DOT) acc += ((const double*)xv)[n] * ((const double*)yv)[n];
      else acc += ((const double*)xv)[n];
    }
  }
  acc = block_sum(acc);
  if (threadIdx.x == 0) partials[blockIdx.x] = acc;
}

__global__ void __launch_bounds__(kRedThreads)
reduce_stage2(const int nparts, const double* __restrict__ partials, double* __restrict__ out, const int root = 0) {
  double acc = 0;
  for (int i = threadIdx.x; i < nparts; i += blockDim.x) acc += partials[i];
  acc = block_sum(acc);
  if (threadIdx.x == 0) *out = root ? sqrt(acc) : acc;
}

static inline int red_blocks(int64_t N) {
  int64_t b = (N + kRedThreads * 4 - 1) / (kRedThreads * 4);
  if (b > kReducePartials) b = kReducePartials;
  if (b < 1) b = 1;
  return (int)b;
}

int reduction_blocks(int64_t N) { return red_blocks(N); }

template <int KIND>
static int reduce(int64_t N, const void* x, const void* y, double* out, double* partials, cudaStream_t s) {
  const int nb = red_blocks(N);
  reduce_stage1<KIND><<<nb, kRedThreads, 0, s>>>(N, x, y, partials);
  LPG_LAUNCH_CHECK("reduce_stage1");
  reduce_stage2<<<1, kRedThreads, 0, s>>>(nb, partials, out);
  LPG_LAUNCH_CHECK("reduce_stage2");
  return LPG_OK;
}

int dot(int64_t N, const double* x, const double* y, double* out, double* partials, cudaStream_t s) {
  return reduce<RED_DOT>(N, x, y, out, partials, s);
}
int dot_f32(int64_t N, const float* x, const float* y, double* out, double* partials, cudaStream_t s) {
  return reduce<RED_DOT32>(N, x, y, out, partials, s);
}
int sum(int64_t N, const double* x, double* out, double* partials, cudaStream_t s) {
  return reduce<RED_SUM>(N, x, nullptr, out, partials, s);
}
int norm2(int64_t N, const double* x, double* out, double* partials, cudaStream_t s) {
  const int nb = red_blocks(N);
  reduce_stage1<RED_DOT><<<nb, kRedThreads, 0, s>>>(N, x, x, partials);
  LPG_LAUNCH_CHECK("reduce_stage1");
  reduce_stage2<<<1, kRedThreads, 0, s>>>(nb, partials, out, 1);
  LPG_LAUNCH_CHECK("reduce_stage2");
  return LPG_OK;
}

// two inner products of x in one pass: out[0] = x.y, out[1] = x.z. FP32 data: products
// summed per thread in FP32 with Kahan compensation (as dot_f32), FP64 across threads.
template <typename T>
__global__ void __launch_bounds__(kRedThreads)
dot2_stage1(const int64_t N, const T* __restrict__ x, const T* __restrict__ y, const T* __restrict__ z,
            double* __restrict__ partials) {
  double a, b;
  if constexpr (std::is_same<T, float>::value) {
    float sa = 0.f, ca = 0.f, sb = 0.f, cb = 0.f;
    for (int64_t n = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; n < N; n += (int64_t)gridDim.x * blockDim.x) {
      const float xv = x[n];
      const float ya = xv * y[n] - ca, yb = xv * z[n] - cb;
      const float ta = sa + ya, tb = sb + yb;
      ca = (ta - sa) - ya;
      cb = (tb - sb) - yb;
      sa = ta;
      sb = tb;
    }
    a = (double)sa - (double)ca;
    b = (double)sb - (double)cb;
  } else {
    a = 0;
    b = 0;
    for (int64_t n = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; n < N; n += (int64_t)gridDim.x * blockDim.x) {
      a += x[n] * y[n];
      b += x[n] * z[n];
    }
  }
  a = block_sum(a);
  b = block_sum(b);
  if (threadIdx.x == 0) {
    partials[blockIdx.x] = a;
    partials[gridDim.x + blockIdx.x] = b;
  }
}
__global__ void __launch_bounds__(kRedThreads)
dot2_stage2(const int nparts, const double* __restrict__ partials, double* __restrict__ out) {
  double a = 0, b = 0;
  for (int i = threadIdx.x; i < nparts; i += blockDim.x) {
    a += partials[i];
    b += partials[nparts + i];
  }
  a = block_sum(a);
  b = block_sum(b);
  if (threadIdx.x == 0) {
    out[0] = a;
    out[1] = b;
  }
}
template <typename T>
int dot2(int64_t N, const T* x, const T* y, const T* z, double* out2, double* partials, cudaStream_t s) {
  const int nb = std::min(red_blocks(N), kReducePartials / 2);
  dot2_stage1<T><<<nb, kRedThreads, 0, s>>>(N, x, y, z, partials);
  LPG_LAUNCH_CHECK("dot2_stage1");
  dot2_stage2<<<1, kRedThreads, 0, s>>>(nb, partials, out2);
  LPG_LAUNCH_CHECK("dot2_stage2");
  return LPG_OK;
}
template int dot2<double>(int64_t, const double*, const double*, const double*, double*, double*, cudaStream_t);
template int dot2<float>(int64_t, const float*, const float*, const float*, double*, double*, cudaStream_t);

// FPCG with an FP32 preconditioner output z: out[0] = r.z, out[1] = z.Ap with z widened
// exactly to FP64 and FP64 products; and p = z + beta p. z is read as FP32 and never
// stored as FP64.
__global__ void __launch_bounds__(kRedThreads)
dot2_mixed_stage1(const int64_t N, const float* __restrict__ z, const double* __restrict__ r,
                  const double* __restrict__ Ap, double* __restrict__ partials) {
  double a = 0, b = 0;
  for (int64_t n = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; n < N; n += (int64_t)gridDim.x * blockDim.x) {
    const double zn = (double)z[n];
    a += r[n] * zn;
    b += zn * Ap[n];
  }
  a = block_sum(a);
  b = block_sum(b);
  if (threadIdx.x == 0) {
    partials[blockIdx.x] = a;
    partials[gridDim.x + blockIdx.x] = b;
  }
}
int dot2_mixed(int64_t N, const float* z, const double* r, const double* Ap, double* out2, double* partials,
               cudaStream_t s) {
  const int nb = std::min(red_blocks(N), kReducePartials / 2);
  dot2_mixed_stage1<<<nb, kRedThreads, 0, s>>>(N, z, r, Ap, partials);
  LPG_LAUNCH_CHECK("dot2_mixed_stage1");
  dot2_stage2<<<1, kRedThreads, 0, s>>>(nb, partials, out2);
  LPG_LAUNCH_CHECK("dot2_stage2");
  return LPG_OK;
}
__global__ void direction_mixed_kernel(const int64_t N, const float* __restrict__ z, const double beta,
                                       double* __restrict__ p) {
  for (int64_t n = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; n < N; n += (int64_t)gridDim.x * blockDim.x)
    p[n] = (double)z[n] + beta * p[n];
}
int direction_mixed(int64_t N, const float* z, double beta, double* p, cudaStream_t s) {
  if (N <= 0) return LPG_OK;
  direction_mixed_kernel<<<grid_for(N, 256, kStreamCap), 256, 0, s>>>(N, z, beta, p);
  LPG_LAUNCH_CHECK("direction_mixed_kernel");
  return LPG_OK;
}

// x += a p; r -= a q
template <typename T>
__global__ void update2_kernel(const int64_t N, const T a, const T* __restrict__ p, const T* __restrict__ q,
                               T* __restrict__ x, T* __restrict__ r) {
  for (int64_t n = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; n < N; n += (int64_t)gridDim.x * blockDim.x) {
    x[n] += a * p[n];
    r[n] -= a * q[n];
  }
}
template <typename T>
int update2(int64_t N, T a, const T* p, const T* q, T* x, T* r, cudaStream_t s) {
  if (N <= 0) return LPG_OK;
  update2_kernel<T><<<grid_for(N, 256, kStreamCap), 256, 0, s>>>(N, a, p, q, x, r);
  LPG_LAUNCH_CHECK("update2_kernel");
  return LPG_OK;
}
template int update2<double>(int64_t, double, const double*, const double*, double*, double*, cudaStream_t);
template int update2<float>(int64_t, float, const float*, const float*, float*, float*, cudaStream_t);

// the same with the step w = num/den read from device memory (sc[0], sc[1]); w = 0 when
// den <= 0 or either is not finite (no host round trip for the step length)
template <typename T>
__global__ void update2_dev_kernel(const int64_t N, const double* __restrict__ sc, const T* __restrict__ p,
                                   const T* __restrict__ q, T* __restrict__ x, T* __restrict__ r) {
  const double num = sc[0], den = sc[1];
  const T a = (T)((den > 0 && isfinite(num) && isfinite(den)) ? num / den : 0.0);
  for (int64_t n = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; n < N; n += (int64_t)gridDim.x * blockDim.x) {
    x[n] += a * p[n];
    r[n] -= a * q[n];
  }
}
template <typename T>
int update2_dev(int64_t N, const double* sc, const T* p, const T* q, T* x, T* r, cudaStream_t s) {
  if (N <= 0) return LPG_OK;
  update2_dev_kernel<T><<<grid_for(N, 256, kStreamCap), 256, 0, s>>>(N, sc, p, q, x, r);
  LPG_LAUNCH_CHECK("update2_dev_kernel");
  return LPG_OK;
}
template int update2_dev<double>(int64_t, const double*, const double*, const double*, double*, double*, cudaStream_t);
template int update2_dev<float>(int64_t, const double*, const float*, const float*, float*, float*, cudaStream_t);

// halo exchange halves (the ogs extract kernel, libs/ogs/okl/ogsKernels.okl:167-): buf[i] =
// v[idx[i]], and v[idx[i]] += buf[i] (the indices of one list are distinct)
__global__ void halo_pack_kernel(const int64_t n, const int32_t* __restrict__ idx, const double* __restrict__ v,
                                 double* __restrict__ buf) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    buf[i] = v[idx[i]];
}
__global__ void halo_unpack_add_kernel(const int64_t n, const int32_t* __restrict__ idx,
                                       const double* __restrict__ buf, double* __restrict__ v) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    v[idx[i]] += buf[i];
}
int halo_pack(int64_t n, const int32_t* idx, const double* v, double* buf, cudaStream_t s) {
  if (n <= 0) return LPG_OK;
  halo_pack_kernel<<<grid_for(n, 256, kStreamCap), 256, 0, s>>>(n, idx, v, buf);
  LPG_LAUNCH_CHECK("halo_pack_kernel");
  return LPG_OK;
}
int halo_unpack_add(int64_t n, const int32_t* idx, const double* buf, double* v, cudaStream_t s) {
  if (n <= 0) return LPG_OK;
  halo_unpack_add_kernel<<<grid_for(n, 256, kStreamCap), 256, 0, s>>>(n, idx, buf, v);
  LPG_LAUNCH_CHECK("halo_unpack_add_kernel");
  return LPG_OK;
}

__global__ void __launch_bounds__(kRedThreads)
pcg_update_stage1(const int64_t N, const double alpha, const double* __restrict__ p,
                  const double* __restrict__ Ap, double* __restrict__ x, double* __restrict__ r,
                  double* __restrict__ partials) {
  double acc = 0;
  for (int64_t n = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; n < N; n += (int64_t)gridDim.x * blockDim.x) {
    x[n] += alpha * p[n];
    const double rn = r[n] - alpha * Ap[n];
    r[n] = rn;
    acc += rn * rn;
  }
  acc = block_sum(acc);
  if (threadIdx.x == 0) partials[blockIdx.x] = acc;
}

int pcg_update(int64_t N, double alpha, const double* p, const double* Ap, double* x, double* r,
               double* out, double* partials, cudaStream_t s) {
  const int nb = red_blocks(N);
  pcg_update_stage1<<<nb, kRedThreads, 0, s>>>(N, alpha, p, Ap, x, r, partials);
  LPG_LAUNCH_CHECK("pcg_update_stage1");
  reduce_stage2<<<1, kRedThreads, 0, s>>>(nb, partials, out);
  LPG_LAUNCH_CHECK("reduce_stage2");
  return LPG_OK;
}

__global__ void add_scalar_kernel(const int64_t N, const double* __restrict__ sdev, const double scale,
                                  double* __restrict__ x) {
  const double v = (*sdev) * scale;
  for (int64_t n = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; n < N; n += (int64_t)gridDim.x * blockDim.x)
    x[n] += v;
}
int add_scalar(int64_t N, const double* scalarDev, double scale, double* x, cudaStream_t s) {
  if (N <= 0) return LPG_OK;
  add_scalar_kernel<<<grid_for(N, 256, kStreamCap), 256, 0, s>>>(N, scalarDev, scale, x);
  LPG_LAUNCH_CHECK("add_scalar_kernel");
  return LPG_OK;
}

// ---------------------------------------------------------------- Chebyshev
// res -= invDiag .* Ad ;  d = a d + b res   (one pass of the level smoother loop)
template <typename T>
__global__ void cheb_update_kernel(const int64_t N, const T* __restrict__ invDiag, const T* __restrict__ Ad,
                                   T* __restrict__ res, T* __restrict__ d, const T a, const T b) {
  for (int64_t n = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; n < N; n += (int64_t)gridDim.x * blockDim.x) {
    const T rn = res[n] - invDiag[n] * Ad[n];
    res[n] = rn;
    d[n] = b * rn + a * d[n];
  }
}
template <typename T>
int cheb_update(int64_t N, const T* invDiag, const T* Ad, T* res, T* d, T a, T b, cudaStream_t s) {
  if (N <= 0) return LPG_OK;
  cheb_update_kernel<T><<<grid_for(N, 256, kStreamCap), 256, 0, s>>>(N, invDiag, Ad, res, d, a, b);
  LPG_LAUNCH_CHECK("cheb_update_kernel");
  return LPG_OK;
}
template int cheb_update<double>(int64_t, const double*, const double*, double*, double*, double, double, cudaStream_t);
template int cheb_update<float>(int64_t, const float*, const float*, float*, float*, float, float, cudaStream_t);

// Fused Chebyshev passes (the same operations as the separate vector kernels, one sweep):
// start: res = invDiag .* (r - Ax) (Ax == nullptr: res = invDiag .* r); d = invTheta res;
//        x = d (xIsZero) or x += d
// step:  res -= invDiag .* Ad; d = a d + b res; x += d
template <typename T>
__global__ void cheb_start_kernel(const int64_t N, const T* __restrict__ invDiag, const T* __restrict__ r,
                                  const T* Ax, T* res, T* __restrict__ d, T* __restrict__ x, const T invTheta,
                                  const int xIsZero) {   // Ax may alias res
  for (int64_t n = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; n < N; n += (int64_t)gridDim.x * blockDim.x) {
    const T rn = Ax ? invDiag[n] * (r[n] - Ax[n]) : invDiag[n] * r[n];
    res[n] = rn;
    const T dn = invTheta * rn;
    d[n] = dn;
    x[n] = xIsZero ? dn : x[n] + dn;
  }
}
// LAST: the smoother's final step, whose res and d nobody reads again: only x is written
template <typename T, bool LAST>
__global__ void cheb_step_kernel(const int64_t N, const T* __restrict__ invDiag, const T* __restrict__ Ad,
                                 T* __restrict__ res, T* __restrict__ d, T* __restrict__ x, const T a, const T b) {
  for (int64_t n = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; n < N; n += (int64_t)gridDim.x * blockDim.x) {
    const T rn = res[n] - invDiag[n] * Ad[n];
    const T dn = b * rn + a * d[n];
    if (!LAST) {
      res[n] = rn;
      d[n] = dn;
    }
    x[n] = x[n] + dn;
  }
}
template <typename T>
int cheb_start(int64_t N, const T* invDiag, const T* r, const T* Ax, T* res, T* d, T* x, T invTheta, bool xIsZero,
               cudaStream_t s) {
  if (N <= 0) return LPG_OK;
  cheb_start_kernel<T><<<grid_for(N, 256, kStreamCap), 256, 0, s>>>(N, invDiag, r, Ax, res, d, x, invTheta,
                                                                     xIsZero ? 1 : 0);
  LPG_LAUNCH_CHECK("cheb_start_kernel");
  return LPG_OK;
}
template <typename T>
int cheb_step(int64_t N, const T* invDiag, const T* Ad, T* res, T* d, T* x, T a, T b, cudaStream_t s, bool last) {
  if (N <= 0) return LPG_OK;
  if (last) cheb_step_kernel<T, true><<<grid_for(N, 256, kStreamCap), 256, 0, s>>>(N, invDiag, Ad, res, d, x, a, b);
  else cheb_step_kernel<T, false><<<grid_for(N, 256, kStreamCap), 256, 0, s>>>(N, invDiag, Ad, res, d, x, a, b);
  LPG_LAUNCH_CHECK("cheb_step_kernel");
  return LPG_OK;
}
// Chebyshev passes on the unscaled residual u = r - A x, which the operator updates in
// place (u -= A d): start u = r - Ax (or r), d = invTheta invDiag u, x = d or x += d; step
// d = a d + b invDiag u, x += d (last: d not written)
template <typename T>
__global__ void cheb_start_u_kernel(const int64_t N, const T* __restrict__ invDiag, const T* __restrict__ r,
                                    const T* Ax, T* u, T* __restrict__ d, T* __restrict__ x, const T invTheta,
                                    const int xIsZero) {   // Ax may alias u
  for (int64_t n = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; n < N; n += (int64_t)gridDim.x * blockDim.x) {
    const T un = Ax ? r[n] - Ax[n] : r[n];
    u[n] = un;
    const T dn = invTheta * (invDiag[n] * un);
    d[n] = dn;
    x[n] = xIsZero ? dn : x[n] + dn;
  }
}
template <typename T, bool LAST>
__global__ void cheb_step_u_kernel(const int64_t N, const T* __restrict__ invDiag, const T* __restrict__ u,
                                   T* __restrict__ d, T* __restrict__ x, const T a, const T b) {
  for (int64_t n = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; n < N; n += (int64_t)gridDim.x * blockDim.x) {
    const T dn = b * (invDiag[n] * u[n]) + a * d[n];
    if (!LAST) d[n] = dn;
    x[n] = x[n] + dn;
  }
}
template <typename T>
int cheb_start_u(int64_t N, const T* invDiag, const T* r, const T* Ax, T* u, T* d, T* x, T invTheta, bool xIsZero,
                 cudaStream_t s) {
  if (N <= 0) return LPG_OK;
  cheb_start_u_kernel<T><<<grid_for(N, 256, kStreamCap), 256, 0, s>>>(N, invDiag, r, Ax, u, d, x, invTheta,
                                                                       xIsZero ? 1 : 0);
  LPG_LAUNCH_CHECK("cheb_start_u_kernel");
  return LPG_OK;
}
template <typename T>
int cheb_step_u(int64_t N, const T* invDiag, const T* u, T* d, T* x, T a, T b, cudaStream_t s, bool last) {
  if (N <= 0) return LPG_OK;
  if (last) cheb_step_u_kernel<T, true><<<grid_for(N, 256, kStreamCap), 256, 0, s>>>(N, invDiag, u, d, x, a, b);
  else cheb_step_u_kernel<T, false><<<grid_for(N, 256, kStreamCap), 256, 0, s>>>(N, invDiag, u, d, x, a, b);
  LPG_LAUNCH_CHECK("cheb_step_u_kernel");
  return LPG_OK;
}
template int cheb_start_u<float>(int64_t, const float*, const float*, const float*, float*, float*, float*, float, bool,
                                 cudaStream_t);
template int cheb_step_u<float>(int64_t, const float*, const float*, float*, float*, float, float, cudaStream_t, bool);

template int cheb_start<double>(int64_t, const double*, const double*, const double*, double*, double*, double*, double,
                                bool, cudaStream_t);
template int cheb_start<float>(int64_t, const float*, const float*, const float*, float*, float*, float*, float, bool,
                               cudaStream_t);
template int cheb_step<double>(int64_t, const double*, const double*, double*, double*, double*, double, double,
                               cudaStream_t, bool);
template int cheb_step<float>(int64_t, const float*, const float*, float*, float*, float*, float, float, cudaStream_t,
                              bool);

// ---------------------------------------------------------------- initial-guess history
// Kernels of the initial-guess strategies (libs/linearSolver/okl/igBasisInnerProducts.okl,
// igReconstruct.okl, igDropQRFirstColumn.okl, igExtrap.okl). History vectors are stored
// contiguously, column m at Q + m N.

// The history kernels are instantiated for a compile-time bound K on the history dimension
// (4, 8, 16 or 32, the smallest that holds k) and unrolled over it: the per-column
// accumulators stay in registers and the k column loads of a node are independent, so each
// thread keeps k loads in flight.
template <typename F>
static int history_dispatch(int k, F&& f) {
  if (k <= 4) return f(std::integral_constant<int, 4>{});
  if (k <= 8) return f(std::integral_constant<int, 8>{});
  if (k <= 16) return f(std::integral_constant<int, 16>{});
  return f(std::integral_constant<int, kMaxHistory>{});
}

// partials[m * nb + b] = block b's share of Q_m . x for m < k (host sums the nb entries)
template <int K>
__global__ void __launch_bounds__(256)
multi_dot_kernel(const int64_t N, const int k, const double* __restrict__ x, const double* __restrict__ Q,
                 double* __restrict__ partials) {
  __shared__ double s_w[8];
  double acc[K];
#pragma unroll
  for (int m = 0; m < K; ++m) acc[m] = 0;
  for (int64_t n = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; n < N; n += (int64_t)gridDim.x * blockDim.x) {
    const double xn = x[n];
#pragma unroll
    for (int m = 0; m < K; ++m)
      if (m < k) acc[m] += Q[(int64_t)m * N + n] * xn;
  }
#pragma unroll
  for (int m = 0; m < K; ++m) {
    if (m < k) {
      double v = acc[m];
      for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
      __syncthreads();
      if ((threadIdx.x & 31) == 0) s_w[threadIdx.x >> 5] = v;
      __syncthreads();
      if (threadIdx.x == 0) {
        double t = 0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += s_w[w];
        partials[(int64_t)m * gridDim.x + blockIdx.x] = t;
      }
    }
  }
}
int multi_dot(int64_t N, int k, const double* x, const double* Q, double* partials, int* nblocks, cudaStream_t s) {
  if (k < 0 || k > kMaxHistory) return set_error(LPG_ERR_INVALID, "multi_dot: history dimension out of range");
  const int nb = (int)std::max<int64_t>(1, std::min<int64_t>((N + 255) / 256, kMultiDotBlocks));
  *nblocks = nb;
  if (k == 0) return LPG_OK;
  return history_dispatch(k, [&](auto kb) {
    multi_dot_kernel<decltype(kb)::value><<<nb, 256, 0, s>>>(N, k, x, Q, partials);
    LPG_LAUNCH_CHECK("multi_dot_kernel");
    return LPG_OK;
  });
}

// out = u + beta * sum_m c[m] Q_m  (out may be u)
template <int K>
__global__ void combine_kernel(const int64_t N, const int k, const double* u, const double beta, const HistCoeffs c,
                               const double* __restrict__ Q, double* out) {
  for (int64_t n = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; n < N; n += (int64_t)gridDim.x * blockDim.x) {
    double q[K];
#pragma unroll
    for (int m = 0; m < K; ++m) q[m] = m < k ? Q[(int64_t)m * N + n] : 0.0;
    double r = u ? u[n] : 0.0;
#pragma unroll
    for (int m = 0; m < K; ++m)
      if (m < k) r += beta * c.v[m] * q[m];
    out[n] = r;
  }
}
int combine(int64_t N, int k, const double* u, double beta, const HistCoeffs& c, const double* Q, double* out,
            cudaStream_t s) {
  if (N <= 0) return LPG_OK;
  if (k < 0 || k > kMaxHistory) return set_error(LPG_ERR_INVALID, "combine: history dimension out of range");
  return history_dispatch(k, [&](auto kb) {
    combine_kernel<decltype(kb)::value><<<grid_for(N, 256, kStreamCap), 256, 0, s>>>(N, k, u, beta, c, Q, out);
    LPG_LAUNCH_CHECK("combine_kernel");
    return LPG_OK;
  });
}

// Rotations i = 0..dim-2 applied in order to columns (i, i+1) of Q and U:
// (Q_i, Q_i+1) <- (c Q_i + s Q_i+1, -s Q_i + c Q_i+1); then column dim-1 = 0.
// A node's dim values of one array are loaded first, rotated in registers and stored;
// Q and U are done one after the other.
template <int K>
__device__ __forceinline__ void givens_node(const int64_t N, const int64_t n, const int dim, const HistCoeffs& c,
                                            const HistCoeffs& sn, double* __restrict__ Q) {
  double q[K];
#pragma unroll
  for (int i = 0; i < K; ++i) q[i] = i < dim ? Q[(int64_t)i * N + n] : 0.0;
#pragma unroll
  for (int i = 0; i + 1 < K; ++i) {
    if (i + 1 < dim) {
      const double q0 = q[i], q1 = q[i + 1];
      q[i] = c.v[i] * q0 + sn.v[i] * q1;
      q[i + 1] = -sn.v[i] * q0 + c.v[i] * q1;
    }
  }
#pragma unroll
  for (int i = 0; i < K; ++i) {
    if (i + 1 < dim) Q[(int64_t)i * N + n] = q[i];
    else if (i + 1 == dim) Q[(int64_t)i * N + n] = 0;
  }
}
template <int K>
__global__ void __launch_bounds__(256)
givens_columns_kernel(const int64_t N, const int dim, const HistCoeffs c, const HistCoeffs sn,
                      double* __restrict__ Q, double* __restrict__ U) {
  for (int64_t n = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; n < N; n += (int64_t)gridDim.x * blockDim.x) {
    givens_node<K>(N, n, dim, c, sn, Q);
    givens_node<K>(N, n, dim, c, sn, U);
  }
}
int givens_columns(int64_t N, int dim, const HistCoeffs& c, const HistCoeffs& sn, double* Q, double* U, cudaStream_t s) {
  if (N <= 0 || dim <= 0) return LPG_OK;
  if (dim > kMaxHistory) return set_error(LPG_ERR_INVALID, "givens_columns: history dimension out of range");
  return history_dispatch(dim, [&](auto kb) {
    givens_columns_kernel<decltype(kb)::value><<<grid_for(N, 256, kStreamCap), 256, 0, s>>>(N, dim, c, sn, Q, U);
    LPG_LAUNCH_CHECK("givens_columns_kernel");
    return LPG_OK;
  });
}

// x = sum_i d[i] * H_{(i + shift) % nh} over the nonzero d[i]
template <int K>
__global__ void extrap_kernel(const int64_t N, const int nh, const int shift, const HistCoeffs d,
                              const double* __restrict__ H, double* __restrict__ x) {
  for (int64_t n = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; n < N; n += (int64_t)gridDim.x * blockDim.x) {
    double h[K];
#pragma unroll
    for (int i = 0; i < K; ++i) h[i] = (i < nh && d.v[i] != 0.0) ? H[(int64_t)((i + shift) % nh) * N + n] : 0.0;
    double r = 0;
#pragma unroll
    for (int i = 0; i < K; ++i)
      if (i < nh && d.v[i] != 0.0) r += d.v[i] * h[i];
    x[n] = r;
  }
}
int extrap(int64_t N, int nh, int shift, const HistCoeffs& d, const double* H, double* x, cudaStream_t s) {
  if (N <= 0) return LPG_OK;
  if (nh < 1 || nh > kMaxHistory) return set_error(LPG_ERR_INVALID, "extrap: history dimension out of range");
  return history_dispatch(nh, [&](auto kb) {
    extrap_kernel<decltype(kb)::value><<<grid_for(N, 256, kStreamCap), 256, 0, s>>>(N, nh, shift, d, H, x);
    LPG_LAUNCH_CHECK("extrap_kernel");
    return LPG_OK;
  });
}

// ---------------------------------------------------------------- NBFPCG
// Fused passes of the non-blocking flexible PCG (okl/linearSolverUpdateNBFPCG.okl):
// block partial sums land in partials[k * nb + b]; the host adds them in block order.
template <int K>
__device__ __forceinline__ void block_partials(double (&v)[K], double* partials) {
  __shared__ double s_w[K][8];
#pragma unroll
  for (int k = 0; k < K; ++k)
    for (int o = 16; o > 0; o >>= 1) v[k] += __shfl_down_sync(0xffffffffu, v[k], o);
  if ((threadIdx.x & 31) == 0)
#pragma unroll
    for (int k = 0; k < K; ++k) s_w[k][threadIdx.x >> 5] = v[k];
  __syncthreads();
  if (threadIdx.x == 0)
#pragma unroll
    for (int k = 0; k < K; ++k) {
      double t = 0;
      for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += s_w[k][w];
      partials[(int64_t)k * gridDim.x + blockIdx.x] = t;
    }
}

// u.r, u.w, r.r (update0NBFPCG)
__global__ void __launch_bounds__(256)
nb_dots3_kernel(const int64_t N, const double* __restrict__ u, const double* __restrict__ r,
                const double* __restrict__ w, double* __restrict__ partials) {
  double v[3] = {0, 0, 0};
  for (int64_t n = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; n < N; n += (int64_t)gridDim.x * blockDim.x) {
    const double un = u[n], rn = r[n];
    v[0] += un * rn;
    v[1] += un * w[n];
    v[2] += rn * rn;
  }
  block_partials<3>(v, partials);
}
// x += a p; r -= a s; u -= a q; w -= a z; nv = w - r; then u.r, u.s, u.w, r.r (update1NBFPCG,
// with the n = w - r of the next preconditioner input folded in)
__global__ void __launch_bounds__(256)
nb_update_kernel(const int64_t N, const double a, const double* __restrict__ p, const double* __restrict__ s,
                 const double* __restrict__ q, const double* __restrict__ z, double* __restrict__ x,
                 double* __restrict__ r, double* __restrict__ u, double* __restrict__ w, double* __restrict__ nv,
                 double* __restrict__ partials) {
  double v[4] = {0, 0, 0, 0};
  for (int64_t n = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; n < N; n += (int64_t)gridDim.x * blockDim.x) {
    const double sn = s[n];
    x[n] += a * p[n];
    const double rn = r[n] - a * sn, un = u[n] - a * q[n], wn = w[n] - a * z[n];
    r[n] = rn;
    u[n] = un;
    w[n] = wn;
    nv[n] = wn - rn;
    v[0] += un * rn;
    v[1] += un * sn;
    v[2] += un * wn;
    v[3] += rn * rn;
  }
  block_partials<4>(v, partials);
}
static int nb_blocks(int64_t N) { return (int)std::max<int64_t>(1, std::min<int64_t>((N + 255) / 256, 1024)); }
int nb_dots3(int64_t N, const double* u, const double* r, const double* w, double* partials, int* nb, cudaStream_t s) {
  *nb = nb_blocks(N);
  nb_dots3_kernel<<<*nb, 256, 0, s>>>(N, u, r, w, partials);
  LPG_LAUNCH_CHECK("nb_dots3_kernel");
  return LPG_OK;
}
int nb_update(int64_t N, double a, const double* p, const double* sv, const double* q, const double* z, double* x,
              double* r, double* u, double* w, double* nv, double* partials, int* nb, cudaStream_t s) {
  *nb = nb_blocks(N);
  nb_update_kernel<<<*nb, 256, 0, s>>>(N, a, p, sv, q, z, x, r, u, w, nv, partials);
  LPG_LAUNCH_CHECK("nb_update_kernel");
  return LPG_OK;
}
// p = u + beta p; s = w + beta s; q = m + beta q; z = n + beta z (the search-direction
// updates of linearSolverNBFPCG.cpp:159-169 in one pass)
__global__ void __launch_bounds__(256)
nb_directions_kernel(const int64_t N, const double beta, const double* __restrict__ u, const double* __restrict__ w,
                     double* __restrict__ m, const double* __restrict__ nv, double* __restrict__ p,
                     double* __restrict__ s, double* __restrict__ q, double* __restrict__ z) {
  for (int64_t n = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; n < N; n += (int64_t)gridDim.x * blockDim.x) {
    const double un = u[n];
    p[n] = un + beta * p[n];
    s[n] = w[n] + beta * s[n];
    q[n] = m[n] + beta * q[n];
    z[n] = nv[n] + beta * z[n];
  }
}
int nb_directions(int64_t N, double beta, const double* u, const double* w, double* m, const double* nv, double* p,
                  double* sv, double* q, double* z, cudaStream_t s) {
  if (N <= 0) return LPG_OK;
  nb_directions_kernel<<<grid_for(N, 256, kStreamCap), 256, 0, s>>>(N, beta, u, w, m, nv, p, sv, q, z);
  LPG_LAUNCH_CHECK("nb_directions_kernel");
  return LPG_OK;
}

}  // namespace lpg
