// Double-word ("double-FP32") arithmetic for FP64-accurate work on the FP32 pipe.
//
// A value is hi + lo with two floats, |lo| <= ulp(hi)/2: 48 significand bits. The
// building blocks are the classical error-free transformations -- Knuth's TwoSum,
// Dekker's Fast2Sum and the FMA-based TwoProd -- and the double-word sum and product
// built from them as analysed by Joldes, Muller and Popescu ("Tight and rigorous error
// bounds for basic building blocks of double-word arithmetic", ACM TOMS 44(2), 2017):
// the "sloppy" DW+DW sum (absolute error of order u^2 (|x| + |y|)) and DW x DW with
// FMA. Dot products accumulate TwoProd products with a TwoSum-chained high part and a
// plain FP32 low part, renormalised once at the end.
//
// All roundings must stay separate: __fadd_rn / __fsub_rn / __fmul_rn are never
// contracted into FMA by the compiler.
//
// Conversions from and to FP64 use integer operations only (GB300's FP64 pipe is the
// scarce unit): x -> hi = x truncated to 24 significant bits (exact in FP32), lo = the
// remaining bits rounded to FP32. Full double-word precision needs 2^-74 <= |x| < 2^128;
// below 2^-74 the low word is dropped (relative error 2^-24), below 2^-126 the value is 0.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

namespace lpg {

struct __align__(8) dw {
  float h, l;
};

__device__ __forceinline__ dw dw_two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  const float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
  return {s, e};
}

// |a| >= |b| (or a == 0)
__device__ __forceinline__ dw dw_fast_two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  return {s, __fsub_rn(b, __fsub_rn(s, a))};
}

// sloppy double-word sum
__device__ __forceinline__ dw dw_add(dw x, dw y) {
  const dw s = dw_two_sum(x.h, y.h);
  const float w = __fadd_rn(s.l, __fadd_rn(x.l, y.l));
  return dw_fast_two_sum(s.h, w);
}
// the sloppy sum without the final renormalisation: s.h exact TwoSum high part, low part
// s.l + x.l + y.l (|low| of order ulp(|x| + |y|)). Every consumer here (products, sums,
// the FP64 rebuild) takes an unnormalised pair; the error bound is that of dw_add.
__device__ __forceinline__ dw dw_add_u(dw x, dw y) {
  const dw s = dw_two_sum(x.h, y.h);
  return {s.h, __fadd_rn(s.l, __fadd_rn(x.l, y.l))};
}
// x + sign * y (sign = +-1) unnormalised, the sign folded into FMAs: fma(sign, b, c) is
// the exactly rounded c + sign * b, so this is dw_add_u(x, {sign y.h, sign y.l}) bit for bit
__device__ __forceinline__ dw dw_add_sign_u(dw x, float sign, dw y) {
  const float s = fmaf(sign, y.h, x.h);
  const float bb = __fsub_rn(s, x.h);
  const float e = __fadd_rn(__fsub_rn(x.h, __fsub_rn(s, bb)), fmaf(sign, y.h, -bb));
  return {s, __fadd_rn(e, fmaf(sign, y.l, x.l))};
}
__device__ __forceinline__ dw dw_neg(dw x) { return {-x.h, -x.l}; }
__device__ __forceinline__ dw dw_sub(dw x, dw y) { return dw_add(x, dw_neg(y)); }
// sign * x for sign = +-1 (exact)
__device__ __forceinline__ dw dw_scale_sign(float sign, dw x) { return {sign * x.h, sign * x.l}; }

// double-word product with FMA (the x.l * y.l term is below the error bound)
__device__ __forceinline__ dw dw_mul(dw x, dw y) {
  const float ch = __fmul_rn(x.h, y.h);
  float cl = fmaf(x.h, y.h, -ch);
  cl = fmaf(x.h, y.l, cl);
  cl = fmaf(x.l, y.h, cl);
  return dw_fast_two_sum(ch, cl);
}

// sum of double-word products
struct dw_acc {
  float h = 0.f, l = 0.f;
  dw_acc() = default;
  // started with its first product (no TwoSum against zero)
  __device__ __forceinline__ dw_acc(dw a, dw b) {
    h = __fmul_rn(a.h, b.h);
    float pl = fmaf(a.h, b.h, -h);
    pl = fmaf(a.h, b.l, pl);
    l = fmaf(a.l, b.h, pl);
  }
  __device__ __forceinline__ void mac(dw a, dw b) {
    const float ph = __fmul_rn(a.h, b.h);
    float pl = fmaf(a.h, b.h, -ph);
    pl = fmaf(a.h, b.l, pl);
    pl = fmaf(a.l, b.h, pl);
    const dw s = dw_two_sum(h, ph);
    h = s.h;
    l = __fadd_rn(l, __fadd_rn(pl, s.l));
  }
  __device__ __forceinline__ dw get() const { return dw_fast_two_sum(h, l); }
  __device__ __forceinline__ dw raw() const { return {h, l}; }   // unnormalised
};

__device__ __forceinline__ dw dw_from_double(double x) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
  const int ex = (int)((b >> 52) & 0x7FF);
  const unsigned sign = (unsigned)(b >> 63) << 31;
  const int fe = ex - 1023 + 127;                                 // FP32 exponent of hi
  const unsigned hbits = (fe <= 0) ? sign : (fe >= 255) ? (sign | 0x7F800000u)
                                                         : (sign | ((unsigned)fe << 23) | (unsigned)((b >> 29) & 0x7FFFFFu));
  const int le = ex - 1075 + 127;                                 // FP32 exponent of 2^(ex-1075)
  float lo = __uint2float_rn((unsigned)(b & 0x1FFFFFFFu));        // the 29 bits below hi
  lo = (le > 0 && fe > 0 && fe < 255) ? __fmul_rn(lo, __uint_as_float((unsigned)le << 23)) : 0.f;
  return dw_fast_two_sum(__uint_as_float(hbits), sign ? -lo : lo);
}

// exact FP32 -> FP64 for normal numbers and zero (FP32 subnormals give 0)
__device__ __forceinline__ double dw_float_to_double(float f) {
  const unsigned u = __float_as_uint(f);
  const unsigned e = (u >> 23) & 0xFFu;
  const unsigned long long s = (unsigned long long)(u >> 31) << 63;
  const unsigned long long bits = (e == 0) ? s
                                  : (e == 255) ? (s | 0x7FF0000000000000ull | ((unsigned long long)(u & 0x7FFFFFu) << 29))
                                               : (s | ((unsigned long long)(e - 127 + 1023) << 52) |
                                                  ((unsigned long long)(u & 0x7FFFFFu) << 29));
  return __longlong_as_double((long long)bits);
}

__device__ __forceinline__ double dw_to_double(dw a) { return dw_float_to_double(a.h) + dw_float_to_double(a.l); }

__device__ __forceinline__ dw dw_shfl_xor(dw v, int mask) {
  return {__shfl_xor_sync(0xffffffffu, v.h, mask), __shfl_xor_sync(0xffffffffu, v.l, mask)};
}

}  // namespace lpg
