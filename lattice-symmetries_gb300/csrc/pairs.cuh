// pairs.cuh -- FP64 values carried as unevaluated pairs of floats (hi + lo, 48 significant
// bits) for multiply-accumulate work on the FP32 pipe.  GB300's FP64 pipe is a small fraction
// of its FP32 rate; kernels whose FP64 multiply-adds dominate (blocks of right-hand sides, the
// eigensolver's tall-skinny products) keep FP64 in memory and accumulate in pairs:
//
//   split_double  FP64 -> (hi, lo): hi = the top 24 significant bits (exact), lo = the next
//                 bits rounded to 24; integer instructions and one int->float conversion.
//   mac           acc += a * b: hi*hi product made error-free with fmaf, first-order cross
//                 terms, two-sum accumulation (relative error per product below 2^-45, 3e-14).
//   renorm        folds the low word back under ulp(hi) (after every few multiply-adds, so that
//                 the low word's own rounding stays at 2^-48 of the running sum).
//   join          (hi, lo) -> FP64 (exact conversions, one FP64 add).
//
// Range: magnitudes below 2^-126 split to 0; products above ~3e38 overflow to inf.
#pragma once

#include <cstdint>

namespace lsg {

struct F2 {
  float h, l;
};

// hi + lo split of a double: hi = its top 24 significant bits (exact), lo = the next bits
// rounded to 24.  Magnitudes below 2^-126 become 0, magnitudes from 2^128 on become +-inf,
// NaN stays NaN.
__device__ __forceinline__ F2 split_double(double a) {
  const unsigned long long u = (unsigned long long)__double_as_longlong(a);
  const unsigned hw = (unsigned)(u >> 32);
  const unsigned sign = hw & 0x80000000u;
  const int e = (int)((hw >> 20) & 0x7ffu);
  const unsigned mant23 = (unsigned)(u >> 29) & 0x7fffffu;
  F2 r;
  if (e <= 896) {
    r.h = __uint_as_float(sign);
    r.l = 0.0f;
    return r;
  }
  if (e >= 1151) {
    const bool nan = e == 2047 && (u & 0xfffffffffffffull) != 0;
    r.h = __uint_as_float(sign | 0x7f800000u | (nan ? 0x400000u : 0u));
    r.l = 0.0f;
    return r;
  }
  const unsigned ebits = (unsigned)(e - 896) << 23;  // 2^(e - 1023) as a float exponent field
  r.h = __uint_as_float(sign | ebits | mant23);
  const unsigned low = (unsigned)u & 0x1fffffffu;    // remaining 29 bits, weight 2^(e - 1075)
  const float lo = __fmul_rn(__fmul_rn(__uint2float_rn(low), 0x1p-52f), __uint_as_float(ebits));
  r.l = __uint_as_float(__float_as_uint(lo) ^ sign);
  return r;
}

// Exact float -> double by bit manipulation (subnormal floats become 0).
__device__ __forceinline__ double float_bits_to_double(float f) {
  const unsigned b = __float_as_uint(f);
  const unsigned e = (b >> 23) & 0xffu;
  const unsigned long long sign = (unsigned long long)(b >> 31) << 63;
  const unsigned long long m = (unsigned long long)(b & 0x7fffffu) << 29;
  if (e == 0) return __longlong_as_double((long long)sign);
  if (e == 255) return __longlong_as_double((long long)(sign | 0x7ff0000000000000ull | m));
  return __longlong_as_double((long long)(sign | ((unsigned long long)(e + 896) << 52) | m));
}

__device__ __forceinline__ double join(F2 v) { return float_bits_to_double(v.h) + float_bits_to_double(v.l); }

// acc += a * b.  The hi*hi product is error-free (fmaf), the cross terms are first order, the
// sum is a two-sum.  Explicit _rn intrinsics keep the compiler from contracting the
// error-free transformations into FMAs.
__device__ __forceinline__ void mac(F2& acc, const float ah, const float al, const float bh, const float bl) {
  const float p = __fmul_rn(ah, bh);
  float e = __fmaf_rn(ah, bh, -p);
  e = __fmaf_rn(ah, bl, e);
  e = __fmaf_rn(al, bh, e);
  const float t = __fadd_rn(acc.h, p);
  const float bp = __fsub_rn(t, acc.h);
  const float err = __fadd_rn(__fsub_rn(acc.h, __fsub_rn(t, bp)), __fsub_rn(p, bp));
  acc.l = __fadd_rn(acc.l, __fadd_rn(err, e));
  acc.h = t;
}

// a + b for pairs (two-sum of the high words).
__device__ __forceinline__ F2 pair_add(F2 a, F2 b) {
  const float t = __fadd_rn(a.h, b.h);
  const float bp = __fsub_rn(t, a.h);
  const float err = __fadd_rn(__fsub_rn(a.h, __fsub_rn(t, bp)), __fsub_rn(b.h, bp));
  return F2{t, __fadd_rn(__fadd_rn(a.l, b.l), err)};
}

__device__ __forceinline__ F2 pair_neg(F2 a) { return F2{-a.h, -a.l}; }

// Moves the low word's accumulated value into the high word (fast two-sum, |h| >= |l|), so that
// later additions to the low word round relative to ulp(h) again.
__device__ __forceinline__ void renorm(F2& a) {
  const float s = __fadd_rn(a.h, a.l);
  a.l = __fsub_rn(a.l, __fsub_rn(s, a.h));
  a.h = s;
}

// Warp butterfly step for a pair (both words exchanged).
__device__ __forceinline__ F2 pair_shfl_xor(F2 a, int d) {
  return F2{__shfl_xor_sync(0xffffffffu, a.h, d), __shfl_xor_sync(0xffffffffu, a.l, d)};
}

__device__ __forceinline__ void mac(F2& acc, F2 a, F2 b) { mac(acc, a.h, a.l, b.h, b.l); }

__device__ __forceinline__ float4 split_c(double2 v) {
  const F2 re = split_double(v.x), im = split_double(v.y);
  return make_float4(re.h, re.l, im.h, im.l);
}

}  // namespace lsg
