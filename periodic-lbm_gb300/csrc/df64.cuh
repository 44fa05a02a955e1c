// df64.cuh -- double-float ("df64") arithmetic: a value is the unevaluated
// sum hi + lo of two binary32 numbers with |lo| <= ulp(hi)/2, about 48
// significant bits.  All operations run on the FP32 pipe.
//
// Algorithms (error-free transformations):
//   two_sum       Knuth, TAOCP vol. 2, 4.2.2 (6 flops)
//   fast_two_sum  Dekker 1971, |a| >= |b| (3 flops)
//   two_prod      with a fused multiply-add: p = a*b, e = fma(a, b, -p)
//   add / mul     the "sloppy" double-length add and the FMA multiply of
//                 Dekker 1971 / Hida-Li-Bailey QD library (2001), renormalised
//                 by fast_two_sum.
//   recip         one Newton step r1 = r0 + r0*(1 - b*r0) on a binary32
//                 seed, evaluated in double-length arithmetic.
// Conversions to and from binary64 use integer bit operations only: on GB300
// F2F conversions between binary32 and binary64 run at the binary64 rate.
//
// Every function is __host__ __device__ so the same code can be checked on
// the CPU.  The error-free transformations assume each + - * is rounded
// separately and the only fused operations are the explicit fmaf calls; the
// one product that feeds an add (two_prod) uses an explicitly rounded
// multiply, so contraction settings of the including translation unit cannot
// fuse it (host code is compiled with -ffp-contract=off).
#pragma once
#include <stdint.h>
#include <string.h>
#ifdef __CUDACC__
#define DF_HD __host__ __device__ __forceinline__
#else
#include <math.h>
#define DF_HD inline
#endif

namespace plbm {
namespace df {

struct df64 {
  float hi, lo;
};

DF_HD float fmaf_(float a, float b, float c) {
#ifdef __CUDA_ARCH__
  return __fmaf_rn(a, b, c);
#else
  return fmaf(a, b, c);
#endif
}

DF_HD uint32_t f2u(float f) {
#ifdef __CUDA_ARCH__
  return __float_as_uint(f);
#else
  uint32_t u;
  memcpy(&u, &f, 4);
  return u;
#endif
}
DF_HD float u2f_bits(uint32_t u) {
#ifdef __CUDA_ARCH__
  return __uint_as_float(u);
#else
  float f;
  memcpy(&f, &u, 4);
  return f;
#endif
}
DF_HD uint64_t d2u(double d) {
#ifdef __CUDA_ARCH__
  return (uint64_t)__double_as_longlong(d);
#else
  uint64_t u;
  memcpy(&u, &d, 8);
  return u;
#endif
}
DF_HD double u2d(uint64_t u) {
#ifdef __CUDA_ARCH__
  return __longlong_as_double((long long)u);
#else
  double d;
  memcpy(&d, &u, 8);
  return d;
#endif
}
DF_HD float uint_to_float_rn(uint32_t u) {
#ifdef __CUDA_ARCH__
  return __uint2float_rn(u);
#else
  return (float)u;
#endif
}

DF_HD df64 make(float hi, float lo) {
  df64 r;
  r.hi = hi;
  r.lo = lo;
  return r;
}

DF_HD df64 two_sum(float a, float b) {
  float s = a + b;
  float bb = s - a;
  float e = (a - (s - bb)) + (b - bb);
  return make(s, e);
}

DF_HD df64 fast_two_sum(float a, float b) {
  float s = a + b;
  float e = b - (s - a);
  return make(s, e);
}

// Product rounded on its own: never fused into a following add, whatever the
// translation unit's contraction setting (the error-free transformations need
// p = RN(a*b) exactly).
DF_HD float mul_rn(float a, float b) {
#ifdef __CUDA_ARCH__
  return __fmul_rn(a, b);
#else
  return a * b;
#endif
}

DF_HD df64 two_prod(float a, float b) {
  float p = mul_rn(a, b);
  float e = fmaf_(a, b, -p);
  return make(p, e);
}

DF_HD df64 neg(df64 a) { return make(-a.hi, -a.lo); }

DF_HD df64 add(df64 a, df64 b) {
  df64 s = two_sum(a.hi, b.hi);
  float e = s.lo + (a.lo + b.lo);
  return fast_two_sum(s.hi, e);
}

DF_HD df64 sub(df64 a, df64 b) { return add(a, neg(b)); }

DF_HD df64 add_f(df64 a, float b) {
  df64 s = two_sum(a.hi, b);
  float e = s.lo + a.lo;
  return fast_two_sum(s.hi, e);
}

DF_HD df64 mul(df64 a, df64 b) {
  df64 p = two_prod(a.hi, b.hi);
  float e = fmaf_(a.hi, b.lo, p.lo);
  e = fmaf_(a.lo, b.hi, e);
  return fast_two_sum(p.hi, e);
}

DF_HD df64 mul_f(df64 a, float b) {
  df64 p = two_prod(a.hi, b);
  float e = fmaf_(a.lo, b, p.lo);
  return fast_two_sum(p.hi, e);
}

DF_HD df64 sqr(df64 a) {
  df64 p = two_prod(a.hi, a.hi);
  float e = fmaf_(a.hi + a.hi, a.lo, p.lo);
  return fast_two_sum(p.hi, e);
}

// Lazy variants: the same error-free first step without the final
// renormalisation (lo may grow to a few ulps of hi).  The pair still holds its
// value to ~2^-46 relative, and a pair's binary64 image (df_to_double) is the
// exact sum of its halves either way; three binary32 operations fewer each.
DF_HD df64 add_lz(df64 a, df64 b) {
  df64 s = two_sum(a.hi, b.hi);
  s.lo += a.lo + b.lo;
  return s;
}
DF_HD df64 sub_lz(df64 a, df64 b) { return add_lz(a, neg(b)); }
DF_HD df64 mul_lz(df64 a, df64 b) {
  df64 p = two_prod(a.hi, b.hi);
  p.lo = fmaf_(a.hi, b.lo, p.lo);
  p.lo = fmaf_(a.lo, b.hi, p.lo);
  return p;
}
DF_HD df64 mul_f_lz(df64 a, float b) {
  df64 p = two_prod(a.hi, b);
  p.lo = fmaf_(a.lo, b, p.lo);
  return p;
}
DF_HD df64 sqr_lz(df64 a) {
  df64 p = two_prod(a.hi, a.hi);
  p.lo = fmaf_(a.hi + a.hi, a.lo, p.lo);
  return p;
}

// Multiplication by a power of two is exact.
DF_HD df64 mul_pow2(df64 a, float p2) { return make(a.hi * p2, a.lo * p2); }

// 1/b: binary32 seed, one Newton step in double length.
DF_HD df64 recip(df64 b) {
  float r0 = 1.0f / b.hi;
  // e = 1 - b*r0 in double length
  df64 br = mul_f(b, r0);
  df64 e = add_f(neg(br), 1.0f);
  // r1 = r0 + r0*e
  df64 re = mul_f(e, r0);
  return add_f(re, r0);
}

// Split of a compile-time binary64 constant into hi + lo.
DF_HD df64 from_double_const(double d) {
  float hi = (float)d;
  float lo = (float)(d - (double)hi);
  return make(hi, lo);
}

// binary64 -> df64 by bit manipulation (no binary64 arithmetic, no F2F).
// hi keeps the leading 24 significand bits (truncated), lo the next 29 bits
// rounded to 24.  Magnitudes below 2^-126 become 0 (never reached by lattice
// populations); NaN/Inf map to NaN/Inf in hi.
DF_HD df64 from_double(double d) {
  const uint64_t u = d2u(d);
  const uint32_t H = (uint32_t)(u >> 32), L = (uint32_t)u;
  const uint32_t sign = H & 0x80000000u;
  const int e = (int)((H >> 20) & 0x7FFu);
  const uint32_t mant23 = ((H & 0xFFFFFu) << 3) | (L >> 29);
  if (e <= 896) return make(0.0f, 0.0f);
  if (e >= 1151) return make(u2f_bits(sign | 0x7F800000u | (e == 2047 && ((H & 0xFFFFFu) | L) ? 0x400000u : 0u)), 0.0f);
  const float hi = u2f_bits(sign | ((uint32_t)(e - 896) << 23) | mant23);
  float lo = 0.0f;
  if (e >= 949) {
    // remainder r * 2^(e - 1075), r < 2^29
    const float r = uint_to_float_rn(L & 0x1FFFFFFFu);
    const float scale = u2f_bits((uint32_t)(e - 948) << 23);
    lo = u2f_bits(f2u(r * scale) | sign);
  }
  return make(hi, lo);
}

// binary32 -> binary64 by bit assembly for finite values (binary32 subnormals
// become 0); integer instructions only, no conversion on the binary64 pipe.
DF_HD double f2d_bits(float f) {
  const uint32_t b = f2u(f);
  const uint32_t ex = (b >> 23) & 0xFFu;
  const uint32_t hi = ex ? ((b & 0x80000000u) | ((ex + 896u) << 20) | ((b & 0x7FFFFFu) >> 3)) : (b & 0x80000000u);
  const uint32_t lo = ex ? ((b & 0x7u) << 29) : 0u;
  return u2d(((uint64_t)hi << 32) | (uint64_t)lo);
}

// hi + lo of a normalised pair as one binary64 addition of the exact binary64
// images of hi and lo (exact whenever lo lies within 29 bits below hi's last
// bit, as it does after renormalisation): one binary64 addition and a few
// integer instructions, the form for kernels whose binary64 pipe has room.
DF_HD double df_to_double(df64 a) { return f2d_bits(a.hi) + f2d_bits(a.lo); }

}  // namespace df
}  // namespace plbm
