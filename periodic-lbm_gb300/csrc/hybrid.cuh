// hybrid.cuh -- binary64 BGK with the binary64 pipe reserved for the final
// linear combination.
//
// GB300 issues binary64 at 1/64 of the binary32 rate, so a straight binary64
// BGK (about 70 FP64 instructions per cell) is bound by the FP64 pipe at ~15 %
// of HBM bandwidth.  This form keeps every term whose size is O(f) exact or
// binary64, and moves the rest to integer and binary32 pipes:
//
//   F_q      = f_q * 2^59 as int64 (exact for f_q >= 2^-7; below that the
//              truncation is < 2^-59)
//   R, JX, JY = sum F_q, sum cx F_q, sum cy F_q         exact integer sums
//   T_q      = R + 3 c_q.J                             exact integer
//   corr_q   = omega w_q rho (4.5 (c_q.u)^2 - 1.5 u^2)  double-float, |corr| <~ 1e-3
//   f'_q     = fma(omega w_q, T_q, fma(1 - omega, f_q, corr_q))   2 binary64 FMAs
//
// which is the BGK update f' = (1 - omega) f + omega feq with
// feq_q = w_q rho (1 + 3 c.u + 4.5 (c.u)^2 - 1.5 u^2) written as
// w_q (rho + 3 c.j + rho (4.5 (c.u)^2 - 1.5 u^2)), j = rho u
// (src/collision_bgk.F90:58-71, src/fvm_bardow.F90:99-126).  Only corr_q is
// evaluated in double-float; its size keeps the absolute error near 1e-18.
//
// Range: |f_q| < 2 for every population (so that the integer sums cannot
// overflow); values outside it set the kernel's range flag.
#pragma once
#include "df64.cuh"

namespace plbm {
namespace hy {

using df::df64;

constexpr int kScale = 59;  // fixed-point scale 2^59

DF_HD double fma_d(double a, double b, double c) {
#ifdef __CUDA_ARCH__
  return __fma_rn(a, b, c);
#else
  return fma(a, b, c);
#endif
}

DF_HD int clz64(uint64_t a) {
#ifdef __CUDA_ARCH__
  return __clzll((long long)a);
#else
  return a ? __builtin_clzll(a) : 64;
#endif
}

// binary64 -> int64 fixed point, scale 2^59, truncating toward zero.
// `bad` is set when |d| >= 2 or d is not finite.
DF_HD int64_t to_fixed(double d, bool& bad) {
  const uint64_t u = df::d2u(d);
  const int e = (int)((u >> 52) & 0x7FF);
  if (e >= 1024) {  // |d| >= 2, Inf, NaN
    bad = true;
    return 0;
  }
  const int64_t m = (int64_t)((u & 0xFFFFFFFFFFFFFull) | 0x10000000000000ull);
  const int sh = e - 1075 + kScale;  // value = m * 2^(e-1075)
  int64_t F;
  if (e == 0) F = 0;
  else if (sh >= 0) F = m << sh;
  else if (sh > -64) F = m >> (-sh);
  else F = 0;
  return (u >> 63) ? -F : F;
}

// int64 fixed point (scale 2^59) -> binary64, round to nearest even.
DF_HD double fixed_to_double(int64_t T) {
  if (T == 0) return 0.0;
  const uint64_t s = T < 0 ? 1ull : 0ull;
  const uint64_t a = s ? (uint64_t)(-T) : (uint64_t)T;
  const int lz = clz64(a);
  const uint64_t n = a << lz;  // bit 63 set
  uint64_t m = n >> 11;
  const uint64_t rem = n & 0x7FF;
  if (rem > 0x400 || (rem == 0x400 && (m & 1))) m += 1;
  int ex = 1086 - lz - kScale;
  if (m >> 53) {
    m >>= 1;
    ex += 1;
  }
  return df::u2d((s << 63) | ((uint64_t)ex << 52) | (m & 0xFFFFFFFFFFFFFull));
}

// int64 fixed point -> double-float (leading 48 bits: hi truncated, lo exact).
DF_HD df64 fixed_to_df(int64_t T) {
  if (T == 0) return df::make(0.0f, 0.0f);
  const uint32_t s = T < 0 ? 0x80000000u : 0u;
  const uint64_t a = s ? (uint64_t)(-T) : (uint64_t)T;
  const int lz = clz64(a);
  const uint64_t n = a << lz;
  const uint32_t mh = (uint32_t)(n >> 40);             // 24 bits, top bit set
  const uint32_t ml = (uint32_t)(n >> 16) & 0xFFFFFFu;  // next 24 bits
  // value = n * 2^(-lz - kScale); hi = mh * 2^(40 - lz - kScale)
  const int eh = 40 - lz - kScale + 23;  // exponent of hi's leading bit
  const float hi = df::u2f_bits(s | ((uint32_t)(eh + 127) << 23) | (mh & 0x7FFFFFu));
  float lo = 0.0f;
  if (ml) {
    const float l = df::uint_to_float_rn(ml);  // exact, < 2^24
    const float sc = df::u2f_bits((uint32_t)(16 - lz - kScale + 127) << 23);
    lo = df::u2f_bits(df::f2u(l * sc) | s);
  }
  return df::make(hi, lo);
}

struct Params {
  double omb;     // 1 - omega
  double omw[3];  // omega * w for w0, ws, wd
  df64 omw_df[3];  // the same as double-float
};

// One BGK collision of the 9 binary64 populations of a cell (in place).
DF_HD void bgk(double (&f)[9], const Params& p, bool& bad) {
  int64_t F[9];
#pragma unroll
  for (int q = 0; q < 9; q++) F[q] = to_fixed(f[q], bad);
  const int64_t R = (((F[5] + F[7]) + (F[6] + F[8])) + ((F[1] + F[3]) + (F[2] + F[4]))) + F[0];
  const int64_t d57 = F[5] - F[7], d86 = F[8] - F[6];
  const int64_t JX = (d57 + d86) + (F[1] - F[3]);
  const int64_t JY = (d57 - d86) + (F[2] - F[4]);
  // nonlinear part in double-float
  const df64 rho = fixed_to_df(R);
  const df64 inv = df::recip(rho);
  const df64 ux = df::mul(fixed_to_df(JX), inv), uy = df::mul(fixed_to_df(JY), inv);
  const df64 u2_15 = df::mul_f(df::add(df::sqr(ux), df::sqr(uy)), 1.5f);
  // q = 0: corr = omega w0 rho (-1.5 u^2)
  {
    const double c0 = df::pack_double(df::neg(df::mul(p.omw_df[0], df::mul(rho, u2_15))));
    f[0] = fma_d(p.omw[0], fixed_to_double(R), fma_d(p.omb, f[0], c0));
  }
#define PLBM_HY_PAIR(QP, QM, CU, CJ, WI)                                                    \
  {                                                                                         \
    const double c = df::pack_double(                                                       \
        df::mul(p.omw_df[WI], df::mul(rho, df::sub(df::mul_f(df::sqr(CU), 4.5f), u2_15))));  \
    const int64_t cj3 = (CJ) + ((CJ) << 1);                                                 \
    f[QP] = fma_d(p.omw[WI], fixed_to_double(R + cj3), fma_d(p.omb, f[QP], c));             \
    f[QM] = fma_d(p.omw[WI], fixed_to_double(R - cj3), fma_d(p.omb, f[QM], c));             \
  }
  PLBM_HY_PAIR(1, 3, ux, JX, 1)
  PLBM_HY_PAIR(2, 4, uy, JY, 1)
  PLBM_HY_PAIR(5, 7, df::add(ux, uy), JX + JY, 2)
  PLBM_HY_PAIR(8, 6, df::sub(ux, uy), JX - JY, 2)
#undef PLBM_HY_PAIR
}

// ---- fast paths for the ranges lattice states live in --------------------
// The general conversions are called out of line from the fast paths, so that
// the compiler branches around them instead of predicating them in.
#ifdef __CUDACC__
#define PLBM_NOINLINE static __host__ __device__ __noinline__
#else
#define PLBM_NOINLINE static __attribute__((noinline))
#endif
PLBM_NOINLINE int64_t to_fixed_slow(double d, int* bad) {
  bool b = false;
  const int64_t r = to_fixed(d, b);
  if (b) *bad = 1;
  return r;
}
PLBM_NOINLINE double fixed_to_double_slow(int64_t T) { return fixed_to_double(T); }

// High word of (hi:lo) << sh, 0 <= sh <= 31.
DF_HD uint32_t funnel_l(uint32_t lo, uint32_t hi, uint32_t sh) {
#ifdef __CUDA_ARCH__
  return __funnelshift_l(lo, hi, sh);
#else
  return sh ? (hi << sh) | (lo >> (32 - sh)) : hi;
#endif
}

// to_fixed for positive f in [2^-7, 2): one 64-bit shift by 0..7, the same
// exact value as the general conversion (which handles everything else).
DF_HD int64_t to_fixed_fast(double d, bool& bad) {
  const uint64_t u = df::d2u(d);
  const uint32_t H = (uint32_t)(u >> 32), L = (uint32_t)u;
  const uint32_t sh = (H >> 20) - 1016u;  // a set sign bit makes this large
  if (sh <= 7u) {
    const uint32_t mh = (H & 0xFFFFFu) | 0x100000u;
    return (int64_t)(((uint64_t)funnel_l(L, mh, sh) << 32) | (uint64_t)(L << sh));
  }
  int b = 0;
  const int64_t r = to_fixed_slow(d, &b);
  if (b) bad = true;
  return r;
}

// fixed_to_double for 2^58 <= T < 2^60 (values in [0.5, 2)): a shift by 6 or
// 7 with round-half-up.  It differs from round-to-nearest-even only on exact
// ties, a few in a thousand values, by one ulp upward (a bias of order 1e-19
// relative, far below the rounding of the stored state).
DF_HD double fixed_to_double_fast(int64_t T) {
  const uint64_t a = (uint64_t)T;
  const uint32_t top = (uint32_t)(a >> 58);
  if (top - 1u <= 2u) {
    const bool big = top >= 2u;
    const uint32_t sh = big ? 7u : 6u;
    uint64_t m = (a + (1ull << (sh - 1u))) >> sh;
    // m <= 2^53; m == 2^53 carries into the exponent through the add below
    const uint64_t ex = big ? 1023ull : 1022ull;
    return df::u2d((ex << 52) + (m - (1ull << 52)));
  }
  return fixed_to_double_slow(T);
}

// BGK of the hybrid arithmetic with the fast conversions: the same update as
// bgk() (rho for the nonlinear term taken from the rounded binary64 R).
DF_HD void bgk_fast(double (&f)[9], const Params& p, bool& bad) {
  int64_t F[9];
#pragma unroll
  for (int q = 0; q < 9; q++) F[q] = to_fixed_fast(f[q], bad);
  const int64_t R = (((F[5] + F[7]) + (F[6] + F[8])) + ((F[1] + F[3]) + (F[2] + F[4]))) + F[0];
  const int64_t d57 = F[5] - F[7], d86 = F[8] - F[6];
  const int64_t JX = (d57 + d86) + (F[1] - F[3]);
  const int64_t JY = (d57 - d86) + (F[2] - F[4]);
  const double Rd = fixed_to_double_fast(R);
  const df64 rho = df::from_double(Rd);
  const df64 inv = df::recip(rho);
  const df64 ux = df::mul(fixed_to_df(JX), inv), uy = df::mul(fixed_to_df(JY), inv);
  const df64 u2_15 = df::mul_f(df::add(df::sqr(ux), df::sqr(uy)), 1.5f);
  {
    const double c0 = df::pack_double(df::neg(df::mul(p.omw_df[0], df::mul(rho, u2_15))));
    f[0] = fma_d(p.omw[0], Rd, fma_d(p.omb, f[0], c0));
  }
#define PLBM_HY_PAIR(QP, QM, CU, CJ, WI)                                                    \
  {                                                                                         \
    const double c = df::pack_double(                                                       \
        df::mul(p.omw_df[WI], df::mul(rho, df::sub(df::mul_f(df::sqr(CU), 4.5f), u2_15))));  \
    const int64_t cj3 = (CJ) + ((CJ) << 1);                                                 \
    f[QP] = fma_d(p.omw[WI], fixed_to_double_fast(R + cj3), fma_d(p.omb, f[QP], c));        \
    f[QM] = fma_d(p.omw[WI], fixed_to_double_fast(R - cj3), fma_d(p.omb, f[QM], c));        \
  }
  PLBM_HY_PAIR(1, 3, ux, JX, 1)
  PLBM_HY_PAIR(2, 4, uy, JY, 1)
  PLBM_HY_PAIR(5, 7, df::add(ux, uy), JX + JY, 2)
  PLBM_HY_PAIR(8, 6, df::sub(ux, uy), JX - JY, 2)
#undef PLBM_HY_PAIR
}

}  // namespace hy
}  // namespace plbm
