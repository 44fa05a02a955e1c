// hybrid.cuh -- binary64 collisions with the binary64 pipe reserved for the
// one operation per population that needs its precision.
//
// GB300 issues binary64 at 1/64 of the binary32 rate, so a straight binary64
// BGK (about 70 FP64 instructions per cell) is bound by the FP64 pipe at ~15 %
// of HBM bandwidth.  These forms keep every term whose size is O(f) exact, and
// do the rest on the integer, XU and binary32 pipes.
//
// Common part:
//   F_q       = f_q * 2^59 as int64 (exact for |f_q| >= 2^-7; below that
//               rounded to nearest, error <= 2^-60)
//   R, JX, JY = sum F_q, sum cx F_q, sum cy F_q          exact integer sums
//   f'_q      = fma(c_q, Y_q 2^-59, f_q)                  ONE binary64 FMA
// where Y_q is an integer bracket holding the whole update of population q
// (the linear part exact, the nonlinear part from double-float or exact
// 128-bit products taken to the fixed point once), c_q a power-of-two multiple
// of one rounded relaxation constant, so that the brackets of the nine
// populations sum to zero with the weights exactly: mass and momentum change
// only by the nine final roundings, plus the drift the reference's own
// binary64 weights cause (sums 1 - 2^-54), which is restored in the integers.
//
//   BGK (bgk_fma, src/collision_bgk.F90:58-71 with the equilibrium of
//     src/fvm_bardow.F90:99-126): the nonlinear terms of all nine populations
//     are integer combinations of three double-float products.
//   TRT (trt_fma, incompressible, src/collision_trt.F90:98-152): symmetric
//     and antisymmetric brackets of each pair, joined by one exact 128-bit
//     product r D (r = lambda_d / lambda_e scaled); |j|^2 and jx jy exact.
//   RR (rr_fma, src/collision_regularized.F90:72-194): the six merged Hermite
//     coefficients of the equilibrium and the regularized part in
//     double-float, taken to the fixed point at half scale.
// Each states its range; a cell outside it reports `bad`, and the kernels then
// evaluate that cell with the binary64 operator of the reference instead.
// Populations stored shifted (h = f - w, the plugin's storage) take the same
// forms with DH = sum h = rho - 1 in place of R in the linear brackets.
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
  return ::fma(a, b, c);
#endif
}

DF_HD int clz64(uint64_t a) {
#ifdef __CUDA_ARCH__
  return __clzll((long long)a);
#else
  return a ? __builtin_clzll(a) : 64;
#endif
}

// m / 2^rs rounded to nearest, ties to even (1 <= rs; 0 for rs >= 64).
DF_HD uint64_t shr_rne(uint64_t m, int rs) {
  if (rs >= 64) return 0;
  const uint64_t q = m >> rs, rem = m - (q << rs), half = 1ull << (rs - 1);
  return q + (uint64_t)((rem > half) | ((rem == half) & (q & 1ull)));
}

// binary64 -> int64 fixed point, scale 2^59, rounded to nearest even below
// 2^-59.  `bad` is set when the biased exponent of d exceeds emax
// (emax <= 1023), or d is not finite.
DF_HD int64_t to_fixed_lim(double d, int emax, bool& bad) {
  const uint64_t u = df::d2u(d);
  const int e = (int)((u >> 52) & 0x7FF);
  if (e > emax) {
    bad = true;
    return 0;
  }
  const int64_t m = (int64_t)((u & 0xFFFFFFFFFFFFFull) | 0x10000000000000ull);
  const int sh = e - 1075 + kScale;  // value = m * 2^(e-1075)
  int64_t F;
  if (e == 0) F = 0;
  else if (sh >= 0) F = m << sh;
  else F = (int64_t)shr_rne((uint64_t)m, -sh);
  return (u >> 63) ? -F : F;
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

// ---- fast paths for the ranges lattice states live in --------------------
// The general conversions are called out of line from the fast paths, so that
// the compiler branches around them instead of predicating them in.
#ifdef __CUDACC__
#define PLBM_NOINLINE static __host__ __device__ __noinline__
#else
#define PLBM_NOINLINE static __attribute__((noinline))
#endif

// High word of (hi:lo) << sh, 0 <= sh <= 31.
DF_HD uint32_t funnel_l(uint32_t lo, uint32_t hi, uint32_t sh) {
#ifdef __CUDA_ARCH__
  return __funnelshift_l(lo, hi, sh);
#else
  return sh ? (hi << sh) | (lo >> (32 - sh)) : hi;
#endif
}



// ---- shifted populations h = f - w (the plugin path) -------------------------
// With h in place of f the exact sums give DH = sum h = rho - 1 and the same
// J; every linear bracket keeps its form with DH in place of R (the w terms
// cancel), and rho = 1 + DH where the nonlinear terms need it.  The range
// limits apply to |h|.

// binary64 h (either sign, |h| < 2^(EMAX-1022)) -> int64 fixed point, scale
// 2^59; below 2^-59 rounded to nearest with ties toward +inf (an arithmetic
// shift of the signed value plus half a unit).  Most h = f - w are below 2^-7,
// where bits drop out.  Truncating toward zero shrank them by half a unit on
// average, and with h of the sign of c.u that damped |J| by ~1e-16 per step
// (2e-12 in u over 10,000 plugin steps); a bias that does not depend on the
// sign of h leaves every odd moment alone.
template <int EMAX>
DF_HD int64_t to_fixed_signed(double d, bool& bad) {
  const uint64_t u = df::d2u(d);
  const int e = (int)((u >> 52) & 0x7FF);
  if (e > EMAX) {
    bad = true;
    return 0;
  }
  const uint64_t m = (u & 0xFFFFFFFFFFFFFull) | 0x10000000000000ull;
  const int sh = e - 1016;  // value * 2^59 = m * 2^(e - 1016)
  const int64_t s = (u >> 63) ? -(int64_t)m : (int64_t)m;
  if (sh >= 0) return (int64_t)((uint64_t)s << sh);
  const int rs = -sh;
  return rs < 64 ? (s + ((int64_t)1 << (rs - 1))) >> rs : 0;
}

// int64 fixed point (any value) -> binary64, rounded to nearest with ties
// away from zero, branch-free apart from zero.  Ties are common (the integers
// are sums of binary64 images whose low bits are often zero) and in the
// shifted forms these values carry the sign of c.J, so the tie rule nudges |J|
// up: 1.5e-13 in u over 10,000 plugin steps (256 x 192 TGV), against 9e-14
// with ties to even, which costs 7 % of the plugin step.
DF_HD double fixed_to_double_any(int64_t T) {
  if (T == 0) return 0.0;
  const uint64_t neg = (uint64_t)T >> 63;
  const uint64_t a = neg ? (uint64_t)(-T) : (uint64_t)T;
  const int lz = clz64(a);
  const uint64_t n = a << lz;                      // bit 63 set
  const uint64_t m = (n >> 11) + ((n >> 10) & 1);  // <= 2^53; 2^53 carries into the exponent
  const uint64_t ex = (uint64_t)(1086 - lz - kScale);
  return df::u2d((neg << 63) | ((ex << 52) + (m - (1ull << 52))));
}

constexpr int64_t kOne = (int64_t)1 << kScale;  // 1.0 in fixed point




// a k / 2^64 rounded to nearest, for the constant corrections below
// (|a| < 2^63, |k| < 2^31; a's low 32 bits do not take part).
DF_HD int64_t scale_2m64(int64_t a, int32_t k) {
  return ((int64_t)(int32_t)(a >> 32) * (int64_t)k + (int64_t(1) << 31)) >> 32;
}


// ---- conversions shaped for the GB300 pipes ----------------------------------
// Measured issue rates per SM and clock: integer add/logic/shift and
// I2F.F32.S32 go to the ALU pipe (64 lanes), IMAD and binary32 arithmetic to
// the FMA pipes (64 / 128), F2I, FRND and FLO (clz) to the XU pipe (16), and
// every conversion to or from a 64-bit type to the binary64 pipe (~2).  The
// one-FMA BGK is bound by its ALU work, so these forms move work to the FMA
// and XU pipes.

// 32-bit count of leading zeros (XU pipe).
DF_HD uint32_t clz32(uint32_t a) {
#ifdef __CUDA_ARCH__
  return (uint32_t)__clz((int)a);
#else
  return a ? (uint32_t)__builtin_clz(a) : 32u;
#endif
}
// Low word of (hi:lo) >> sh, 0 <= sh <= 31.
DF_HD uint32_t funnel_r(uint32_t lo, uint32_t hi, uint32_t sh) {
#ifdef __CUDA_ARCH__
  return __funnelshift_r(lo, hi, sh);
#else
  return sh ? (lo >> sh) | (hi << (32 - sh)) : lo;
#endif
}
DF_HD int32_t f2i_trunc(float v) {
#ifdef __CUDA_ARCH__
  return __float2int_rz(v);
#else
  return (int32_t)v;
#endif
}
DF_HD float i2f(int32_t v) {
#ifdef __CUDA_ARCH__
  return __int2float_rn(v);
#else
  return (float)v;
#endif
}

PLBM_NOINLINE double fixed_to_double_any_slow(int64_t T) { return fixed_to_double_any(T); }

// int64 fixed point (scale 2^59) -> binary64 for |T| >= 2^32 (others out of
// line, exactly): the magnitude taken in one's complement (a negative T comes
// out 2^-59 smaller in magnitude) and truncated to 53 bits.  The error is below
// 2^-52 relative plus 2^-59 absolute -- for the non-equilibrium brackets it
// converts, negligible against the binary64 rounding of the populations.
DF_HD double fixed_to_double_tr(int64_t T) {
  const uint32_t hi = (uint32_t)((uint64_t)T >> 32), lo = (uint32_t)(uint64_t)T;
  const uint32_t s = (uint32_t)((int32_t)hi >> 31);  // 0 or ~0
  const uint32_t ah = hi ^ s, al = lo ^ s;
  if (ah == 0u) return fixed_to_double_any_slow(T);
  const uint32_t lz = clz32(ah);  // 0..31
  const uint32_t nh = funnel_l(al, ah, lz), nl = al << lz;  // bit 63 of (nh:nl) set
  const uint32_t mh = nh >> 11, ml = funnel_r(nl, nh, 11);  // 53 bits, leading one at bit 52
  // value = (nh:nl) 2^(-lz - 59): biased exponent 1027 - lz; the leading one of
  // mh (bit 20) adds the final 1 to the exponent field
  const uint32_t eh = (1026u - lz) * 0x100000u + mh;
  return df::u2d(((uint64_t)(eh | (s & 0x80000000u)) << 32) | (uint64_t)ml);
}

// binary32 v, |v| < 16 -> int64 fixed point (scale 2^59), truncated toward
// zero below 2^-58: the integer part of v 2^27 (F2I) is the high word and its
// fraction 2^31 (F2I, signed) the low word shifted by one.  The fraction
// t - trunc(t) is exact for either sign.  Exact for |v| >= 2^-35.
DF_HD int64_t float_to_fixed_xu(float v) {
  const float t = v * 0x1p27f;  // exact
  const int32_t h = f2i_trunc(t);
  const int32_t l = f2i_trunc((t - i2f(h)) * 0x1p31f);  // |l| < 2^31
  return (int64_t)((uint64_t)(uint32_t)h << 32) + 2 * (int64_t)l;
}
// A double-float (|value| < 16) in the fixed point: the sum of its halves' images.
DF_HD int64_t df_to_fixed_xu(df64 c) { return float_to_fixed_xu(c.hi) + float_to_fixed_xu(c.lo); }

PLBM_NOINLINE df64 fixed_to_df_slow(int64_t T) { return fixed_to_df(T); }

// int64 fixed point -> double-float (leading 48 bits: hi and lo truncated)
// for |T| >= 2^32 (others out of line).
DF_HD df64 fixed_to_df_x(int64_t T) {
  const uint32_t hi = (uint32_t)((uint64_t)T >> 32), lo = (uint32_t)(uint64_t)T;
  const uint32_t s = (uint32_t)((int32_t)hi >> 31);
  const uint64_t a = ((((uint64_t)hi << 32) | lo) ^ (((uint64_t)s << 32) | s)) + (uint64_t)(s & 1u);
  const uint32_t ah = (uint32_t)(a >> 32), al = (uint32_t)a;
  if (ah == 0u) return fixed_to_df_slow(T);
  const uint32_t lz = clz32(ah);
  const uint32_t nh = funnel_l(al, ah, lz), nl = al << lz;  // bit 31 of nh set
  // value = (nh:nl) 2^(-lz - 59) = nh 2^(-lz - 27) + ...: hi = top 24 bits of
  // nh, leading one at bit 23 (it adds the final 1 to the exponent field)
  const uint32_t sgn = s & 0x80000000u;
  const float fhi = df::u2f_bits(((130u - lz) * 0x800000u + (nh >> 8)) | sgn);
  const uint32_t ml = funnel_r(nl, nh, 16) & 0xFFFFFFu;  // next 24 bits
  // lo = ml 2^(16 - lz - 59): a signed scale (biased exponent 84 - lz) times
  // the exact I2F of the 24-bit integer
  const float sc = df::u2f_bits(((84u - lz) * 0x800000u) | sgn);
  return df::make(fhi, i2f((int32_t)ml) * sc);
}

// ---- BGK with one binary64 FMA per population --------------------------------
// f'_q = f_q + omega (feq_q - f_q), feq_q = w_q T_q, T_q = R + 3 c_q.J + C_q,
// C_q = rho (4.5 (c_q.u)^2 - 1.5 u^2) (src/collision_bgk.F90:58-71 with the
// equilibrium of src/fvm_bardow.F90:99-126, rearranged).  The nonlinear terms
// of all nine populations are integer combinations of three products,
//   A = 1.5 jx^2 / rho,  B = 1.5 jy^2 / rho,  X = 4.5 jx jy / rho,
//   C_0 = -(A + B),  C_x = 2A - B,  C_y = 2B - A,  C_(+-diag) = 2 (A + B) +- 2X,
// evaluated in double-float and taken to the fixed point once each.  With
// every F_q and the C images integers, 36 (w_q T_q - F_q) is an integer, and
//   rest      4 Y_0,  Y_0 = 4 (R + C_0) - 9 F_0
//   axis      4 Y_q,  Y_q = T_q - 9 F_q
//   diagonal    Y_q,  Y_q = T_q - 36 F_q
// so f'_q = fma(k_q c, Y_q 2^-59, f_q) with c = RN(omega / 36), k_q = 4 or 1:
// the only rounding of the linear part is the final one, and the integers
// satisfy sum k_q Y_q = 0 and sum k_q c_q Y_q = 0 exactly (the nonlinear
// combinations above sum to zero with the weights), so mass and momentum
// change only by the nine final roundings.  Y_q is taken to binary64 by
// integer instructions (53 leading bits); its error is relative to the small
// non-equilibrium term, not to f.
//
// The reference relaxes with its binary64 weights, whose sum W0 + 4 WS + 4 WD
// and first-moment factor 3 (2 WS + 4 WD) are both 1 - 2^-54: each step its
// mass and momentum lose omega 2^-54 of themselves, 1e-12 over 10,000 steps
// -- the size of the tolerance.  The same relaxation is restored in the
// integers: the rest bracket gains omega eps_m R / (4c) (mass_k), and the
// x-axis pair gains +- omega eps_j JX / (8c) (mom_k; the y pair likewise), so
// the mass changes by omega eps_m R and JX by omega eps_j JX per step.
//
// Range.  The loads take 0 <= f_0 < 1, 0 <= f_axis < 1/4, 0 <= f_diag < 1/8
// (biased exponents at most 1022, 1020, 1019), and the cell must satisfy
// A + B < 0.2 (7.5 rho |u|^2 < 1, which bounds every |C_q| below 1).  Then,
// in units of 2^59, R < 2.5, |JX|, |JY| < 1/2, |JX +- JY| < 3/4, and
// |Y_0| < 10, |Y_axis| < 7.25, |Y_diag| < 10.25: every bracket fits int64
// (intermediate products such as 4 R may wrap; two's complement sums of
// wrapped terms are exact when the result fits).  Other cells report `bad`.
struct BgkParams {
  double c1;       // RN(omega / 36)
  double c4;       // 4 RN(omega / 36), exact
  int32_t mass_k;  // omega eps_m / c4 2^64, rounded (bgk_fma_params)
  int32_t mom_k;   // omega eps_j / (2 c4) 2^64, rounded
};

// a + b = s + e exactly (Knuth's two-sum).
inline void two_sum_d(double a, double b, double& s, double& e) {
  s = a + b;
  const double bb = s - a;
  e = (a - (s - bb)) + (b - bb);
}

// eps_m = W0 + 4 WS + 4 WD - 1 and eps_j = 3 (2 WS + 4 WD) - 1 of the binary64
// weights, evaluated without rounding error (both are -2^-54 for 4/9, 1/9,
// 1/36: the sums are within 2^-50 of 1, so the final subtraction is exact).
inline double weight_sum_error(const double (&w)[3]) {
  double s1, e1, s2, e2;
  two_sum_d(w[0], 4.0 * w[1], s1, e1);
  two_sum_d(s1, 4.0 * w[2], s2, e2);
  return (s2 - 1.0) + (e1 + e2);
}
inline double first_moment_error(const double (&w)[3]) {
  double s, e;
  two_sum_d(2.0 * w[1], 4.0 * w[2], s, e);
  const double p = 3.0 * s, ep = ::fma(3.0, s, -p);
  return (p - 1.0) + (ep + 3.0 * e);
}

inline BgkParams bgk_fma_params(double omega, const double (&w)[3]) {
  BgkParams p;
  p.c1 = omega / 36.0;
  p.c4 = 4.0 * p.c1;
  const double eps_m = weight_sum_error(w), eps_j = first_moment_error(w);
  const double km = ldexp(omega * eps_m / p.c4, 64), kj = ldexp(0.5 * omega * eps_j / p.c4, 64);
  p.mass_k = fabs(km) < 0x1p30 ? (int32_t)llrint(km) : 0;
  p.mom_k = fabs(kj) < 0x1p30 ? (int32_t)llrint(kj) : 0;
  return p;
}

// Exact fixed-point image of a non-negative population below 2^(EMAX-1022);
// `bad` for negative values, values past the limit and non-finite ones.
PLBM_NOINLINE int64_t to_fixed_nonneg_slow(double d, int emax, int* bad) {
  bool b = false;
  const int64_t r = to_fixed_lim(d, emax, b);
  if (b || r < 0) *bad = 1;
  return r;
}
template <int EMAX>
DF_HD int64_t to_fixed_nonneg(double d, bool& bad) {
  const uint64_t u = df::d2u(d);
  const uint32_t H = (uint32_t)(u >> 32), L = (uint32_t)u;
  const uint32_t sh = (H >> 20) - 1016u;  // a set sign bit makes this large
  if (sh <= (uint32_t)(EMAX - 1016)) {
    const uint32_t mh = (H & 0xFFFFFu) | 0x100000u;
    return (int64_t)(((uint64_t)funnel_l(L, mh, sh) << 32) | (uint64_t)(L << sh));
  }
  int b = 0;
  const int64_t r = to_fixed_nonneg_slow(d, EMAX, &b);
  if (b) bad = true;
  return r;
}

// SHIFTED: f holds h = f - w (the plugin's storage, sim/sim.F90:131).  The
// linear brackets then take DH = sum h = rho - 1 in place of R (the w terms
// cancel) and the nonlinear terms rho = 1 + DH.  Range for h: |h_0| < 1/2,
// |h_axis| < 1/8, |h_diag| < 1/16 (biased exponents at most 1021, 1019, 1018),
// rho >= 1/4 and A + B < 0.2; then |DH| < 1.25, |JX|, |JY| < 1/2,
// |JX +- JY| < 3/4 and |Y_0| < 10.3, |Y_axis| < 4.9, |Y_diag| < 6.75 (units of
// 2^59).  Small h are rounded to the fixed point with ties toward +infinity,
// a bias that leaves the odd moments alone (to_fixed_signed).
template <bool SHIFTED = false>
DF_HD void bgk_fma(double (&f)[9], const BgkParams& p, bool& bad) {
  using namespace df;
  int64_t F[9];
  if constexpr (SHIFTED) {
    F[0] = to_fixed_signed<1021>(f[0], bad);
    F[1] = to_fixed_signed<1019>(f[1], bad);
    F[2] = to_fixed_signed<1019>(f[2], bad);
    F[3] = to_fixed_signed<1019>(f[3], bad);
    F[4] = to_fixed_signed<1019>(f[4], bad);
    F[5] = to_fixed_signed<1018>(f[5], bad);
    F[6] = to_fixed_signed<1018>(f[6], bad);
    F[7] = to_fixed_signed<1018>(f[7], bad);
    F[8] = to_fixed_signed<1018>(f[8], bad);
  } else {
    F[0] = to_fixed_nonneg<1022>(f[0], bad);
    F[1] = to_fixed_nonneg<1020>(f[1], bad);
    F[2] = to_fixed_nonneg<1020>(f[2], bad);
    F[3] = to_fixed_nonneg<1020>(f[3], bad);
    F[4] = to_fixed_nonneg<1020>(f[4], bad);
    F[5] = to_fixed_nonneg<1019>(f[5], bad);
    F[6] = to_fixed_nonneg<1019>(f[6], bad);
    F[7] = to_fixed_nonneg<1019>(f[7], bad);
    F[8] = to_fixed_nonneg<1019>(f[8], bad);
  }
  // R: the zeroth moment of the stored values (rho, or DH when shifted)
  const int64_t R = (((F[5] + F[7]) + (F[6] + F[8])) + ((F[1] + F[3]) + (F[2] + F[4]))) + F[0];
  const int64_t d57 = F[5] - F[7], d86 = F[8] - F[6];
  const int64_t JX = (d57 + d86) + (F[1] - F[3]);
  const int64_t JY = (d57 - d86) + (F[2] - F[4]);
  const int64_t Rrho = SHIFTED ? R + kOne : R;
  if constexpr (SHIFTED) bad |= Rrho < (kOne >> 2);
  const df64 s15 = mul_f(recip(fixed_to_df_x(Rrho)), 1.5f);  // 1.5 / rho
  const df64 jx = fixed_to_df_x(JX), jy = fixed_to_df_x(JY);
  const df64 A = mul_lz(sqr_lz(jx), s15);
  const df64 B = mul_lz(sqr_lz(jy), s15);
  const df64 X = mul_f_lz(mul_lz(mul_lz(jx, jy), s15), 3.0f);
  bad |= !(A.hi + B.hi < 0.2f);  // NaN (R = 0) fails too
  const int64_t Ai = df_to_fixed_xu(A), Bi = df_to_fixed_xu(B), Xi = df_to_fixed_xu(X);
  const int64_t AB = Ai + Bi;
  f[0] = fma_d(p.c4, fixed_to_double_tr(4 * (R - AB) - 9 * F[0] + scale_2m64(R, p.mass_k)), f[0]);
  const int64_t cx = R + (2 * Ai - Bi), cy = R + (2 * Bi - Ai);
  const int64_t jx3 = 3 * JX, jy3 = 3 * JY;
  const int64_t ax = jx3 + scale_2m64(JX, p.mom_k), ay = jy3 + scale_2m64(JY, p.mom_k);
  f[1] = fma_d(p.c4, fixed_to_double_tr(cx + ax - 9 * F[1]), f[1]);
  f[3] = fma_d(p.c4, fixed_to_double_tr(cx - ax - 9 * F[3]), f[3]);
  f[2] = fma_d(p.c4, fixed_to_double_tr(cy + ay - 9 * F[2]), f[2]);
  f[4] = fma_d(p.c4, fixed_to_double_tr(cy - ay - 9 * F[4]), f[4]);
  const int64_t dp = R + 2 * (AB + Xi), dm = R + 2 * (AB - Xi);
  const int64_t sp = jx3 + jy3, sm = jy3 - jx3;
  f[5] = fma_d(p.c1, fixed_to_double_tr(dp + sp - 36 * F[5]), f[5]);
  f[7] = fma_d(p.c1, fixed_to_double_tr(dp - sp - 36 * F[7]), f[7]);
  f[6] = fma_d(p.c1, fixed_to_double_tr(dm + sm - 36 * F[6]), f[6]);
  f[8] = fma_d(p.c1, fixed_to_double_tr(dm - sm - 36 * F[8]), f[8]);
}

// Recursive-regularized constants (rr_fma).
struct RrParams {
  double w[3];   // 4/9, 1/9, 1/36 in binary64
  df64 wdf[3];   // the same as double-float
  df64 omb;      // 1 - omega
  df64 third;    // 1/3
};


// Recursive regularized collision with one binary64 FMA per population.
// f'_q = w_q (T_q + N_q), T_q = R + 3 c_q.J, N_q the Hermite combination of
// the six merged coefficients M = rho (u product) + (1 - omega) a of the
// second-, third- and fourth-order Hermite terms (the equilibrium's and the
// regularized non-equilibrium part's, src/collision_regularized.F90:99-194),
// with a_xx = (3 Pxx - R)/3 - jx ux, a_yy alike, a_xy = Pxy - jx uy from exact
// integer moments and the recursive third and fourth orders; so with the
// fixed-point images of
// M / 2 (exact halving in double-float), h.., every 36 (f'_q - f_q) / k_q is
// an integer bracket:
//   rest      4 Y_0,  Y_0 = 4 R - 9 F_0 - 12 (hxx + hyy) + 18 hxxyy
//   axis      4 Y_q,  Y_q = T_q - 9 F_q + 6 hxx - 3 hyy - 9 hxxyy -+ 9 hyyx  (x; y alike)
//   diagonal    Y_q,  Y_q = T_q - 36 F_q + 6 (hxx + hyy) + 18 hxxyy
//                            +- 18 hxy +- 18 (hxxy +- hyyx)
// and f'_q = fma(k_q RN(1/36), Y_q 2^-59, f_q).  The Hermite parts of the
// brackets sum to zero with the weights exactly, as T_q - 36 w_q F_q does; the
// reference's binary64 weights (sums 1 - 2^-54) take 2^-54 of the mass and
// momentum each step, restored by p.mass_k / p.mom_k (bgk_fma_params at
// omega = 1).  Range as bgk_fma, and sum |M / 2| < 0.1 (checked on the
// binary32 heads): then the Hermite parts add at most 3, 0.9 and 1.8 (units of
// 2^59) to the rest, axis and diagonal brackets, which stay below 13 x 2^59.
template <bool SHIFTED = false>
DF_HD void rr_fma(double (&f)[9], const RrParams& r, const BgkParams& p, bool& bad) {
  using namespace df;
  int64_t F[9];
  if constexpr (SHIFTED) {
    F[0] = to_fixed_signed<1021>(f[0], bad);
    F[1] = to_fixed_signed<1019>(f[1], bad);
    F[2] = to_fixed_signed<1019>(f[2], bad);
    F[3] = to_fixed_signed<1019>(f[3], bad);
    F[4] = to_fixed_signed<1019>(f[4], bad);
    F[5] = to_fixed_signed<1018>(f[5], bad);
    F[6] = to_fixed_signed<1018>(f[6], bad);
    F[7] = to_fixed_signed<1018>(f[7], bad);
    F[8] = to_fixed_signed<1018>(f[8], bad);
  } else {
    F[0] = to_fixed_nonneg<1022>(f[0], bad);
    F[1] = to_fixed_nonneg<1020>(f[1], bad);
    F[2] = to_fixed_nonneg<1020>(f[2], bad);
    F[3] = to_fixed_nonneg<1020>(f[3], bad);
    F[4] = to_fixed_nonneg<1020>(f[4], bad);
    F[5] = to_fixed_nonneg<1019>(f[5], bad);
    F[6] = to_fixed_nonneg<1019>(f[6], bad);
    F[7] = to_fixed_nonneg<1019>(f[7], bad);
    F[8] = to_fixed_nonneg<1019>(f[8], bad);
  }
  const int64_t s57 = F[5] + F[7], s68 = F[6] + F[8];
  const int64_t sd = s57 + s68;
  const int64_t R = ((s57 + s68) + ((F[1] + F[3]) + (F[2] + F[4]))) + F[0];
  const int64_t d57 = F[5] - F[7], d86 = F[8] - F[6];
  const int64_t JX = (d57 + d86) + (F[1] - F[3]);
  const int64_t JY = (d57 - d86) + (F[2] - F[4]);
  const int64_t PXX3 = 3 * ((F[1] + F[3]) + sd) - R;
  const int64_t PYY3 = 3 * ((F[2] + F[4]) + sd) - R;
  const int64_t PXY = s57 - s68;
  const int64_t Rrho = SHIFTED ? R + kOne : R;
  if constexpr (SHIFTED) bad |= Rrho < (kOne >> 2);
  const df64 rho = fixed_to_df_x(Rrho);
  const df64 inv = recip(rho);
  const df64 jx = fixed_to_df_x(JX), jy = fixed_to_df_x(JY);
  const df64 ux = mul_lz(jx, inv), uy = mul_lz(jy, inv);
  // rho times the velocity products: rho ux^2 = jx ux, rho ux uy = jx uy, ...
  const df64 qxx = mul_lz(jx, ux), qyy = mul_lz(jy, uy), qxy = mul_lz(jx, uy);
  const df64 uxx = sqr_lz(ux), uyy = sqr_lz(uy), uxy = mul_lz(ux, uy);
  const df64 axx = sub_lz(mul_lz(fixed_to_df_x(PXX3), r.third), qxx);
  const df64 ayy = sub_lz(mul_lz(fixed_to_df_x(PYY3), r.third), qyy);
  const df64 axy = sub_lz(fixed_to_df_x(PXY), qxy);
  const df64 axxy = add_lz(mul_pow2(mul_lz(ux, axy), 2.0f), mul_lz(uy, axx));
  const df64 ayyx = add_lz(mul_pow2(mul_lz(uy, axy), 2.0f), mul_lz(ux, ayy));
  const df64 axxyy =
      sub_lz(sub_lz(sub_lz(mul_pow2(add_lz(mul_lz(ux, ayyx), mul_lz(uy, axxy)), 2.0f), mul_lz(uxx, ayy)),
                    mul_lz(uyy, axx)),
             mul_pow2(mul_lz(uxy, axy), 4.0f));
  // M / 2 = (rho (u product) + (1 - omega) a) / 2
  const df64 mxx = mul_pow2(add_lz(qxx, mul_lz(r.omb, axx)), 0.5f);
  const df64 myy = mul_pow2(add_lz(qyy, mul_lz(r.omb, ayy)), 0.5f);
  const df64 mxy = mul_pow2(add_lz(qxy, mul_lz(r.omb, axy)), 0.5f);
  const df64 mxxy = mul_pow2(add_lz(mul_lz(qxx, uy), mul_lz(r.omb, axxy)), 0.5f);
  const df64 myyx = mul_pow2(add_lz(mul_lz(qyy, ux), mul_lz(r.omb, ayyx)), 0.5f);
  const df64 mxxyy = mul_pow2(add_lz(mul_lz(qxx, uyy), mul_lz(r.omb, axxyy)), 0.5f);
  // sum |M / 2| < 0.1 (NaN fails too)
  bad |= !(fabsf(mxx.hi) + fabsf(myy.hi) + fabsf(mxy.hi) + fabsf(mxxy.hi) + fabsf(myyx.hi) + fabsf(mxxyy.hi) < 0.1f);
  const int64_t hxx = df_to_fixed_xu(mxx), hyy = df_to_fixed_xu(myy), hxy = df_to_fixed_xu(mxy);
  const int64_t hxxy = df_to_fixed_xu(mxxy), hyyx = df_to_fixed_xu(myyx), hxxyy = df_to_fixed_xu(mxxyy);
  f[0] = fma_d(p.c4, fixed_to_double_tr(4 * R - 9 * F[0] - 12 * (hxx + hyy) + 18 * hxxyy + scale_2m64(R, p.mass_k)),
               f[0]);
  const int64_t jx3 = 3 * JX + scale_2m64(JX, p.mom_k), jy3 = 3 * JY + scale_2m64(JY, p.mom_k);
  const int64_t nx_ = R + 6 * hxx - 3 * hyy - 9 * hxxyy, nxo = 9 * hyyx;
  const int64_t ny_ = R + 6 * hyy - 3 * hxx - 9 * hxxyy, nyo = 9 * hxxy;
  f[1] = fma_d(p.c4, fixed_to_double_tr(nx_ + jx3 - nxo - 9 * F[1]), f[1]);
  f[3] = fma_d(p.c4, fixed_to_double_tr(nx_ - jx3 + nxo - 9 * F[3]), f[3]);
  f[2] = fma_d(p.c4, fixed_to_double_tr(ny_ + jy3 - nyo - 9 * F[2]), f[2]);
  f[4] = fma_d(p.c4, fixed_to_double_tr(ny_ - jy3 + nyo - 9 * F[4]), f[4]);
  // diagonal pairs without the momentum correction (the axis pairs carry it):
  // q=5 (+x,+y): +18 hxy + 18 (hxxy + hyyx); q=7: +18 hxy - 18 (hxxy + hyyx)
  // q=6 (-x,+y): -18 hxy + 18 (hxxy - hyyx); q=8: -18 hxy - 18 (hxxy - hyyx)
  const int64_t dsum = R + 6 * (hxx + hyy) + 18 * hxxyy;
  const int64_t sp = 3 * (JX + JY), sm = 3 * (JY - JX);
  const int64_t a5 = 18 * (hxy + hxxy + hyyx), a6 = 18 * (hxy - hxxy + hyyx);
  f[5] = fma_d(p.c1, fixed_to_double_tr(dsum + sp + a5 - 36 * F[5]), f[5]);
  f[7] = fma_d(p.c1, fixed_to_double_tr(dsum - sp + 36 * hxy - a5 - 36 * F[7]), f[7]);
  f[6] = fma_d(p.c1, fixed_to_double_tr(dsum + sm - a6 - 36 * F[6]), f[6]);
  f[8] = fma_d(p.c1, fixed_to_double_tr(dsum - sm - 36 * hxy + a6 - 36 * F[8]), f[8]);
}

// (a b) / 2^sh, 0 < sh < 64, of the exact 128-bit product, rounded to nearest
// (ties toward +infinity); the caller keeps the result within int64.  Rounding
// toward -infinity instead biases every product by half a unit in one
// direction: in the antisymmetric brackets that is a uniform force on the flow
// (about 3e-19 per step in J), which grew to 2e-12 of the decaying u over
// 10,000 steps.
DF_HD int64_t mul_shr(int64_t a, int64_t b, int sh) {
#ifdef __CUDA_ARCH__
  int64_t hi = __mul64hi(a, b);
#else
  int64_t hi = (int64_t)(((__int128)a * b) >> 64);
#endif
  const uint64_t lo = (uint64_t)a * (uint64_t)b;
  const uint64_t lo2 = lo + (1ull << (sh - 1));
  hi += (int64_t)(lo2 < lo);
  return (int64_t)(((uint64_t)hi << (64 - sh)) | (lo2 >> sh));
}

// Incompressible TRT with one binary64 FMA per population
// (src/collision_trt.F90:98-152).  With c = RN(lambda_e / 18) and the exact
// integer brackets of the pairs (axis: weights 1/9, diagonal: 1/36; J2 = |J|^2,
// XY = JX JY as exact 128-bit products taken to the fixed point)
//   axis x    Sb = 9 (F_1 + F_3) - 2 R - 6 JX^2 + 3 JY^2,   D = 3 (F_1 - F_3) - 2 JX
//   diagonal  Sb = 18 (F_5 + F_7) - R - 3 J2 -+ 9 XY,       D = 6 (F_5 - F_7) - (JX +- JY)
// the reference's sym = les (...) is c Sb (axis) and c/2 Sb (diagonal), its
// asym the same constants times r D with r = lambda_d / (6 c) (one exact
// 64 x 64-bit product per pair), so
//   f'_p = fma(c_k, -(Sb + r D), f_p),  f'_m = fma(c_k, -(Sb - r D), f_m),
//   f'_0 = fma(2c, 4 R - 6 J2 - 9 F_0, f_0)
// (c_k = c on the axis pairs, c/2 on the diagonal ones).  The integer brackets
// sum to zero with the weights; the reference's binary64 weights relax the
// mass by lambda_e (sum w - 1) R per step (the sum is 1 - 2^-54), restored in
// the rest bracket (mass_k).  Range: the loads of bgk_fma, and |Sb| < 2^61,
// |D| < dmax = 2^61 / r (checked), so every bracket stays below 2^62.
struct TrtFmaParams {
  double c, c2, ch;  // RN(lambda_e / 18), 2c, c/2
  int64_t r_fx;      // r = lambda_d / (6c) = r_fx 2^-r_sh
  int64_t dmax;      // largest |D| with |r D| < 2^61 (0: every cell falls back)
  int32_t r_sh;
  int32_t mass_k;    // lambda_e eps_m / (2c) 2^64
  int32_t mom_k;     // lambda_d eps_j / (2c) 2^64
};

inline TrtFmaParams trt_fma_params(double lambda_e, double lambda_d, const double (&w)[3]) {
  TrtFmaParams p;
  p.c = lambda_e / 18.0;
  p.c2 = 2.0 * p.c;
  p.ch = 0.5 * p.c;
  const double r = lambda_d / (6.0 * p.c);
  int e = 0;
  frexp(r, &e);  // r in [2^(e-1), 2^e)
  int sh = 61 - e;
  if (sh > 63) sh = 63;
  if (sh < 1) sh = 1;
  const double rf = ldexp(r, sh);
  p.r_sh = sh;
  p.r_fx = rf < 0x1p62 ? (int64_t)llrint(rf) : 0;
  p.dmax = r > 0 ? (int64_t)fmin(0x1p61 / r, 0x1p62) : ((int64_t)1 << 62);
  if (!(rf < 0x1p62) || !(r >= 0)) p.dmax = 0;
  const double km = ldexp(lambda_e * weight_sum_error(w) / p.c2, 64);
  const double kj = ldexp(lambda_d * first_moment_error(w) / p.c2, 64);
  p.mass_k = fabs(km) < 0x1p30 ? (int32_t)llrint(km) : 0;
  p.mom_k = fabs(kj) < 0x1p30 ? (int32_t)llrint(kj) : 0;
  return p;
}

DF_HD int64_t abs64(int64_t v) { return v < 0 ? -v : v; }

template <bool SHIFTED = false>
DF_HD void trt_fma(double (&f)[9], const TrtFmaParams& p, bool& bad) {
  int64_t F[9];
  if constexpr (SHIFTED) {
    F[0] = to_fixed_signed<1021>(f[0], bad);
    F[1] = to_fixed_signed<1019>(f[1], bad);
    F[2] = to_fixed_signed<1019>(f[2], bad);
    F[3] = to_fixed_signed<1019>(f[3], bad);
    F[4] = to_fixed_signed<1019>(f[4], bad);
    F[5] = to_fixed_signed<1018>(f[5], bad);
    F[6] = to_fixed_signed<1018>(f[6], bad);
    F[7] = to_fixed_signed<1018>(f[7], bad);
    F[8] = to_fixed_signed<1018>(f[8], bad);
  } else {
    F[0] = to_fixed_nonneg<1022>(f[0], bad);
    F[1] = to_fixed_nonneg<1020>(f[1], bad);
    F[2] = to_fixed_nonneg<1020>(f[2], bad);
    F[3] = to_fixed_nonneg<1020>(f[3], bad);
    F[4] = to_fixed_nonneg<1020>(f[4], bad);
    F[5] = to_fixed_nonneg<1019>(f[5], bad);
    F[6] = to_fixed_nonneg<1019>(f[6], bad);
    F[7] = to_fixed_nonneg<1019>(f[7], bad);
    F[8] = to_fixed_nonneg<1019>(f[8], bad);
  }
  const int64_t R = (((F[5] + F[7]) + (F[6] + F[8])) + ((F[1] + F[3]) + (F[2] + F[4]))) + F[0];
  const int64_t d57 = F[5] - F[7], d86 = F[8] - F[6];
  const int64_t JX = (d57 + d86) + (F[1] - F[3]);
  const int64_t JY = (d57 - d86) + (F[2] - F[4]);
  const int64_t X2 = mul_shr(JX, JX, kScale), Y2 = mul_shr(JY, JY, kScale), XY = mul_shr(JX, JY, kScale);
  const int64_t J2 = X2 + Y2;
  const int64_t sx = 9 * (F[1] + F[3]) - 2 * R - 6 * X2 + 3 * Y2, dx = 3 * (F[1] - F[3]) - 2 * JX;
  const int64_t sy = 9 * (F[2] + F[4]) - 2 * R - 6 * Y2 + 3 * X2, dy = 3 * (F[2] - F[4]) - 2 * JY;
  const int64_t sp = 18 * (F[5] + F[7]) - R - 3 * J2 - 9 * XY, dp = 6 * d57 - (JX + JY);
  const int64_t sm = 18 * (F[8] + F[6]) - R - 3 * J2 + 9 * XY, dm = 6 * d86 - (JX - JY);
  const int64_t lim = (int64_t)1 << 61;
  bad |= (abs64(sx) | abs64(sy) | abs64(sp) | abs64(sm)) >= lim;
  bad |= (abs64(dx) | abs64(dy) | abs64(dp) | abs64(dm)) >= p.dmax;
  f[0] = fma_d(p.c2, fixed_to_double_tr(4 * R - 6 * J2 - 9 * F[0] + scale_2m64(R, p.mass_k)), f[0]);
  const int64_t rx = mul_shr(dx, p.r_fx, p.r_sh) - scale_2m64(JX, p.mom_k);
  const int64_t ry = mul_shr(dy, p.r_fx, p.r_sh) - scale_2m64(JY, p.mom_k);
  const int64_t rp = mul_shr(dp, p.r_fx, p.r_sh), rm = mul_shr(dm, p.r_fx, p.r_sh);
  f[1] = fma_d(p.c, fixed_to_double_tr(-(sx + rx)), f[1]);
  f[3] = fma_d(p.c, fixed_to_double_tr(rx - sx), f[3]);
  f[2] = fma_d(p.c, fixed_to_double_tr(-(sy + ry)), f[2]);
  f[4] = fma_d(p.c, fixed_to_double_tr(ry - sy), f[4]);
  f[5] = fma_d(p.ch, fixed_to_double_tr(-(sp + rp)), f[5]);
  f[7] = fma_d(p.ch, fixed_to_double_tr(rp - sp), f[7]);
  f[8] = fma_d(p.ch, fixed_to_double_tr(-(sm + rm)), f[8]);
  f[6] = fma_d(p.ch, fixed_to_double_tr(rm - sm), f[6]);
}

}  // namespace hy
}  // namespace plbm
