// exact_fields.cuh -- moments and equilibria of binary64 lattices on the
// integer pipes.
//
// The reference evaluates update_macros (src/fvm_bardow.F90:368-382) and
// equilibrium() (src/fvm_bardow.F90:99-126; the shifted forms of
// sim/sim.F90:160-173 and :353-401) in binary64: about 30 and 50 binary64
// instructions per cell, which GB300 issues at 1/64 of the binary32 rate, so
// the two field kernels ran at 32 % and 17 % of HBM bandwidth.  These forms
// compute the same quantities without the binary64 pipe:
//
//   moments      F_q = f_q 2^59 (exact for f_q >= 2^-7), R, JX, JY exact
//                integer sums; rho = RN(R 2^-59) and u = RN(J / R) by an
//                integer division with an exact remainder: every output is the
//                correctly rounded value of the exact moments.
//   equilibrium  P = rho 2^60, U = u 2^62 (exact for rho >= 2^-8,
//                |u| >= 2^-10); j = rho u and the three nonlinear products
//                (1.5 rho ux^2, 1.5 rho uy^2, 4.5 rho ux uy) as exact 128-bit
//                products rounded once to 2^-60; the bracket
//                T_q = rho (1 + 3 c.u + 4.5 (c.u)^2 - 1.5 u^2) an integer
//                combination of them; feq_q = RN(w_q T_q) from the exact
//                product of T_q and the binary64 weight's significand.  Error
//                below 0.5 ulp plus w_q 2^-58 (1/32 ulp for rho ~ 1).
//
// Either reports `bad` for a cell outside its range and the kernels evaluate
// that cell with the reference's binary64 expressions instead.
#pragma once
#include "hybrid.cuh"

namespace plbm {
namespace ex {

using hy::clz64;

DF_HD uint64_t umulhi(uint64_t a, uint64_t b) {
#ifdef __CUDA_ARCH__
  return __umul64hi(a, b);
#else
  return (uint64_t)(((unsigned __int128)a * b) >> 64);
#endif
}

DF_HD float rcp_approx(float x) {
#ifdef __CUDA_ARCH__
  float r;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
#else
  return 1.0f / x;
#endif
}

// The binary64 (-1)^neg n 2^(e2 - 63), n with bit 63 set, rounded to nearest
// even on the bits below n's top 53 and `sticky` (nonzero bits further down).
// The result must be a normal number.
DF_HD double pack_rne(uint64_t neg, uint64_t n, bool sticky, int e2) {
  uint64_t m = n >> 11;  // 53 bits, leading one at bit 52
  const uint64_t rb = (n >> 10) & 1ull;
  const uint64_t st = (uint64_t)(((n & 0x3FFull) != 0) | sticky);
  m += rb & (st | (m & 1ull));  // 2^53 carries into the exponent below
  return df::u2d((neg << 63) | (((uint64_t)(1022 + e2) << 52) + m));
}

// RN(T 2^-scale) of an int64 fixed-point value.
DF_HD double fixed_to_double_rne(int64_t T, int scale) {
  if (T == 0) return 0.0;
  const uint64_t neg = (uint64_t)T >> 63;
  const uint64_t a = neg ? (uint64_t)0 - (uint64_t)T : (uint64_t)T;
  const int lz = clz64(a);
  return pack_rne(neg, a << lz, false, 63 - lz - scale);
}

// binary64 d -> int64 d 2^SCALE, rounded to nearest (ties toward +inf) below
// 2^-SCALE; `bad` when |d| >= 2^(EMAX - 1022) or d is not finite.
template <int SCALE, int EMAX>
DF_HD int64_t to_fixed_rn(double d, bool& bad) {
  const uint64_t u = df::d2u(d);
  const int e = (int)((u >> 52) & 0x7FF);
  if (e > EMAX) {
    bad = true;
    return 0;
  }
  if (e == 0) return 0;  // zero or subnormal: below any fixed-point unit used here
  const uint64_t m = (u & 0xFFFFFFFFFFFFFull) | 0x10000000000000ull;
  const int sh = e - 1075 + SCALE;  // d 2^SCALE = m 2^sh
  const int64_t s = (u >> 63) ? -(int64_t)m : (int64_t)m;
  if (sh >= 0) return (int64_t)((uint64_t)s << sh);
  const int rs = -sh;
  return rs < 64 ? (s + ((int64_t)1 << (rs - 1))) >> rs : 0;
}

// ---- division ------------------------------------------------------------------
// The reciprocal of a divisor 1 <= b < 2^62: bn = b 2^lb (bit 63 set) and
// v ~ 2^127 / bn within a few units.  A binary32 seed refined once in
// double-float (~44 bits), then one Newton step on the integers
// (v += v (2^127 - bn v) / 2^127).
struct Recip {
  uint64_t b, bn, v;
  int lb;
};

DF_HD Recip recip(uint64_t b) {
  Recip r;
  r.b = b;
  r.lb = clz64(b);
  r.bn = b << r.lb;
  // bn / 2^64 in [1/2, 1) as bh + bl, its leading 48 bits (both exact)
  const float bh = hy::i2f((int32_t)(r.bn >> 40)) * 0x1p-24f;
  const float bl = hy::i2f((int32_t)((r.bn >> 16) & 0xFFFFFFull)) * 0x1p-48f;
  float y = fminf(rcp_approx(bh), 0x1.fffffcp0f);  // in (1, 2): v stays below 2^64
  float e = df::fmaf_(-bh, y, 1.0f);
  e = df::fmaf_(-bl, y, e);
  const float lo = y * e;  // 1 / (bh + bl) ~ y + lo
  // v1 = (y + lo) 2^63: y = my 2^(ey - 23) with a 24-bit my
  const uint32_t uy = df::f2u(y);
  const int ey = (int)(uy >> 23) - 127;  // 0, or -1 for a seed just below 1
  const uint64_t my = (uint64_t)((uy & 0x7FFFFFu) | 0x800000u);
  uint64_t v = (my << (40 + ey)) + (uint64_t)((int64_t)hy::f2i_trunc(lo * 0x1p44f) * ((int64_t)1 << 19));
  // E = 2^127 - bn v: |E| < 2^84 with the seed's 2^-22, below 2^91 for a
  // seed within 2^-18; E >> 28 as int64
  const uint64_t ph = umulhi(r.bn, v), pl = r.bn * v;
  const uint64_t ehi = (1ull << 63) - ph - (uint64_t)(pl != 0), elo = (uint64_t)0 - pl;
  const int64_t es = (int64_t)((ehi << 36) | (elo >> 28));
  // v E / 2^127 = ((v / 2) es / 2^64) / 2^34
#ifdef __CUDA_ARCH__
  const int64_t c = __mul64hi((int64_t)(v >> 1), es);
#else
  const int64_t c = (int64_t)(((__int128)(int64_t)(v >> 1) * es) >> 64);
#endif
  r.v = v + (uint64_t)(c >> 34);
  return r;
}

// RN(a / b) for |a| < 2^63 and the divisor of r.  `bad` if the estimate was
// off by more than the one correction step allows (not expected; the caller
// then evaluates the cell another way).
DF_HD double div_rn(int64_t sa, const Recip& r, bool& bad) {
  if (sa == 0) return 0.0;
  const uint64_t neg = (uint64_t)sa >> 63;
  const uint64_t a = neg ? (uint64_t)0 - (uint64_t)sa : (uint64_t)sa;
  const int la = clz64(a);
  const uint64_t an = a << la;
  // q = floor(an 2^s / bn) in [2^53, 2^54): s = 53 when an >= bn, else 54
  const int s = 54 - (int)(an >= r.bn);
  uint64_t q = umulhi(an, r.v) >> (63 - s);
  // exact remainder an 2^(s - lb) - q b (|.| < 2 b < 2^63) in wrapping arithmetic
  int64_t rem = (int64_t)((an << (s - r.lb)) - q * r.b);
  if (rem < 0) {
    q -= 1;
    rem += (int64_t)r.b;
  } else if (rem >= (int64_t)r.b) {
    q += 1;
    rem -= (int64_t)r.b;
  }
  bad |= (rem < 0) | (rem >= (int64_t)r.b);
  // a / b = (an / bn) 2^(lb - la) ~ q 2^(lb - la - s)
  return pack_rne(neg, q << 10, rem != 0, 53 + r.lb - la - s);
}

// ---- moments -------------------------------------------------------------------
// rho and u of one cell, correctly rounded from the exact sums of the
// fixed-point populations.  Unshifted: 0 <= f_q < 1 (update_macros,
// src/fvm_bardow.F90:368-382).  SHIFTED (h = f - w, lbm_macros of
// sim/sim.F90:160-173): |h_q| < 1/2, rho = 1 + sum h; small h rounded to
// 2^-59 (ties toward +inf).  Range: 2^32 <= R < 2^62 (2^-27 <= rho < 8).
template <bool SHIFTED>
DF_HD void macros_exact(const double (&f)[9], double& rho, double& ux, double& uy, bool& bad) {
  int64_t F[9];
#pragma unroll
  for (int q = 0; q < 9; q++) {
    if constexpr (SHIFTED) F[q] = hy::to_fixed_signed<1021>(f[q], bad);
    else F[q] = hy::to_fixed_nonneg<1022>(f[q], bad);
  }
  const int64_t d57 = F[5] - F[7], d86 = F[8] - F[6];
  int64_t R = ((F[1] + F[3]) + (F[2] + F[4])) + ((F[5] + F[7]) + (F[6] + F[8])) + F[0];
  if constexpr (SHIFTED) R += hy::kOne;
  const int64_t JX = (d57 + d86) + (F[1] - F[3]);
  const int64_t JY = (d57 - d86) + (F[2] - F[4]);
  bad |= (R < ((int64_t)1 << 32)) | (R >= ((int64_t)1 << 62));
  if (bad) return;
  rho = fixed_to_double_rne(R, hy::kScale);
  const Recip r = recip((uint64_t)R);
  ux = div_rn(JX, r, bad);
  uy = div_rn(JY, r, bad);
}

// ---- equilibrium ---------------------------------------------------------------
// RN(w T 2^-scale) for a positive binary64 weight w and |T| < 2^63: the exact
// product of T and w's 53-bit significand, rounded once.  SIGNED = false
// takes T >= 0 (the unshifted brackets) and skips the sign handling.
template <bool SIGNED = true>
DF_HD double weighted_rne(double w, int64_t T, int scale) {
  if (T == 0) return 0.0;
  const uint64_t neg = SIGNED ? (uint64_t)T >> 63 : 0ull;
  const uint64_t a = neg ? (uint64_t)0 - (uint64_t)T : (uint64_t)T;
  const uint64_t uw = df::d2u(w);
  const uint64_t mw = (uw & 0xFFFFFFFFFFFFFull) | 0x10000000000000ull;
  const int ew = (int)((uw >> 52) & 0x7FF) - 1075;  // w = mw 2^ew
  const uint64_t ph = umulhi(a, mw), pl = a * mw;  // a mw < 2^116
  if (ph == 0) {
    const int lz = clz64(pl);
    return pack_rne(neg, pl << lz, false, 63 - lz + ew - scale);
  }
  const int lz = clz64(ph);  // >= 12
  const uint64_t n = (ph << lz) | (pl >> (64 - lz));
  return pack_rne(neg, n, (pl << lz) != 0, 127 - lz + ew - scale);
}

// The reference's binary64 weights 4/9, 1/9, 1/36 (src/fvm_bardow.F90:90-92).
DF_HD double eq_weight(int q) { return q == 0 ? 4.0 / 9.0 : (q < 5 ? 1.0 / 9.0 : 1.0 / 36.0); }

constexpr int kEqScale = 60;
constexpr int64_t kEqOne = (int64_t)1 << kEqScale;

// The nine brackets T_q = rho (1 + 3 c_q.u + 4.5 (c_q.u)^2 - 1.5 u^2) at scale
// 2^60 from rho 2^60 (P) and u 2^62 (U, V):
//   X3, Y3 = 3 rho u, A = 1.5 rho ux^2, B = 1.5 rho uy^2, X = 4.5 rho ux uy
//   (each one product rounded to nearest: at most half a unit off),
//   T_0 = P - (A + B), T_(+-x) = P +- X3 + 2A - B, T_(+-y) = P +- Y3 + 2B - A,
//   T_(diag) = P + c.(X3, Y3) + 2 (A + B) +- 2 X,
// within 1 (rest), 2 (axis) and 4 (diagonal) units of 2^-60 of exact.
// Range: 0 < rho < 2, |ux|, |uy| < 1/4; then rho / 3 < T_q < 7 (no int64
// overflow in any term).
DF_HD void eq_brackets(int64_t P, int64_t U, int64_t V, int64_t (&T)[9]) {
  using hy::mul_shr;
  const int64_t X3 = mul_shr(3 * P, U, 62), Y3 = mul_shr(3 * P, V, 62);  // 3 rho u
  const int64_t A = mul_shr(X3, U, 63), B = mul_shr(Y3, V, 63), X = mul_shr(3 * X3, V, 63);
  const int64_t S = 2 * (A + B), X2 = 2 * X;
  const int64_t Cx = 2 * A - B, Cy = 2 * B - A;
  T[0] = P - (A + B);
  T[1] = P + X3 + Cx;
  T[3] = P - X3 + Cx;
  T[2] = P + Y3 + Cy;
  T[4] = P - Y3 + Cy;
  T[5] = P + (X3 + Y3) + S + X2;
  T[7] = P - (X3 + Y3) + S + X2;
  T[6] = P - (X3 - Y3) + S - X2;
  T[8] = P + (X3 - Y3) + S - X2;
}

// feq_q (SHIFTED = false) or h_q = feq_q - w_q (SHIFTED) of rho and u.  With
// SHIFTED the bracket loses 1 exactly before the weight is applied:
// h_q = RN(w_q (T_q - 1)), the equilibrium of sim/sim.F90:357-384 (which is
// w rho (...) + w (rho - 1) with indp = -1.5 u^2).  P = rho 2^60
// (rho_fixed, or rho_fixed_from_pressure for a pressure field).
template <bool SHIFTED>
DF_HD void equilibrium_exact(int64_t P, double ux, double uy, double (&out)[9], bool& bad) {
  const int64_t U = to_fixed_rn<62, 1020>(ux, bad), V = to_fixed_rn<62, 1020>(uy, bad);
  bad |= (P <= 0) | (P >= 2 * kEqOne);
  if (bad) return;
  int64_t T[9];
  eq_brackets(P, U, V, T);
#pragma unroll
  for (int q = 0; q < 9; q++) out[q] = weighted_rne<SHIFTED>(eq_weight(q), SHIFTED ? T[q] - kEqOne : T[q], kEqScale);
}

// rho 2^60 of a binary64 rho (0 < rho < 2).
DF_HD int64_t rho_fixed(double rho, bool& bad) {
  const int64_t P = to_fixed_rn<kEqScale, 1023>(rho, bad);
  bad |= P <= 0;
  return P;
}

// rho 2^60 = 2^60 + p / cs^2 with the reference's binary64 cs^2 = RN(1/3)
// = (1 - 2^-54) / 3 (sim/sim.F90:193): p / cs^2 = 3p (1 + 2^-54 + 2^-108 ...),
// the last terms below 2^-100 p; formed at 2^62 and rounded to 2^-60 (within
// one unit of 2^-60; 5/8 for |p| >= 2^-10).  Range |p| < 1/4.
DF_HD int64_t rho_fixed_from_pressure(double p, bool& bad) {
  int64_t t = 3 * to_fixed_rn<kEqScale + 2, 1020>(p, bad);
  t += (t + ((int64_t)1 << 53)) >> 54;
  return kEqOne + ((t + 2) >> 2);
}

}  // namespace ex
}  // namespace plbm
