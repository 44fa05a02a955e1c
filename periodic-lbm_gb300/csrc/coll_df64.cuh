// coll_df64.cuh -- collision operators in double-float arithmetic on the
// shifted populations h_q = f_q - w_q.
//
// A binary64 population f_q is brought in as h_q = f_q - w_q (one binary64
// subtraction, exact whenever f_q is within a factor two of w_q, i.e. for
// every physical state) and split into a df64 pair; the collision is evaluated
// in df64; the result is packed back to binary64 and w_q added (one binary64
// addition, the single rounding of the stored value).  Working on h keeps the
// roughly 48-bit df64 precision relative to |h| (~1e-2), i.e. absolute errors
// around 1e-17, below the binary64 spacing of f itself.
//
// The operators are algebraic rewrites of the reference kernels
// (src/collision_bgk.F90:58-71, src/collision_trt.F90:98-152,
// src/collision_regularized.F90:72-194) for h = f - w; they agree with them
// to rounding (the parity tests bound the difference at 1e-12).
#pragma once
#include "df64.cuh"

namespace plbm {
namespace df {

// df64 constants of one launch, formed on the host.
struct DfParams {
  df64 om, omb;        // omega, 1 - omega (BGK, RR); TRT: lambda_e, 1 - lambda_e
  df64 les, lds;       // TRT: 0.5 lambda_e, 0.5 lambda_d
  df64 rr0, rrs, rrd;  // RR: w (1 - omega)
  df64 w0, ws, wd;     // 4/9, 1/9, 1/36
  df64 ws3, wd3;       // 3/9, 3/36
  double w0d, wsd, wdd;  // the same weights in binary64 for the I/O shift
};

// BGK, src/collision_bgk.F90:58-71 with equilibrium() of
// src/fvm_bardow.F90:99-126, for h = f - w:
//   rho = 1 + sum h,  u = j / rho,
//   heq_q = w_q [ drho + 3 c_q.j + rho (4.5 (c_q.u)^2 - 1.5 u^2) ]
//   h'_q  = (1 - omega) h_q + omega heq_q
DF_HD void bgk(df64 (&h)[9], const DfParams& p) {
  const df64 s13 = add(h[1], h[3]), s24 = add(h[2], h[4]);
  const df64 s57 = add(h[5], h[7]), s68 = add(h[6], h[8]);
  const df64 drho = add(add(add(s57, s68), add(s13, s24)), h[0]);
  const df64 d13 = sub(h[1], h[3]), d24 = sub(h[2], h[4]);
  const df64 d57 = sub(h[5], h[7]), d86 = sub(h[8], h[6]);
  const df64 jx = add(add(d57, d86), d13);
  const df64 jy = add(sub(d57, d86), d24);
  const df64 rho = add_f(drho, 1.0f);
  const df64 inv = recip(rho);
  const df64 ux = mul(jx, inv), uy = mul(jy, inv);
  const df64 u2_15 = mul_f(add(sqr(ux), sqr(uy)), 1.5f);
  // rest population
  {
    const df64 heq = mul(p.w0, sub(drho, mul(rho, u2_15)));
    h[0] = add(mul(p.omb, h[0]), mul(p.om, heq));
  }
  // a +/- pair: c.u = +-cu, c.j = +-cj, weight w, 3w
#define PLBM_DF_PAIR(QP, QM, CU, CJ, W, W3)                                          \
  {                                                                                  \
    const df64 g = mul(rho, sub(mul_f(sqr(CU), 4.5f), u2_15));                       \
    const df64 omA = mul(p.om, mul(W, add(drho, g)));                                \
    const df64 omB = mul(p.om, mul(W3, CJ));                                         \
    h[QP] = add(add(mul(p.omb, h[QP]), omA), omB);                                   \
    h[QM] = sub(add(mul(p.omb, h[QM]), omA), omB);                                   \
  }
  PLBM_DF_PAIR(1, 3, ux, jx, p.ws, p.ws3)
  PLBM_DF_PAIR(2, 4, uy, jy, p.ws, p.ws3)
  PLBM_DF_PAIR(5, 7, add(ux, uy), add(jx, jy), p.wd, p.wd3)
  PLBM_DF_PAIR(8, 6, sub(ux, uy), sub(jx, jy), p.wd, p.wd3)
#undef PLBM_DF_PAIR
}

// ---- compensated binary32 BGK for deviation storage --------------------------
// The result is rounded to binary32 (or binary16) storage, so the collision
// only needs to be accurate well below the spacing of the stored h, not to
// 48 bits.  The O(h) linear part of the update -- moments, w (drho +- 3 c.j),
// (1-omega) h -- is carried as an unnormalised hi+lo pair (lazy double-float:
// no renormalisation, ~44 bits); the nonlinear term
// omega w rho (4.5 (c.u)^2 - 1.5 u^2), at most ~1e-3, is plain binary32.
struct DevParams {
  df64 w[3];     // w0, ws, wd as double-float
  df64 w3[3];    // 3 w
  float om_hi;   // omega = om_hi + om_lo
  float om_lo;
};

DF_HD df64 add_lazy(df64 a, df64 b) {
  df64 s = two_sum(a.hi, b.hi);
  s.lo += a.lo + b.lo;
  return s;
}
DF_HD df64 mul_lazy(df64 a, df64 b) {
  df64 p = two_prod(a.hi, b.hi);
  p.lo = fmaf_(a.hi, b.lo, p.lo);
  p.lo = fmaf_(a.lo, b.hi, p.lo);
  return p;
}
DF_HD df64 mul_lazy_f(df64 a, float b) {
  df64 p = two_prod(a.hi, b);
  p.lo = fmaf_(a.lo, b, p.lo);
  return p;
}

// h + omega d rounded once: t = RN(h + om_hi d), its rounding error from one
// more FMA (h - t is exact, t being close to h), plus om_lo d.  Rounding omega
// to binary32 instead biased the relaxation rate by ~1e-8, which at
// tau = 0.52 (viscosity 26x as sensitive as omega) let the shear layer's
// velocity error grow to 1e-6 over 20,000 steps.
DF_HD float relax(float h, float d, float om_hi, float om_lo) {
  const float t = fmaf_(om_hi, d, h);
  const float c = fmaf_(om_lo, d, fmaf_(om_hi, d, h - t));
  return t + c;
}

// The update of a pair (q, qbar = -q): heq = a +- b with a = w (drho + rho nl_q)
// (nl_q = 4.5 (c_q.u)^2 - 1.5 u^2) and b = 3 w c_q.j.  With the pair's exact
// sum S = h_q + h_qbar and difference D = h_q - h_qbar (the error-free sums
// the moments are built from),
//   heq_q - h_q = (a - S/2) + (b - D/2),  heq_qbar - h_qbar = (a - S/2) - (b - D/2):
// a - S/2 and b - D/2 are the symmetric and antisymmetric non-equilibrium
// parts, small against a and b, so their high parts subtract exactly (the
// operands are within a factor two; the FMA with -1/2 forms S/2 exactly) and
// their low parts add in binary32.  This replaces the double-float sums
// a + b, a - b of the two equilibria and 12 binary32 operations per pair.
DF_HD void bgk_dev_comp(float (&h)[9], const DevParams& p) {
  // exact pairwise sums and differences of the stored values
  const df64 s13 = two_sum(h[1], h[3]), s24 = two_sum(h[2], h[4]);
  const df64 s57 = two_sum(h[5], h[7]), s68 = two_sum(h[6], h[8]);
  const df64 d13 = two_sum(h[1], -h[3]), d24 = two_sum(h[2], -h[4]);
  const df64 d57 = two_sum(h[5], -h[7]), d86 = two_sum(h[8], -h[6]);
  const df64 drho = add_lazy(add_lazy(add_lazy(s57, s68), add_lazy(s13, s24)), make(h[0], 0.0f));
  const df64 jx = add_lazy(add_lazy(d57, d86), d13);
  const df64 jy = add_lazy(add_lazy(d57, neg(d86)), d24);
  // nonlinear part in binary32: u = j / (1 + drho)
  const float dr = drho.hi + drho.lo;
  const float inv = 1.0f / (1.0f + dr);
  const float jxf = jx.hi + jx.lo, jyf = jy.hi + jy.lo;
  const float ux = jxf * inv, uy = jyf * inv;
  const float rho = 1.0f + dr;
  const float u2 = 1.5f * (ux * ux + uy * uy);
  // h' = h + omega (heq - h), heq = w (drho + rho (4.5 (c.u)^2 - 1.5 u^2)) + 3 w c.j.
  // The equilibrium's O(h) part is formed in double-float, the nonlinear term
  // (binary32) joining the exact drho before the product with w (binary32
  // weights in that product biased the relaxation rate by ~1e-8); heq - h is a
  // small difference of nearby values and takes binary32; relax() adds
  // omega (heq - h) with one rounding, to the storage format.
  {
    const df64 e = mul_lazy(p.w[0], add_lazy(drho, make(rho * -u2, 0.0f)));
    h[0] = relax(h[0], (e.hi - h[0]) + e.lo, p.om_hi, p.om_lo);
  }
#define PLBM_COMP_PAIR(QP, QM, CUF, CJ, S, D, WI)                                                       \
  {                                                                                                    \
    const float cu = (CUF);                                                                            \
    const df64 a = mul_lazy(p.w[WI], add_lazy(drho, make(rho * fmaf_(4.5f * cu, cu, -u2), 0.0f)));    \
    const df64 b = mul_lazy(p.w3[WI], CJ);                                                             \
    const float sym = fmaf_(-0.5f, S.hi, a.hi) + fmaf_(-0.5f, S.lo, a.lo);                             \
    const float asym = fmaf_(-0.5f, D.hi, b.hi) + fmaf_(-0.5f, D.lo, b.lo);                            \
    h[QP] = relax(h[QP], sym + asym, p.om_hi, p.om_lo);                                                \
    h[QM] = relax(h[QM], sym - asym, p.om_hi, p.om_lo);                                                \
  }
  PLBM_COMP_PAIR(1, 3, ux, jx, s13, d13, 1)
  PLBM_COMP_PAIR(2, 4, uy, jy, s24, d24, 1)
  PLBM_COMP_PAIR(5, 7, ux + uy, add_lazy(jx, jy), s57, d57, 2)
  PLBM_COMP_PAIR(8, 6, ux - uy, add_lazy(jx, neg(jy)), s68, d86, 2)
#undef PLBM_COMP_PAIR
}

// ---- compensated binary32 reverse step of the BGK adjoint ---------------------
// One cell of the discrete adjoint's reverse step on binary32 deviation
// storage: g = the pulled pre-collision populations (h = f - w), l = lambda_{n+1}
// at the cell.  Returns mu (the nine values scattered to lambda_n) and the
// cell's dL/domega term sum_q lambda_q (feq_q - g_q).  The BGK Jacobian
// transpose, mu_q = lambda_q + omega (X_q - lambda_q) with
//   X_q = A + c_q.E,  A = S0 - N,  E = 3 M1 + 9 Q - 3 S0 u,
//   S0 = sum w lambda, M1 = sum w lambda c, Q = sum w lambda (c.u) c,
//   N = sum w lambda (4.5 (c.u)^2 - 1.5 u^2),
// is evaluated like the compensated forward collision: S0 and 3 M1 (the O(lambda)
// terms) in double-float from exact pairwise sums of lambda, Q and N (O(u lambda))
// in binary32, and X_q - lambda_q of each pair from the pair's exact sum and
// difference, (S0 - L/2 - N) +- (c.3M1 - D/2 + c.F), so that only the small
// non-equilibrium part of lambda is rounded before the single rounding of mu.
// feq_q - g_q takes the forward's pair form.
struct AdjDevParams {
  df64 w[3], w3[3];  // w0, ws, wd and 3 w as double-float
  float om_hi, om_lo;
};

DF_HD float adj_step_comp(const float (&g)[9], const float (&l)[9], float (&mu)[9], const AdjDevParams& p) {
  // forward state of the cell
  const df64 s13 = two_sum(g[1], g[3]), s24 = two_sum(g[2], g[4]);
  const df64 s57 = two_sum(g[5], g[7]), s68 = two_sum(g[6], g[8]);
  const df64 d13 = two_sum(g[1], -g[3]), d24 = two_sum(g[2], -g[4]);
  const df64 d57 = two_sum(g[5], -g[7]), d86 = two_sum(g[8], -g[6]);
  const df64 drho = add_lazy(add_lazy(add_lazy(s57, s68), add_lazy(s13, s24)), make(g[0], 0.0f));
  const df64 jx = add_lazy(add_lazy(d57, d86), d13);
  const df64 jy = add_lazy(add_lazy(d57, neg(d86)), d24);
  const float dr = drho.hi + drho.lo;
  const float inv = 1.0f / (1.0f + dr);
  const float ux = (jx.hi + jx.lo) * inv, uy = (jy.hi + jy.lo) * inv;
  const float rho = 1.0f + dr;
  const float u2 = 1.5f * (ux * ux + uy * uy);
  const float upp = ux + uy, upm = ux - uy;
  // exact pairwise sums and differences of lambda
  const df64 L13 = two_sum(l[1], l[3]), L24 = two_sum(l[2], l[4]);
  const df64 L57 = two_sum(l[5], l[7]), L68 = two_sum(l[6], l[8]);
  const df64 M13 = two_sum(l[1], -l[3]), M24 = two_sum(l[2], -l[4]);
  const df64 M57 = two_sum(l[5], -l[7]), M86 = two_sum(l[8], -l[6]);
  // S0 and 3 M1 in double-float
  const df64 S0 = add_lazy(add_lazy(mul_lazy(p.w[1], add_lazy(L13, L24)), mul_lazy(p.w[2], add_lazy(L57, L68))),
                           mul_lazy_f(p.w[0], l[0]));
  const df64 Mp = add_lazy(M57, M86), Mm = add_lazy(M57, neg(M86));
  const df64 E3x = add_lazy(mul_lazy(p.w3[1], M13), mul_lazy(p.w3[2], Mp));
  const df64 E3y = add_lazy(mul_lazy(p.w3[1], M24), mul_lazy(p.w3[2], Mm));
  // O(u lambda) terms in binary32
  const float ws = p.w[1].hi, wd = p.w[2].hi;
  const float l13 = L13.hi + L13.lo, l24 = L24.hi + L24.lo, l57 = L57.hi + L57.lo, l68 = L68.hi + L68.lo;
  const float s0 = S0.hi + S0.lo;
  const float Qx = ws * ux * l13 + wd * (upp * l57 + upm * l68);
  const float Qy = ws * uy * l24 + wd * (upp * l57 - upm * l68);
  const float N = 4.5f * (ws * (ux * ux * l13 + uy * uy * l24) + wd * (upp * upp * l57 + upm * upm * l68)) - u2 * s0;
  const float Fx = 9.0f * Qx - 3.0f * s0 * ux, Fy = 9.0f * Qy - 3.0f * s0 * uy;
  float dterm;
  {  // rest population
    const df64 e = mul_lazy(p.w[0], add_lazy(drho, make(rho * -u2, 0.0f)));
    dterm = l[0] * ((e.hi - g[0]) + e.lo);
    mu[0] = relax(l[0], ((S0.hi - l[0]) + S0.lo) - N, p.om_hi, p.om_lo);
  }
#define PLBM_ADJ_PAIR(QP, QM, CUF, CJ, S, D, WI, LS, LD, E3C, CF)                                      \
  {                                                                                                   \
    const float cu = (CUF);                                                                           \
    const df64 a = mul_lazy(p.w[WI], add_lazy(drho, make(rho * fmaf_(4.5f * cu, cu, -u2), 0.0f)));   \
    const df64 b = mul_lazy(p.w3[WI], CJ);                                                            \
    const float sym = fmaf_(-0.5f, S.hi, a.hi) + fmaf_(-0.5f, S.lo, a.lo);                            \
    const float asym = fmaf_(-0.5f, D.hi, b.hi) + fmaf_(-0.5f, D.lo, b.lo);                           \
    dterm += (l[QP] + l[QM]) * sym + (l[QP] - l[QM]) * asym;                                          \
    const df64 e3 = (E3C);                                                                            \
    const float ls = (fmaf_(-0.5f, LS.hi, S0.hi) + fmaf_(-0.5f, LS.lo, S0.lo)) - N;                   \
    const float la = (fmaf_(-0.5f, LD.hi, e3.hi) + fmaf_(-0.5f, LD.lo, e3.lo)) + (CF);                \
    mu[QP] = relax(l[QP], ls + la, p.om_hi, p.om_lo);                                                 \
    mu[QM] = relax(l[QM], ls - la, p.om_hi, p.om_lo);                                                 \
  }
  PLBM_ADJ_PAIR(1, 3, ux, jx, s13, d13, 1, L13, M13, E3x, Fx)
  PLBM_ADJ_PAIR(2, 4, uy, jy, s24, d24, 1, L24, M24, E3y, Fy)
  PLBM_ADJ_PAIR(5, 7, upp, add_lazy(jx, jy), s57, d57, 2, L57, M57, add_lazy(E3x, E3y), Fx + Fy)
  PLBM_ADJ_PAIR(8, 6, upm, add_lazy(jx, neg(jy)), s68, d86, 2, L68, M86, add_lazy(E3x, neg(E3y)), Fx - Fy)
#undef PLBM_ADJ_PAIR
  return dterm;
}

}  // namespace df
}  // namespace plbm
