// schemes.cuh -- the finite-volume / finite-difference streaming formulas of
// src/fvm_bardow.F90:393-886 as one function of a population's 3x3
// neighbourhood, usable on host and device.
//
// The neighbourhood of population q at (x, y) is v[k] = f_q(x + ex_k, y + ey_k)
// in the order c, e, n, w, s, ne, nw, sw, se (the reference's fc, fe, fn, fw,
// fs, fne, fnw, fsw, fse).  scheme_value() evaluates the reference's
// expression for the new f_q in the reference's association; the kernels of
// the strict build call it directly.
//
// Every scheme is linear in v, so scheme_value(delta_k) is the coefficient of
// v[k]; stencil_coefficients() tabulates them (9 per population) for the
// stencil-form kernels of the FMA and hybrid builds, which then need 9 fused
// multiply-adds per population.
#pragma once
#include <math.h>

#ifdef __CUDACC__
#define SCH_HD __host__ __device__ __forceinline__
#else
#define SCH_HD inline
#endif

namespace plbm {
namespace sch {

enum { FVM = 1, FDM = 2, FDM_ISO = 3, FDM_WLS = 4, SOFONEA = 5, FDM_WLS_G1 = 6, FDM_WLS_G2 = 7 };
enum { C = 0, E = 1, N = 2, W = 3, S = 4, NE = 5, NW = 6, SW = 7, SE = 8 };

// Neighbour offsets of the order above.
SCH_HD int ex(int k) { return k == E || k == NE || k == SE ? 1 : (k == W || k == NW || k == SW ? -1 : 0); }
SCH_HD int ey(int k) { return k == N || k == NE || k == NW ? 1 : (k == S || k == SW || k == SE ? -1 : 0); }
// The neighbour at offset (dx, dy).
SCH_HD int nb(int dx, int dy) {
  if (dx == 0) return dy > 0 ? N : (dy < 0 ? S : C);
  if (dx > 0) return dy > 0 ? NE : (dy < 0 ? SE : E);
  return dy > 0 ? NW : (dy < 0 ? SW : W);
}

SCH_HD double qcx(int q) { return (double)((q == 1 || q == 5 || q == 8) ? 1 : (q == 3 || q == 6 || q == 7) ? -1 : 0); }
SCH_HD double qcy(int q) { return (double)((q == 2 || q == 5 || q == 6) ? 1 : (q == 4 || q == 7 || q == 8) ? -1 : 0); }

// New f_q (q = 1..8) of scheme `scheme` from the neighbourhood v.
SCH_HD double scheme_value(int scheme, const double (&v)[9], int q, double dt) {
  const double cxq = dt * qcx(q), cyq = dt * qcy(q);
  const double fc = v[C];
  if (scheme == SOFONEA) {
    // stream_fdm_sofonea, src/fvm_bardow.F90:721-882: fu = f(x + c), fd = f(x - c)
    const int cxi = (int)qcx(q), cyi = (int)qcy(q);
    const double fu = v[nb(cxi, cyi)], fd = v[nb(-cxi, -cyi)];
    double du1, du2;
    if (q <= 4) {
      du1 = 0.5 * (fu - fd);
      du2 = fu - 2 * fc + fd;
    } else {
      const double p2 = 0.35355339059327373;  // 0.5/sqrt(2) rounded to binary64 (:713)
      du1 = p2 * (fu - fd);
      du2 = 0.5 * (fu - 2 * fc + fd);
    }
    return fc + dt * (0.5 * dt * du2 - du1);
  }
  const double fe = v[E], fn = v[N], fw = v[W], fs = v[S], fne = v[NE], fnw = v[NW], fsw = v[SW], fse = v[SE];
  if (scheme == FVM) {
    // stream_fvm_bardow, src/fvm_bardow.F90:459-494: bilinear face values
    const double p2 = 0.5, p8 = 0.125;
    const double cfw = p2 * (fc + fw) - p2 * cxq * (fc - fw) - p8 * cyq * (fnw + fn - fsw - fs);
    const double cfn = p2 * (fc + fn) - p2 * cyq * (fn - fc) - p8 * cxq * (fne + fe - fnw - fw);
    const double cfe = p2 * (fc + fe) - p2 * cxq * (fe - fc) - p8 * cyq * (fne + fn - fse - fs);
    const double cfs = p2 * (fc + fs) - p2 * cyq * (fc - fs) - p8 * cxq * (fse + fe - fsw - fw);
    return fc - cxq * (cfe - cfw) - cyq * (cfn - cfs);
  }
  // stream_fdm_bardow, src/fvm_bardow.F90:563-678
  const double cxxq = 0.5 * cxq * cxq, cyyq = 0.5 * cyq * cyq, cxyq = cxq * cyq;
  double dfx, dfy, dfxx, dfyy, dfxy;
  if (scheme == FDM_ISO) {
    const double p2 = 0.5, two_thirds = 2.0 / 3.0, one_sixth = 1.0 / 6.0, five_sixths = 10.0 / 12.0,
                 one_twelth = 1.0 / 12.0;
    dfx = p2 * (one_sixth * (fne - fnw) + two_thirds * (fe - fw) + one_sixth * (fse - fsw));
    dfy = p2 * (one_sixth * (fne - fse) + two_thirds * (fn - fs) + one_sixth * (fnw - fsw));
    dfxx = one_twelth * (fne - 2 * fn + fnw) + five_sixths * (fe - 2 * fc + fw) + one_twelth * (fse - 2 * fs + fsw);
    dfyy = one_twelth * (fne - 2 * fe + fse) + five_sixths * (fn - 2 * fc + fs) + one_twelth * (fnw - 2 * fw + fsw);
    dfxy = 0.25 * (fne - fse - fnw + fsw);
  } else if (scheme == FDM_WLS) {
    const double one_sixth = 1.0 / 6.0, one_third = 1.0 / 3.0;
    dfx = one_sixth * ((fne - fnw) + (fe - fw) + (fse - fsw));
    dfy = one_sixth * ((fne - fse) + (fn - fs) + (fnw - fsw));
    dfxx = one_third * (fne - 2 * fn + fnw) + one_third * (fe - 2 * fc + fw) + one_third * (fse - 2 * fs + fsw);
    dfyy = one_third * (fne - 2 * fe + fse) + one_third * (fn - 2 * fc + fs) + one_third * (fnw - 2 * fw + fsw);
    dfxy = 0.25 * (fne - fnw + fsw - fse);
  } else if (scheme == FDM_WLS_G1 || scheme == FDM_WLS_G2) {
    // Gaussian-weighted least squares: FDM_WLS_GAUSS_V1 (weight scaled to the
    // farthest node, src/fvm_bardow.F90:604-624) and FDM_WLS_GAUSS_V2 (to the
    // closest node, :625-644); the fitted weights are the reference's binary64
    // constants.
    const bool v1 = scheme == FDM_WLS_G1;
    const double p1s = v1 ? 0.2880584423829145035434 : 0.3934930210807994210853;
    const double p1d = v1 ? 0.1059707788085427065949 : 0.05325348945960039354075;
    const double p2c = v1 ? -1.152233769531658458263 : -1.573972084323197018207;
    const double p2d1 = v1 ? 0.5761168847658292291314 : 0.7869860421615988421706;
    const double p2d2 = v1 ? -0.4238831152341712149578 : -0.2130139578384016019186;
    const double p2d = v1 ? 0.2119415576170855242122 : 0.1065069789192007732037;
    dfx = p1s * (fe - fw) + p1d * (fne - fnw) + p1d * (fse - fsw);
    dfy = p1s * (fn - fs) + p1d * (fne - fse) + p1d * (fnw - fsw);
    dfxx = p2c * fc + p2d1 * (fe + fw) + p2d2 * (fn + fs) + p2d * (fne + fnw + fsw + fse);
    dfyy = p2c * fc + p2d2 * (fe + fw) + p2d1 * (fn + fs) + p2d * (fne + fnw + fsw + fse);
    dfxy = 0.25 * (fne - fnw + fsw - fse);
  } else {
    dfx = 0.5 * (fe - fw);
    dfy = 0.5 * (fn - fs);
    dfxx = fe - 2 * fc + fw;
    dfyy = fn - 2 * fc + fs;
    dfxy = 0.25 * (fne - fse - fnw + fsw);
  }
  return fc - cxq * dfx - cyq * dfy + (cxxq * dfxx + cxyq * dfxy + cyyq * dfyy);
}

// Stencil coefficients a[q][k] (q = 1..8; row 0 is the identity) of the
// scheme at time step dt.
struct Stencil {
  double a[9][9];
};

inline Stencil stencil_coefficients(int scheme, double dt) {
  Stencil s;
  for (int q = 0; q < 9; q++)
    for (int k = 0; k < 9; k++) s.a[q][k] = 0.0;
  s.a[0][C] = 1.0;
  for (int q = 1; q < 9; q++)
    for (int k = 0; k < 9; k++) {
      double v[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
      v[k] = 1.0;
      s.a[q][k] = scheme_value(scheme, v, q, dt);
    }
  return s;
}

#ifdef __CUDACC__
// The 3x3 neighbourhood of population q around (x, y) of a YFast lattice
// (xp/xm/yp/ym: the periodic neighbours).  Unused entries are dead loads the
// compiler drops.
template <class L>
__device__ __forceinline__ void gather(const double* __restrict__ a, int q, int x, int y, int xp, int xm, int yp,
                                       int ym, int nx, int ny, int ld, double (&v)[9]) {
  v[C] = __ldg(a + L::off(x, y, q, nx, ny, ld));
  v[E] = __ldg(a + L::off(xp, y, q, nx, ny, ld));
  v[N] = __ldg(a + L::off(x, yp, q, nx, ny, ld));
  v[W] = __ldg(a + L::off(xm, y, q, nx, ny, ld));
  v[S] = __ldg(a + L::off(x, ym, q, nx, ny, ld));
  v[NE] = __ldg(a + L::off(xp, yp, q, nx, ny, ld));
  v[NW] = __ldg(a + L::off(xm, yp, q, nx, ny, ld));
  v[SW] = __ldg(a + L::off(xm, ym, q, nx, ny, ld));
  v[SE] = __ldg(a + L::off(xp, ym, q, nx, ny, ld));
}

// Tap patterns of the stencil form:
//   TAPS_FULL  all nine taps for every population (FDM isotropic / least squares)
//   TAPS_AXIS3 three taps (c and the two along the axis) for the axis
//              populations, nine for the diagonal ones (FVM, FDM central: their
//              cross-direction terms carry a factor cy_q or cx_q = 0, so the
//              other coefficients are exactly zero)
//   TAPS_LINE  three taps along c_q for every population (Sofonea)
enum { TAPS_FULL = 0, TAPS_AXIS3 = 1, TAPS_LINE = 2 };

inline int taps_of(int scheme) {
  return scheme == SOFONEA ? TAPS_LINE : (scheme == FVM || scheme == FDM) ? TAPS_AXIS3 : TAPS_FULL;
}

// Streamed populations of cell (x, y) in stencil form: f_q = sum_k a[q][k] v_k
// with explicit fused multiply-adds (the same result in every build).
template <class L, int TAPS>
__device__ __forceinline__ void stencil_pull(const double* __restrict__ src, int x, int y, int nx, int ny, int ld,
                                             const Stencil& st, double (&f)[9]) {
  const int xp = x + 1 == nx ? 0 : x + 1, xm = x == 0 ? nx - 1 : x - 1;
  const int yp = y + 1 == ny ? 0 : y + 1, ym = y == 0 ? ny - 1 : y - 1;
  f[0] = __ldg(src + L::off(x, y, 0, nx, ny, ld));
#pragma unroll
  for (int q = 1; q < 9; q++) {
    double v[9];
    gather<L>(src, q, x, y, xp, xm, yp, ym, nx, ny, ld, v);
    if (TAPS == TAPS_LINE || (TAPS == TAPS_AXIS3 && q <= 4)) {
      const int cxi = (int)qcx(q), cyi = (int)qcy(q);
      const int ku = nb(cxi, cyi), kd = nb(-cxi, -cyi);
      f[q] = __fma_rn(st.a[q][kd], v[kd], __fma_rn(st.a[q][ku], v[ku], st.a[q][C] * v[C]));
    } else {
      double acc = st.a[q][C] * v[C];
#pragma unroll
      for (int k = 1; k < 9; k++) acc = __fma_rn(st.a[q][k], v[k], acc);
      f[q] = acc;
    }
  }
}
#endif

}  // namespace sch
}  // namespace plbm
