// plbm_device.cuh -- device building blocks of the D2Q9 periodic hot path:
// lattice constants, the two lattice layouts, storage conversion, and the
// per-cell collision operators.
//
// Velocity set and weights follow src/fvm_bardow.F90:87-92:
//   q : 0  1  2  3  4  5  6  7  8
//   cx: 0  1  0 -1  0  1 -1 -1  1
//   cy: 0  0  1  0 -1  1  1 -1 -1
//   w : 4/9, 1/9 (q=1..4), 1/36 (q=5..8)
//
// The binary64 "reference" operators (coll_*_ref) evaluate exactly the
// expressions of the Fortran kernels they cite, with the Fortran association
// (left to right, parentheses kept).  Compiled with --fmad=false they perform
// the same IEEE operations as the Fortran built without FMA contraction and
// give bit-identical results; compiled with contraction they differ by
// rounding only.
#pragma once
#include <cuda_runtime.h>
#include <cuda_fp16.h>
#include <stdint.h>

namespace plbm {

constexpr double W0 = 4.0 / 9.0;
constexpr double WS = 1.0 / 9.0;
constexpr double WD = 1.0 / 36.0;
constexpr double CSQR = 1.0 / 3.0;

__host__ __device__ constexpr int cx_of(int q) {
  return q == 1 || q == 5 || q == 8 ? 1 : (q == 3 || q == 6 || q == 7 ? -1 : 0);
}
__host__ __device__ constexpr int cy_of(int q) {
  return q == 2 || q == 5 || q == 6 ? 1 : (q == 4 || q == 7 || q == 8 ? -1 : 0);
}
__host__ __device__ constexpr double w_of(int q) { return q == 0 ? W0 : (q < 5 ? WS : WD); }
__host__ __device__ constexpr float wf_of(int q) {
  return q == 0 ? 4.0f / 9.0f : (q < 5 ? 1.0f / 9.0f : 1.0f / 36.0f);
}

// ---------------------------------------------------------------------------
// Layouts.  YFast is the src/ convention f(ld,nx,0:8): offset y + ld*(x + nx*q).
// XFast is the sim/ plugin convention without halo: offset x + ld*(y + ny*q)
// with ld = nx rounded up to 16.  `ld` is the padded fast extent in both.
struct YFast {
  static constexpr bool x_fast = false;
  __device__ __forceinline__ static size_t off(int x, int y, int q, int nx, int ny, int ld) {
    return (size_t)y + (size_t)ld * ((size_t)x + (size_t)nx * (size_t)q);
  }
  __device__ __forceinline__ static size_t plane(int nx, int ny, int ld) { return (size_t)ld * nx; }
  // cell offset within a plane
  __device__ __forceinline__ static size_t cell(int x, int y, int ld) { return (size_t)y + (size_t)ld * x; }
};
struct XFast {
  static constexpr bool x_fast = true;
  __device__ __forceinline__ static size_t off(int x, int y, int q, int nx, int ny, int ld) {
    return (size_t)x + (size_t)ld * ((size_t)y + (size_t)ny * (size_t)q);
  }
  __device__ __forceinline__ static size_t plane(int nx, int ny, int ld) { return (size_t)ld * ny; }
  __device__ __forceinline__ static size_t cell(int x, int y, int ld) { return (size_t)x + (size_t)ld * y; }
};

// Periodic neighbours by index arithmetic (no modulo): the 0-based forms of
// the reference maps xp1 = mod(x,nx)+1, xm1 = mod(nx+x-2,nx)+1
// (src/periodic_lbm.f90:63-64,79-80).
__device__ __forceinline__ int wrap_p(int v, int n) { return v + 1 == n ? 0 : v + 1; }
__device__ __forceinline__ int wrap_m(int v, int n) { return v == 0 ? n - 1 : v - 1; }
__device__ __forceinline__ int wrap_add(int v, int d, int n) {
  return d > 0 ? wrap_p(v, n) : (d < 0 ? wrap_m(v, n) : v);
}

// ---------------------------------------------------------------------------
// Storage traits: how one population is held in HBM.
struct StoreF64 {
  typedef double elem;
  typedef double real;
  static constexpr bool ddf = false;
  __device__ __forceinline__ static double load(const double* p, size_t i) { return __ldg(p + i); }
  __device__ __forceinline__ static void store(double* p, size_t i, double v) { p[i] = v; }
};
// binary64 populations stored shifted (h = f - w), sim/sim.F90:131
struct StoreF64Shift {
  typedef double elem;
  typedef double real;
  static constexpr bool ddf = true;
  __device__ __forceinline__ static double load(const double* p, size_t i) { return __ldg(p + i); }
  __device__ __forceinline__ static void store(double* p, size_t i, double v) { p[i] = v; }
};
struct StoreF32Dev {
  typedef float elem;
  typedef float real;
  static constexpr bool ddf = true;
  __device__ __forceinline__ static float load(const float* p, size_t i) { return __ldg(p + i); }
  __device__ __forceinline__ static void store(float* p, size_t i, float v) { p[i] = v; }
};
constexpr float F16_SCALE = 32768.0f;          // 2^15, PLBM_F16_SCALE_LOG2
constexpr float F16_INV_SCALE = 1.0f / 32768.0f;
struct StoreF16Dev {
  typedef __half elem;
  typedef float real;
  static constexpr bool ddf = true;
  __device__ __forceinline__ static float load(const __half* p, size_t i) {
    return __half2float(__ldg(p + i)) * F16_INV_SCALE;
  }
  __device__ __forceinline__ static void store(__half* p, size_t i, float v) {
    p[i] = __float2half_rn(v * F16_SCALE);
  }
};

// ---------------------------------------------------------------------------
// Collision parameters, resolved on the host once per launch.
struct CollParams {
  double omega;      // BGK / RR relaxation rate, TRT lambda_e
  double omegabar;   // 1 - omega
  double lambda_d;   // TRT odd rate, src/collision_trt.F90:30-34
  double les, lds;   // 0.5*lambda_e, 0.5*lambda_d (src/collision_trt.F90:90-91)
  double rr_w0, rr_ws, rr_wd;  // w*(1-omega), src/collision_regularized.F90:63-65
  double bgki_fac;   // 4.5 - 2.25*omega, src/collision_bgk_improved.f90:39
};

// ---- binary64 reference operators -----------------------------------------

// src/collision_bgk.F90:58-71 with equilibrium() of src/fvm_bardow.F90:99-126
__device__ __forceinline__ void coll_bgk_ref(double (&fs)[9], const CollParams& p) {
  double rho = (((fs[5] + fs[7]) + (fs[6] + fs[8])) + ((fs[1] + fs[3]) + (fs[2] + fs[4]))) + fs[0];
  double invrho = 1.0 / rho;
  double ux = invrho * (((fs[5] - fs[7]) + (fs[8] - fs[6])) + (fs[1] - fs[3]));
  double uy = invrho * (((fs[5] - fs[7]) + (fs[6] - fs[8])) + (fs[2] - fs[4]));
  double uxx = ux * ux;
  double uyy = uy * uy;
  double indp = 1.0 - 1.5 * (uxx + uyy);
  double feq[9];
  feq[0] = W0 * rho * (indp);
  feq[1] = WS * rho * (indp + 3.0 * ux + 4.5 * uxx);
  feq[2] = WS * rho * (indp + 3.0 * uy + 4.5 * uyy);
  feq[3] = WS * rho * (indp - 3.0 * ux + 4.5 * uxx);
  feq[4] = WS * rho * (indp - 3.0 * uy + 4.5 * uyy);
  double uxpy = ux + uy;
  feq[5] = WD * rho * (indp + 3.0 * uxpy + 4.5 * uxpy * uxpy);
  feq[7] = WD * rho * (indp - 3.0 * uxpy + 4.5 * uxpy * uxpy);
  double uxmy = ux - uy;
  feq[6] = WD * rho * (indp - 3.0 * uxmy + 4.5 * uxmy * uxmy);
  feq[8] = WD * rho * (indp + 3.0 * uxmy + 4.5 * uxmy * uxmy);
#pragma unroll
  for (int q = 0; q < 9; q++) fs[q] = p.omegabar * fs[q] + p.omega * feq[q];
}

// src/collision_trt.F90:12-20 constants
constexpr double TRT_T0 = 4.0 / 9.0;
constexpr double TRT_T1X2 = (1.0 / 9.0) * 2.0;
constexpr double TRT_T2X2 = (1.0 / 36.0) * 2.0;
constexpr double TRT_INV2CSQ2 = 1.0 / (2.0 * (1.0 / 3.0) * (1.0 / 3.0));
constexpr double TRT_FAC1 = TRT_T1X2 * TRT_INV2CSQ2;
constexpr double TRT_FAC2 = TRT_T2X2 * TRT_INV2CSQ2;

// src/collision_trt.F90:98-152 (trt_naive, incompressible equilibrium)
__device__ __forceinline__ void coll_trt_ref(double (&v)[9], const CollParams& p) {
  const double vC = v[0], vE = v[1], vN = v[2], vW = v[3], vS = v[4];
  const double vNE = v[5], vNW = v[6], vSW = v[7], vSE = v[8];
  const double le = p.omega, les = p.les, lds = p.lds;
  double rho = (((vNE + vSW) + (vNW + vSE)) + ((vE + vW) + (vN + vS))) + vC;
  double velX = (((vNE - vSW) + (vSE - vNW)) + (vE - vW));
  double velY = (((vNE - vSW) + (vNW - vSE)) + (vN - vS));
  double velX2 = velX * velX;
  double velY2 = velY * velY;
  double feq_common = rho - 1.5 * (velX2 + velY2);
  v[0] = vC * (1.0 - le) + le * TRT_T0 * feq_common;
  double velXPY = velX + velY;
  double sym = les * (vNE + vSW - TRT_FAC2 * velXPY * velXPY - TRT_T2X2 * feq_common);
  double asym = lds * (vNE - vSW - 3.0 * TRT_T2X2 * velXPY);
  v[5] = vNE - sym - asym;
  v[7] = vSW - sym + asym;
  double velXMY = velX - velY;
  sym = les * (vSE + vNW - TRT_FAC2 * velXMY * velXMY - TRT_T2X2 * feq_common);
  asym = lds * (vSE - vNW - 3.0 * TRT_T2X2 * velXMY);
  v[8] = vSE - sym - asym;
  v[6] = vNW - sym + asym;
  sym = les * (vN + vS - TRT_FAC1 * velY2 - TRT_T1X2 * feq_common);
  asym = lds * (vN - vS - 3.0 * TRT_T1X2 * velY);
  v[2] = vN - sym - asym;
  v[4] = vS - sym + asym;
  sym = les * (vE + vW - TRT_FAC1 * velX2 - TRT_T1X2 * feq_common);
  asym = lds * (vE - vW - 3.0 * TRT_T1X2 * velX);
  v[1] = vE - sym - asym;
  v[3] = vW - sym + asym;
}

// src/collision_regularized.F90:72-194 (rr_kernel_naive)
__device__ __forceinline__ void coll_rr_ref(double (&f)[9], const CollParams& p) {
  double vC = f[0], vE = f[1], vN = f[2], vW = f[3], vS = f[4];
  double vNE = f[5], vNW = f[6], vSW = f[7], vSE = f[8];
  double feq[9];
  double rho = (((vNE + vSW) + (vNW + vSE)) + ((vE + vW) + (vN + vS))) + vC;
  double invrho = 1.0 / rho;
  double ux = invrho * (((vNE - vSW) + (vSE - vNW)) + (vE - vW));
  double uy = invrho * (((vNE - vSW) + (vNW - vSE)) + (vN - vS));
  double uxx = ux * ux;
  double uyy = uy * uy;
  double uxxy = uxx * uy;
  double uyyx = uyy * ux;
  double uxxyy = uxx * uyy;
  double indp0 = 1.0 - 1.5 * (uxx + uyy);
  double indps = indp0 - 4.5 * uxxyy;
  double indpd = indp0 + 9.0 * uxxyy;
  indp0 = indp0 + 2.25 * uxxyy;
  feq[0] = W0 * rho * indp0;
  feq[1] = WS * rho * (indps + 3.0 * ux + 4.5 * (uxx - uyyx));
  feq[3] = WS * rho * (indps - 3.0 * ux + 4.5 * (uxx + uyyx));
  feq[2] = WS * rho * (indps + 3.0 * uy + 4.5 * (uyy - uxxy));
  feq[4] = WS * rho * (indps - 3.0 * uy + 4.5 * (uyy + uxxy));
  vC = vC - feq[0];
  vE = vE - feq[1];
  vN = vN - feq[2];
  vW = vW - feq[3];
  vS = vS - feq[4];
  double axx = CSQR * (2.0 * (vE + vW) - (vN + vS) - vC);
  double ayy = CSQR * (2.0 * (vN + vS) - (vE + vW) - vC);
  double u3p = uxxy + uyyx;
  double uxpy = ux + uy;
  double indp57 = indpd + 4.5 * uxpy * uxpy;
  feq[5] = WD * rho * (indp57 + 3.0 * uxpy + 9.0 * u3p);
  feq[7] = WD * rho * (indp57 - 3.0 * uxpy - 9.0 * u3p);
  double u3m = uxxy - uyyx;
  double uxmy = ux - uy;
  double indp68 = indpd + 4.5 * uxmy * uxmy;
  feq[6] = WD * rho * (indp68 - 3.0 * uxmy + 9.0 * u3m);
  feq[8] = WD * rho * (indp68 + 3.0 * uxmy - 9.0 * u3m);
  vNE = vNE - feq[5];
  vNW = vNW - feq[6];
  vSW = vSW - feq[7];
  vSE = vSE - feq[8];
  double tmp = 2.0 * CSQR * (vNE + vNW + vSW + vSE);
  axx = axx + tmp;
  ayy = ayy + tmp;
  double axy = ((vNE + vSW) - (vNW + vSE));
  double axxy = 2.0 * ux * axy + uy * axx;
  double ayyx = 2.0 * uy * axy + ux * ayy;
  double axxyy = 2.0 * (ux * ayyx + uy * axxy) - uxx * ayy - uyy * axx - 4.0 * ux * uy * axy;
  indp0 = -1.5 * (axx + ayy);
  indps = indp0 - 4.5 * axxyy;
  indpd = 9.0 * axxyy - 2.0 * indp0;
  indp0 = indp0 + 2.25 * axxyy;
  vC = indp0;
  vE = indps + 4.5 * (axx - ayyx);
  vW = indps + 4.5 * (axx + ayyx);
  vN = indps + 4.5 * (ayy - axxy);
  vS = indps + 4.5 * (ayy + axxy);
  vNE = indpd + 9.0 * (axxy + ayyx + axy);
  vSW = indpd - 9.0 * (axxy + ayyx - axy);
  vNW = indpd + 9.0 * (axxy - ayyx - axy);
  vSE = indpd - 9.0 * (axxy - ayyx + axy);
  f[0] = feq[0] + p.rr_w0 * vC;
  f[1] = feq[1] + p.rr_ws * vE;
  f[2] = feq[2] + p.rr_ws * vN;
  f[3] = feq[3] + p.rr_ws * vW;
  f[4] = feq[4] + p.rr_ws * vS;
  f[5] = feq[5] + p.rr_wd * vNE;
  f[6] = feq[6] + p.rr_wd * vNW;
  f[7] = feq[7] + p.rr_wd * vSW;
  f[8] = feq[8] + p.rr_wd * vSE;
}

// src/collision_bgk_improved.f90:45-102
__device__ __forceinline__ void coll_bgki_ref(double (&f)[9], const CollParams& p) {
  const double one_third = 1.0 / 3.0, two_thirds = 2.0 / 3.0;
  const double vC = f[0], vE = f[1], vN = f[2], vW = f[3], vS = f[4];
  const double vNE = f[5], vNW = f[6], vSW = f[7], vSE = f[8];
  double rho = (((vNE + vSW) + (vNW + vSE)) + ((vE + vW) + (vN + vS))) + vC;
  double invrho = 1.0 / rho;
  double sumX1 = vE + vNE + vSE;
  double sumXN = vW + vNW + vSW;
  double sumY1 = vN + vNE + vNW;
  double sumYN = vS + vSE + vSW;
  double m10 = invrho * (sumX1 - sumXN);
  double m01 = invrho * (sumY1 - sumYN);
  double u2 = m10 * m10;
  double v2 = m01 * m01;
  double m20 = invrho * (sumX1 + sumXN);
  double m02 = invrho * (sumY1 + sumYN);
  double Gx = p.bgki_fac * u2 * (m20 - one_third - u2);
  double Gy = p.bgki_fac * v2 * (m02 - one_third - v2);
  double X0 = -two_thirds + u2 + Gx;
  double X1 = -(X0 + 1.0 + m10) * 0.5;
  double XN = X1 + m10;
  double Y0 = -two_thirds + v2 + Gy;
  double Y1 = -(Y0 + 1.0 + m01) * 0.5;
  double YN = Y1 + m01;
  double rho_omega = rho * p.omega;
  X0 = X0 * rho_omega;
  X1 = X1 * rho_omega;
  XN = XN * rho_omega;
  const double ob = p.omegabar;
  f[0] = ob * vC + X0 * Y0;
  f[1] = ob * vE + X1 * Y0;
  f[2] = ob * vN + X0 * Y1;
  f[3] = ob * vW + XN * Y0;
  f[4] = ob * vS + X0 * YN;
  f[5] = ob * vNE + X1 * Y1;
  f[6] = ob * vNW + XN * Y1;
  f[7] = ob * vSW + XN * YN;
  f[8] = ob * vSE + X1 * YN;
}

// ---- shifted-population operators (h = f - w) -------------------------------
// BGK of the plugin path, sim/sim.F90:445-499 (ddf_shift = .true.): rho = sum h
// + 1, u = j/rho by division, feq shifted by w*(rho - 1), h' = omega*(feq-h)+h.
// Instantiated in binary64 (plugin parity) and binary32 (deviation storage).
template <typename R>
__device__ __forceinline__ void coll_bgk_shift(R (&f)[9], R omega) {
  const R w0 = R(4) / R(9), ws = R(1) / R(9), wd = R(1) / R(36);
  R rho = (((f[5] + f[7]) + (f[6] + f[8])) + ((f[1] + f[3]) + (f[2] + f[4]))) + f[0];
  rho = rho + R(1);
  R ux = (((f[5] - f[7]) + (f[8] - f[6])) + (f[1] - f[3])) / rho;
  R uy = (((f[5] - f[7]) + (f[6] - f[8])) + (f[2] - f[4])) / rho;
  R uxx = ux * ux;
  R uyy = uy * uy;
  R indp = R(-1.5) * (uxx + uyy);
  R feq[9];
  feq[0] = w0 * rho * (indp);
  feq[1] = ws * rho * (indp + R(3) * ux + R(4.5) * uxx);
  feq[2] = ws * rho * (indp + R(3) * uy + R(4.5) * uyy);
  feq[3] = ws * rho * (indp - R(3) * ux + R(4.5) * uxx);
  feq[4] = ws * rho * (indp - R(3) * uy + R(4.5) * uyy);
  R uxpy = ux + uy;
  feq[5] = wd * rho * (indp + R(3) * uxpy + R(4.5) * uxpy * uxpy);
  feq[7] = wd * rho * (indp - R(3) * uxpy + R(4.5) * uxpy * uxpy);
  R uxmy = ux - uy;
  feq[6] = wd * rho * (indp - R(3) * uxmy + R(4.5) * uxmy * uxmy);
  feq[8] = wd * rho * (indp + R(3) * uxmy + R(4.5) * uxmy * uxmy);
  const R drho = rho - R(1);
  feq[0] = feq[0] + w0 * drho;
#pragma unroll
  for (int q = 1; q < 5; q++) feq[q] = feq[q] + ws * drho;
#pragma unroll
  for (int q = 5; q < 9; q++) feq[q] = feq[q] + wd * drho;
#pragma unroll
  for (int q = 0; q < 9; q++) f[q] = omega * (feq[q] - f[q]) + f[q];
}

// TRT of src/collision_trt.F90:98-152 rewritten for shifted populations.
// With v = h + w, the constant parts cancel exactly:
//   v_a + v_b - t*feq_common = h_a + h_b - t*(drho - 1.5 j^2),  v_a - v_b = h_a - h_b,
// so the operator is the reference's with h for v and drho for rho.
// SC: populations held scaled by 2^15 (binary16 storage); the operator is
// linear in them except for its squares of j, which take one factor 2^-15
// (q = 2^-15 j is the second factor of each).
template <typename R, bool SC = false>
__device__ __forceinline__ void coll_trt_shift(R (&v)[9], R le, R les, R lds) {
  const R t0 = R(4) / R(9), t1x2 = R(2) / R(9), t2x2 = R(2) / R(36);
  const R fac1 = t1x2 * R(4.5), fac2 = t2x2 * R(4.5);
  const R vC = v[0], vE = v[1], vN = v[2], vW = v[3], vS = v[4];
  const R vNE = v[5], vNW = v[6], vSW = v[7], vSE = v[8];
  R drho = (((vNE + vSW) + (vNW + vSE)) + ((vE + vW) + (vN + vS))) + vC;
  R velX = (((vNE - vSW) + (vSE - vNW)) + (vE - vW));
  R velY = (((vNE - vSW) + (vNW - vSE)) + (vN - vS));
  R qx = velX, qy = velY;
  if constexpr (SC) {
    qx = velX * R(1.0 / 32768.0);
    qy = velY * R(1.0 / 32768.0);
  }
  R velX2 = velX * qx, velY2 = velY * qy;
  R fc = drho - R(1.5) * (velX2 + velY2);
  v[0] = vC * (R(1) - le) + le * t0 * fc;
  R velXPY = velX + velY;
  R sym = les * (vNE + vSW - fac2 * velXPY * (qx + qy) - t2x2 * fc);
  R asym = lds * (vNE - vSW - R(3) * t2x2 * velXPY);
  v[5] = vNE - sym - asym;
  v[7] = vSW - sym + asym;
  R velXMY = velX - velY;
  sym = les * (vSE + vNW - fac2 * velXMY * (qx - qy) - t2x2 * fc);
  asym = lds * (vSE - vNW - R(3) * t2x2 * velXMY);
  v[8] = vSE - sym - asym;
  v[6] = vNW - sym + asym;
  sym = les * (vN + vS - fac1 * velY2 - t1x2 * fc);
  asym = lds * (vN - vS - R(3) * t1x2 * velY);
  v[2] = vN - sym - asym;
  v[4] = vS - sym + asym;
  sym = les * (vE + vW - fac1 * velX2 - t1x2 * fc);
  asym = lds * (vE - vW - R(3) * t1x2 * velX);
  v[1] = vE - sym - asym;
  v[3] = vW - sym + asym;
}

// Recursive-regularised operator of src/collision_regularized.F90:72-194 for
// shifted populations.  The equilibrium is split as feq_i = w_i*(rho + rho*P_i)
// with P_i the velocity polynomial, so heq_i = feq_i - w_i = w_i*(drho + rho*P_i);
// non-equilibrium parts h_i - heq_i equal f_i - feq_i exactly in real arithmetic.
// SC: populations held scaled by S = 2^15 (binary16 storage); the operator is
// linear in them except through rho and u: rho = 1 + drho/S, u = j/(S rho),
// and heq scaled is w*(drho + S rho P).  SC is binary32 only: 1/rho takes the
// approximate division (2 ulp), far below the storage's 2^-11 rounding.
template <typename R, bool SC = false>
__device__ __forceinline__ void coll_rr_shift(R (&f)[9], R rr_w0, R rr_ws, R rr_wd) {
  const R w0 = R(4) / R(9), ws = R(1) / R(9), wd = R(1) / R(36), csqr = R(1) / R(3);
  R vC = f[0], vE = f[1], vN = f[2], vW = f[3], vS = f[4];
  R vNE = f[5], vNW = f[6], vSW = f[7], vSE = f[8];
  R drho = (((vNE + vSW) + (vNW + vSE)) + ((vE + vW) + (vN + vS))) + vC;
  R rho, invrho;
  if constexpr (SC) {
    rho = drho * R(1.0 / 32768.0) + R(1);
    invrho = __fdividef(R(1.0 / 32768.0), rho);
  } else {
    rho = drho + R(1);
    invrho = R(1) / rho;
  }
  R ux = invrho * (((vNE - vSW) + (vSE - vNW)) + (vE - vW));
  R uy = invrho * (((vNE - vSW) + (vNW - vSE)) + (vN - vS));
  R uxx = ux * ux, uyy = uy * uy;
  R uxxy = uxx * uy, uyyx = uyy * ux, uxxyy = uxx * uyy;
  // P terms: indp0 - 1 etc.
  if constexpr (SC) rho = rho * R(32768);
  R p0 = R(-1.5) * (uxx + uyy);
  R ps = p0 - R(4.5) * uxxyy;
  R pd = p0 + R(9) * uxxyy;
  p0 = p0 + R(2.25) * uxxyy;
  R heq[9];
  heq[0] = w0 * (drho + rho * p0);
  heq[1] = ws * (drho + rho * (ps + R(3) * ux + R(4.5) * (uxx - uyyx)));
  heq[3] = ws * (drho + rho * (ps - R(3) * ux + R(4.5) * (uxx + uyyx)));
  heq[2] = ws * (drho + rho * (ps + R(3) * uy + R(4.5) * (uyy - uxxy)));
  heq[4] = ws * (drho + rho * (ps - R(3) * uy + R(4.5) * (uyy + uxxy)));
  vC = vC - heq[0];
  vE = vE - heq[1];
  vN = vN - heq[2];
  vW = vW - heq[3];
  vS = vS - heq[4];
  R axx = csqr * (R(2) * (vE + vW) - (vN + vS) - vC);
  R ayy = csqr * (R(2) * (vN + vS) - (vE + vW) - vC);
  R u3p = uxxy + uyyx, uxpy = ux + uy;
  R p57 = pd + R(4.5) * uxpy * uxpy;
  heq[5] = wd * (drho + rho * (p57 + R(3) * uxpy + R(9) * u3p));
  heq[7] = wd * (drho + rho * (p57 - R(3) * uxpy - R(9) * u3p));
  R u3m = uxxy - uyyx, uxmy = ux - uy;
  R p68 = pd + R(4.5) * uxmy * uxmy;
  heq[6] = wd * (drho + rho * (p68 - R(3) * uxmy + R(9) * u3m));
  heq[8] = wd * (drho + rho * (p68 + R(3) * uxmy - R(9) * u3m));
  vNE = vNE - heq[5];
  vNW = vNW - heq[6];
  vSW = vSW - heq[7];
  vSE = vSE - heq[8];
  R tmp = R(2) * csqr * (vNE + vNW + vSW + vSE);
  axx = axx + tmp;
  ayy = ayy + tmp;
  R axy = ((vNE + vSW) - (vNW + vSE));
  R axxy = R(2) * ux * axy + uy * axx;
  R ayyx = R(2) * uy * axy + ux * ayy;
  R axxyy = R(2) * (ux * ayyx + uy * axxy) - uxx * ayy - uyy * axx - R(4) * ux * uy * axy;
  R i0 = R(-1.5) * (axx + ayy);
  R is = i0 - R(4.5) * axxyy;
  R id = R(9) * axxyy - R(2) * i0;
  i0 = i0 + R(2.25) * axxyy;
  f[0] = heq[0] + rr_w0 * i0;
  f[1] = heq[1] + rr_ws * (is + R(4.5) * (axx - ayyx));
  f[3] = heq[3] + rr_ws * (is + R(4.5) * (axx + ayyx));
  f[2] = heq[2] + rr_ws * (is + R(4.5) * (ayy - axxy));
  f[4] = heq[4] + rr_ws * (is + R(4.5) * (ayy + axxy));
  f[5] = heq[5] + rr_wd * (id + R(9) * (axxy + ayyx + axy));
  f[7] = heq[7] + rr_wd * (id - R(9) * (axxy + ayyx - axy));
  f[6] = heq[6] + rr_wd * (id + R(9) * (axxy - ayyx - axy));
  f[8] = heq[8] + rr_wd * (id - R(9) * (axxy - ayyx + axy));
}

// ---- dispatch -----------------------------------------------------------------
enum { K_BGK = 0, K_TRT = 1, K_RR = 2, K_BGKI = 3 };

template <int KIND>
__device__ __forceinline__ void collide_ref(double (&f)[9], const CollParams& p) {
  if (KIND == K_BGK) coll_bgk_ref(f, p);
  else if (KIND == K_TRT) coll_trt_ref(f, p);
  else if (KIND == K_RR) coll_rr_ref(f, p);
  else coll_bgki_ref(f, p);
}

template <int KIND, typename R>
__device__ __forceinline__ void collide_shift(R (&f)[9], const CollParams& p) {
  if (KIND == K_BGK) coll_bgk_shift<R>(f, (R)p.omega);
  else if (KIND == K_TRT) coll_trt_shift<R>(f, (R)p.omega, (R)p.les, (R)p.lds);
  else coll_rr_shift<R>(f, (R)p.rr_w0, (R)p.rr_ws, (R)p.rr_wd);
}

}  // namespace plbm
