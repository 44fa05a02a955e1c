// step_df64.cu -- binary64-storage fused step in the "hybrid" arithmetic of
// hybrid.cuh (exact integer moments, double-float small terms, binary64 only
// for the final combination), BGK, TRT and RR.  Cells outside the hybrid range
// are evaluated with the binary64 operator of the reference (and set the
// range flag).
//
// Also the deviation-storage steps whose collision runs in more than binary32:
// double-float (PLBM_MATH_HYBRID) or binary64 (PLBM_MATH_STRICT) arithmetic on
// h = f - w, stored back in binary32 / scaled binary16.
//
// Compiled with --fmad=false: the double-float error-free transformations
// need every + - * rounded on its own; the fused operations are explicit.
#include "coll_df64.cuh"
#include "hybrid.cuh"
#include "plbm_launch.h"
#include "schemes.cuh"

namespace plbm {

// Set to 1 by a hybrid kernel that met a population outside |f| < 2.
__device__ int g_hybrid_range_flag = 0;

namespace {

// Deviation storage, BGK evaluated in double-float on h.
template <class S>
__global__ void __launch_bounds__(kBlock) k_step_dev_df(const typename S::elem* __restrict__ src,
                                                       typename S::elem* __restrict__ dst, int nx, int ny, int ld,
                                                       int ftiles, df::DfParams p) {
  const int x = blockIdx.x / ftiles;
  const int y = (blockIdx.x - x * ftiles) * blockDim.x + threadIdx.x;
  if (y >= ny) return;
  df::df64 h[9];
#pragma unroll
  for (int q = 0; q < 9; q++) {
    const int sx = wrap_add(x, -cx_of(q), nx), sy = wrap_add(y, -cy_of(q), ny);
    h[q] = df::make(S::load(src, YFast::off(sx, sy, q, nx, ny, ld)), 0.0f);
  }
  df::bgk(h, p);
#pragma unroll
  for (int q = 0; q < 9; q++) S::store(dst, YFast::off(x, y, q, nx, ny, ld), h[q].hi + h[q].lo);
}

// Deviation storage, BGK with the compensated binary32 operator.  I: offset
// type (32-bit when the lattice has fewer than 2^32 elements).
template <class S, typename I>
__global__ void __launch_bounds__(kBlock) k_step_dev_comp(const typename S::elem* __restrict__ src,
                                                         typename S::elem* __restrict__ dst, int nx, int ny, int ld,
                                                         int ftiles, df::DevParams p) {
  const int x = blockIdx.x / ftiles;
  const int y = (blockIdx.x - x * ftiles) * blockDim.x + threadIdx.x;
  if (y >= ny) return;
  const I L = (I)ld, P = (I)ld * (I)nx;
  const I c0 = (I)x * L, cm = (I)wrap_m(x, nx) * L, cp = (I)wrap_p(x, nx) * L;
  const I y0 = (I)y, ym = (I)wrap_m(y, ny), yp = (I)wrap_p(y, ny);
  float h[9];
  h[0] = S::load(src, c0 + y0);
  h[1] = S::load(src, P + cm + y0);
  h[2] = S::load(src, 2 * P + c0 + ym);
  h[3] = S::load(src, 3 * P + cp + y0);
  h[4] = S::load(src, 4 * P + c0 + yp);
  h[5] = S::load(src, 5 * P + cm + ym);
  h[6] = S::load(src, 6 * P + cp + ym);
  h[7] = S::load(src, 7 * P + cp + yp);
  h[8] = S::load(src, 8 * P + cm + yp);
  df::bgk_dev_comp(h, p);
  const I o = c0 + y0;
#pragma unroll
  for (int q = 0; q < 9; q++) S::store(dst, (I)q * P + o, h[q]);
}

// Deviation storage, collision evaluated in binary64 on h (any kind but BGKI).
template <class S, int KIND>
__global__ void __launch_bounds__(kBlock) k_step_dev_d(const typename S::elem* __restrict__ src,
                                                      typename S::elem* __restrict__ dst, int nx, int ny, int ld,
                                                      int ftiles, CollParams p) {
  const int x = blockIdx.x / ftiles;
  const int y = (blockIdx.x - x * ftiles) * blockDim.x + threadIdx.x;
  if (y >= ny) return;
  double h[9];
#pragma unroll
  for (int q = 0; q < 9; q++) {
    const int sx = wrap_add(x, -cx_of(q), nx), sy = wrap_add(y, -cy_of(q), ny);
    h[q] = (double)S::load(src, YFast::off(sx, sy, q, nx, ny, ld));
  }
  collide_shift<KIND, double>(h, p);
#pragma unroll
  for (int q = 0; q < 9; q++) S::store(dst, YFast::off(x, y, q, nx, ny, ld), (float)h[q]);
}

df::df64 split_const(double d) {
  const float hi = (float)d;
  return df::make(hi, (float)(d - (double)hi));
}

// Constants of one hybrid launch: the hybrid operator's and the binary64
// operator's (for cells outside the hybrid range).
struct HybridArgs {
  hy::BgkParams bgk1;  // BGK (bgk_fma, populations or shifted populations)
  hy::BgkParams rr1;   // RR (rr_fma): the one-FMA constants at omega = 1
  hy::TrtFmaParams trt;  // TRT (trt_fma)
  hy::RrParams rr;
  CollParams ref;
};

// One cell outside the hybrid range: pull, the binary64 operator of the
// reference, store.  Out of line so that the hot kernel's registers and code
// are not shaped by this rarely taken path.
template <int KIND>
__device__ __noinline__ void hybrid_fallback_cell(const double* __restrict__ src, double* __restrict__ dst, int x,
                                                  int y, int nx, int ny, int ld, const CollParams& p) {
  double f[9];
#pragma unroll
  for (int q = 0; q < 9; q++) {
    const int sx = wrap_add(x, -cx_of(q), nx), sy = wrap_add(y, -cy_of(q), ny);
    f[q] = src[YFast::off(sx, sy, q, nx, ny, ld)];
  }
  collide_ref<KIND>(f, p);
#pragma unroll
  for (int q = 0; q < 9; q++) dst[YFast::off(x, y, q, nx, ny, ld)] = f[q];
  g_hybrid_range_flag = 1;
}

// Resident CTAs per SM the hybrid kernels are compiled for: BGK (bgk_fma) and
// TRT (trt_fma) at 4, RR (rr_fma) at 3 (register caps 64 and 80).  Capped at
// 48 registers for 5 CTAs the BGK kernel spills and runs 2 % slower at 8192^2.
constexpr int hybrid_min_blocks(int kind) { return kind == K_RR ? 3 : 4; }

// I: index type of the lattice offsets; 32-bit when the whole lattice has
// fewer than 2^32 elements (one multiply-add per address instead of 64-bit
// arithmetic).
template <typename I, int KIND>
__global__ void __launch_bounds__(kBlock, hybrid_min_blocks(KIND)) k_step_hybrid(const double* __restrict__ src, double* __restrict__ dst,
                                                       int nx, int ny, int ld, int ftiles, HybridArgs a) {
  const int x = blockIdx.x / ftiles;
  const int y = (blockIdx.x - x * ftiles) * blockDim.x + threadIdx.x;
  if (y >= ny) return;
  const I L = (I)ld, P = (I)ld * (I)nx;
  const I c0 = (I)x * L, cm = (I)wrap_m(x, nx) * L, cp = (I)wrap_p(x, nx) * L;
  const I y0 = (I)y, ym = (I)wrap_m(y, ny), yp = (I)wrap_p(y, ny);
  double f[9];
  // pull: f_q(x, y) = f_q(x - cx_q, y - cy_q) of the source lattice
  f[0] = __ldg(src + (c0 + y0));
  f[1] = __ldg(src + (P + cm + y0));
  f[2] = __ldg(src + (2 * P + c0 + ym));
  f[3] = __ldg(src + (3 * P + cp + y0));
  f[4] = __ldg(src + (4 * P + c0 + yp));
  f[5] = __ldg(src + (5 * P + cm + ym));
  f[6] = __ldg(src + (6 * P + cp + ym));
  f[7] = __ldg(src + (7 * P + cp + yp));
  f[8] = __ldg(src + (8 * P + cm + yp));
  bool bad = false;
  if (KIND == K_TRT) hy::trt_fma(f, a.trt, bad);
  else if (KIND == K_RR) hy::rr_fma(f, a.rr, a.rr1, bad);
  else hy::bgk_fma(f, a.bgk1, bad);
  if (bad) {  // outside the hybrid range: the binary64 operator on the same inputs
    hybrid_fallback_cell<KIND>(src, dst, x, y, nx, ny, ld, a.ref);
    return;
  }
  const I o = c0 + y0;
#pragma unroll
  for (int q = 0; q < 9; q++) dst[(I)q * P + o] = f[q];
}

// A finite-volume / finite-difference streaming scheme in stencil form fused
// with the hybrid collision (binary64 storage).  Out-of-range cells take the
// binary64 collision (out of line, the stencil evaluated again).
template <int TAPS, int KIND>
__device__ __noinline__ void scheme_fallback_cell(const double* __restrict__ src, double* __restrict__ dst, int x,
                                                  int y, int nx, int ny, int ld, const sch::Stencil& st,
                                                  const CollParams& p) {
  double f[9];
  sch::stencil_pull<YFast, TAPS>(src, x, y, nx, ny, ld, st, f);
  collide_ref<KIND>(f, p);
#pragma unroll
  for (int q = 0; q < 9; q++) dst[YFast::off(x, y, q, nx, ny, ld)] = f[q];
  g_hybrid_range_flag = 1;
}

template <int TAPS, int KIND>
__global__ void __launch_bounds__(kBlock) k_step_scheme_hybrid(const double* __restrict__ src,
                                                              double* __restrict__ dst, int nx, int ny, int ld,
                                                              int ftiles, sch::Stencil st, HybridArgs a) {
  const int x = blockIdx.x / ftiles;
  const int y = (blockIdx.x - x * ftiles) * blockDim.x + threadIdx.x;
  if (y >= ny) return;
  double f[9];
  sch::stencil_pull<YFast, TAPS>(src, x, y, nx, ny, ld, st, f);
  bool bad = false;
  if (KIND == K_TRT) hy::trt_fma(f, a.trt, bad);
  else if (KIND == K_RR) hy::rr_fma(f, a.rr, a.rr1, bad);
  else hy::bgk_fma(f, a.bgk1, bad);
  if (bad) {
    scheme_fallback_cell<TAPS, KIND>(src, dst, x, y, nx, ny, ld, st, a.ref);
    return;
  }
#pragma unroll
  for (int q = 0; q < 9; q++) dst[YFast::off(x, y, q, nx, ny, ld)] = f[q];
}

// The plugin step (sim/sim.F90:404-505 + :568-624) in the hybrid arithmetic:
// shifted binary64 populations h = f - w in the x-fastest layout, collide at
// the cell, push along c_q.  Out-of-range cells take the shifted binary64
// operator of the FMA plugin kernel (out of line).
template <int KIND>
__device__ __noinline__ void push_fallback_cell(const double* __restrict__ src, double* __restrict__ dst, int x,
                                                int y, int nx, int ny, int ld, const CollParams& p) {
  double f[9];
#pragma unroll
  for (int q = 0; q < 9; q++) f[q] = src[XFast::off(x, y, q, nx, ny, ld)];
  collide_shift<KIND, double>(f, p);
#pragma unroll
  for (int q = 0; q < 9; q++) dst[XFast::off(wrap_add(x, cx_of(q), nx), wrap_add(y, cy_of(q), ny), q, nx, ny, ld)] = f[q];
  g_hybrid_range_flag = 1;
}

template <typename I, int KIND>
__global__ void __launch_bounds__(kBlock, hybrid_min_blocks(KIND)) k_push_hybrid(const double* __restrict__ src,
                                                                                double* __restrict__ dst, int nx,
                                                                                int ny, int ld, int ftiles,
                                                                                HybridArgs a) {
  const int y = blockIdx.x / ftiles;
  const int x = (blockIdx.x - y * ftiles) * blockDim.x + threadIdx.x;
  if (x >= nx) return;
  const I L = (I)ld, P = (I)ld * (I)ny;
  const I o = (I)y * L + (I)x;
  double f[9];
#pragma unroll
  for (int q = 0; q < 9; q++) f[q] = __ldg(src + ((I)q * P + o));
  bool bad = false;
  if (KIND == K_TRT) hy::trt_fma<true>(f, a.trt, bad);
  else if (KIND == K_RR) hy::rr_fma<true>(f, a.rr, a.rr1, bad);
  else hy::bgk_fma<true>(f, a.bgk1, bad);
  if (bad) {
    push_fallback_cell<KIND>(src, dst, x, y, nx, ny, ld, a.ref);
    return;
  }
  const I xm = (I)wrap_m(x, nx), xp = (I)wrap_p(x, nx), x0 = (I)x;
  const I rm = (I)wrap_m(y, ny) * L, rp = (I)wrap_p(y, ny) * L, r0 = (I)y * L;
  // push: f_q goes to (x + cx_q, y + cy_q)
  dst[r0 + x0] = f[0];
  dst[P + r0 + xp] = f[1];
  dst[2 * P + rp + x0] = f[2];
  dst[3 * P + r0 + xm] = f[3];
  dst[4 * P + rm + x0] = f[4];
  dst[5 * P + rp + xp] = f[5];
  dst[6 * P + rp + xm] = f[6];
  dst[7 * P + rm + xm] = f[7];
  dst[8 * P + rm + xp] = f[8];
}

template <int KIND>
cudaError_t launch_hybrid(const Sweep& s, unsigned blocks, int bs, int ft, const HybridArgs& a) {
  const double* src = static_cast<const double*>(s.src);
  double* dst = static_cast<double*>(s.dst);
  if ((unsigned long long)s.ld * (unsigned long long)s.nx * 9ull < (1ull << 32))
    k_step_hybrid<uint32_t, KIND><<<blocks, bs, 0, s.stream>>>(src, dst, s.nx, s.ny, s.ld, ft, a);
  else
    k_step_hybrid<size_t, KIND><<<blocks, bs, 0, s.stream>>>(src, dst, s.nx, s.ny, s.ld, ft, a);
  return cudaGetLastError();
}

}  // namespace

hy::BgkParams hybrid_bgk_params(double omega) {
  const double w[3] = {W0, WS, WD};
  return hy::bgk_fma_params(omega, w);
}

// Constants of the hybrid TRT from the launch's binary64 parameters
// (le = omega, les = omega/2, lds = lambda_d/2 as the reference forms them).
// Constants of the one-FMA TRT from the launch's binary64 parameters
// (lambda_e = omega, lambda_d as the reference forms it).
hy::TrtFmaParams hybrid_trt_params(const CollParams& cp) {
  const double w[3] = {W0, WS, WD};
  return hy::trt_fma_params(cp.omega, cp.lambda_d, w);
}

hy::RrParams hybrid_rr_params(const CollParams& cp) {
  hy::RrParams p;
  const double w[3] = {W0, WS, WD};
  for (int i = 0; i < 3; i++) {
    p.w[i] = w[i];
    p.wdf[i] = split_const(w[i]);
  }
  p.omb = split_const(1.0 - cp.omega);
  p.third = split_const(1.0 / 3.0);
  return p;
}

cudaError_t step_pull_df64(int kind, const Sweep& s, const CollParams& cp) {
  if (kind != K_BGK && kind != K_TRT && kind != K_RR) return cudaErrorNotSupported;
  const int bs = block_for((long long)s.nx * s.ny);
  const int ft = (s.ny + bs - 1) / bs;
  const long long blocks = (long long)ft * s.nx;
  if (blocks <= 0 || blocks > 0x7fffffffLL) return cudaErrorInvalidConfiguration;
  HybridArgs a;
  a.bgk1 = hybrid_bgk_params(cp.omega);
  a.rr1 = hybrid_bgk_params(1.0);
  a.trt = hybrid_trt_params(cp);
  a.rr = hybrid_rr_params(cp);
  a.ref = cp;
  if (kind == K_TRT) return launch_hybrid<K_TRT>(s, (unsigned)blocks, bs, ft, a);
  if (kind == K_RR) return launch_hybrid<K_RR>(s, (unsigned)blocks, bs, ft, a);
  return launch_hybrid<K_BGK>(s, (unsigned)blocks, bs, ft, a);
}

cudaError_t step_push_hybrid(int kind, const Sweep& s, const CollParams& cp) {
  if (kind != K_BGK && kind != K_TRT && kind != K_RR) return cudaErrorNotSupported;
  const int bs = block_for((long long)s.nx * s.ny);
  const int ft = (s.nx + bs - 1) / bs;
  const long long blocks = (long long)ft * s.ny;
  if (blocks <= 0 || blocks > 0x7fffffffLL) return cudaErrorInvalidConfiguration;
  HybridArgs a;
  a.bgk1 = hybrid_bgk_params(cp.omega);
  a.rr1 = hybrid_bgk_params(1.0);
  a.trt = hybrid_trt_params(cp);
  a.rr = hybrid_rr_params(cp);
  a.ref = cp;
  const double* src = static_cast<const double*>(s.src);
  double* dst = static_cast<double*>(s.dst);
  const unsigned nb = (unsigned)blocks;
  const bool small = (unsigned long long)s.ld * (unsigned long long)s.ny * 9ull < (1ull << 32);
#define PLBM_PUSH_HY(I)                                                                                      \
  switch (kind) {                                                                                            \
    case K_BGK: k_push_hybrid<I, K_BGK><<<nb, bs, 0, s.stream>>>(src, dst, s.nx, s.ny, s.ld, ft, a); break; \
    case K_TRT: k_push_hybrid<I, K_TRT><<<nb, bs, 0, s.stream>>>(src, dst, s.nx, s.ny, s.ld, ft, a); break; \
    default: k_push_hybrid<I, K_RR><<<nb, bs, 0, s.stream>>>(src, dst, s.nx, s.ny, s.ld, ft, a); break;     \
  }
  if (small) {
    PLBM_PUSH_HY(uint32_t)
  } else {
    PLBM_PUSH_HY(size_t)
  }
#undef PLBM_PUSH_HY
  return cudaGetLastError();
}

cudaError_t step_scheme_hybrid(int scheme, int kind, const Sweep& s, double dt, const CollParams& cp) {
  if (kind != K_BGK && kind != K_TRT && kind != K_RR) return cudaErrorNotSupported;
  if (scheme < sch::FVM || scheme > sch::FDM_WLS_G2) return cudaErrorInvalidValue;
  const int ft = (s.ny + kBlock - 1) / kBlock;
  const long long blocks = (long long)ft * s.nx;
  if (blocks <= 0 || blocks > 0x7fffffffLL) return cudaErrorInvalidConfiguration;
  const sch::Stencil st = sch::stencil_coefficients(scheme, dt);
  HybridArgs a;
  a.bgk1 = hybrid_bgk_params(cp.omega);
  a.rr1 = hybrid_bgk_params(1.0);
  a.trt = hybrid_trt_params(cp);
  a.rr = hybrid_rr_params(cp);
  a.ref = cp;
  const double* src = static_cast<const double*>(s.src);
  double* dst = static_cast<double*>(s.dst);
  const unsigned nb = (unsigned)blocks;
#define PLBM_SCH_HY(T)                                                                                        \
  switch (kind) {                                                                                             \
    case K_BGK: k_step_scheme_hybrid<T, K_BGK><<<nb, kBlock, 0, s.stream>>>(src, dst, s.nx, s.ny, s.ld, ft, st, a); break; \
    case K_TRT: k_step_scheme_hybrid<T, K_TRT><<<nb, kBlock, 0, s.stream>>>(src, dst, s.nx, s.ny, s.ld, ft, st, a); break; \
    default: k_step_scheme_hybrid<T, K_RR><<<nb, kBlock, 0, s.stream>>>(src, dst, s.nx, s.ny, s.ld, ft, st, a); break;     \
  }
  switch (sch::taps_of(scheme)) {
    case sch::TAPS_LINE: PLBM_SCH_HY(sch::TAPS_LINE) break;
    case sch::TAPS_AXIS3: PLBM_SCH_HY(sch::TAPS_AXIS3) break;
    default: PLBM_SCH_HY(sch::TAPS_FULL) break;
  }
#undef PLBM_SCH_HY
  return cudaGetLastError();
}

cudaError_t step_pull_dev_hi(int storage, int math, int kind, const Sweep& s, const CollParams& cp) {
  const int ft = (s.ny + kBlock - 1) / kBlock;
  const long long blocks = (long long)ft * s.nx;
  if (blocks <= 0 || blocks > 0x7fffffffLL) return cudaErrorInvalidConfiguration;
  const unsigned nb = (unsigned)blocks;
  if (math == 2) {  // compensated binary32
    if (kind != K_BGK) return cudaErrorNotSupported;
    df::DevParams p;
    const double w[3] = {W0, WS, WD};
    for (int i = 0; i < 3; i++) {
      p.w[i] = split_const(w[i]);
      p.w3[i] = split_const(3.0 * w[i]);
    }
    p.om_hi = (float)cp.omega;
    p.om_lo = (float)(cp.omega - (double)p.om_hi);
    const bool small = (unsigned long long)s.ld * (unsigned long long)s.nx * 9ull < (1ull << 32);
    if (storage == ST_F32DEV) {
      const float* a = static_cast<const float*>(s.src);
      float* b = static_cast<float*>(s.dst);
      if (small) k_step_dev_comp<StoreF32Dev, uint32_t><<<nb, kBlock, 0, s.stream>>>(a, b, s.nx, s.ny, s.ld, ft, p);
      else k_step_dev_comp<StoreF32Dev, size_t><<<nb, kBlock, 0, s.stream>>>(a, b, s.nx, s.ny, s.ld, ft, p);
    } else if (storage == ST_F16DEV) {
      const __half* a = static_cast<const __half*>(s.src);
      __half* b = static_cast<__half*>(s.dst);
      if (small) k_step_dev_comp<StoreF16Dev, uint32_t><<<nb, kBlock, 0, s.stream>>>(a, b, s.nx, s.ny, s.ld, ft, p);
      else k_step_dev_comp<StoreF16Dev, size_t><<<nb, kBlock, 0, s.stream>>>(a, b, s.nx, s.ny, s.ld, ft, p);
    } else {
      return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
  }
  if (math == 3) {  // double-float
    if (kind != K_BGK) return cudaErrorNotSupported;
    df::DfParams p;
    p.om = split_const(cp.omega);
    p.omb = split_const(cp.omegabar);
    p.w0 = split_const(W0);
    p.ws = split_const(WS);
    p.wd = split_const(WD);
    p.ws3 = split_const(3.0 * WS);
    p.wd3 = split_const(3.0 * WD);
    if (storage == ST_F32DEV)
      k_step_dev_df<StoreF32Dev><<<nb, kBlock, 0, s.stream>>>(static_cast<const float*>(s.src),
                                                              static_cast<float*>(s.dst), s.nx, s.ny, s.ld, ft, p);
    else if (storage == ST_F16DEV)
      k_step_dev_df<StoreF16Dev><<<nb, kBlock, 0, s.stream>>>(static_cast<const __half*>(s.src),
                                                              static_cast<__half*>(s.dst), s.nx, s.ny, s.ld, ft, p);
    else
      return cudaErrorInvalidValue;
    return cudaGetLastError();
  }
#define PLBM_DEVD(S, E)                                                                                      \
  switch (kind) {                                                                                            \
    case K_BGK: k_step_dev_d<S, K_BGK><<<nb, kBlock, 0, s.stream>>>(static_cast<const E*>(s.src),            \
                                                                    static_cast<E*>(s.dst), s.nx, s.ny, s.ld, \
                                                                    ft, cp); break;                           \
    case K_TRT: k_step_dev_d<S, K_TRT><<<nb, kBlock, 0, s.stream>>>(static_cast<const E*>(s.src),            \
                                                                    static_cast<E*>(s.dst), s.nx, s.ny, s.ld, \
                                                                    ft, cp); break;                           \
    case K_RR: k_step_dev_d<S, K_RR><<<nb, kBlock, 0, s.stream>>>(static_cast<const E*>(s.src),              \
                                                                  static_cast<E*>(s.dst), s.nx, s.ny, s.ld,   \
                                                                  ft, cp); break;                             \
    default: return cudaErrorNotSupported;                                                                   \
  }
  if (storage == ST_F32DEV) {
    PLBM_DEVD(StoreF32Dev, float)
  } else if (storage == ST_F16DEV) {
    PLBM_DEVD(StoreF16Dev, __half)
  } else {
    return cudaErrorInvalidValue;
  }
#undef PLBM_DEVD
  return cudaGetLastError();
}

cudaError_t hybrid_range_flag(int* flag, int reset) {
  cudaError_t e = cudaMemcpyFromSymbol(flag, g_hybrid_range_flag, sizeof(int));
  if (e == cudaSuccess && reset) {
    const int z = 0;
    e = cudaMemcpyToSymbol(g_hybrid_range_flag, &z, sizeof(int));
  }
  return e;
}

}  // namespace plbm
