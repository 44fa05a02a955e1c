// step_f64.cu -- binary64 stream/collide kernels with reference arithmetic.
//
// This translation unit is compiled twice: with FMA contraction into
// namespace plbm::fma, and with --fmad=false -DPLBM_STRICT into
// plbm::strict.  The strict build performs exactly the IEEE operations of the
// Fortran kernels (no contraction; CUDA binary64 division is correctly
// rounded), so its results are bit-identical to them.
//
// Kernels
//   k_step<YFast, pull>   fused lbm_stream + collide_*: one read and one write
//                         of the 9 populations per cell (144 B/cell).
//   k_stream              lbm_stream alone (src/periodic_lbm.f90:45-127).
//   k_collide             collide_* alone, in place (src/collision_*.F90).
//   k_collide_bgki_seq    collide_bgk_improved on its (ny,nx,0:8) dummy view.
//   k_step_pre            perform_triple_step: fused step that also stores the
//                         pre-collision populations.
//   k_stream_scheme       finite-volume / finite-difference streaming schemes
//                         (src/fvm_bardow.F90:393-886).
//   k_step<XFast, push>   the plugin step of sim/sim.F90:404-505 + :568-624:
//                         shifted populations, collide, then push along c_i.
#include "plbm_launch.h"

#ifdef PLBM_STRICT
#define PLBM_NS strict
#else
#define PLBM_NS fma
#endif

namespace plbm {
namespace PLBM_NS {
namespace {

template <class L>
__device__ __forceinline__ bool cell_of(int ftiles, int nx, int ny, int& x, int& y);

template <>
__device__ __forceinline__ bool cell_of<YFast>(int ftiles, int nx, int ny, int& x, int& y) {
  x = blockIdx.x / ftiles;
  y = (blockIdx.x - x * ftiles) * blockDim.x + threadIdx.x;
  return y < ny;
}
template <>
__device__ __forceinline__ bool cell_of<XFast>(int ftiles, int nx, int ny, int& x, int& y) {
  y = blockIdx.x / ftiles;
  x = (blockIdx.x - y * ftiles) * blockDim.x + threadIdx.x;
  return x < nx;
}

// Fused step.  PUSH=false: pull-stream then collide at the destination cell
// (src/ semantics).  PUSH=true: collide at the source cell, then push.
template <class L, int KIND, bool SHIFT, bool PUSH>
__global__ void __launch_bounds__(kBlock) k_step(const double* __restrict__ src, double* __restrict__ dst,
                                                int nx, int ny, int ld, int ftiles, CollParams p) {
  int x, y;
  if (!cell_of<L>(ftiles, nx, ny, x, y)) return;
  double f[9];
#pragma unroll
  for (int q = 0; q < 9; q++) {
    const int sx = PUSH ? x : wrap_add(x, -cx_of(q), nx);
    const int sy = PUSH ? y : wrap_add(y, -cy_of(q), ny);
    f[q] = __ldg(src + L::off(sx, sy, q, nx, ny, ld));
  }
  if (SHIFT) collide_shift<KIND, double>(f, p);
  else collide_ref<KIND>(f, p);
#pragma unroll
  for (int q = 0; q < 9; q++) {
    const int dx = PUSH ? wrap_add(x, cx_of(q), nx) : x;
    const int dy = PUSH ? wrap_add(y, cy_of(q), ny) : y;
    dst[L::off(dx, dy, q, nx, ny, ld)] = f[q];
  }
}

// perform_triple_step fused (src/fvm_bardow.F90:322-340): pull-stream from
// src, store the streamed (pre-collision) populations to pre, collide, store
// the result to dst.  Reads 72 B and writes 144 B per cell; the reference's
// three passes (stream, copy, collide) move 432 B.
template <int KIND>
__global__ void __launch_bounds__(kBlock) k_step_pre(const double* __restrict__ src, double* __restrict__ pre,
                                                    double* __restrict__ dst, int nx, int ny, int ld, int ftiles,
                                                    CollParams p) {
  int x, y;
  if (!cell_of<YFast>(ftiles, nx, ny, x, y)) return;
  double f[9];
#pragma unroll
  for (int q = 0; q < 9; q++) {
    const int sx = wrap_add(x, -cx_of(q), nx), sy = wrap_add(y, -cy_of(q), ny);
    f[q] = __ldg(src + YFast::off(sx, sy, q, nx, ny, ld));
    pre[YFast::off(x, y, q, nx, ny, ld)] = f[q];
  }
  collide_ref<KIND>(f, p);
#pragma unroll
  for (int q = 0; q < 9; q++) dst[YFast::off(x, y, q, nx, ny, ld)] = f[q];
}

// Finite-volume / finite-difference streaming (src/fvm_bardow.F90:393-886),
// one thread per cell, populations 1..8; each population's new value is a
// 9-point (FVM, FDM) or 3-point (Sofonea) stencil of the same population.
// The arithmetic is the Fortran's expression by expression (the strict build
// reproduces it exactly).  Loops cover the whole nx x ny grid.
enum { SCH_FVM = 1, SCH_FDM = 2, SCH_FDM_ISO = 3, SCH_FDM_WLS = 4, SCH_SOFONEA = 5 };

template <int SCHEME>
__device__ __forceinline__ double scheme_cell(const double* __restrict__ a, int q, int x, int y, int xp, int xm,
                                              int yp, int ym, int nx, int ny, int ld, double dt) {
  auto at = [&](int yy, int xx) { return __ldg(a + YFast::off(xx, yy, q, nx, ny, ld)); };
  const double cxq = dt * (double)cx_of(q), cyq = dt * (double)cy_of(q);
  if (SCHEME == SCH_SOFONEA) {
    const int cxi = cx_of(q), cyi = cy_of(q);
    const int xu = cxi > 0 ? xp : (cxi < 0 ? xm : x), xd = cxi > 0 ? xm : (cxi < 0 ? xp : x);
    const int yu = cyi > 0 ? yp : (cyi < 0 ? ym : y), yd = cyi > 0 ? ym : (cyi < 0 ? yp : y);
    const double fc = at(y, x), fu = at(yu, xu), fd = at(yd, xd);
    double du1, du2;
    if (q <= 4) {
      du1 = 0.5 * (fu - fd);
      du2 = fu - 2 * fc + fd;
    } else {
      const double p2 = 0.35355339059327373;  // 0.5/sqrt(2) rounded to binary64
      du1 = p2 * (fu - fd);
      du2 = 0.5 * (fu - 2 * fc + fd);
    }
    return fc + dt * (0.5 * dt * du2 - du1);
  }
  const double fc = at(y, x), fe = at(y, xp), fn = at(yp, x), fw = at(y, xm), fs = at(ym, x);
  const double fne = at(yp, xp), fnw = at(yp, xm), fsw = at(ym, xm), fse = at(ym, xp);
  if (SCHEME == SCH_FVM) {
    const double p2 = 0.5, p8 = 0.125;
    const double cfw = p2 * (fc + fw) - p2 * cxq * (fc - fw) - p8 * cyq * (fnw + fn - fsw - fs);
    const double cfn = p2 * (fc + fn) - p2 * cyq * (fn - fc) - p8 * cxq * (fne + fe - fnw - fw);
    const double cfe = p2 * (fc + fe) - p2 * cxq * (fe - fc) - p8 * cyq * (fne + fn - fse - fs);
    const double cfs = p2 * (fc + fs) - p2 * cyq * (fc - fs) - p8 * cxq * (fse + fe - fsw - fw);
    return fc - cxq * (cfe - cfw) - cyq * (cfn - cfs);
  }
  const double cxxq = 0.5 * cxq * cxq, cyyq = 0.5 * cyq * cyq, cxyq = cxq * cyq;
  double dfx, dfy, dfxx, dfyy, dfxy;
  if (SCHEME == SCH_FDM_ISO) {
    const double p2 = 0.5, two_thirds = 2.0 / 3.0, one_sixth = 1.0 / 6.0, five_sixths = 10.0 / 12.0,
                 one_twelth = 1.0 / 12.0;
    dfx = p2 * (one_sixth * (fne - fnw) + two_thirds * (fe - fw) + one_sixth * (fse - fsw));
    dfy = p2 * (one_sixth * (fne - fse) + two_thirds * (fn - fs) + one_sixth * (fnw - fsw));
    dfxx = one_twelth * (fne - 2 * fn + fnw) + five_sixths * (fe - 2 * fc + fw) + one_twelth * (fse - 2 * fs + fsw);
    dfyy = one_twelth * (fne - 2 * fe + fse) + five_sixths * (fn - 2 * fc + fs) + one_twelth * (fnw - 2 * fw + fsw);
    dfxy = 0.25 * (fne - fse - fnw + fsw);
  } else if (SCHEME == SCH_FDM_WLS) {
    const double one_sixth = 1.0 / 6.0, one_third = 1.0 / 3.0;
    dfx = one_sixth * ((fne - fnw) + (fe - fw) + (fse - fsw));
    dfy = one_sixth * ((fne - fse) + (fn - fs) + (fnw - fsw));
    dfxx = one_third * (fne - 2 * fn + fnw) + one_third * (fe - 2 * fc + fw) + one_third * (fse - 2 * fs + fsw);
    dfyy = one_third * (fne - 2 * fe + fse) + one_third * (fn - 2 * fc + fs) + one_third * (fnw - 2 * fw + fsw);
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

// grid%streaming => stream_fvm_bardow / stream_fdm_bardow / stream_fdm_sofonea.
// The rest population of the finite-difference schemes (all ld rows) is
// copied by the launcher; the finite-volume one copies rows 1:ny here.
template <int SCHEME>
__global__ void __launch_bounds__(kBlock) k_stream_scheme(const double* __restrict__ src, double* __restrict__ dst,
                                                         int nx, int ny, int ld, int ftiles, double dt) {
  int x, y;
  if (!cell_of<YFast>(ftiles, nx, ny, x, y)) return;
  const int xp = wrap_p(x, nx), xm = wrap_m(x, nx), yp = wrap_p(y, ny), ym = wrap_m(y, ny);
  if (SCHEME == SCH_FVM) dst[YFast::off(x, y, 0, nx, ny, ld)] = __ldg(src + YFast::off(x, y, 0, nx, ny, ld));
#pragma unroll
  for (int q = 1; q < 9; q++)
    dst[YFast::off(x, y, q, nx, ny, ld)] = scheme_cell<SCHEME>(src, q, x, y, xp, xm, yp, ym, nx, ny, ld, dt);
}

// lbm_stream: fdst(y,x,q) = fsrc(y - cy, x - cx, q) for rows 1:ny.
__global__ void __launch_bounds__(kBlock) k_stream(const double* __restrict__ src, double* __restrict__ dst,
                                                  int nx, int ny, int ld, int ftiles) {
  int x, y;
  if (!cell_of<YFast>(ftiles, nx, ny, x, y)) return;
#pragma unroll
  for (int q = 0; q < 9; q++) {
    const int sx = wrap_add(x, -cx_of(q), nx), sy = wrap_add(y, -cy_of(q), ny);
    dst[YFast::off(x, y, q, nx, ny, ld)] = __ldg(src + YFast::off(sx, sy, q, nx, ny, ld));
  }
}

template <int KIND>
__global__ void __launch_bounds__(kBlock) k_collide(double* __restrict__ f, int nx, int ny, int ld,
                                                   int ftiles, CollParams p) {
  int x, y;
  if (!cell_of<YFast>(ftiles, nx, ny, x, y)) return;
  double v[9];
#pragma unroll
  for (int q = 0; q < 9; q++) v[q] = f[YFast::off(x, y, q, nx, ny, ld)];
  collide_ref<KIND>(v, p);
#pragma unroll
  for (int q = 0; q < 9; q++) f[YFast::off(x, y, q, nx, ny, ld)] = v[q];
}

// collide_bgk_improved addresses the lattice through the dummy f1(ny,nx,0:8)
// (src/collision_bgk_improved.f90:26): row stride ny and plane stride ny*nx,
// whatever ld is.  Linear cell index c = y + ny*x.
__global__ void __launch_bounds__(kBlock) k_collide_bgki_seq(double* __restrict__ f, long long ncell,
                                                            CollParams p) {
  long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= ncell) return;
  double v[9];
#pragma unroll
  for (int q = 0; q < 9; q++) v[q] = f[c + ncell * q];
  coll_bgki_ref(v, p);
#pragma unroll
  for (int q = 0; q < 9; q++) f[c + ncell * q] = v[q];
}

inline int tiles(int n) { return (n + kBlock - 1) / kBlock; }

template <class L, bool SHIFT, bool PUSH>
cudaError_t launch_step(int kind, const Sweep& s, const CollParams& p) {
  const int ft = tiles(L::x_fast ? s.nx : s.ny);
  const int nslow = L::x_fast ? s.ny : s.nx;
  const long long blocks = (long long)ft * nslow;
  if (blocks <= 0 || blocks > 0x7fffffffLL) return cudaErrorInvalidConfiguration;
  const double* a = static_cast<const double*>(s.src);
  double* b = static_cast<double*>(s.dst);
  switch (kind) {
    case K_BGK: k_step<L, K_BGK, SHIFT, PUSH><<<(unsigned)blocks, kBlock, 0, s.stream>>>(a, b, s.nx, s.ny, s.ld, ft, p); break;
    case K_TRT: k_step<L, K_TRT, SHIFT, PUSH><<<(unsigned)blocks, kBlock, 0, s.stream>>>(a, b, s.nx, s.ny, s.ld, ft, p); break;
    case K_RR: k_step<L, K_RR, SHIFT, PUSH><<<(unsigned)blocks, kBlock, 0, s.stream>>>(a, b, s.nx, s.ny, s.ld, ft, p); break;
    case K_BGKI:
      if (SHIFT) return cudaErrorNotSupported;
      k_step<L, K_BGKI, false, PUSH><<<(unsigned)blocks, kBlock, 0, s.stream>>>(a, b, s.nx, s.ny, s.ld, ft, p);
      break;
    default: return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

}  // namespace

cudaError_t step_pull_f64(int kind, const Sweep& s, const CollParams& p) {
  return launch_step<YFast, false, false>(kind, s, p);
}

cudaError_t step_push_shift_f64(int kind, const Sweep& s, const CollParams& p) {
  return launch_step<XFast, true, true>(kind, s, p);
}

cudaError_t step_pull_pre_f64(int kind, const Sweep& s, void* pre, const CollParams& p) {
  const int ft = tiles(s.ny);
  const long long blocks = (long long)ft * s.nx;
  if (blocks <= 0 || blocks > 0x7fffffffLL) return cudaErrorInvalidConfiguration;
  const double* a = static_cast<const double*>(s.src);
  double* b = static_cast<double*>(s.dst);
  double* c = static_cast<double*>(pre);
  const unsigned nb = (unsigned)blocks;
  switch (kind) {
    case K_BGK: k_step_pre<K_BGK><<<nb, kBlock, 0, s.stream>>>(a, c, b, s.nx, s.ny, s.ld, ft, p); break;
    case K_TRT: k_step_pre<K_TRT><<<nb, kBlock, 0, s.stream>>>(a, c, b, s.nx, s.ny, s.ld, ft, p); break;
    case K_RR: k_step_pre<K_RR><<<nb, kBlock, 0, s.stream>>>(a, c, b, s.nx, s.ny, s.ld, ft, p); break;
    case K_BGKI: k_step_pre<K_BGKI><<<nb, kBlock, 0, s.stream>>>(a, c, b, s.nx, s.ny, s.ld, ft, p); break;
    default: return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

cudaError_t stream_scheme_f64(int scheme, const Sweep& s, double dt) {
  const int ft = tiles(s.ny);
  const long long blocks = (long long)ft * s.nx;
  if (blocks <= 0 || blocks > 0x7fffffffLL) return cudaErrorInvalidConfiguration;
  const double* a = static_cast<const double*>(s.src);
  double* b = static_cast<double*>(s.dst);
  const unsigned nb = (unsigned)blocks;
  if (scheme != SCH_FVM) {  // fnew(:,:,0) = fold(:,:,0), padding rows included
    cudaError_t e = cudaMemcpyAsync(b, a, sizeof(double) * (size_t)s.ld * s.nx, cudaMemcpyDeviceToDevice, s.stream);
    if (e != cudaSuccess) return e;
  }
  switch (scheme) {
    case SCH_FVM: k_stream_scheme<SCH_FVM><<<nb, kBlock, 0, s.stream>>>(a, b, s.nx, s.ny, s.ld, ft, dt); break;
    case SCH_FDM: k_stream_scheme<SCH_FDM><<<nb, kBlock, 0, s.stream>>>(a, b, s.nx, s.ny, s.ld, ft, dt); break;
    case SCH_FDM_ISO: k_stream_scheme<SCH_FDM_ISO><<<nb, kBlock, 0, s.stream>>>(a, b, s.nx, s.ny, s.ld, ft, dt); break;
    case SCH_FDM_WLS: k_stream_scheme<SCH_FDM_WLS><<<nb, kBlock, 0, s.stream>>>(a, b, s.nx, s.ny, s.ld, ft, dt); break;
    case SCH_SOFONEA: k_stream_scheme<SCH_SOFONEA><<<nb, kBlock, 0, s.stream>>>(a, b, s.nx, s.ny, s.ld, ft, dt); break;
    default: return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

cudaError_t stream_f64(const Sweep& s) {
  const int ft = tiles(s.ny);
  const long long blocks = (long long)ft * s.nx;
  if (blocks <= 0 || blocks > 0x7fffffffLL) return cudaErrorInvalidConfiguration;
  k_stream<<<(unsigned)blocks, kBlock, 0, s.stream>>>(static_cast<const double*>(s.src),
                                                      static_cast<double*>(s.dst), s.nx, s.ny, s.ld, ft);
  return cudaGetLastError();
}

cudaError_t collide_f64(int kind, const Sweep& s, const CollParams& p) {
  double* f = static_cast<double*>(s.dst);
  if (kind == K_BGKI) {
    const long long ncell = (long long)s.nx * s.ny;
    const long long blocks = (ncell + kBlock - 1) / kBlock;
    if (blocks <= 0 || blocks > 0x7fffffffLL) return cudaErrorInvalidConfiguration;
    k_collide_bgki_seq<<<(unsigned)blocks, kBlock, 0, s.stream>>>(f, ncell, p);
    return cudaGetLastError();
  }
  const int ft = tiles(s.ny);
  const long long blocks = (long long)ft * s.nx;
  if (blocks <= 0 || blocks > 0x7fffffffLL) return cudaErrorInvalidConfiguration;
  switch (kind) {
    case K_BGK: k_collide<K_BGK><<<(unsigned)blocks, kBlock, 0, s.stream>>>(f, s.nx, s.ny, s.ld, ft, p); break;
    case K_TRT: k_collide<K_TRT><<<(unsigned)blocks, kBlock, 0, s.stream>>>(f, s.nx, s.ny, s.ld, ft, p); break;
    case K_RR: k_collide<K_RR><<<(unsigned)blocks, kBlock, 0, s.stream>>>(f, s.nx, s.ny, s.ld, ft, p); break;
    default: return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

}  // namespace PLBM_NS
}  // namespace plbm
