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
#include "schemes.cuh"

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
// one thread per cell, populations 1..8, each the reference's expression of
// its 3x3 neighbourhood (sch::scheme_value; the strict build reproduces the
// Fortran exactly).  The rest population of the finite-difference schemes
// (all ld rows) is copied by the launcher; the finite-volume one copies rows
// 1:ny here.
template <int SCHEME>
__global__ void __launch_bounds__(kBlock) k_stream_scheme(const double* __restrict__ src, double* __restrict__ dst,
                                                         int nx, int ny, int ld, int ftiles, double dt) {
  int x, y;
  if (!cell_of<YFast>(ftiles, nx, ny, x, y)) return;
  const int xp = wrap_p(x, nx), xm = wrap_m(x, nx), yp = wrap_p(y, ny), ym = wrap_m(y, ny);
  if (SCHEME == sch::FVM) dst[YFast::off(x, y, 0, nx, ny, ld)] = __ldg(src + YFast::off(x, y, 0, nx, ny, ld));
#pragma unroll
  for (int q = 1; q < 9; q++) {
    double v[9];
    sch::gather<YFast>(src, q, x, y, xp, xm, yp, ym, nx, ny, ld, v);
    dst[YFast::off(x, y, q, nx, ny, ld)] = sch::scheme_value(SCHEME, v, q, dt);
  }
}

// Fused stencil-form streaming + collide_* (FMA build): one read pass of the
// 3x3 neighbourhoods (L1/L2 reuse), one write of the 9 collided populations.
template <int TAPS, int KIND>
__global__ void __launch_bounds__(kBlock) k_step_scheme(const double* __restrict__ src, double* __restrict__ dst,
                                                       int nx, int ny, int ld, int ftiles, sch::Stencil st,
                                                       CollParams p) {
  int x, y;
  if (!cell_of<YFast>(ftiles, nx, ny, x, y)) return;
  double f[9];
  sch::stencil_pull<YFast, TAPS>(src, x, y, nx, ny, ld, st, f);
  collide_ref<KIND>(f, p);
#pragma unroll
  for (int q = 0; q < 9; q++) dst[YFast::off(x, y, q, nx, ny, ld)] = f[q];
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
  const int bs = block_for((long long)s.nx * s.ny);
  const int nfast = L::x_fast ? s.nx : s.ny;
  const int ft = (nfast + bs - 1) / bs;
  const int nslow = L::x_fast ? s.ny : s.nx;
  const long long blocks = (long long)ft * nslow;
  if (blocks <= 0 || blocks > 0x7fffffffLL) return cudaErrorInvalidConfiguration;
  const double* a = static_cast<const double*>(s.src);
  double* b = static_cast<double*>(s.dst);
  switch (kind) {
    case K_BGK: k_step<L, K_BGK, SHIFT, PUSH><<<(unsigned)blocks, bs, 0, s.stream>>>(a, b, s.nx, s.ny, s.ld, ft, p); break;
    case K_TRT: k_step<L, K_TRT, SHIFT, PUSH><<<(unsigned)blocks, bs, 0, s.stream>>>(a, b, s.nx, s.ny, s.ld, ft, p); break;
    case K_RR: k_step<L, K_RR, SHIFT, PUSH><<<(unsigned)blocks, bs, 0, s.stream>>>(a, b, s.nx, s.ny, s.ld, ft, p); break;
    case K_BGKI:
      if (SHIFT) return cudaErrorNotSupported;
      k_step<L, K_BGKI, false, PUSH><<<(unsigned)blocks, bs, 0, s.stream>>>(a, b, s.nx, s.ny, s.ld, ft, p);
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
  if (scheme != sch::FVM) {  // fnew(:,:,0) = fold(:,:,0), padding rows included
    cudaError_t e = cudaMemcpyAsync(b, a, sizeof(double) * (size_t)s.ld * s.nx, cudaMemcpyDeviceToDevice, s.stream);
    if (e != cudaSuccess) return e;
  }
  switch (scheme) {
    case sch::FVM: k_stream_scheme<sch::FVM><<<nb, kBlock, 0, s.stream>>>(a, b, s.nx, s.ny, s.ld, ft, dt); break;
    case sch::FDM: k_stream_scheme<sch::FDM><<<nb, kBlock, 0, s.stream>>>(a, b, s.nx, s.ny, s.ld, ft, dt); break;
    case sch::FDM_ISO: k_stream_scheme<sch::FDM_ISO><<<nb, kBlock, 0, s.stream>>>(a, b, s.nx, s.ny, s.ld, ft, dt); break;
    case sch::FDM_WLS: k_stream_scheme<sch::FDM_WLS><<<nb, kBlock, 0, s.stream>>>(a, b, s.nx, s.ny, s.ld, ft, dt); break;
    case sch::SOFONEA: k_stream_scheme<sch::SOFONEA><<<nb, kBlock, 0, s.stream>>>(a, b, s.nx, s.ny, s.ld, ft, dt); break;
    case sch::FDM_WLS_G1: k_stream_scheme<sch::FDM_WLS_G1><<<nb, kBlock, 0, s.stream>>>(a, b, s.nx, s.ny, s.ld, ft, dt); break;
    case sch::FDM_WLS_G2: k_stream_scheme<sch::FDM_WLS_G2><<<nb, kBlock, 0, s.stream>>>(a, b, s.nx, s.ny, s.ld, ft, dt); break;
    default: return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

cudaError_t step_scheme_f64(int scheme, int kind, const Sweep& s, double dt, const CollParams& p) {
  const int ft = tiles(s.ny);
  const long long blocks = (long long)ft * s.nx;
  if (blocks <= 0 || blocks > 0x7fffffffLL) return cudaErrorInvalidConfiguration;
  if (kind == K_BGKI && s.ld != s.ny) return cudaErrorNotSupported;
  const sch::Stencil st = sch::stencil_coefficients(scheme, dt);
  const double* a = static_cast<const double*>(s.src);
  double* b = static_cast<double*>(s.dst);
  const unsigned nb = (unsigned)blocks;
#define PLBM_SCH_KIND(SC)                                                                                     \
  switch (kind) {                                                                                             \
    case K_BGK: k_step_scheme<SC, K_BGK><<<nb, kBlock, 0, s.stream>>>(a, b, s.nx, s.ny, s.ld, ft, st, p); break; \
    case K_TRT: k_step_scheme<SC, K_TRT><<<nb, kBlock, 0, s.stream>>>(a, b, s.nx, s.ny, s.ld, ft, st, p); break; \
    case K_RR: k_step_scheme<SC, K_RR><<<nb, kBlock, 0, s.stream>>>(a, b, s.nx, s.ny, s.ld, ft, st, p); break;   \
    case K_BGKI: k_step_scheme<SC, K_BGKI><<<nb, kBlock, 0, s.stream>>>(a, b, s.nx, s.ny, s.ld, ft, st, p); break; \
    default: return cudaErrorInvalidValue;                                                                    \
  }
  if (scheme < sch::FVM || scheme > sch::FDM_WLS_G2) return cudaErrorInvalidValue;
  switch (sch::taps_of(scheme)) {
    case sch::TAPS_LINE: PLBM_SCH_KIND(sch::TAPS_LINE) break;
    case sch::TAPS_AXIS3: PLBM_SCH_KIND(sch::TAPS_AXIS3) break;
    default: PLBM_SCH_KIND(sch::TAPS_FULL) break;
  }
#undef PLBM_SCH_KIND
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
