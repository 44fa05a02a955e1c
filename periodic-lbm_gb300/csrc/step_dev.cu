// step_dev.cu -- deviation-storage stream/collide kernels.
//
// Populations are held as h_i = f_i - w_i (the shifted form of
// sim/sim.F90:131,384) in binary32 or in binary16 scaled by 2^15, and the
// collision runs in binary32 on the shifted form (coll_*_shift).  The
// traffic per cell update is 72 B (binary32) or 36 B (binary16).
#include "plbm_launch.h"

namespace plbm {
namespace {

template <class L>
__device__ __forceinline__ bool dev_cell(int ftiles, int nx, int ny, int& x, int& y) {
  if (L::x_fast) {
    y = blockIdx.x / ftiles;
    x = (blockIdx.x - y * ftiles) * blockDim.x + threadIdx.x;
    return x < nx;
  }
  x = blockIdx.x / ftiles;
  y = (blockIdx.x - x * ftiles) * blockDim.x + threadIdx.x;
  return y < ny;
}

template <class L, class S, int KIND, bool PUSH>
__global__ void __launch_bounds__(kBlock) k_step_dev(const typename S::elem* __restrict__ src,
                                                    typename S::elem* __restrict__ dst, int nx, int ny,
                                                    int ld, int ftiles, CollParams p) {
  int x, y;
  if (!dev_cell<L>(ftiles, nx, ny, x, y)) return;
  float h[9];
#pragma unroll
  for (int q = 0; q < 9; q++) {
    const int sx = PUSH ? x : wrap_add(x, -cx_of(q), nx);
    const int sy = PUSH ? y : wrap_add(y, -cy_of(q), ny);
    h[q] = S::load(src, L::off(sx, sy, q, nx, ny, ld));
  }
  collide_shift<KIND, float>(h, p);
#pragma unroll
  for (int q = 0; q < 9; q++) {
    const int dx = PUSH ? wrap_add(x, cx_of(q), nx) : x;
    const int dy = PUSH ? wrap_add(y, cy_of(q), ny) : y;
    S::store(dst, L::off(dx, dy, q, nx, ny, ld), h[q]);
  }
}

template <class S>
__global__ void __launch_bounds__(kBlock) k_stream_dev(const typename S::elem* __restrict__ src,
                                                      typename S::elem* __restrict__ dst, int nx, int ny,
                                                      int ld, int ftiles) {
  int x, y;
  if (!dev_cell<YFast>(ftiles, nx, ny, x, y)) return;
#pragma unroll
  for (int q = 0; q < 9; q++) {
    const int sx = wrap_add(x, -cx_of(q), nx), sy = wrap_add(y, -cy_of(q), ny);
    dst[YFast::off(x, y, q, nx, ny, ld)] = src[YFast::off(sx, sy, q, nx, ny, ld)];
  }
}

template <class S, int KIND>
__global__ void __launch_bounds__(kBlock) k_collide_dev(typename S::elem* __restrict__ f, int nx, int ny,
                                                       int ld, int ftiles, CollParams p) {
  int x, y;
  if (!dev_cell<YFast>(ftiles, nx, ny, x, y)) return;
  float h[9];
#pragma unroll
  for (int q = 0; q < 9; q++) {
    const size_t o = YFast::off(x, y, q, nx, ny, ld);
    h[q] = S::load(f, o);
  }
  collide_shift<KIND, float>(h, p);
#pragma unroll
  for (int q = 0; q < 9; q++) S::store(f, YFast::off(x, y, q, nx, ny, ld), h[q]);
}

inline int tiles(int n) { return (n + kBlock - 1) / kBlock; }

template <class L, class S, bool PUSH>
cudaError_t launch_dev(int kind, const Sweep& s, const CollParams& p) {
  const int ft = tiles(L::x_fast ? s.nx : s.ny);
  const long long blocks = (long long)ft * (L::x_fast ? s.ny : s.nx);
  if (blocks <= 0 || blocks > 0x7fffffffLL) return cudaErrorInvalidConfiguration;
  typedef typename S::elem E;
  const E* a = static_cast<const E*>(s.src);
  E* b = static_cast<E*>(s.dst);
  switch (kind) {
    case K_BGK: k_step_dev<L, S, K_BGK, PUSH><<<(unsigned)blocks, kBlock, 0, s.stream>>>(a, b, s.nx, s.ny, s.ld, ft, p); break;
    case K_TRT: k_step_dev<L, S, K_TRT, PUSH><<<(unsigned)blocks, kBlock, 0, s.stream>>>(a, b, s.nx, s.ny, s.ld, ft, p); break;
    case K_RR: k_step_dev<L, S, K_RR, PUSH><<<(unsigned)blocks, kBlock, 0, s.stream>>>(a, b, s.nx, s.ny, s.ld, ft, p); break;
    default: return cudaErrorNotSupported;
  }
  return cudaGetLastError();
}

template <class S>
cudaError_t launch_collide_dev(int kind, const Sweep& s, const CollParams& p) {
  const int ft = tiles(s.ny);
  const long long blocks = (long long)ft * s.nx;
  if (blocks <= 0 || blocks > 0x7fffffffLL) return cudaErrorInvalidConfiguration;
  typedef typename S::elem E;
  E* f = static_cast<E*>(s.dst);
  switch (kind) {
    case K_BGK: k_collide_dev<S, K_BGK><<<(unsigned)blocks, kBlock, 0, s.stream>>>(f, s.nx, s.ny, s.ld, ft, p); break;
    case K_TRT: k_collide_dev<S, K_TRT><<<(unsigned)blocks, kBlock, 0, s.stream>>>(f, s.nx, s.ny, s.ld, ft, p); break;
    case K_RR: k_collide_dev<S, K_RR><<<(unsigned)blocks, kBlock, 0, s.stream>>>(f, s.nx, s.ny, s.ld, ft, p); break;
    default: return cudaErrorNotSupported;
  }
  return cudaGetLastError();
}

}  // namespace

cudaError_t step_pull_dev(int storage, int kind, const Sweep& s, const CollParams& p) {
  if (storage == ST_F32DEV) return launch_dev<YFast, StoreF32Dev, false>(kind, s, p);
  if (storage == ST_F16DEV) return launch_dev<YFast, StoreF16Dev, false>(kind, s, p);
  return cudaErrorInvalidValue;
}

cudaError_t step_push_dev(int storage, int kind, const Sweep& s, const CollParams& p) {
  if (storage == ST_F32DEV) return launch_dev<XFast, StoreF32Dev, true>(kind, s, p);
  if (storage == ST_F16DEV) return launch_dev<XFast, StoreF16Dev, true>(kind, s, p);
  return cudaErrorInvalidValue;
}

cudaError_t stream_dev(int storage, const Sweep& s) {
  const int ft = tiles(s.ny);
  const long long blocks = (long long)ft * s.nx;
  if (blocks <= 0 || blocks > 0x7fffffffLL) return cudaErrorInvalidConfiguration;
  if (storage == ST_F32DEV)
    k_stream_dev<StoreF32Dev><<<(unsigned)blocks, kBlock, 0, s.stream>>>(
        static_cast<const float*>(s.src), static_cast<float*>(s.dst), s.nx, s.ny, s.ld, ft);
  else if (storage == ST_F16DEV)
    k_stream_dev<StoreF16Dev><<<(unsigned)blocks, kBlock, 0, s.stream>>>(
        static_cast<const __half*>(s.src), static_cast<__half*>(s.dst), s.nx, s.ny, s.ld, ft);
  else
    return cudaErrorInvalidValue;
  return cudaGetLastError();
}

cudaError_t collide_dev(int storage, int kind, const Sweep& s, const CollParams& p) {
  if (storage == ST_F32DEV) return launch_collide_dev<StoreF32Dev>(kind, s, p);
  if (storage == ST_F16DEV) return launch_collide_dev<StoreF16Dev>(kind, s, p);
  return cudaErrorInvalidValue;
}

}  // namespace plbm
