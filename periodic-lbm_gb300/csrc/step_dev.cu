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

// Relaxation constants of the shifted operators, rounded to binary32 once
// on the host: BGK (omega), TRT (le, les, lds), RR (w (1 - omega) x 3).
struct ShiftParamsF {
  float a, b, c;
};

ShiftParamsF shift_params(int kind, const CollParams& p) {
  if (kind == K_TRT) return {(float)p.omega, (float)p.les, (float)p.lds};
  if (kind == K_RR) return {(float)p.rr_w0, (float)p.rr_ws, (float)p.rr_wd};
  return {(float)p.omega, 0.0f, 0.0f};
}

// The pull step of the src/ layout (YFast) with explicit pull offsets: I is
// the offset type, 32-bit when the lattice has fewer than 2^32 elements (one
// multiply-add per address instead of 64-bit index arithmetic).
template <class S, int KIND, typename I>
__global__ void __launch_bounds__(kBlock) k_step_dev_pull(const typename S::elem* __restrict__ src,
                                                         typename S::elem* __restrict__ dst, int nx, int ny,
                                                         int ld, int ftiles, ShiftParamsF p) {
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
  if (KIND == K_TRT) coll_trt_shift<float>(h, p.a, p.b, p.c);
  else if (KIND == K_RR) coll_rr_shift<float>(h, p.a, p.b, p.c);
  else coll_bgk_shift<float>(h, p.a);
  const I o = c0 + y0;
#pragma unroll
  for (int q = 0; q < 9; q++) S::store(dst, (I)q * P + o, h[q]);
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
  const int bs = block_for((long long)s.nx * s.ny);
  const int ft = ((L::x_fast ? s.nx : s.ny) + bs - 1) / bs;
  const long long blocks = (long long)ft * (L::x_fast ? s.ny : s.nx);
  if (blocks <= 0 || blocks > 0x7fffffffLL) return cudaErrorInvalidConfiguration;
  typedef typename S::elem E;
  const E* a = static_cast<const E*>(s.src);
  E* b = static_cast<E*>(s.dst);
  switch (kind) {
    case K_BGK: k_step_dev<L, S, K_BGK, PUSH><<<(unsigned)blocks, bs, 0, s.stream>>>(a, b, s.nx, s.ny, s.ld, ft, p); break;
    case K_TRT: k_step_dev<L, S, K_TRT, PUSH><<<(unsigned)blocks, bs, 0, s.stream>>>(a, b, s.nx, s.ny, s.ld, ft, p); break;
    case K_RR: k_step_dev<L, S, K_RR, PUSH><<<(unsigned)blocks, bs, 0, s.stream>>>(a, b, s.nx, s.ny, s.ld, ft, p); break;
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

template <class S, typename I>
cudaError_t launch_pull_dev(int kind, const Sweep& s, const CollParams& cp) {
  const int bs = block_for((long long)s.nx * s.ny);
  const int ft = (s.ny + bs - 1) / bs;
  const long long blocks = (long long)ft * s.nx;
  if (blocks <= 0 || blocks > 0x7fffffffLL) return cudaErrorInvalidConfiguration;
  typedef typename S::elem E;
  const E* a = static_cast<const E*>(s.src);
  E* b = static_cast<E*>(s.dst);
  const ShiftParamsF p = shift_params(kind, cp);
  const unsigned nb = (unsigned)blocks;
  switch (kind) {
    case K_BGK: k_step_dev_pull<S, K_BGK, I><<<nb, bs, 0, s.stream>>>(a, b, s.nx, s.ny, s.ld, ft, p); break;
    case K_TRT: k_step_dev_pull<S, K_TRT, I><<<nb, bs, 0, s.stream>>>(a, b, s.nx, s.ny, s.ld, ft, p); break;
    case K_RR: k_step_dev_pull<S, K_RR, I><<<nb, bs, 0, s.stream>>>(a, b, s.nx, s.ny, s.ld, ft, p); break;
    default: return cudaErrorNotSupported;
  }
  return cudaGetLastError();
}

}  // namespace

cudaError_t step_pull_dev(int storage, int kind, const Sweep& s, const CollParams& p) {
  const bool small = (unsigned long long)s.ld * (unsigned long long)s.nx * 9ull < (1ull << 32);
  if (storage == ST_F32DEV)
    return small ? launch_pull_dev<StoreF32Dev, uint32_t>(kind, s, p) : launch_pull_dev<StoreF32Dev, size_t>(kind, s, p);
  if (storage == ST_F16DEV)
    return small ? launch_pull_dev<StoreF16Dev, uint32_t>(kind, s, p) : launch_pull_dev<StoreF16Dev, size_t>(kind, s, p);
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
