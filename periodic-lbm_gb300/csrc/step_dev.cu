// step_dev.cu -- deviation-storage stream/collide kernels.
//
// Populations are held as h_i = f_i - w_i (the shifted form of
// sim/sim.F90:131,384) in binary32 or in binary16 scaled by 2^15, and the
// collision runs in binary32 on the shifted form (coll_*_shift).  The fused
// binary16 pull step collides in the stored scale (H = 2^15 h) and, on even
// ny, updates two y-adjacent cells per thread (k_step_f16_pull2).  The
// traffic per cell update is 72 B (binary32) or 36 B (binary16).
#include <type_traits>

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

// BGK on binary16 deviations kept in their stored scale, H = 2^15 h: the
// scale enters the constants instead of 18 multiplies per cell.  rho = 1 +
// 2^-15 sum H, u = j / rho, and H' = (1 - omega) H + omega Heq with Heq =
// w (sum H + 2^15 rho P), P = -1.5 u^2 + 3 c.u + 4.5 (c.u)^2 -- the shifted
// equilibrium of coll_bgk_shift, scaled, with omega w folded into the two
// per-cell factors.  u takes the approximate division (2 ulp): binary16
// storage rounds the populations to 2^-11 relative, far above it.
__device__ __forceinline__ void coll_bgk_shift_f16scaled(float (&H)[9], float omega) {
  const float dh = (((H[5] + H[7]) + (H[6] + H[8])) + ((H[1] + H[3]) + (H[2] + H[4]))) + H[0];
  const float rho = fmaf(dh, F16_INV_SCALE, 1.0f);
  const float r = __fdividef(F16_INV_SCALE, rho);
  const float ux = (((H[5] - H[7]) + (H[8] - H[6])) + (H[1] - H[3])) * r;
  const float uy = (((H[5] - H[7]) + (H[6] - H[8])) + (H[2] - H[4])) * r;
  const float uxx = ux * ux, uyy = uy * uy;
  const float indp = -1.5f * (uxx + uyy);
  const float sr = F16_SCALE * rho, omb = 1.0f - omega;
  const float a0 = omega * (4.0f / 9.0f), as = omega * (1.0f / 9.0f), ad = omega * (1.0f / 36.0f);
  const float k00 = a0 * dh, k10 = a0 * sr, k0s = as * dh, k1s = as * sr, k0d = ad * dh, k1d = ad * sr;
  H[0] = fmaf(omb, H[0], fmaf(k10, indp, k00));
  const float bx = fmaf(4.5f, uxx, indp), by = fmaf(4.5f, uyy, indp);
  H[1] = fmaf(omb, H[1], fmaf(k1s, fmaf(3.0f, ux, bx), k0s));
  H[3] = fmaf(omb, H[3], fmaf(k1s, fmaf(-3.0f, ux, bx), k0s));
  H[2] = fmaf(omb, H[2], fmaf(k1s, fmaf(3.0f, uy, by), k0s));
  H[4] = fmaf(omb, H[4], fmaf(k1s, fmaf(-3.0f, uy, by), k0s));
  const float uxpy = ux + uy, uxmy = ux - uy;
  const float bp = fmaf(4.5f * uxpy, uxpy, indp), bm = fmaf(4.5f * uxmy, uxmy, indp);
  H[5] = fmaf(omb, H[5], fmaf(k1d, fmaf(3.0f, uxpy, bp), k0d));
  H[7] = fmaf(omb, H[7], fmaf(k1d, fmaf(-3.0f, uxpy, bp), k0d));
  H[6] = fmaf(omb, H[6], fmaf(k1d, fmaf(-3.0f, uxmy, bm), k0d));
  H[8] = fmaf(omb, H[8], fmaf(k1d, fmaf(3.0f, uxmy, bm), k0d));
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
  const I offs[9] = {c0 + y0,         P + cm + y0,     2 * P + c0 + ym, 3 * P + cp + y0, 4 * P + c0 + yp,
                     5 * P + cm + ym, 6 * P + cp + ym, 7 * P + cp + yp, 8 * P + cm + yp};
  const I o = c0 + y0;
  if constexpr (std::is_same<S, StoreF16Dev>::value) {
    float H[9];
#pragma unroll
    for (int q = 0; q < 9; q++) H[q] = __half2float(__ldg(src + offs[q]));
    if constexpr (KIND == K_TRT) coll_trt_shift<float, true>(H, p.a, p.b, p.c);
    else if constexpr (KIND == K_RR) coll_rr_shift<float, true>(H, p.a, p.b, p.c);
    else coll_bgk_shift_f16scaled(H, p.a);
#pragma unroll
    for (int q = 0; q < 9; q++) dst[(I)q * P + o] = __float2half_rn(H[q]);
    return;
  }
  float h[9];
#pragma unroll
  for (int q = 0; q < 9; q++) h[q] = S::load(src, offs[q]);
  if (KIND == K_TRT) coll_trt_shift<float>(h, p.a, p.b, p.c);
  else if (KIND == K_RR) coll_rr_shift<float>(h, p.a, p.b, p.c);
  else coll_bgk_shift<float>(h, p.a);
#pragma unroll
  for (int q = 0; q < 9; q++) S::store(dst, (I)q * P + o, h[q]);
}

// The binary16 pull step with two y-adjacent cells per thread (y even): the
// nine stores and the three loads without a y shift move as half2, one
// 4-byte access and one conversion for both cells.  The cell operations are
// those of k_step_dev_pull<StoreF16Dev>.  Needs ny even (y + 1 < ny), ld even
// and 4-byte aligned lattices, so that every half2 offset is even.
template <int KIND, typename I>
__global__ void __launch_bounds__(kBlock) k_step_f16_pull2(const __half* __restrict__ src, __half* __restrict__ dst,
                                                          int nx, int ny, int ld, int ftiles, ShiftParamsF p) {
  const int x = blockIdx.x / ftiles;
  const int y = 2 * ((blockIdx.x - x * ftiles) * blockDim.x + threadIdx.x);
  if (y >= ny) return;
  const I L = (I)ld, P = (I)ld * (I)nx;
  const I c0 = (I)x * L, cm = (I)wrap_m(x, nx) * L, cp = (I)wrap_p(x, nx) * L;
  const I y0 = (I)y, y1 = (I)(y + 1), ym = (I)wrap_m(y, ny), yp = (I)wrap_p(y + 1, ny);
  const __half2* s2 = reinterpret_cast<const __half2*>(src);
  float A[9], B[9];
  const float2 v0 = __half22float2(__ldg(s2 + (c0 + y0) / 2));
  const float2 v1 = __half22float2(__ldg(s2 + (P + cm + y0) / 2));
  const float2 v3 = __half22float2(__ldg(s2 + (3 * P + cp + y0) / 2));
  A[0] = v0.x, B[0] = v0.y, A[1] = v1.x, B[1] = v1.y, A[3] = v3.x, B[3] = v3.y;
  A[2] = __half2float(__ldg(src + 2 * P + c0 + ym)), B[2] = __half2float(__ldg(src + 2 * P + c0 + y0));
  A[4] = __half2float(__ldg(src + 4 * P + c0 + y1)), B[4] = __half2float(__ldg(src + 4 * P + c0 + yp));
  A[5] = __half2float(__ldg(src + 5 * P + cm + ym)), B[5] = __half2float(__ldg(src + 5 * P + cm + y0));
  A[6] = __half2float(__ldg(src + 6 * P + cp + ym)), B[6] = __half2float(__ldg(src + 6 * P + cp + y0));
  A[7] = __half2float(__ldg(src + 7 * P + cp + y1)), B[7] = __half2float(__ldg(src + 7 * P + cp + yp));
  A[8] = __half2float(__ldg(src + 8 * P + cm + y1)), B[8] = __half2float(__ldg(src + 8 * P + cm + yp));
  if constexpr (KIND == K_TRT) {
    coll_trt_shift<float, true>(A, p.a, p.b, p.c);
    coll_trt_shift<float, true>(B, p.a, p.b, p.c);
  } else if constexpr (KIND == K_RR) {
    coll_rr_shift<float, true>(A, p.a, p.b, p.c);
    coll_rr_shift<float, true>(B, p.a, p.b, p.c);
  } else {
    coll_bgk_shift_f16scaled(A, p.a);
    coll_bgk_shift_f16scaled(B, p.a);
  }
  __half2* d2 = reinterpret_cast<__half2*>(dst) + (c0 + y0) / 2;
#pragma unroll
  for (int q = 0; q < 9; q++) d2[(I)q * (P / 2)] = __floats2half2_rn(A[q], B[q]);
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

template <typename I>
cudaError_t launch_f16_pull2(int kind, const Sweep& s, const CollParams& cp) {
  const int bs = block_for((long long)s.nx * (s.ny / 2));
  const int ft = (s.ny / 2 + bs - 1) / bs;
  const long long blocks = (long long)ft * s.nx;
  if (blocks <= 0 || blocks > 0x7fffffffLL) return cudaErrorInvalidConfiguration;
  const __half* a = static_cast<const __half*>(s.src);
  __half* b = static_cast<__half*>(s.dst);
  const ShiftParamsF p = shift_params(kind, cp);
  const unsigned nb = (unsigned)blocks;
  switch (kind) {
    case K_BGK: k_step_f16_pull2<K_BGK, I><<<nb, bs, 0, s.stream>>>(a, b, s.nx, s.ny, s.ld, ft, p); break;
    case K_TRT: k_step_f16_pull2<K_TRT, I><<<nb, bs, 0, s.stream>>>(a, b, s.nx, s.ny, s.ld, ft, p); break;
    case K_RR: k_step_f16_pull2<K_RR, I><<<nb, bs, 0, s.stream>>>(a, b, s.nx, s.ny, s.ld, ft, p); break;
    default: return cudaErrorNotSupported;
  }
  return cudaGetLastError();
}

}  // namespace

cudaError_t step_pull_dev(int storage, int kind, const Sweep& s, const CollParams& p) {
  const bool small = (unsigned long long)s.ld * (unsigned long long)s.nx * 9ull < (1ull << 32);
  const bool pairs = s.ny % 2 == 0 && s.ld % 2 == 0 &&
                     (((uintptr_t)s.src | (uintptr_t)s.dst) & 3) == 0;
  if (storage == ST_F16DEV && pairs)
    return small ? launch_f16_pull2<uint32_t>(kind, s, p) : launch_f16_pull2<size_t>(kind, s, p);
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
