// fields.cu -- per-cell field kernels around the step: moments, equilibrium
// initialisation, storage conversion, vorticity and binary64 reductions.
// Compiled with --fmad=false: the moments and equilibria then perform the
// same IEEE operations as update_macros / equilibrium() of the reference.
// With `exact` (grids in hybrid arithmetic) the binary64 lattices take the
// integer forms of exact_fields.cuh instead, correctly rounded from the exact
// moments, cell by cell back to the reference's expressions outside their range.
#include "plbm_launch.h"
#include "exact_fields.cuh"

namespace plbm {
namespace {

inline int tiles(int n) { return (n + kBlock - 1) / kBlock; }

// Cell of a (fast, slow) launch: blocks are ftiles per slow line, the first
// line is slow0 (a slab of slow lines when the work is split).
__device__ __forceinline__ bool fs_cell(int ftiles, int nfast, int& fast, int& slow, int slow0 = 0) {
  const int b = blockIdx.x / ftiles;
  fast = (blockIdx.x - b * ftiles) * blockDim.x + threadIdx.x;
  slow = slow0 + b;
  return fast < nfast;
}

template <int ST>
__device__ __forceinline__ double load_pop(const void* f, size_t i) {
  if (ST == ST_F64 || ST == ST_F64SHIFT) return __ldg(static_cast<const double*>(f) + i);
  if (ST == ST_F32DEV) return (double)__ldg(static_cast<const float*>(f) + i);
  return (double)(__half2float(__ldg(static_cast<const __half*>(f) + i)) * F16_INV_SCALE);
}

template <int ST>
__device__ __forceinline__ void store_pop(void* f, size_t i, double v) {
  if (ST == ST_F64 || ST == ST_F64SHIFT) static_cast<double*>(f)[i] = v;
  else if (ST == ST_F32DEV) static_cast<float*>(f)[i] = (float)v;
  else static_cast<__half*>(f)[i] = __float2half_rn((float)v * F16_SCALE);
}

// Moments of one cell.  Unshifted binary64: update_macros order,
// src/fvm_bardow.F90:368-382.  Shifted storage: lbm_macros order,
// sim/sim.F90:160-173 (rho = sum h + 1, u = j/rho).
template <int ST>
__device__ __forceinline__ void cell_moments(const double (&fs)[9], double& rho, double& ux, double& uy) {
  if (ST == ST_F64) {
    rho = fs[0] + (((fs[5] + fs[7]) + (fs[6] + fs[8])) + ((fs[1] + fs[3]) + (fs[2] + fs[4])));
    double invrho = 1.0 / rho;
    ux = invrho * (((fs[5] - fs[7]) + (fs[8] - fs[6])) + (fs[1] - fs[3]));
    uy = invrho * (((fs[5] - fs[7]) + (fs[6] - fs[8])) + (fs[2] - fs[4]));
  } else {
    rho = (((fs[5] + fs[7]) + (fs[6] + fs[8])) + ((fs[1] + fs[3]) + (fs[2] + fs[4]))) + fs[0];
    rho = rho + 1.0;
    ux = (((fs[5] - fs[7]) + (fs[8] - fs[6])) + (fs[1] - fs[3])) / rho;
    uy = (((fs[5] - fs[7]) + (fs[6] - fs[8])) + (fs[2] - fs[4])) / rho;
  }
}

// The reference's moments of a cell outside the exact forms' range, out of
// line so that the fast path does not carry them.
template <int ST>
__device__ __noinline__ void cell_moments_ref(const double* fs, double* out) {
  double g[9];
#pragma unroll
  for (int q = 0; q < 9; q++) g[q] = fs[q];
  cell_moments<ST>(g, out[0], out[1], out[2]);
}

template <int ST, class L, bool EXACT>
__global__ void __launch_bounds__(kBlock) k_macros(const void* __restrict__ f, double* __restrict__ rho,
                                                  double* __restrict__ ux, double* __restrict__ uy, int nx,
                                                  int ny, int ld, int ftiles, int slow0) {
  const int nfast = L::x_fast ? nx : ny;
  int fast, slow;
  if (!fs_cell(ftiles, nfast, fast, slow, slow0)) return;
  const int x = L::x_fast ? fast : slow, y = L::x_fast ? slow : fast;
  double fs[9];
#pragma unroll
  for (int q = 0; q < 9; q++) fs[q] = load_pop<ST>(f, L::off(x, y, q, nx, ny, ld));
  double r, u, v;
  if constexpr (EXACT) {
    bool bad = false;
    ex::macros_exact<ST == ST_F64SHIFT>(fs, r, u, v, bad);
    if (bad) {
      double m[3];
      cell_moments_ref<ST>(fs, m);
      r = m[0], u = m[1], v = m[2];
    }
  } else {
    cell_moments<ST>(fs, r, u, v);
  }
  const size_t o = (size_t)fast + (size_t)nfast * slow;
  if (rho) rho[o] = r;
  if (ux) ux[o] = u;
  if (uy) uy[o] = v;
}

// equilibrium(), src/fvm_bardow.F90:99-126
__device__ __forceinline__ void eq_ref(double rho, double ux, double uy, double (&feq)[9]) {
  double uxx = ux * ux;
  double uyy = uy * uy;
  double indp = 1.0 - 1.5 * (uxx + uyy);
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
}

// equilibrium() with ddf_shift, sim/sim.F90:357-384
__device__ __forceinline__ void eq_shift(double rho, double ux, double uy, double (&feq)[9]) {
  double uxx = ux * ux, uyy = uy * uy;
  double uxpy = ux + uy, uxmy = ux - uy;
  double indp = -1.5 * (uxx + uyy);
  feq[0] = W0 * rho * (indp);
  feq[1] = WS * rho * (indp + 3.0 * ux + 4.5 * uxx);
  feq[2] = WS * rho * (indp + 3.0 * uy + 4.5 * uyy);
  feq[3] = WS * rho * (indp - 3.0 * ux + 4.5 * uxx);
  feq[4] = WS * rho * (indp - 3.0 * uy + 4.5 * uyy);
  feq[5] = WD * rho * (indp + 3.0 * uxpy + 4.5 * uxpy * uxpy);
  feq[7] = WD * rho * (indp - 3.0 * uxpy + 4.5 * uxpy * uxpy);
  feq[6] = WD * rho * (indp - 3.0 * uxmy + 4.5 * uxmy * uxmy);
  feq[8] = WD * rho * (indp + 3.0 * uxmy + 4.5 * uxmy * uxmy);
#pragma unroll
  for (int q = 0; q < 9; q++) feq[q] = feq[q] + w_of(q) * (rho - 1.0);
}

// The reference's equilibrium of one cell for storage ST (below).
template <int ST>
__device__ __forceinline__ void cell_equilibrium(double r, double u, double v, int from_pressure,
                                                 double (&feq)[9]) {
  if (ST == ST_F64) {
    eq_ref(r, u, v, feq);
  } else if (from_pressure) {
    eq_shift(1.0 + r / CSQR, u, v, feq);
  } else {
    eq_ref(r, u, v, feq);
#pragma unroll
    for (int q = 0; q < 9; q++) feq[q] = feq[q] - w_of(q);
  }
}
template <int ST>
__device__ __noinline__ void cell_equilibrium_ref(double r, double u, double v, int from_pressure, double* out) {
  double feq[9];
  cell_equilibrium<ST>(r, u, v, from_pressure, feq);
#pragma unroll
  for (int q = 0; q < 9; q++) out[q] = feq[q];
}

// ST_F64: reference equilibrium of rho.  Shifted storages: from_pressure
// selects rho = 1 + p/cs^2 (sim/sim.F90:193) and the shifted equilibrium of
// sim/sim.F90; otherwise the reference equilibrium minus w_i.  EXACT (binary64
// storages only): the integer forms, the reference's expressions for a cell
// outside their range.
template <int ST, class L, bool EXACT>
__global__ void __launch_bounds__(kBlock) k_equilibrium(const double* __restrict__ rho,
                                                       const double* __restrict__ ux,
                                                       const double* __restrict__ uy, int from_pressure,
                                                       void* __restrict__ f, int nx, int ny, int ld,
                                                       int ftiles, int slow0) {
  const int nfast = L::x_fast ? nx : ny;
  int fast, slow;
  if (!fs_cell(ftiles, nfast, fast, slow, slow0)) return;
  const int x = L::x_fast ? fast : slow, y = L::x_fast ? slow : fast;
  const size_t o = (size_t)fast + (size_t)nfast * slow;
  double feq[9];
  if constexpr (EXACT) {
    const double r = rho[o], u = ux[o], v = uy[o];
    bool bad = false;
    const int64_t P = (ST == ST_F64SHIFT && from_pressure) ? ex::rho_fixed_from_pressure(r, bad)
                                                           : ex::rho_fixed(r, bad);
    ex::equilibrium_exact<ST == ST_F64SHIFT>(P, u, v, feq, bad);
    if (bad) cell_equilibrium_ref<ST>(r, u, v, from_pressure, feq);
  } else {
    cell_equilibrium<ST>(rho[o], ux[o], uy[o], from_pressure, feq);
  }
#pragma unroll
  for (int q = 0; q < 9; q++) store_pop<ST>(f, L::off(x, y, q, nx, ny, ld), feq[q]);
}

// f (binary64, YFast) <-> h = f - w (deviation storage), over rows 0..ny-1.
template <int ST, bool TO_DEV>
__global__ void __launch_bounds__(kBlock) k_convert(const void* __restrict__ a, void* __restrict__ b, int nx,
                                                   int ny, int ld, int ftiles) {
  int y, x;
  if (!fs_cell(ftiles, ny, y, x)) return;
#pragma unroll
  for (int q = 0; q < 9; q++) {
    const size_t i = YFast::off(x, y, q, nx, ny, ld);
    if (TO_DEV) store_pop<ST>(b, i, static_cast<const double*>(a)[i] - w_of(q));
    else static_cast<double*>(b)[i] = load_pop<ST>(a, i) + w_of(q);
  }
}

// vorticity_2nd / vorticity_4th, src/vorticity.f90:13-87 ((ny,nx) arrays).
// ORDER 4 keeps the reference weights t1 = 1/12 on +-1 and t2 = 2/3 on +-2;
// ORDER 44 uses t1 = 2/3, t2 = 1/12 (the standard fourth-order stencil).
template <int ORDER>
__global__ void __launch_bounds__(kBlock) k_vorticity(const double* __restrict__ ux,
                                                     const double* __restrict__ uy, double* __restrict__ w,
                                                     int nx, int ny, int ftiles) {
  int y, x;
  if (!fs_cell(ftiles, ny, y, x)) return;
  const int xp1 = (x + 1) % nx, xm1 = (x - 1 + nx) % nx;
  const int yp1 = (y + 1) % ny, ym1 = (y - 1 + ny) % ny;
#define A(a, yy, xx) a[(size_t)(yy) + (size_t)ny * (size_t)(xx)]
  double duydx, duxdy;
  if (ORDER == 2) {
    duydx = 0.5 * (A(uy, y, xp1) - A(uy, y, xm1));
    duxdy = 0.5 * (A(ux, yp1, x) - A(ux, ym1, x));
  } else {
    const double t1 = ORDER == 4 ? 1.0 / 12.0 : 2.0 / 3.0;
    const double t2 = ORDER == 4 ? 2.0 / 3.0 : 1.0 / 12.0;
    const int xp2 = (x + 2) % nx, xm2 = (x - 2 + 2 * nx) % nx;
    const int yp2 = (y + 2) % ny, ym2 = (y - 2 + 2 * ny) % ny;
    duydx = t1 * (A(uy, y, xp1) - A(uy, y, xm1)) + t2 * (A(uy, y, xm2) - A(uy, y, xp2));
    duxdy = t1 * (A(ux, yp1, x) - A(ux, ym1, x)) + t2 * (A(ux, ym2, x) - A(ux, yp2, x));
  }
  A(w, y, x) = duydx - duxdy;
#undef A
}


__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  return v;
}

// Grid-stride binary64 partial sums of [0.5 rho |u|^2, |u - ua|^2, |ua|^2].
template <int ST, class L>
__global__ void __launch_bounds__(kBlock) k_energy_error(const void* __restrict__ f,
                                                        const double* __restrict__ uxa,
                                                        const double* __restrict__ uya, int nx, int ny,
                                                        int ld, double* __restrict__ partial) {
  const int nfast = L::x_fast ? nx : ny;
  const long long ncell = (long long)nx * ny;
  double e = 0.0, num = 0.0, den = 0.0;
  for (long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x; c < ncell;
       c += (long long)gridDim.x * blockDim.x) {
    const int slow = (int)(c / nfast), fast = (int)(c - (long long)slow * nfast);
    const int x = L::x_fast ? fast : slow, y = L::x_fast ? slow : fast;
    double fs[9];
#pragma unroll
    for (int q = 0; q < 9; q++) fs[q] = load_pop<ST>(f, L::off(x, y, q, nx, ny, ld));
    double r, u, v;
    cell_moments<ST>(fs, r, u, v);
    e += r * (u * u + v * v);
    if (uxa) {
      const double a = uxa[c], b = uya[c];
      num += (u - a) * (u - a) + (v - b) * (v - b);
      den += a * a + b * b;
    }
  }
  __shared__ double sh[3][kBlock / 32];
  e = warp_sum(e);
  num = warp_sum(num);
  den = warp_sum(den);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (lane == 0) {
    sh[0][warp] = e;
    sh[1][warp] = num;
    sh[2][warp] = den;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double a = 0.0, b = 0.0, d = 0.0;
    for (int i = 0; i < kBlock / 32; i++) {
      a += sh[0][i];
      b += sh[1][i];
      d += sh[2][i];
    }
    partial[3 * blockIdx.x + 0] = 0.5 * a;
    partial[3 * blockIdx.x + 1] = b;
    partial[3 * blockIdx.x + 2] = d;
  }
}

}  // namespace

cudaError_t macros(int storage, int layout, int nx, int ny, int ld, const void* f, double* rho, double* ux,
                   double* uy, cudaStream_t st, bool exact) {
  return macros_range(storage, layout, nx, ny, ld, f, rho, ux, uy, 0, layout ? ny : nx, st, exact);
}

cudaError_t macros_range(int storage, int layout, int nx, int ny, int ld, const void* f, double* rho, double* ux,
                         double* uy, int slow0, int slow1, cudaStream_t st, bool exact) {
  const int nfast = layout ? nx : ny, nslow = layout ? ny : nx;
  if (slow0 < 0 || slow1 > nslow || slow0 >= slow1) return cudaErrorInvalidValue;
  const int ft = tiles(nfast);
  const long long blocks = (long long)ft * (slow1 - slow0);
  if (blocks <= 0 || blocks > 0x7fffffffLL) return cudaErrorInvalidConfiguration;
#define L_(ST, LL, EX) \
  k_macros<ST, LL, EX><<<(unsigned)blocks, kBlock, 0, st>>>(f, rho, ux, uy, nx, ny, ld, ft, slow0)
#define SW_(LL)                                                                \
  switch (storage) {                                                           \
    case ST_F64: if (exact) L_(ST_F64, LL, true); else L_(ST_F64, LL, false); break;                  \
    case ST_F64SHIFT: if (exact) L_(ST_F64SHIFT, LL, true); else L_(ST_F64SHIFT, LL, false); break;   \
    case ST_F32DEV: L_(ST_F32DEV, LL, false); break;                           \
    case ST_F16DEV: L_(ST_F16DEV, LL, false); break;                           \
    default: return cudaErrorInvalidValue;                                     \
  }
  if (layout) { SW_(XFast) } else { SW_(YFast) }
#undef SW_
#undef L_
  return cudaGetLastError();
}

cudaError_t equilibrium(int storage, int layout, int nx, int ny, int ld, const double* rho, const double* ux,
                        const double* uy, int from_pressure, void* f, cudaStream_t st, bool exact) {
  return equilibrium_range(storage, layout, nx, ny, ld, rho, ux, uy, from_pressure, f, 0, layout ? ny : nx, st,
                           exact);
}

cudaError_t equilibrium_range(int storage, int layout, int nx, int ny, int ld, const double* rho, const double* ux,
                              const double* uy, int from_pressure, void* f, int slow0, int slow1, cudaStream_t st,
                              bool exact) {
  const int nfast = layout ? nx : ny, nslow = layout ? ny : nx;
  if (slow0 < 0 || slow1 > nslow || slow0 >= slow1) return cudaErrorInvalidValue;
  const int ft = tiles(nfast);
  const long long blocks = (long long)ft * (slow1 - slow0);
  if (blocks <= 0 || blocks > 0x7fffffffLL) return cudaErrorInvalidConfiguration;
#define L_(ST, LL, EX)                                                                                   \
  k_equilibrium<ST, LL, EX><<<(unsigned)blocks, kBlock, 0, st>>>(rho, ux, uy, from_pressure, f, nx, ny, ld, ft, \
                                                                 slow0)
#define SW_(LL)                                                                \
  switch (storage) {                                                           \
    case ST_F64: if (exact) L_(ST_F64, LL, true); else L_(ST_F64, LL, false); break;                  \
    case ST_F64SHIFT: if (exact) L_(ST_F64SHIFT, LL, true); else L_(ST_F64SHIFT, LL, false); break;   \
    case ST_F32DEV: L_(ST_F32DEV, LL, false); break;                           \
    case ST_F16DEV: L_(ST_F16DEV, LL, false); break;                           \
    default: return cudaErrorInvalidValue;                                     \
  }
  if (layout) { SW_(XFast) } else { SW_(YFast) }
#undef SW_
#undef L_
  return cudaGetLastError();
}

namespace {
__global__ void __launch_bounds__(kBlock) k_copy2(const double2* __restrict__ s, double2* __restrict__ d, size_t n) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    d[i] = s[i];
}
__global__ void __launch_bounds__(kBlock) k_copy1(const double* __restrict__ s, double* __restrict__ d, size_t n) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    d[i] = s[i];
}
}  // namespace

cudaError_t copy_doubles(const double* src, double* dst, size_t n, cudaStream_t st) {
  if (n == 0) return cudaSuccess;
  int dev = 0, sms = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (e != cudaSuccess) return e;
  const unsigned blocks = (unsigned)(sms > 0 ? sms * 8 : 1024);
  if ((((uintptr_t)src | (uintptr_t)dst) & 15u) == 0 && n % 2 == 0)
    k_copy2<<<blocks, kBlock, 0, st>>>(reinterpret_cast<const double2*>(src), reinterpret_cast<double2*>(dst), n / 2);
  else
    k_copy1<<<blocks, kBlock, 0, st>>>(src, dst, n);
  return cudaGetLastError();
}

cudaError_t f64_to_dev(int storage, int nx, int ny, int ld, const double* f, void* h, cudaStream_t st) {
  const int ft = tiles(ny);
  const long long blocks = (long long)ft * nx;
  if (blocks <= 0 || blocks > 0x7fffffffLL) return cudaErrorInvalidConfiguration;
  if (storage == ST_F32DEV) k_convert<ST_F32DEV, true><<<(unsigned)blocks, kBlock, 0, st>>>(f, h, nx, ny, ld, ft);
  else if (storage == ST_F16DEV) k_convert<ST_F16DEV, true><<<(unsigned)blocks, kBlock, 0, st>>>(f, h, nx, ny, ld, ft);
  else return cudaErrorInvalidValue;
  return cudaGetLastError();
}

cudaError_t dev_to_f64(int storage, int nx, int ny, int ld, const void* h, double* f, cudaStream_t st) {
  const int ft = tiles(ny);
  const long long blocks = (long long)ft * nx;
  if (blocks <= 0 || blocks > 0x7fffffffLL) return cudaErrorInvalidConfiguration;
  if (storage == ST_F32DEV) k_convert<ST_F32DEV, false><<<(unsigned)blocks, kBlock, 0, st>>>(h, f, nx, ny, ld, ft);
  else if (storage == ST_F16DEV) k_convert<ST_F16DEV, false><<<(unsigned)blocks, kBlock, 0, st>>>(h, f, nx, ny, ld, ft);
  else return cudaErrorInvalidValue;
  return cudaGetLastError();
}

cudaError_t vorticity(int order, int nx, int ny, const double* ux, const double* uy, double* w, cudaStream_t st) {
  const int ft = tiles(ny);
  const long long blocks = (long long)ft * nx;
  if (blocks <= 0 || blocks > 0x7fffffffLL) return cudaErrorInvalidConfiguration;
  if (order == 2) k_vorticity<2><<<(unsigned)blocks, kBlock, 0, st>>>(ux, uy, w, nx, ny, ft);
  else if (order == 4) k_vorticity<4><<<(unsigned)blocks, kBlock, 0, st>>>(ux, uy, w, nx, ny, ft);
  else if (order == 44) k_vorticity<44><<<(unsigned)blocks, kBlock, 0, st>>>(ux, uy, w, nx, ny, ft);
  else return cudaErrorInvalidValue;
  return cudaGetLastError();
}

int reduce_blocks(int nx, int ny) {
  const long long need = ((long long)nx * ny + kBlock - 1) / kBlock;
  return (int)(need < kReduceBlocks ? (need > 0 ? need : 1) : kReduceBlocks);
}

cudaError_t energy_error_partials(int storage, int layout, int nx, int ny, int ld, const void* f,
                                  const double* uxa, const double* uya, double* partial, cudaStream_t st) {
  const int nb = reduce_blocks(nx, ny);
#define L_(ST, LL) k_energy_error<ST, LL><<<nb, kBlock, 0, st>>>(f, uxa, uya, nx, ny, ld, partial)
#define SW_(LL)                                          \
  switch (storage) {                                     \
    case ST_F64: L_(ST_F64, LL); break;                  \
    case ST_F64SHIFT: L_(ST_F64SHIFT, LL); break;        \
    case ST_F32DEV: L_(ST_F32DEV, LL); break;            \
    case ST_F16DEV: L_(ST_F16DEV, LL); break;            \
    default: return cudaErrorInvalidValue;               \
  }
  if (layout) { SW_(XFast) } else { SW_(YFast) }
#undef SW_
#undef L_
  return cudaGetLastError();
}

}  // namespace plbm
