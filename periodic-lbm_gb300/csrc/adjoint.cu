// adjoint.cu -- discrete adjoint of the BGK stream-collide time stepper.
//
// Forward model (pull form, src/periodic_lbm.f90:15-29 with collide_bgk):
//   f_0 = feq(1, u0),   f_{n+1} = C(S(f_n)),   u_T = j/rho of f_T,
// S the periodic pull stream, C the BGK collision.  Reverse mode:
//   lambda_T,q = sum_a G_a (c_qa - u_a) / rho                 G = dL/du_T
//   mu(x)      = J_C(g(x))^T lambda_{n+1}(x),  g = S(f_n)
//   lambda_n,q(x - c_q) = mu_q(x)            (S^T: push along -c_q)
//   dL/domega += sum_x sum_q lambda_{n+1,q}(x) (feq_q - g_q)(x)
//   dL/du0_a(x) = sum_q lambda_0,q(x) w_q (3 c_qa + 9 (c_q.u0) c_qa - 3 u0_a)
// with the BGK Jacobian transpose applied matrix-free:
//   mu_p = (1-omega) lambda_p + omega (A + c_p.(B - 3 S0 u)),
//   S0 = sum w_q lambda_q, A = sum w_q lambda_q (1 - 4.5 (c_q.u)^2 + 1.5 u^2),
//   B = sum w_q lambda_q (3 + 9 c_q.u) c_q.
// The per-cell adjoint arithmetic runs in the storage's type (binary64 for
// PLBM_F64, binary32 for PLBM_F32DEV): lambda, its weighted sums and mu; with
// plbm_adjoint_set_math(PLBM_MATH_HYBRID) the binary32 reverse step is the
// compensated one of coll_df64.cuh (k_adj_step_comp).  The
// gradients are accumulated in binary64: each cell's dL/domega term is taken
// to binary64 and summed over the warp in binary64 into the warp's own slot
// (the host adds the slots in a fixed order), and dL/du0 is assembled from
// lambda_0 in binary64 (k_adj_u0).
#include <cuda_runtime.h>

#include "../../include/plbm_gpu.h"
#include "coll_df64.cuh"
#include "plbm_adjoint.h"
#include "plbm_launch.h"

namespace plbm {
namespace {

inline int tiles(int n) { return (n + kBlock - 1) / kBlock; }

__device__ __forceinline__ bool yfast_cell(int ftiles, int ny, int& x, int& y) {
  x = blockIdx.x / ftiles;
  y = (blockIdx.x - x * ftiles) * blockDim.x + threadIdx.x;
  return y < ny;
}

// Population q of the model as a value of f (binary64) or of h = f - w.
template <int ST>
struct AdjTraits;
template <>
struct AdjTraits<ST_F64> {
  typedef double elem;
  typedef double real;
  static constexpr bool shift = false;
};
template <>
struct AdjTraits<ST_F32DEV> {
  typedef float elem;
  typedef float real;
  static constexpr bool shift = true;
};

// rho, u and feq_q - g_q of a cell (g in the storage's form).
template <typename R, bool SHIFT>
__device__ __forceinline__ void cell_state(const R (&g)[9], R& rho, R& ux, R& uy, R (&neq)[9]) {
  R s = 0, jx = 0, jy = 0;
#pragma unroll
  for (int q = 0; q < 9; q++) {
    s += g[q];
    jx += (R)cx_of(q) * g[q];
    jy += (R)cy_of(q) * g[q];
  }
  const R drho = SHIFT ? s : s - R(1);
  rho = drho + R(1);
  ux = jx / rho;
  uy = jy / rho;
  const R u2 = ux * ux + uy * uy;
#pragma unroll
  for (int q = 0; q < 9; q++) {
    const R cu = (R)cx_of(q) * ux + (R)cy_of(q) * uy;
    const R w = (R)w_of(q);
    // feq - w = w (drho + rho (3cu + 4.5 cu^2 - 1.5 u^2)); g - w = h (shifted) or f - w
    const R heq = w * (drho + rho * (R(3) * cu + R(4.5) * cu * cu - R(1.5) * u2));
    const R hg = SHIFT ? g[q] : g[q] - w;
    neq[q] = heq - hg;  // feq_q - g_q
  }
}

// Warp sum in binary64 of the cells' dL/domega terms.  Each warp adds its sum
// to its own binary64 slot: no block barrier, and the host adds the slots in a
// fixed order, so the result does not depend on scheduling.
__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  return v;
}

// f_0 = feq(1, u0) (src/fvm_bardow.F90:99-126 with rho = 1), stored as f or h.
template <int ST>
__global__ void __launch_bounds__(kBlock) k_adj_init(const double* __restrict__ u0, void* __restrict__ f, int nx,
                                                    int ny, int ld, int ftiles) {
  int x, y;
  if (!yfast_cell(ftiles, ny, x, y)) return;
  const size_t o = (size_t)y + (size_t)ny * x;
  const double ux = u0[o], uy = u0[(size_t)nx * ny + o];
  const double uxx = ux * ux, uyy = uy * uy;
  const double indp = -1.5 * (uxx + uyy);
  typedef typename AdjTraits<ST>::elem E;
  E* fe = static_cast<E*>(f);
#pragma unroll
  for (int q = 0; q < 9; q++) {
    const double cu = cx_of(q) * ux + cy_of(q) * uy;
    const double h = w_of(q) * (indp + 3.0 * cu + 4.5 * cu * cu);  // feq - w at rho = 1
    fe[YFast::off(x, y, q, nx, ny, ld)] = AdjTraits<ST>::shift ? (E)h : (E)(h + w_of(q));
  }
}

// u_T and lambda_T from f_T and G = dL/du_T (either output may be skipped).
template <int ST>
__global__ void __launch_bounds__(kBlock) k_adj_final(const void* __restrict__ f, const double* __restrict__ G,
                                                     double* __restrict__ uT, void* __restrict__ lam, int nx, int ny,
                                                     int ld, int ftiles) {
  typedef typename AdjTraits<ST>::real R;
  typedef typename AdjTraits<ST>::elem E;
  int x, y;
  if (!yfast_cell(ftiles, ny, x, y)) return;
  const E* fe = static_cast<const E*>(f);
  R g[9], neq[9], rho, ux, uy;
#pragma unroll
  for (int q = 0; q < 9; q++) g[q] = (R)fe[YFast::off(x, y, q, nx, ny, ld)];
  cell_state<R, AdjTraits<ST>::shift>(g, rho, ux, uy, neq);
  const size_t o = (size_t)y + (size_t)ny * x, n = (size_t)nx * ny;
  if (uT) {
    uT[o] = (double)ux;
    uT[n + o] = (double)uy;
  }
  if (lam) {
    const R gx = (R)G[o], gy = (R)G[n + o];
    E* le = static_cast<E*>(lam);
#pragma unroll
    for (int q = 0; q < 9; q++)
      le[YFast::off(x, y, q, nx, ny, ld)] = (E)((gx * ((R)cx_of(q) - ux) + gy * ((R)cy_of(q) - uy)) / rho);
  }
}

// One reverse step: lambda_n from lambda_{n+1} and f_n; adds this step's
// dL/domega to the warp's binary64 slot.  I: offset type (32-bit when the
// lattice has fewer than 2^32 elements).  The pull sources of the forward
// step are also where the reverse step scatters mu_p, so one offset table
// serves the loads of f and the stores of lambda_n.
template <int ST, typename I>
__global__ void __launch_bounds__(kBlock) k_adj_step(const void* __restrict__ f, const void* __restrict__ lam_in,
                                                    void* __restrict__ lam_out, double* __restrict__ dom,
                                                    typename AdjTraits<ST>::real om, int nx, int ny, int ld,
                                                    int ftiles) {
  typedef typename AdjTraits<ST>::real R;
  typedef typename AdjTraits<ST>::elem E;
  int x, y;
  const bool in = yfast_cell(ftiles, ny, x, y);
  R part = R(0);
  if (in) {
    const E* fe = static_cast<const E*>(f);
    const E* li = static_cast<const E*>(lam_in);
    E* lo = static_cast<E*>(lam_out);
    const I L = (I)ld, P = (I)ld * (I)nx;
    const I c0 = (I)x * L, cm = (I)wrap_m(x, nx) * L, cp = (I)wrap_p(x, nx) * L;
    const I y0 = (I)y, ym = (I)wrap_m(y, ny), yp = (I)wrap_p(y, ny);
    const I off[9] = {c0 + y0,         P + cm + y0,     2 * P + c0 + ym, 3 * P + cp + y0, 4 * P + c0 + yp,
                      5 * P + cm + ym, 6 * P + cp + ym, 7 * P + cp + yp, 8 * P + cm + yp};
    R g[9], l[9], neq[9], rho, ux, uy;
#pragma unroll
    for (int q = 0; q < 9; q++) {
      g[q] = (R)__ldg(fe + off[q]);
      l[q] = (R)__ldg(li + ((I)q * P + c0 + y0));
    }
    cell_state<R, AdjTraits<ST>::shift>(g, rho, ux, uy, neq);
    const R u2 = ux * ux + uy * uy;
    R s0 = 0, A = 0, Bx = 0, By = 0, d = 0;
#pragma unroll
    for (int q = 0; q < 9; q++) {
      d += l[q] * neq[q];
      const R cu = (R)cx_of(q) * ux + (R)cy_of(q) * uy;
      const R wl = (R)w_of(q) * l[q];
      s0 += wl;
      A += wl * (R(1) - R(4.5) * cu * cu + R(1.5) * u2);
      const R b = wl * (R(3) + R(9) * cu);
      Bx += b * (R)cx_of(q);
      By += b * (R)cy_of(q);
    }
    part = d;
    const R omb = R(1) - om;
    const R ex = Bx - R(3) * s0 * ux, ey = By - R(3) * s0 * uy;
#pragma unroll
    for (int p = 0; p < 9; p++) {
      const R mu = omb * l[p] + om * (A + (R)cx_of(p) * ex + (R)cy_of(p) * ey);
      lo[off[p]] = (E)mu;
    }
  }
  const double t = warp_sum((double)part);
  if ((threadIdx.x & 31) == 0) dom[(size_t)blockIdx.x * (kBlock / 32) + (threadIdx.x >> 5)] += t;
}

// The reverse step in compensated binary32 (binary32 storage; df::adj_step_comp
// of coll_df64.cuh): the same loads, scatter and dL/domega slots as k_adj_step.
// Compiled for 4 CTAs of 256 per SM (64 registers): uncapped it takes 73 and
// runs at 3, capped at 48 it spills; 4 measured fastest.
template <typename I>
__global__ void __launch_bounds__(kBlock, 4) k_adj_step_comp(const float* __restrict__ fe, const float* __restrict__ li,
                                                         float* __restrict__ lo, double* __restrict__ dom,
                                                         df::AdjDevParams cpar, int nx, int ny, int ld,
                                                         int ftiles) {
  int x, y;
  const bool in = yfast_cell(ftiles, ny, x, y);
  float part = 0.0f;
  if (in) {
    const I L = (I)ld, P = (I)ld * (I)nx;
    const I c0 = (I)x * L, cm = (I)wrap_m(x, nx) * L, cp = (I)wrap_p(x, nx) * L;
    const I y0 = (I)y, ym = (I)wrap_m(y, ny), yp = (I)wrap_p(y, ny);
    const I off[9] = {c0 + y0,         P + cm + y0,     2 * P + c0 + ym, 3 * P + cp + y0, 4 * P + c0 + yp,
                      5 * P + cm + ym, 6 * P + cp + ym, 7 * P + cp + yp, 8 * P + cm + yp};
    float g[9], l[9], mu[9];
#pragma unroll
    for (int q = 0; q < 9; q++) {
      g[q] = __ldg(fe + off[q]);
      l[q] = __ldg(li + ((I)q * P + c0 + y0));
    }
    part = df::adj_step_comp(g, l, mu, cpar);
#pragma unroll
    for (int q = 0; q < 9; q++) lo[off[q]] = mu[q];
  }
  const double t = warp_sum((double)part);
  if ((threadIdx.x & 31) == 0) dom[(size_t)blockIdx.x * (kBlock / 32) + (threadIdx.x >> 5)] += t;
}

// dL/du0 from lambda_0 and u0.
template <int ST>
__global__ void __launch_bounds__(kBlock) k_adj_u0(const void* __restrict__ lam, const double* __restrict__ u0,
                                                  double* __restrict__ grad, int nx, int ny, int ld, int ftiles) {
  typedef typename AdjTraits<ST>::elem E;
  int x, y;
  if (!yfast_cell(ftiles, ny, x, y)) return;
  const E* le = static_cast<const E*>(lam);
  const size_t o = (size_t)y + (size_t)ny * x, n = (size_t)nx * ny;
  const double ux = u0[o], uy = u0[n + o];
  double ax = 0.0, ay = 0.0;
#pragma unroll
  for (int q = 0; q < 9; q++) {
    const double cu = cx_of(q) * ux + cy_of(q) * uy;
    const double wl = w_of(q) * (double)le[YFast::off(x, y, q, nx, ny, ld)];
    ax += wl * (3.0 * cx_of(q) + 9.0 * cu * cx_of(q) - 3.0 * ux);
    ay += wl * (3.0 * cy_of(q) + 9.0 * cu * cy_of(q) - 3.0 * uy);
  }
  grad[o] = ax;
  grad[n + o] = ay;
}

template <int ST>
cudaError_t dispatch(int what, const AdjLaunch& a) {
  const int ft = tiles(a.ny);
  const long long blocks = (long long)ft * a.nx;
  if (blocks <= 0 || blocks > 0x7fffffffLL) return cudaErrorInvalidConfiguration;
  const unsigned nb = (unsigned)blocks;
  switch (what) {
    case 0: k_adj_init<ST><<<nb, kBlock, 0, a.stream>>>(a.u, const_cast<void*>(a.f), a.nx, a.ny, a.ld, ft); break;
    case 1: k_adj_final<ST><<<nb, kBlock, 0, a.stream>>>(a.f, a.g, a.out, a.lam_out, a.nx, a.ny, a.ld, ft); break;
    case 2:
      if (ST == ST_F32DEV && a.comp) {
        df::AdjDevParams cpar;
        const double w[3] = {W0, WS, WD};
        for (int i = 0; i < 3; i++) {
          const float hi = (float)w[i], hi3 = (float)(3.0 * w[i]);
          cpar.w[i] = df::make(hi, (float)(w[i] - (double)hi));
          cpar.w3[i] = df::make(hi3, (float)(3.0 * w[i] - (double)hi3));
        }
        cpar.om_hi = (float)a.omega;
        cpar.om_lo = (float)(a.omega - (double)cpar.om_hi);
        const float* fa = static_cast<const float*>(a.f);
        const float* la = static_cast<const float*>(a.lam_in);
        float* lb = static_cast<float*>(a.lam_out);
        if ((unsigned long long)a.ld * (unsigned long long)a.nx * 9ull < (1ull << 32))
          k_adj_step_comp<uint32_t><<<nb, kBlock, 0, a.stream>>>(fa, la, lb, a.dom, cpar, a.nx, a.ny, a.ld, ft);
        else
          k_adj_step_comp<size_t><<<nb, kBlock, 0, a.stream>>>(fa, la, lb, a.dom, cpar, a.nx, a.ny, a.ld, ft);
        break;
      }
      if ((unsigned long long)a.ld * (unsigned long long)a.nx * 9ull < (1ull << 32))
        k_adj_step<ST, uint32_t><<<nb, kBlock, 0, a.stream>>>(a.f, a.lam_in, a.lam_out, a.dom,
                                                              (typename AdjTraits<ST>::real)a.omega, a.nx, a.ny,
                                                              a.ld, ft);
      else
        k_adj_step<ST, size_t><<<nb, kBlock, 0, a.stream>>>(a.f, a.lam_in, a.lam_out, a.dom,
                                                            (typename AdjTraits<ST>::real)a.omega, a.nx, a.ny, a.ld,
                                                            ft);
      break;
    case 3: k_adj_u0<ST><<<nb, kBlock, 0, a.stream>>>(a.lam_in, a.u, a.out, a.nx, a.ny, a.ld, ft); break;
    default: return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

}  // namespace

int adjoint_blocks(int nx, int ny) { return tiles(ny) * nx * (kBlock / 32); }

cudaError_t adjoint_launch(int storage, int what, const AdjLaunch& a) {
  if (storage == ST_F64) return dispatch<ST_F64>(what, a);
  if (storage == ST_F32DEV) return dispatch<ST_F32DEV>(what, a);
  return cudaErrorNotSupported;
}

}  // namespace plbm
