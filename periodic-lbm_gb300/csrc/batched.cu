// batched.cu -- many independent periodic D2Q9 grids of uneven sizes and
// relaxation times advanced together.
//
// Layout: every grid keeps the reference layout f(ld,nx,0:8) (ld = pad16(ny))
// with two lattices A and B, all grids packed into one device allocation.
// Work unit: a tile of TY x TX cells of one grid (TY rows along the fast y
// axis, TX = threads / TY columns), TY chosen per grid by the schedule.  The
// tiles of all grids are numbered 0..T-1, the BGK grids' first; a table holds
// each tile's grid and first cell.  Persistent CTA b takes tiles b, b + nCTA,
// ...; the per-step launch gives each tile its own CTA.
//
// Two launch modes, both capturable in a CUDA graph:
//   * persistent: ONE cooperative launch runs all steps; the CTAs meet at a
//     grid-wide barrier between steps.  Every wait on the barrier is bounded:
//     after kSpinLimit polls the CTA records a timeout in the control block and
//     the kernel returns, so a lost CTA cannot hang the GPU.
//   * per-step: ordinary launches, one per collision kind and step (the graph
//     then holds those nodes); with 128-thread CTAs each kind runs a kernel
//     compiled for it alone.
//
// Lattice loads use ld.global.cg (L2 only): in the persistent kernel a lattice
// written in step s by other SMs is read in step s+1, and the non-coherent L1 /
// read-only path could return lines cached before it was written.
#include <cooperative_groups.h>
#include <cuda_runtime.h>

#include "../../include/plbm_gpu.h"
#include "plbm_batched.h"
#include "plbm_launch.h"

namespace plbm {
namespace {

constexpr unsigned kSpinLimit = 1u << 24;  // polls of the barrier word (~seconds)

struct alignas(16) Ctrl {
  unsigned count;     // CTAs arrived at the current barrier
  unsigned gen;       // barrier generation
  int error;          // 0 ok, 1 barrier timeout
  int where;          // step at which the timeout happened
};

// Population load: ld.global.cg (L2 only) inside the persistent kernel, the
// read-only path in the per-step kernel.
template <bool CG, typename E>
__device__ __forceinline__ E load_pop(const E* p) {
  if constexpr (CG) return __ldcg(p);
  else return __ldg(p);
}

// One binary64 cell outside the hybrid range: pull, the binary64 operator,
// store.  Out of line so that the hot path's registers and code are not
// shaped by this rarely taken path.  gp points at the grid's table entry.
template <bool CG>
__device__ __noinline__ void fallback_cell(const double* __restrict__ src, double* __restrict__ dst, int x, int y,
                                           const BatchGrid* __restrict__ gp) {
  const int nx = gp->nx, ny = gp->ny, ld = gp->ld;
  double f[9];
#pragma unroll
  for (int q = 0; q < 9; q++) {
    const int sx = wrap_add(x, -cx_of(q), nx), sy = wrap_add(y, -cy_of(q), ny);
    f[q] = load_pop<CG>(src + YFast::off(sx, sy, q, nx, ny, ld));
  }
  if (gp->kind == K_TRT) collide_ref<K_TRT>(f, gp->p);
  else collide_ref<K_BGK>(f, gp->p);
#pragma unroll
  for (int q = 0; q < 9; q++) dst[YFast::off(x, y, q, nx, ny, ld)] = f[q];
}

// Process one tile of one grid for one step.  I: index type inside one grid's
// lattice pair (32-bit when every grid's pair has fewer than 2^32 elements).
// KIND: K_BGK or K_TRT, or -1 for the grid's own (read at run time); HY: 1
// hybrid binary64, 0 the binary64 operator, -1 the grid's flag.  gp is the
// grid's table entry; its relaxation constants are read where they are used
// (through the read-only path) rather than held in registers.  (x0, y0) is
// the tile's first cell; its TY = 2^lty rows run along y.
template <class S, bool CG, typename I, int KIND = -1, int HY = -1>
__device__ __forceinline__ void do_tile(const BatchGrid* __restrict__ gp, int2 xy, int parity,
                                        typename S::elem* __restrict__ base) {
  const int nx = __ldg(&gp->nx), ny = __ldg(&gp->ny), ld = __ldg(&gp->ld);
  const int lty = __ldg(&gp->lty);
  const int y = xy.y + (int)(threadIdx.x & ((1u << lty) - 1u));
  const int x = xy.x + (int)(threadIdx.x >> lty);
  if (x >= nx || y >= ny) return;
  const int kind = KIND >= 0 ? KIND : __ldg(&gp->kind);
  const long long goff = __ldg(&gp->off);
  const I L = (I)ld, P = (I)ld * (I)nx, lat = 9 * P;
  const typename S::elem* src = base + goff + (parity ? lat : 0);
  typename S::elem* dst = base + goff + (parity ? 0 : lat);
  const I c0 = (I)x * L, cm = (I)wrap_m(x, nx) * L, cp = (I)wrap_p(x, nx) * L;
  const I y0 = (I)y, ym = (I)wrap_m(y, ny), yp = (I)wrap_p(y, ny);
  typedef typename S::elem E;
  E e[9];
  e[0] = load_pop<CG>(src + (c0 + y0));
  e[1] = load_pop<CG>(src + (P + cm + y0));
  e[2] = load_pop<CG>(src + (2 * P + c0 + ym));
  e[3] = load_pop<CG>(src + (3 * P + cp + y0));
  e[4] = load_pop<CG>(src + (4 * P + c0 + yp));
  e[5] = load_pop<CG>(src + (5 * P + cm + ym));
  e[6] = load_pop<CG>(src + (6 * P + cp + ym));
  e[7] = load_pop<CG>(src + (7 * P + cp + yp));
  e[8] = load_pop<CG>(src + (8 * P + cm + yp));
  typename S::real f[9];
#pragma unroll
  for (int q = 0; q < 9; q++) f[q] = (typename S::real)e[q];
  if constexpr (S::ddf) {
    if (kind == K_TRT) collide_shift<K_TRT, typename S::real>(f, gp->p);
    else collide_shift<K_BGK, typename S::real>(f, gp->p);
  } else {
    if (HY > 0 || (HY < 0 && __ldg(&gp->hybrid))) {
      bool bad = false;
      if (kind == K_TRT) hy::trt_fma(f, gp->ht, bad);
      else hy::bgk_fma(f, gp->hp, bad);
      if (bad) {  // outside the hybrid range: the binary64 operator on the same inputs
        fallback_cell<CG>(src, dst, x, y, gp);
        return;
      }
    } else if (kind == K_TRT) {
      collide_ref<K_TRT>(f, gp->p);
    } else {
      collide_ref<K_BGK>(f, gp->p);
    }
  }
  const I o = c0 + y0;
#pragma unroll
  for (int q = 0; q < 9; q++) S::store(dst, (size_t)((I)q * P + o), f[q]);
}

// Tiles t = blockIdx.x, blockIdx.x + gridDim.x, ...; the grid of tile t is
// tile_grid[t], its first cell tile_xy[t] (both precomputed).
template <class S, bool CG, typename I>
__device__ __forceinline__ void sweep(const BatchGrid* __restrict__ grids, const int2* __restrict__ tile_xy,
                                      const int* __restrict__ tile_grid, int ntiles, int parity,
                                      typename S::elem* base) {
  for (int t = blockIdx.x; t < ntiles; t += gridDim.x)
    do_tile<S, CG, I>(grids + __ldg(tile_grid + t), __ldg(tile_xy + t), parity, base);
}

// Grid-wide barrier with a bounded wait.  Returns false when the wait ran out
// (then Ctrl::error is set and every CTA leaves the kernel).
__device__ __forceinline__ bool barrier(Ctrl* ctrl, int step) {
  __shared__ int ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    ok = 1;
    volatile unsigned* vgen = &ctrl->gen;
    const unsigned gen = *vgen;
    __threadfence();
    const unsigned arrived = atomicAdd(&ctrl->count, 1u);
    if (arrived == gridDim.x - 1) {
      ctrl->count = 0;
      __threadfence();
      atomicAdd(&ctrl->gen, 1u);
    } else {
      unsigned n = 0;
      while (*vgen == gen) {
        if (++n > kSpinLimit || *(volatile int*)&ctrl->error) {
          atomicExch(&ctrl->error, 1);
          atomicExch(&ctrl->where, step);
          ok = 0;
          break;
        }
        __nanosleep(64);
      }
    }
    __threadfence();
  }
  __syncthreads();
  return ok != 0;
}

template <class S, typename I>
__global__ void __launch_bounds__(kBatchMaxThreads) k_batch_persistent(const BatchGrid* __restrict__ grids,
                                                                      const int2* __restrict__ tile_xy,
                                                                      const int* __restrict__ tile_grid,
                                                                      int ntiles, int nsteps, int parity0,
                                                                      typename S::elem* base, Ctrl* ctrl) {
  for (int s = 0; s < nsteps; s++) {
    sweep<S, true, I>(grids, tile_xy, tile_grid, ntiles, (parity0 + s) & 1, base);
    if (s + 1 < nsteps && !barrier(ctrl, s)) return;
  }
}

template <class S, typename I>
__global__ void __launch_bounds__(kBatchMaxThreads) k_batch_step(const BatchGrid* __restrict__ grids,
                                                                const int2* __restrict__ tile_xy,
                                                                const int* __restrict__ tile_grid, int ntiles,
                                                                int parity, typename S::elem* base) {
  sweep<S, false, I>(grids, tile_xy, tile_grid, ntiles, parity, base);
}

// Per-step launch of 128-thread CTAs over the tiles of one collision kind
// (tile t0 + blockIdx.x), compiled for that kind and arithmetic alone with
// MINB resident CTAs per SM: the binary64 hybrid BGK tiles (bgk_fma) take 64
// registers (8 CTAs) and the TRT tiles (trt_fma) 72 (7).  One kernel for both
// kinds needed far more registers than either (97 for the earlier forms, 80
// under a cap with spills, 20.9k MLUPS on the 512-grid batch against 24.5k
// split by kind).
template <class S, typename I, int KIND, int HY, int MINB>
__global__ void __launch_bounds__(128, MINB) k_batch_kind(const BatchGrid* __restrict__ grids,
                                                         const int2* __restrict__ tile_xy,
                                                         const int* __restrict__ tile_grid, int t0, int parity,
                                                         typename S::elem* base) {
  const int t = t0 + (int)blockIdx.x;
  do_tile<S, false, I, KIND, HY>(grids + __ldg(tile_grid + t), __ldg(tile_xy + t), parity, base);
}

template <class S, typename I, int HY>
cudaError_t launch_kinds(const BatchLaunch& L, int parity) {
  typedef typename S::elem E;
  E* base = static_cast<E*>(L.base);
  const int ntrt = L.ntiles - L.nt_bgk;
  if (L.nt_bgk > 0)
    k_batch_kind<S, I, K_BGK, HY, 8><<<L.nt_bgk, 128, 0, L.stream>>>(L.grids, L.tile_xy, L.tile_grid,
                                                                                    0, parity, base);
  if (ntrt > 0)
    k_batch_kind<S, I, K_TRT, HY, 7><<<ntrt, 128, 0, L.stream>>>(L.grids, L.tile_xy, L.tile_grid, L.nt_bgk, parity,
                                                                 base);
  return cudaGetLastError();
}

template <class S, typename I>
cudaError_t launch_batch(const BatchLaunch& L, int nsteps, int parity0) {
  typedef typename S::elem E;
  E* base = static_cast<E*>(L.base);
  if (L.persistent) {
    Ctrl* ctrl = static_cast<Ctrl*>(L.ctrl);
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(L.ctas);
    cfg.blockDim = dim3(L.threads);
    cfg.stream = L.stream;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, k_batch_persistent<S, I>, L.grids, L.tile_xy, L.tile_grid, L.ntiles, nsteps,
                              parity0, base, ctrl);
  }
  // one tile per CTA; 128-thread CTAs run one kernel per collision kind
  for (int s = 0; s < nsteps; s++) {
    const int parity = (parity0 + s) & 1;
    cudaError_t e;
    if (L.threads == 128) {
      e = (!S::ddf && L.hybrid) ? launch_kinds<S, I, 1>(L, parity) : launch_kinds<S, I, 0>(L, parity);
    } else {
      k_batch_step<S, I><<<L.ntiles, L.threads, 0, L.stream>>>(L.grids, L.tile_xy, L.tile_grid, L.ntiles, parity,
                                                               base);
      e = cudaGetLastError();
    }
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}

template <class S>
cudaError_t launch_batch_i(const BatchLaunch& L, int nsteps, int parity0) {
  if (L.small_index) return launch_batch<S, uint32_t>(L, nsteps, parity0);
  return launch_batch<S, size_t>(L, nsteps, parity0);
}

}  // namespace

size_t batch_ctrl_bytes() { return sizeof(Ctrl); }

cudaError_t batch_max_ctas(int storage, int threads, int small_index, int* per_sm) {
  if (storage == ST_F64)
    return small_index ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(per_sm, k_batch_persistent<StoreF64, uint32_t>,
                                                                     threads, 0)
                       : cudaOccupancyMaxActiveBlocksPerMultiprocessor(per_sm, k_batch_persistent<StoreF64, size_t>,
                                                                     threads, 0);
  return small_index ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(per_sm, k_batch_persistent<StoreF32Dev, uint32_t>,
                                                                   threads, 0)
                     : cudaOccupancyMaxActiveBlocksPerMultiprocessor(per_sm, k_batch_persistent<StoreF32Dev, size_t>,
                                                                   threads, 0);
}

cudaError_t batch_run(int storage, const BatchLaunch& L, int nsteps, int parity0) {
  if (nsteps <= 0) return cudaSuccess;
  if (L.threads <= 0 || L.threads > kBatchMaxThreads || (L.threads & 31)) return cudaErrorInvalidConfiguration;
  if (storage == ST_F64) return launch_batch_i<StoreF64>(L, nsteps, parity0);
  if (storage == ST_F32DEV) return launch_batch_i<StoreF32Dev>(L, nsteps, parity0);
  return cudaErrorNotSupported;
}

cudaError_t batch_arm_stall(void* ctrl, cudaStream_t st) {
  // arrival count far above any CTA count: the first barrier never completes
  // and every CTA's wait runs out (kSpinLimit polls)
  static const Ctrl stalled = {0x80000000u, 0u, 0, 0};
  return cudaMemcpyAsync(ctrl, &stalled, sizeof stalled, cudaMemcpyHostToDevice, st);
}

cudaError_t batch_read_ctrl(const void* ctrl, int* error, int* where, cudaStream_t st) {
  Ctrl h;
  cudaError_t e = cudaMemcpyAsync(&h, ctrl, sizeof h, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return e;
  *error = h.error;
  *where = h.where;
  return cudaSuccess;
}

}  // namespace plbm
