// batched.cu -- many independent periodic D2Q9 grids of uneven sizes and
// relaxation times advanced together.
//
// Layout: every grid keeps the reference layout f(ld,nx,0:8) (ld = pad16(ny))
// with two lattices A and B, all grids packed into one device allocation.
// Work unit: a tile of TY x TX cells of one grid (TY rows along the fast y
// axis, TX = threads / TY columns), TY chosen per grid by the schedule.  The
// tiles of all grids are numbered 0..T-1; CTA b takes tiles b, b + nCTA, ...
//
// Two launch modes, both capturable in a CUDA graph:
//   * persistent: ONE cooperative launch runs all steps; the CTAs meet at a
//     grid-wide barrier between steps.  Every wait on the barrier is bounded:
//     after kSpinLimit polls the CTA records a timeout in the control block and
//     the kernel returns, so a lost CTA cannot hang the GPU.
//   * per-step: one ordinary launch per step (the graph then holds one node
//     per step).
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

template <class S>
__device__ __forceinline__ typename S::real load_cg(const typename S::elem* p, size_t i);
template <>
__device__ __forceinline__ double load_cg<StoreF64>(const double* p, size_t i) { return __ldcg(p + i); }
template <>
__device__ __forceinline__ float load_cg<StoreF32Dev>(const float* p, size_t i) { return __ldcg(p + i); }

// Process one tile of one grid for one step.
template <class S>
__device__ __forceinline__ void do_tile(const BatchGrid& g, int local_tile, int parity,
                                        typename S::elem* __restrict__ base) {
  const int ty = g.ty;
  const int tx = blockDim.x / ty;
  const int tiles_y = (g.ny + ty - 1) / ty;
  const int txi = local_tile / tiles_y, tyi = local_tile - txi * tiles_y;
  const int y = tyi * ty + (int)(threadIdx.x % ty);
  const int x = txi * tx + (int)(threadIdx.x / ty);
  if (x >= g.nx || y >= g.ny) return;
  const size_t lat = (size_t)g.ld * g.nx * 9;
  const typename S::elem* src = base + g.off + (parity ? lat : 0);
  typename S::elem* dst = base + g.off + (parity ? 0 : lat);
  typename S::real f[9];
#pragma unroll
  for (int q = 0; q < 9; q++) {
    const int sx = wrap_add(x, -cx_of(q), g.nx), sy = wrap_add(y, -cy_of(q), g.ny);
    f[q] = load_cg<S>(src, YFast::off(sx, sy, q, g.nx, g.ny, g.ld));
  }
  if constexpr (S::ddf) {
    if (g.kind == K_TRT) collide_shift<K_TRT, typename S::real>(f, g.p);
    else collide_shift<K_BGK, typename S::real>(f, g.p);
  } else {
    if (g.kind == K_TRT) collide_ref<K_TRT>(f, g.p);
    else collide_ref<K_BGK>(f, g.p);
  }
#pragma unroll
  for (int q = 0; q < 9; q++) S::store(dst, YFast::off(x, y, q, g.nx, g.ny, g.ld), f[q]);
}

__device__ __forceinline__ int find_grid(const int* __restrict__ tile_start, int ngrids, int t) {
  // largest g with tile_start[g] <= t
  int lo = 0, hi = ngrids - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (__ldg(tile_start + mid) <= t) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}

template <class S>
__device__ __forceinline__ void sweep(const BatchGrid* __restrict__ grids, const int* __restrict__ tile_start,
                                      int ngrids, int ntiles, int parity, typename S::elem* base) {
  __shared__ BatchGrid sg;
  __shared__ int sgi;
  for (int t = blockIdx.x; t < ntiles; t += gridDim.x) {
    __syncthreads();
    if (threadIdx.x == 0) {
      const int gi = find_grid(tile_start, ngrids, t);
      sgi = gi;
      sg = grids[gi];
    }
    __syncthreads();
    do_tile<S>(sg, t - __ldg(tile_start + sgi), parity, base);
  }
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

template <class S>
__global__ void __launch_bounds__(kBatchMaxThreads) k_batch_persistent(const BatchGrid* __restrict__ grids,
                                                                      const int* __restrict__ tile_start,
                                                                      int ngrids, int ntiles, int nsteps,
                                                                      int parity0, typename S::elem* base,
                                                                      Ctrl* ctrl) {
  for (int s = 0; s < nsteps; s++) {
    sweep<S>(grids, tile_start, ngrids, ntiles, (parity0 + s) & 1, base);
    if (s + 1 < nsteps && !barrier(ctrl, s)) return;
  }
}

template <class S>
__global__ void __launch_bounds__(kBatchMaxThreads) k_batch_step(const BatchGrid* __restrict__ grids,
                                                                const int* __restrict__ tile_start, int ngrids,
                                                                int ntiles, int parity, typename S::elem* base) {
  sweep<S>(grids, tile_start, ngrids, ntiles, parity, base);
}

template <class S>
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
    return cudaLaunchKernelEx(&cfg, k_batch_persistent<S>, L.grids, L.tile_start, L.ngrids, L.ntiles, nsteps,
                              parity0, base, ctrl);
  }
  for (int s = 0; s < nsteps; s++) {
    k_batch_step<S><<<L.ctas, L.threads, 0, L.stream>>>(L.grids, L.tile_start, L.ngrids, L.ntiles,
                                                         (parity0 + s) & 1, base);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}

}  // namespace

size_t batch_ctrl_bytes() { return sizeof(Ctrl); }

cudaError_t batch_max_ctas(int storage, int threads, int* per_sm) {
  if (storage == ST_F64)
    return cudaOccupancyMaxActiveBlocksPerMultiprocessor(per_sm, k_batch_persistent<StoreF64>, threads, 0);
  return cudaOccupancyMaxActiveBlocksPerMultiprocessor(per_sm, k_batch_persistent<StoreF32Dev>, threads, 0);
}

cudaError_t batch_run(int storage, const BatchLaunch& L, int nsteps, int parity0) {
  if (nsteps <= 0) return cudaSuccess;
  if (L.threads <= 0 || L.threads > kBatchMaxThreads || (L.threads & 31)) return cudaErrorInvalidConfiguration;
  if (storage == ST_F64) return launch_batch<StoreF64>(L, nsteps, parity0);
  if (storage == ST_F32DEV) return launch_batch<StoreF32Dev>(L, nsteps, parity0);
  return cudaErrorNotSupported;
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
