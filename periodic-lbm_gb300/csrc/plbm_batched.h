// plbm_batched.h -- internal interface of the batched multi-grid stepper.
#pragma once
#include <cuda_runtime.h>
#include <stddef.h>
#include "hybrid.cuh"
#include "plbm_device.cuh"

namespace plbm {

constexpr int kBatchMaxThreads = 512;

// One grid of a batch, as the kernels see it.
struct alignas(16) BatchGrid {
  CollParams p;       // relaxation parameters (grid's omega / TRT magic)
  hy::BgkParams hp;   // the same for the hybrid binary64 BGK (bgk_fma)
  hy::TrtFmaParams ht;  // ... and TRT (trt_fma)
  long long off;      // element offset of lattice A; lattice B follows it
  int nx, ny, ld;
  int kind;           // K_BGK or K_TRT
  int ty;             // tile rows along y; tile columns = threads / ty
  int hybrid;         // binary64 grid in hybrid arithmetic
  int lty;            // log2(ty)
  int pad;
};

hy::BgkParams hybrid_bgk_params(double omega);
hy::TrtFmaParams hybrid_trt_params(const CollParams& p);

struct BatchLaunch {
  const BatchGrid* grids;  // device
  const int2* tile_xy;     // device, first cell (x0, y0) of each tile
  const int* tile_grid;    // device, grid index of each tile
  int ngrids, ntiles;
  int nt_bgk;              // tiles [0, nt_bgk) belong to BGK grids, the rest to TRT grids
  int hybrid;              // binary64 grids in hybrid arithmetic (batch-wide)
  int threads, ctas;       // ctas: persistent mode only (per-step: one CTA per tile)
  int persistent;          // 1: one cooperative launch for all steps
  int small_index;         // every grid's lattice pair has < 2^32 elements
  void* base;              // device, all lattices
  void* ctrl;              // device barrier/control block (persistent mode)
  cudaStream_t stream;
};

size_t batch_ctrl_bytes();
cudaError_t batch_max_ctas(int storage, int threads, int small_index, int* per_sm);
// Advance nsteps; parity0 = 0 reads lattice A first.
cudaError_t batch_run(int storage, const BatchLaunch& L, int nsteps, int parity0);
cudaError_t batch_read_ctrl(const void* ctrl, int* error, int* where, cudaStream_t st);
// Make the next persistent run's first grid barrier unreachable (its waits
// run out): the failure-path test of the bounded wait.
cudaError_t batch_arm_stall(void* ctrl, cudaStream_t st);

}  // namespace plbm
