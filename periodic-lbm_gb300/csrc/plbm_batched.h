// plbm_batched.h -- internal interface of the batched multi-grid stepper.
#pragma once
#include <cuda_runtime.h>
#include <stddef.h>
#include "plbm_device.cuh"

namespace plbm {

constexpr int kBatchMaxThreads = 512;

// One grid of a batch, as the kernels see it.
struct alignas(16) BatchGrid {
  CollParams p;       // relaxation parameters (grid's omega / TRT magic)
  long long off;      // element offset of lattice A; lattice B follows it
  int nx, ny, ld;
  int kind;           // K_BGK or K_TRT
  int ty;             // tile rows along y; tile columns = threads / ty
  int pad[3];
};

struct BatchLaunch {
  const BatchGrid* grids;  // device
  const int* tile_start;   // device, ngrids + 1 prefix sums of tiles
  int ngrids, ntiles;
  int threads, ctas;
  int persistent;          // 1: one cooperative launch for all steps
  void* base;              // device, all lattices
  void* ctrl;              // device barrier/control block (persistent mode)
  cudaStream_t stream;
};

size_t batch_ctrl_bytes();
cudaError_t batch_max_ctas(int storage, int threads, int* per_sm);
// Advance nsteps; parity0 = 0 reads lattice A first.
cudaError_t batch_run(int storage, const BatchLaunch& L, int nsteps, int parity0);
cudaError_t batch_read_ctrl(const void* ctrl, int* error, int* where, cudaStream_t st);

}  // namespace plbm
