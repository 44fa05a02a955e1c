// grid_internal.h -- the plbm_grid handle and the helpers shared by the
// translation units of the plbm_* C ABI (grid.cpp, grid_io.cpp).
#pragma once
#include <cuda_runtime.h>
#include <stddef.h>

#include "../../include/plbm_gpu.h"

namespace plbm_internal {
int fail(int code, const char* fmt, ...);
int cuda_fail(cudaError_t e, const char* what);
inline int ok() { return PLBM_OK; }
}  // namespace plbm_internal

#define PLBM_CUDA_TRY(expr, what)                                         \
  do {                                                                    \
    cudaError_t e_ = (expr);                                              \
    if (e_ != cudaSuccess) return plbm_internal::cuda_fail(e_, what);     \
  } while (0)

constexpr int kMaxLattices = 16;

// Device-resident mirror of lattice_grid (src/fvm_bardow.F90:37-69).
// Most x-column slabs the moment-field transfers are split into.
constexpr int kMaxSlabs = 16;

struct plbm_grid {
  int nx, ny, ld, nf, storage;
  int kind = PLBM_BGK, math = PLBM_MATH_FMA;
  int streaming = PLBM_STREAM_LBM;    // grid%streaming
  int iold = 2, inew = 1, imid = -1;  // 1-based, as alloc_grid sets them
  double nu = 0, dt = 1, tau = 0, omega = 1, trt_magic = 0.25;
  int device = 0;
  void* f = nullptr;           // nf lattices, contiguous
  void* spare = nullptr;       // one more lattice, allocated by the first triple step
  // Buffer index (1-based) -> physical lattice (0..nf-1, nf = the spare).
  // The identity until a triple step remaps it (see plbm_perform_triple_step).
  int slot[kMaxLattices] = {0, 1, 2, 3, 4, 5, 6, 7, 8, 9, 10, 11, 12, 13, 14, 15};
  int spare_slot = -1;         // physical slot currently unused (the spare)
  size_t lat_elems = 0;        // ld*nx*9
  size_t elem_bytes = 8;
  cudaStream_t own = nullptr;  // stream created by the handle
  cudaStream_t stream = nullptr;
  // Host transfers of set_pdf_to_equilibrium / update_macros on large grids:
  // a second stream and one event per x-column slab (created on first use).
  cudaStream_t xfer = nullptr;
  cudaEvent_t slab_ev[kMaxSlabs + 1] = {};
  double* scratch = nullptr;   // 3*nx*ny doubles + reduction partials
  size_t scratch_elems = 0;
  // Captured step loop of a small grid (plbm_perform_lbm_step) and what it
  // was captured for; recaptured when any of it changes.
  cudaGraphExec_t step_graph = nullptr;
  struct {
    const void* a = nullptr;
    const void* b = nullptr;
    cudaStream_t stream = nullptr;
    int kind = -1, math = -1, streaming = -1;
    double omega = 0, trt_magic = 0, dt = 0;
  } step_key;
};

namespace plbm_internal {

inline int pad16(int n) {
  int r = n % 16;
  return r > 0 ? n + (16 - r) : n;
}

inline int check_grid(const plbm_grid_t* g) {
  if (!g) return fail(PLBM_E_INVALID, "NULL grid handle");
  return PLBM_OK;
}

inline int check_buf(const plbm_grid_t* g, int ibuf) {
  if (ibuf < 1 || ibuf > g->nf) return fail(PLBM_E_INVALID, "buffer index %d outside 1..%d", ibuf, g->nf);
  return PLBM_OK;
}

// Physical lattice `p` (0..nf-1 in the main allocation, nf = the spare).
inline void* physical(const plbm_grid_t* g, int p) {
  if (p == g->nf) return g->spare;
  return static_cast<char*>(g->f) + (size_t)p * g->lat_elems * g->elem_bytes;
}

// Device lattice of buffer index ibuf (1-based).
inline void* lattice(const plbm_grid_t* g, int ibuf) { return physical(g, g->slot[ibuf - 1]); }

inline int use_device(const plbm_grid_t* g) {
  PLBM_CUDA_TRY(cudaSetDevice(g->device), "cudaSetDevice");
  return PLBM_OK;
}

inline int ensure_scratch(plbm_grid_t* g, size_t elems) {
  if (g->scratch_elems >= elems) return PLBM_OK;
  if (g->scratch) cudaFree(g->scratch);
  g->scratch = nullptr;
  g->scratch_elems = 0;
  PLBM_CUDA_TRY(cudaMalloc(&g->scratch, elems * sizeof(double)), "cudaMalloc(scratch)");
  g->scratch_elems = elems;
  return PLBM_OK;
}

inline int internal_storage(int storage) { return storage; }  // PLBM_F64/F32DEV/F16DEV == ST_*

// Grids in hybrid arithmetic take their moments and equilibria in the exact
// integer forms too (binary64 storage only).
inline bool exact_fields(const plbm_grid_t* g) { return g->math == PLBM_MATH_HYBRID && g->storage == PLBM_F64; }

}  // namespace plbm_internal
