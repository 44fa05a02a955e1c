// plbm_launch.h -- internal launcher interface shared by the translation units
// of libplbmgpu.so.  Not part of the public C ABI.
#pragma once
#include <cuda_runtime.h>
#include <stddef.h>
#include "plbm_device.cuh"

namespace plbm {

// One lattice sweep: nx, ny, ld and the two lattices.
struct Sweep {
  int nx, ny, ld;
  const void* src;
  void* dst;
  cudaStream_t stream;
};

// Threads per block of the per-cell kernels.
constexpr int kBlock = 256;
// Blocks of the binary64 field reductions (152 SMs x 8); each writes one
// partial triple (the staging of plbm_velocity_l2_error_noalloc holds them).
constexpr int kReduceBlocks = 1216;

// Threads per block for a fused step over `cells` cells: kBlock, or, for a
// grid with fewer than kBlock cells per SM, the smallest multiple of 32 that
// covers the grid with one CTA per SM.  A small grid then spreads over every
// SM instead of a few: each SM's binary64 pipe retires about 2 FMAs per
// cycle, so a 64^2 grid in 16 CTAs of 256 threads spent ~4.5 us per step in
// its collision arithmetic.
int block_for(long long cells);

// The binary64 reference kernels exist twice, once compiled with FMA
// contraction (namespace fma) and once without (namespace strict).
#define PLBM_DECLARE_F64(NS)                                                              \
  namespace NS {                                                                          \
  /* fused lbm_stream + collide_* (src/periodic_lbm.f90:15-29), YFast layout */            \
  cudaError_t step_pull_f64(int kind, const Sweep& s, const CollParams& p);               \
  /* lbm_stream alone (src/periodic_lbm.f90:45-127) */                                   \
  cudaError_t stream_f64(const Sweep& s);                                                 \
  /* collide_* alone, in place on s.dst (s.src ignored) */                                \
  cudaError_t collide_f64(int kind, const Sweep& s, const CollParams& p);                 \
  /* plugin step: shifted binary64 collide + push (sim/sim.F90:404-505), XFast */          \
  cudaError_t step_push_shift_f64(int kind, const Sweep& s, const CollParams& p);         \
  /* perform_triple_step fused: also stores the pre-collision populations to pre */       \
  cudaError_t step_pull_pre_f64(int kind, const Sweep& s, void* pre, const CollParams& p); \
  /* grid%streaming => stream_fvm_bardow (1), stream_fdm_bardow (2, 3 iso,    */          \
  /* 4 least squares), stream_fdm_sofonea (5): src/fvm_bardow.F90:393-886     */          \
  cudaError_t stream_scheme_f64(int scheme, const Sweep& s, double dt);                   \
  /* the same fused with collide_* in stencil form (9 FMAs per population) */             \
  cudaError_t step_scheme_f64(int scheme, int kind, const Sweep& s, double dt, const CollParams& p); \
  }
PLBM_DECLARE_F64(fma)
PLBM_DECLARE_F64(strict)
#undef PLBM_DECLARE_F64

// binary64 storage, hybrid arithmetic (hybrid.cuh), YFast pull, BGK, TRT and RR
cudaError_t step_pull_df64(int kind, const Sweep& s, const CollParams& p);
// The plugin step (shifted binary64, x-fastest, collide then push) in the
// hybrid arithmetic (BGK, TRT, RR).
cudaError_t step_push_hybrid(int kind, const Sweep& s, const CollParams& p);
// A finite-volume / finite-difference streaming scheme (stencil form) fused
// with the hybrid collision (BGK, TRT, RR).
cudaError_t step_scheme_hybrid(int scheme, int kind, const Sweep& s, double dt, const CollParams& p);
cudaError_t hybrid_range_flag(int* flag, int reset);

// Deviation storage (storage = 1 float, 2 half), binary32 arithmetic.
cudaError_t step_pull_dev(int storage, int kind, const Sweep& s, const CollParams& p);
cudaError_t stream_dev(int storage, const Sweep& s);
cudaError_t collide_dev(int storage, int kind, const Sweep& s, const CollParams& p);
cudaError_t step_push_dev(int storage, int kind, const Sweep& s, const CollParams& p);
// Deviation storage with the collision in binary64 (math 1, BGK/TRT/RR),
// compensated binary32 (math 2, BGK) or double-float (math 3, BGK)
// arithmetic; compiled in step_df64.cu.
cudaError_t step_pull_dev_hi(int storage, int math, int kind, const Sweep& s, const CollParams& p);

// Field kernels (fields.cu).  layout: 0 = YFast (src/), 1 = XFast (sim/).
// storage 0 = binary64 f (unshifted), 3 = binary64 shifted, 1/2 = deviation.
enum { ST_F64 = 0, ST_F32DEV = 1, ST_F16DEV = 2, ST_F64SHIFT = 3 };
// Moments of one lattice into (fast,slow) arrays; reference order of
// update_macros (YFast, unshifted) or lbm_macros (shifted).  exact (binary64
// storages 0 and 3): correctly rounded from the exact integer moments instead
// (exact_fields.cuh), the arithmetic of grids in hybrid mode.
cudaError_t macros(int storage, int layout, int nx, int ny, int ld, const void* f, double* rho,
                   double* ux, double* uy, cudaStream_t st, bool exact = false);
// Equilibrium from (fast,slow) rho/ux/uy arrays into a lattice.
//   storage 0: equilibrium() of src/fvm_bardow.F90:99-126;
//   storage 3/1/2: shifted equilibrium of sim/sim.F90:353-401 with rho = 1 + p/cs^2
//   when from_pressure != 0.
// exact (storages 0 and 3): the integer form of exact_fields.cuh.
cudaError_t equilibrium(int storage, int layout, int nx, int ny, int ld, const double* rho,
                        const double* ux, const double* uy, int from_pressure, void* f,
                        cudaStream_t st, bool exact = false);
// The same over the slow lines [slow0, slow1) only (x columns of the YFast
// layout): a slab of the grid, for pipelining with host transfers.  The
// field pointers still address the whole (fast, slow) arrays.
cudaError_t macros_range(int storage, int layout, int nx, int ny, int ld, const void* f, double* rho,
                         double* ux, double* uy, int slow0, int slow1, cudaStream_t st, bool exact = false);
cudaError_t equilibrium_range(int storage, int layout, int nx, int ny, int ld, const double* rho,
                              const double* ux, const double* uy, int from_pressure, void* f, int slow0,
                              int slow1, cudaStream_t st, bool exact = false);
// n doubles from src to dst (device addresses; either may be a mapped host
// array), by a kernel: 16-byte accesses when both are 16-byte aligned.
cudaError_t copy_doubles(const double* src, double* dst, size_t n, cudaStream_t st);
// binary64 f (YFast) <-> deviation storage conversion: h = f - w_i.
cudaError_t f64_to_dev(int storage, int nx, int ny, int ld, const double* f, void* h, cudaStream_t st);
cudaError_t dev_to_f64(int storage, int nx, int ny, int ld, const void* h, double* f, cudaStream_t st);
// Vorticity on (ny,nx) device arrays.
cudaError_t vorticity(int order, int nx, int ny, const double* ux, const double* uy, double* w,
                      cudaStream_t st);
// Per-block binary64 partial sums of 0.5*rho*|u|^2 and of |u-ua|^2, |ua|^2
// over the moments of a lattice; partial has room for reduce_blocks() triples.
int reduce_blocks(int nx, int ny);
cudaError_t energy_error_partials(int storage, int layout, int nx, int ny, int ld, const void* f,
                                  const double* uxa, const double* uya, double* partial,
                                  cudaStream_t st);

}  // namespace plbm
