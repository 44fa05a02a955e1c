// plbm_adjoint.h -- internal interface of the adjoint kernels (adjoint.cu).
#pragma once
#include <cuda_runtime.h>

namespace plbm {

struct AdjLaunch {
  int nx, ny, ld;
  const void* f;        // lattice read (init: written)
  const void* lam_in;   // lambda_{n+1} (u0 kernel: lambda_0)
  void* lam_out;        // lambda_n (final kernel: lambda_T)
  const double* u;      // u0, (2,nx,ny)
  const double* g;      // dL/du_T, (2,nx,ny)
  double* out;          // u_T or dL/du0, (2,nx,ny)
  double* dom;          // per-block dL/domega slots
  double omega;
  int comp;             // reverse step in compensated binary32 (binary32 storage)
  cudaStream_t stream;
};

// what: 0 init f_0 into a.f (cast away const), 1 final (u_T -> out, lambda_T -> lam_out),
//       2 reverse step, 3 dL/du0.
cudaError_t adjoint_launch(int storage, int what, const AdjLaunch& a);
// binary64 slots for dL/domega (one per warp of the reverse-step launch)
int adjoint_blocks(int nx, int ny);

}  // namespace plbm
