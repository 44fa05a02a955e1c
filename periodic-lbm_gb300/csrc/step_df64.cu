// step_df64.cu -- binary64-storage fused step in the "hybrid" arithmetic of
// hybrid.cuh (exact integer moments, double-float nonlinear term, binary64
// FMAs for the final linear combination).  BGK only.
//
// Compiled with --fmad=false: the double-float error-free transformations
// need every + - * rounded on its own; the fused operations are explicit.
#include "hybrid.cuh"
#include "plbm_launch.h"

namespace plbm {

// Set to 1 by a hybrid kernel that met a population outside |f| < 2.
__device__ int g_hybrid_range_flag = 0;

namespace {

__global__ void __launch_bounds__(kBlock) k_step_hybrid_bgk(const double* __restrict__ src,
                                                           double* __restrict__ dst, int nx, int ny, int ld,
                                                           int ftiles, hy::Params p) {
  const int x = blockIdx.x / ftiles;
  const int y = (blockIdx.x - x * ftiles) * blockDim.x + threadIdx.x;
  if (y >= ny) return;
  double f[9];
#pragma unroll
  for (int q = 0; q < 9; q++) {
    const int sx = wrap_add(x, -cx_of(q), nx), sy = wrap_add(y, -cy_of(q), ny);
    f[q] = __ldg(src + YFast::off(sx, sy, q, nx, ny, ld));
  }
  bool bad = false;
  hy::bgk(f, p, bad);
  if (bad) g_hybrid_range_flag = 1;
#pragma unroll
  for (int q = 0; q < 9; q++) dst[YFast::off(x, y, q, nx, ny, ld)] = f[q];
}

}  // namespace

hy::Params hybrid_params(double omega) {
  hy::Params p;
  p.omb = 1.0 - omega;
  const double w[3] = {W0, WS, WD};
  for (int i = 0; i < 3; i++) {
    p.omw[i] = omega * w[i];
    const float hi = (float)p.omw[i];
    p.omw_df[i] = df::make(hi, (float)(p.omw[i] - (double)hi));
  }
  return p;
}

cudaError_t step_pull_df64(int kind, const Sweep& s, const CollParams& cp) {
  if (kind != K_BGK) return cudaErrorNotSupported;
  const int ft = (s.ny + kBlock - 1) / kBlock;
  const long long blocks = (long long)ft * s.nx;
  if (blocks <= 0 || blocks > 0x7fffffffLL) return cudaErrorInvalidConfiguration;
  k_step_hybrid_bgk<<<(unsigned)blocks, kBlock, 0, s.stream>>>(static_cast<const double*>(s.src),
                                                               static_cast<double*>(s.dst), s.nx, s.ny, s.ld, ft,
                                                               hybrid_params(cp.omega));
  return cudaGetLastError();
}

cudaError_t hybrid_range_flag(int* flag, int reset) {
  cudaError_t e = cudaMemcpyFromSymbol(flag, g_hybrid_range_flag, sizeof(int));
  if (e == cudaSuccess && reset) {
    const int z = 0;
    e = cudaMemcpyToSymbol(g_hybrid_range_flag, &z, sizeof(int));
  }
  return e;
}

}  // namespace plbm
