// Host build of the compensated binary32 cell operators of
// periodic-lbm_gb300/csrc/coll_df64.cuh (the forward BGK collision on
// deviation storage and the adjoint's reverse step) for the CPU tests in
// test_df_cells_host.py: the same source the kernels compile.
#include <stdint.h>
#include "coll_df64.cuh"
using namespace plbm::df;

namespace {
df64 split(double d) {
  const float hi = (float)d;
  return make(hi, (float)(d - (double)hi));
}
const double kW[3] = {4.0 / 9.0, 1.0 / 9.0, 1.0 / 36.0};
}  // namespace

// One compensated BGK collision of the stored deviations h (binary32).
extern "C" void dc_bgk_comp(float* h, double omega) {
  DevParams p;
  for (int i = 0; i < 3; i++) {
    p.w[i] = split(kW[i]);
    p.w3[i] = split(3.0 * kW[i]);
  }
  p.om_hi = (float)omega;
  p.om_lo = (float)(omega - (double)p.om_hi);
  float v[9];
  for (int q = 0; q < 9; q++) v[q] = h[q];
  bgk_dev_comp(v, p);
  for (int q = 0; q < 9; q++) h[q] = v[q];
}

// One cell of the compensated adjoint reverse step: mu from the pulled
// deviations g and lambda l; returns the dL/domega term.
extern "C" float dc_adj_comp(const float* g, const float* l, float* mu, double omega) {
  AdjDevParams p;
  for (int i = 0; i < 3; i++) {
    p.w[i] = split(kW[i]);
    p.w3[i] = split(3.0 * kW[i]);
  }
  p.om_hi = (float)omega;
  p.om_lo = (float)(omega - (double)p.om_hi);
  float gg[9], ll[9], mm[9];
  for (int q = 0; q < 9; q++) {
    gg[q] = g[q];
    ll[q] = l[q];
  }
  const float d = adj_step_comp(gg, ll, mm, p);
  for (int q = 0; q < 9; q++) mu[q] = mm[q];
  return d;
}
