// Host build of the integer field forms (periodic-lbm_gb300/csrc/exact_fields.cuh)
// for the CPU tests in test_exact_fields_host.py: the same source the field
// kernels compile, with the host branches of its few device intrinsics.
#include <stdint.h>
#include <math.h>
#include "exact_fields.cuh"
using namespace plbm;

extern "C" int xf_macros(const double* f, int shifted, double* out) {
  double g[9];
  for (int q = 0; q < 9; q++) g[q] = f[q];
  bool bad = false;
  if (shifted) ex::macros_exact<true>(g, out[0], out[1], out[2], bad);
  else ex::macros_exact<false>(g, out[0], out[1], out[2], bad);
  return bad;
}
extern "C" int xf_equilibrium(double rho, double ux, double uy, int shifted, int from_pressure, double* out) {
  bool bad = false;
  const int64_t P = from_pressure ? ex::rho_fixed_from_pressure(rho, bad) : ex::rho_fixed(rho, bad);
  double o[9];
  if (shifted) ex::equilibrium_exact<true>(P, ux, uy, o, bad);
  else ex::equilibrium_exact<false>(P, ux, uy, o, bad);
  for (int q = 0; q < 9; q++) out[q] = o[q];
  return bad;
}
extern "C" int64_t xf_rho_fixed_from_pressure(double p) {
  bool bad = false;
  return ex::rho_fixed_from_pressure(p, bad);
}
extern "C" int xf_div(int64_t a, uint64_t b, double* out) {
  bool bad = false;
  *out = ex::div_rn(a, ex::recip(b), bad);
  return bad;
}
extern "C" uint64_t xf_recip(uint64_t b, uint64_t* bn) {
  const ex::Recip r = ex::recip(b);
  *bn = r.bn;
  return r.v;
}
extern "C" double xf_fixed_to_double(int64_t t, int scale) { return ex::fixed_to_double_rne(t, scale); }
extern "C" double xf_weighted(double w, int64_t t, int scale) { return ex::weighted_rne(w, t, scale); }

// Whole fields, cell by cell: n cells of (rho, ux, uy) into out[q * n + i];
// the cells outside the range get NaN.  Returns the number of such cells.
extern "C" long xf_equilibrium_field(long n, const double* rho, const double* ux, const double* uy, int shifted,
                                     int from_pressure, double* out) {
  long nbad = 0;
  for (long i = 0; i < n; i++) {
    double o[9];
    const int bad = xf_equilibrium(rho[i], ux[i], uy[i], shifted, from_pressure, o);
    nbad += bad;
    for (int q = 0; q < 9; q++) out[q * n + i] = bad ? NAN : o[q];
  }
  return nbad;
}
// n cells of f[q * n + i] into out[k * n + i] (rho, ux, uy).
extern "C" long xf_macros_field(long n, const double* f, int shifted, double* out) {
  long nbad = 0;
  for (long i = 0; i < n; i++) {
    double g[9], m[3];
    for (int q = 0; q < 9; q++) g[q] = f[q * n + i];
    const int bad = xf_macros(g, shifted, m);
    nbad += bad;
    for (int k = 0; k < 3; k++) out[k * n + i] = bad ? NAN : m[k];
  }
  return nbad;
}
