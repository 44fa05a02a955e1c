// grid.cpp -- the plbm_* C ABI: a device-resident mirror of the reference's
// lattice_grid (src/fvm_bardow.F90:37-69) and the routines that act on it.
//
// The handle owns `nf` device lattices of the reference layout f(ld,nx,0:8)
// and the integer buffer indices iold/inew (1-based, as in the Fortran).  The
// host copy of grid%f stays with the caller; transfers happen only in
// plbm_upload / plbm_download / plbm_update_macros.
//
// Compiled with -ffp-contract=off so that the scalar relaxation parameters
// (omega, lambda_d, w*(1-omega), ...) are the same binary64 values the
// Fortran computes.
#include <cuda_runtime.h>
#include <math.h>
#include <stdarg.h>
#include <stdio.h>
#include <string.h>
#include <atomic>
#include <string>
#include <vector>

#include "../../include/plbm_gpu.h"
#include "grid_internal.h"
#include "plbm_launch.h"

using namespace plbm;

int plbm::block_for(long long cells) {
  static std::atomic<int> sms[64];  // SM count per device, 0 until first asked
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return kBlock;
  int n = sms[dev].load(std::memory_order_relaxed);
  if (n < 1) {
    if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n < 1) return kBlock;
    sms[dev].store(n, std::memory_order_relaxed);
  }
  const long long per_sm = (cells + n - 1) / n;
  if (per_sm >= kBlock) return kBlock;
  return (int)(per_sm < 32 ? 32 : (per_sm + 31) / 32 * 32);
}

// ---------------------------------------------------------------------------
// error reporting
namespace plbm_internal {
thread_local std::string g_last_error;

int fail(int code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  g_last_error = buf;
  return code;
}
int cuda_fail(cudaError_t e, const char* what) {
  const int code = e == cudaErrorMemoryAllocation ? PLBM_E_NOMEM
                   : e == cudaErrorNotSupported   ? PLBM_E_UNSUPPORTED
                                                  : PLBM_E_CUDA;
  return fail(code, "%s: %s (%s)", what, cudaGetErrorString(e), cudaGetErrorName(e));
}
}  // namespace plbm_internal
using namespace plbm_internal;

#define CUDA_TRY(expr, what) PLBM_CUDA_TRY(expr, what)

extern "C" const char* plbm_last_error(void) { return g_last_error.c_str(); }
extern "C" int plbm_version(void) { return 1 * 10000 + 1 * 100 + 0; }

// Relaxation parameters of one launch, as the Fortran forms them:
//   BGK  omegabar = 1 - omega                      (src/collision_bgk.F90:26)
//   TRT  lambda_e = omega, lambda_d(omega, magic)  (src/collision_trt.F90:47-48)
//   RR   w*(1 - omega)                             (src/collision_regularized.F90:63-65)
//   BGKI fac = 4.5 - 2.25*omega                    (src/collision_bgk_improved.f90:39)
CollParams plbm_make_params(double omega, double trt_magic) {
  CollParams p;
  p.omega = omega;
  p.omegabar = 1.0 - omega;
  p.lambda_d = (4.0 - 2.0 * omega) / (4.0 * trt_magic * omega + 2.0 - omega);
  p.les = 0.5 * omega;
  p.lds = 0.5 * p.lambda_d;
  p.rr_w0 = W0 * (1.0 - omega);
  p.rr_ws = WS * (1.0 - omega);
  p.rr_wd = WD * (1.0 - omega);
  p.bgki_fac = 4.5 - 2.25 * omega;
  return p;
}

extern "C" int plbm_grid_create(int nx, int ny, int nf, int storage, plbm_grid_t** out) {
  if (!out) return fail(PLBM_E_INVALID, "out is NULL");
  *out = nullptr;
  if (nx < 1 || ny < 1) return fail(PLBM_E_INVALID, "grid size %dx%d: nx and ny must be >= 1", nx, ny);
  if (nx > PLBM_MAX_EXTENT || ny > PLBM_MAX_EXTENT)
    return fail(PLBM_E_INVALID, "grid size %dx%d: nx and ny must be <= %d", nx, ny, PLBM_MAX_EXTENT);
  if (nf < 2 || nf > 16) return fail(PLBM_E_INVALID, "nf = %d: need 2 <= nf <= 16", nf);
  if (storage != PLBM_F64 && storage != PLBM_F32DEV && storage != PLBM_F16DEV)
    return fail(PLBM_E_INVALID, "unknown storage %d", storage);
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev < 1) {
    cudaGetLastError();
    return fail(PLBM_E_NODEVICE, "no CUDA device visible");
  }
  const int ld = pad16(ny);
  const size_t lat = (size_t)ld * (size_t)nx * 9u;
  if ((double)lat * nf > 4.0e11) return fail(PLBM_E_INVALID, "lattice of %zu elements x %d is too large", lat, nf);
  plbm_grid_t* g = new plbm_grid_t();
  g->nx = nx;
  g->ny = ny;
  g->ld = ld;
  g->nf = nf;
  g->storage = storage;
  g->lat_elems = lat;
  g->elem_bytes = storage == PLBM_F64 ? 8 : (storage == PLBM_F32DEV ? 4 : 2);
  cudaGetDevice(&g->device);
  cudaError_t e = cudaMalloc(&g->f, lat * nf * g->elem_bytes);
  if (e != cudaSuccess) {
    delete g;
    cudaGetLastError();
    return cuda_fail(e, "cudaMalloc(lattices)");
  }
  // allocate() leaves the Fortran array undefined; zero is a deterministic stand-in.
  e = cudaMemset(g->f, 0, lat * nf * g->elem_bytes);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&g->own, cudaStreamNonBlocking);
  if (e != cudaSuccess) {
    cudaFree(g->f);
    delete g;
    return cuda_fail(e, "grid setup");
  }
  g->stream = g->own;
  g->imid = nf > 2 ? 3 : -1;  // src/fvm_bardow.F90:172-177
  *out = g;
  return ok();
}

extern "C" int plbm_grid_destroy(plbm_grid_t* g) {
  if (!g) return PLBM_OK;
  cudaSetDevice(g->device);
  cudaStreamSynchronize(g->stream);
  if (g->f) cudaFree(g->f);
  if (g->spare) cudaFree(g->spare);
  if (g->scratch) cudaFree(g->scratch);
  if (g->step_graph) cudaGraphExecDestroy(g->step_graph);
  if (g->xfer) {
    cudaStreamSynchronize(g->xfer);
    cudaStreamDestroy(g->xfer);
  }
  for (cudaEvent_t ev : g->slab_ev)
    if (ev) cudaEventDestroy(ev);
  if (g->own) cudaStreamDestroy(g->own);
  delete g;
  return PLBM_OK;
}

extern "C" int plbm_grid_info(const plbm_grid_t* g, int* nx, int* ny, int* ld, int* nf, int* storage) {
  if (int r = check_grid(g)) return r;
  if (nx) *nx = g->nx;
  if (ny) *ny = g->ny;
  if (ld) *ld = g->ld;
  if (nf) *nf = g->nf;
  if (storage) *storage = g->storage;
  return PLBM_OK;
}

extern "C" int plbm_grid_indices(const plbm_grid_t* g, int* iold, int* inew) {
  if (int r = check_grid(g)) return r;
  if (iold) *iold = g->iold;
  if (inew) *inew = g->inew;
  return PLBM_OK;
}

extern "C" int plbm_grid_set_indices(plbm_grid_t* g, int iold, int inew) {
  if (int r = check_grid(g)) return r;
  if (int r = check_buf(g, iold)) return r;
  if (int r = check_buf(g, inew)) return r;
  if (iold == inew) return fail(PLBM_E_INVALID, "iold and inew must differ");
  g->iold = iold;
  g->inew = inew;
  return PLBM_OK;
}

extern "C" int plbm_grid_indices3(const plbm_grid_t* g, int* iold, int* inew, int* imid) {
  if (int r = check_grid(g)) return r;
  if (iold) *iold = g->iold;
  if (inew) *inew = g->inew;
  if (imid) *imid = g->imid;
  return PLBM_OK;
}

extern "C" int plbm_grid_set_indices3(plbm_grid_t* g, int iold, int inew, int imid) {
  if (int r = check_grid(g)) return r;
  if (int r = check_buf(g, iold)) return r;
  if (int r = check_buf(g, inew)) return r;
  if (imid != -1) {
    if (int r = check_buf(g, imid)) return r;
    if (imid == iold || imid == inew) return fail(PLBM_E_INVALID, "imid must differ from iold and inew");
  }
  if (iold == inew) return fail(PLBM_E_INVALID, "iold and inew must differ");
  g->iold = iold;
  g->inew = inew;
  g->imid = imid;
  return PLBM_OK;
}

extern "C" int plbm_grid_set_stream(plbm_grid_t* g, void* s) {
  if (int r = check_grid(g)) return r;
  g->stream = s ? static_cast<cudaStream_t>(s) : g->own;
  return PLBM_OK;
}

extern "C" int plbm_grid_device_ptr(const plbm_grid_t* g, int ibuf, void** dptr) {
  if (int r = check_grid(g)) return r;
  if (int r = check_buf(g, ibuf)) return r;
  if (!dptr) return fail(PLBM_E_INVALID, "dptr is NULL");
  *dptr = lattice(g, ibuf);
  return PLBM_OK;
}

extern "C" int plbm_set_properties(plbm_grid_t* g, double nu, double dt, const double* magic) {
  if (int r = check_grid(g)) return r;
  if (!(dt > 0.0) || !(nu > 0.0)) return fail(PLBM_E_INVALID, "nu and dt must be > 0 (nu=%g dt=%g)", nu, dt);
  // src/fvm_bardow.F90:249-265
  const double csqr = 1.0 / 3.0, invcsqr = 1.0 / csqr;
  g->nu = nu;
  g->dt = dt;
  const double tau = invcsqr * nu;
  g->tau = tau;
  g->omega = dt / (tau + 0.5 * dt);
  if (magic) g->trt_magic = *magic;
  else {
    const double r = tau / dt;
    g->trt_magic = r * r;
  }
  return PLBM_OK;
}

extern "C" int plbm_get_properties(const plbm_grid_t* g, double* nu, double* dt, double* tau, double* omega,
                                   double* trt_magic) {
  if (int r = check_grid(g)) return r;
  if (nu) *nu = g->nu;
  if (dt) *dt = g->dt;
  if (tau) *tau = g->tau;
  if (omega) *omega = g->omega;
  if (trt_magic) *trt_magic = g->trt_magic;
  return PLBM_OK;
}

extern "C" int plbm_set_relaxation(plbm_grid_t* g, double omega, double trt_magic) {
  if (int r = check_grid(g)) return r;
  if (!(omega > 0.0 && omega < 2.0)) return fail(PLBM_E_INVALID, "omega = %g outside (0,2)", omega);
  g->omega = omega;
  g->trt_magic = trt_magic;
  return PLBM_OK;
}

extern "C" int plbm_set_collision(plbm_grid_t* g, int kind) {
  if (int r = check_grid(g)) return r;
  if (kind < PLBM_BGK || kind > PLBM_BGKI) return fail(PLBM_E_INVALID, "unknown collision kind %d", kind);
  if (kind == PLBM_BGKI && g->storage != PLBM_F64)
    return fail(PLBM_E_UNSUPPORTED, "collide_bgk_improved is offered for PLBM_F64 storage only");
  g->kind = kind;
  return PLBM_OK;
}

extern "C" int plbm_set_time_step(plbm_grid_t* g, double dt) {
  if (int r = check_grid(g)) return r;
  if (!(dt > 0.0)) return fail(PLBM_E_INVALID, "dt = %g must be > 0", dt);
  g->dt = dt;
  return PLBM_OK;
}

extern "C" int plbm_set_streaming(plbm_grid_t* g, int scheme) {
  if (int r = check_grid(g)) return r;
  if (scheme < PLBM_STREAM_LBM || scheme > PLBM_STREAM_FDM_BARDOW_WLS_GAUSS_V2)
    return fail(PLBM_E_INVALID, "unknown streaming scheme %d", scheme);
  g->streaming = scheme;
  return PLBM_OK;
}

extern "C" int plbm_set_math(plbm_grid_t* g, int math) {
  if (int r = check_grid(g)) return r;
  if (math < PLBM_MATH_FMA || math > PLBM_MATH_DF64) return fail(PLBM_E_INVALID, "unknown math mode %d", math);
  if (math == PLBM_MATH_DF64 && g->storage == PLBM_F64)
    return fail(PLBM_E_UNSUPPORTED, "PLBM_MATH_DF64 applies to deviation storage only");
  g->math = math;
  return PLBM_OK;
}

// ---------------------------------------------------------------------------
namespace {
// Device address of a host array that is page-locked and mapped (cudaHostAlloc
// / cudaMallocHost / cudaHostRegister under unified addressing), else NULL
// (pageable memory, or NULL).  The field kernels then read or write the host
// array directly over the host link: no staging buffer, and no copy engine.
const void* mapped_host(const void* p) {
  if (!p) return nullptr;
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  return a.type == cudaMemoryTypeHost ? a.devicePointer : nullptr;
}

}  // namespace

extern "C" int plbm_upload(plbm_grid_t* g, const double* f_host, int ibuf) {
  if (int r = check_grid(g)) return r;
  if (int r = check_buf(g, ibuf)) return r;
  if (!f_host) return fail(PLBM_E_INVALID, "f_host is NULL");
  if (int r = use_device(g)) return r;
  const size_t bytes64 = g->lat_elems * sizeof(double);
  if (const void* m = mapped_host(f_host)) {  // page-locked: read in place by the kernel
    const double* src = static_cast<const double*>(m);
    if (g->storage == PLBM_F64)
      CUDA_TRY(copy_doubles(src, static_cast<double*>(lattice(g, ibuf)), g->lat_elems, g->stream), "upload");
    else
      CUDA_TRY(f64_to_dev(internal_storage(g->storage), g->nx, g->ny, g->ld, src, lattice(g, ibuf), g->stream),
               "upload (deviation conversion)");
    CUDA_TRY(cudaStreamSynchronize(g->stream), "upload sync");
    return ok();
  }
  if (g->storage == PLBM_F64) {
    CUDA_TRY(cudaMemcpyAsync(lattice(g, ibuf), f_host, bytes64, cudaMemcpyHostToDevice, g->stream), "upload");
    CUDA_TRY(cudaStreamSynchronize(g->stream), "upload sync");
    return ok();
  }
  double* tmp = nullptr;
  CUDA_TRY(cudaMalloc(&tmp, bytes64), "cudaMalloc(upload staging)");
  cudaError_t e = cudaMemcpyAsync(tmp, f_host, bytes64, cudaMemcpyHostToDevice, g->stream);
  if (e == cudaSuccess) e = f64_to_dev(internal_storage(g->storage), g->nx, g->ny, g->ld, tmp, lattice(g, ibuf), g->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(g->stream);
  cudaFree(tmp);
  if (e != cudaSuccess) return cuda_fail(e, "upload (deviation conversion)");
  return ok();
}

extern "C" int plbm_download(plbm_grid_t* g, double* f_host, int ibuf) {
  if (int r = check_grid(g)) return r;
  if (int r = check_buf(g, ibuf)) return r;
  if (!f_host) return fail(PLBM_E_INVALID, "f_host is NULL");
  if (int r = use_device(g)) return r;
  const size_t bytes64 = g->lat_elems * sizeof(double);
  const void* m = g->storage == PLBM_F64 ? mapped_host(f_host) : nullptr;
  if (m) {  // page-locked: written in place by the kernel
    CUDA_TRY(copy_doubles(static_cast<const double*>(lattice(g, ibuf)), static_cast<double*>(const_cast<void*>(m)),
                          g->lat_elems, g->stream),
             "download");
    CUDA_TRY(cudaStreamSynchronize(g->stream), "download sync");
    return ok();
  }
  if (g->storage == PLBM_F64) {
    CUDA_TRY(cudaMemcpyAsync(f_host, lattice(g, ibuf), bytes64, cudaMemcpyDeviceToHost, g->stream), "download");
    CUDA_TRY(cudaStreamSynchronize(g->stream), "download sync");
    return ok();
  }
  double* tmp = nullptr;
  CUDA_TRY(cudaMalloc(&tmp, bytes64), "cudaMalloc(download staging)");
  // padding rows are not converted; give them a defined value
  cudaError_t e = cudaMemsetAsync(tmp, 0, bytes64, g->stream);
  if (e == cudaSuccess) e = dev_to_f64(internal_storage(g->storage), g->nx, g->ny, g->ld, lattice(g, ibuf), tmp, g->stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(f_host, tmp, bytes64, cudaMemcpyDeviceToHost, g->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(g->stream);
  cudaFree(tmp);
  if (e != cudaSuccess) return cuda_fail(e, "download (deviation conversion)");
  return ok();
}

namespace {

// Large grids move their (ny,nx) moment fields in x-column slabs -- each a
// contiguous range of the host arrays -- on a second stream, so that the
// copy of one slab overlaps the kernel of the previous one
// (set_pdf_to_equilibrium: copy then equilibrium; update_macros: moments
// then copy).  About 96 MB of fields per slab, at most kMaxSlabs.
int slab_count(const plbm_grid_t* g) {
  const size_t n = (size_t)g->nx * g->ny;
  if (n < ((size_t)1 << 22) || g->nx < 4) return 1;
  const size_t s = 3 * n * 8 / ((size_t)96 << 20);
  const size_t lim = (size_t)kMaxSlabs < (size_t)g->nx ? (size_t)kMaxSlabs : (size_t)g->nx;
  return (int)(s < 2 ? 2 : (s > lim ? lim : s));
}

int ensure_xfer(plbm_grid_t* g) {
  if (!g->xfer) CUDA_TRY(cudaStreamCreateWithFlags(&g->xfer, cudaStreamNonBlocking), "transfer stream");
  for (cudaEvent_t& ev : g->slab_ev)
    if (!ev) CUDA_TRY(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming), "slab event");
  return PLBM_OK;
}

inline void slab_bounds(const plbm_grid_t* g, int s, int S, int& x0, int& x1) {
  x0 = (int)((long long)g->nx * s / S);
  x1 = (int)((long long)g->nx * (s + 1) / S);
}

}  // namespace

extern "C" int plbm_set_pdf_to_equilibrium(plbm_grid_t* g, const double* rho, const double* ux, const double* uy) {
  if (int r = check_grid(g)) return r;
  if (!rho || !ux || !uy) return fail(PLBM_E_INVALID, "rho, ux and uy must be non-NULL");
  if (int r = use_device(g)) return r;
  const void *mr = mapped_host(rho), *mu = mapped_host(ux), *mv = mapped_host(uy);
  if (mr && mu && mv) {  // page-locked host fields: the kernel reads them in place
    CUDA_TRY(equilibrium(internal_storage(g->storage), 0, g->nx, g->ny, g->ld, static_cast<const double*>(mr),
                         static_cast<const double*>(mu), static_cast<const double*>(mv), 0, lattice(g, g->iold),
                         g->stream, exact_fields(g)),
             "equilibrium kernel");
    CUDA_TRY(cudaStreamSynchronize(g->stream), "equilibrium sync");
    return ok();
  }
  const size_t n = (size_t)g->nx * g->ny;
  if (int r = ensure_scratch(g, 3 * n)) return r;
  double* d = g->scratch;
  const int S = slab_count(g);
  if (S > 1) {
    if (int r = ensure_xfer(g)) return r;
    // the copies start after the grid's earlier work (which may read the scratch)
    CUDA_TRY(cudaEventRecord(g->slab_ev[kMaxSlabs], g->stream), "equilibrium order");
    CUDA_TRY(cudaStreamWaitEvent(g->xfer, g->slab_ev[kMaxSlabs], 0), "equilibrium order");
    const double* src[3] = {rho, ux, uy};
    for (int s = 0; s < S; s++) {
      int x0, x1;
      slab_bounds(g, s, S, x0, x1);
      const size_t off = (size_t)x0 * g->ny, cnt = (size_t)(x1 - x0) * g->ny;
      for (int k = 0; k < 3; k++)
        CUDA_TRY(cudaMemcpyAsync(d + k * n + off, src[k] + off, cnt * 8, cudaMemcpyHostToDevice, g->xfer),
                 "upload fields");
      CUDA_TRY(cudaEventRecord(g->slab_ev[s], g->xfer), "slab event");
      CUDA_TRY(cudaStreamWaitEvent(g->stream, g->slab_ev[s], 0), "slab wait");
      CUDA_TRY(equilibrium_range(internal_storage(g->storage), 0, g->nx, g->ny, g->ld, d, d + n, d + 2 * n, 0,
                                 lattice(g, g->iold), x0, x1, g->stream, exact_fields(g)),
               "equilibrium kernel");
    }
    CUDA_TRY(cudaStreamSynchronize(g->stream), "equilibrium sync");
    return ok();
  }
  CUDA_TRY(cudaMemcpyAsync(d, rho, n * 8, cudaMemcpyHostToDevice, g->stream), "upload rho");
  CUDA_TRY(cudaMemcpyAsync(d + n, ux, n * 8, cudaMemcpyHostToDevice, g->stream), "upload ux");
  CUDA_TRY(cudaMemcpyAsync(d + 2 * n, uy, n * 8, cudaMemcpyHostToDevice, g->stream), "upload uy");
  CUDA_TRY(equilibrium(internal_storage(g->storage), 0, g->nx, g->ny, g->ld, d, d + n, d + 2 * n, 0,
                       lattice(g, g->iold), g->stream, exact_fields(g)),
           "equilibrium kernel");
  CUDA_TRY(cudaStreamSynchronize(g->stream), "equilibrium sync");
  return ok();
}

namespace {

// Finite-volume / finite-difference streaming of the handle's scheme.
cudaError_t stream_scheme(const plbm_grid_t* g, const Sweep& s) {
  return g->math == PLBM_MATH_STRICT ? strict::stream_scheme_f64(g->streaming, s, g->dt)
                                     : fma::stream_scheme_f64(g->streaming, s, g->dt);
}

// One fused step from lattice a to lattice b with the handle's settings.
cudaError_t fused_step(plbm_grid_t* g, const void* a, void* b, const CollParams& p) {
  Sweep s{g->nx, g->ny, g->ld, a, b, g->stream};
  if (g->streaming != PLBM_STREAM_LBM) {
    // FMA arithmetic: one fused kernel, the scheme in stencil form then the
    // collision; strict: the reference's two passes, expression by expression
    if (g->math == PLBM_MATH_FMA && !(g->kind == PLBM_BGKI && g->ld != g->ny))
      return fma::step_scheme_f64(g->streaming, g->kind, s, g->dt, p);
    if (g->math == PLBM_MATH_HYBRID) return step_scheme_hybrid(g->streaming, g->kind, s, g->dt, p);
    cudaError_t e = stream_scheme(g, s);
    if (e != cudaSuccess) return e;
    return g->math == PLBM_MATH_STRICT ? strict::collide_f64(g->kind, s, p) : fma::collide_f64(g->kind, s, p);
  }
  if (g->storage != PLBM_F64) {
    if (g->math == PLBM_MATH_FMA) return step_pull_dev(g->storage, g->kind, s, p);
    return step_pull_dev_hi(g->storage, g->math, g->kind, s, p);
  }
  if (g->kind == PLBM_BGKI && g->ld != g->ny) {
    // The (ny,nx,0:8) dummy of collide_bgk_improved does not coincide with the
    // padded lattice: keep the two reference passes.
    cudaError_t e = fma::stream_f64(s);
    if (e != cudaSuccess) return e;
    return g->math == PLBM_MATH_STRICT ? strict::collide_f64(g->kind, s, p) : fma::collide_f64(g->kind, s, p);
  }
  switch (g->math) {
    case PLBM_MATH_STRICT: return strict::step_pull_f64(g->kind, s, p);
    case PLBM_MATH_HYBRID: return step_pull_df64(g->kind, s, p);
    default: return fma::step_pull_f64(g->kind, s, p);
  }
}

// The finite-volume / finite-difference schemes: binary64 storage, FMA or
// strict arithmetic.
int check_scheme(const plbm_grid_t* g) {
  if (g->streaming == PLBM_STREAM_LBM) return PLBM_OK;
  if (g->storage != PLBM_F64) return fail(PLBM_E_UNSUPPORTED, "streaming scheme %d needs PLBM_F64 storage", g->streaming);
  if (g->math == PLBM_MATH_HYBRID && g->kind == PLBM_BGKI)
    return fail(PLBM_E_UNSUPPORTED, "PLBM_MATH_HYBRID is not offered for collide_bgk_improved");
  if (g->math != PLBM_MATH_FMA && g->math != PLBM_MATH_STRICT && g->math != PLBM_MATH_HYBRID)
    return fail(PLBM_E_UNSUPPORTED, "streaming scheme %d runs with PLBM_MATH_FMA, _STRICT or _HYBRID", g->streaming);
  return PLBM_OK;
}

}  // namespace

extern "C" int plbm_stream(plbm_grid_t* g) {
  if (int r = check_grid(g)) return r;
  if (int r = use_device(g)) return r;
  Sweep s{g->nx, g->ny, g->ld, lattice(g, g->iold), lattice(g, g->inew), g->stream};
  if (g->streaming != PLBM_STREAM_LBM) {
    if (int r = check_scheme(g)) return r;
    CUDA_TRY(stream_scheme(g, s), "streaming-scheme kernel");
    return ok();
  }
  cudaError_t e = g->storage == PLBM_F64 ? fma::stream_f64(s) : stream_dev(g->storage, s);
  if (e != cudaSuccess) return cuda_fail(e, "lbm_stream kernel");
  return ok();
}

extern "C" int plbm_collide(plbm_grid_t* g) {
  if (int r = check_grid(g)) return r;
  if (int r = use_device(g)) return r;
  const CollParams p = plbm_make_params(g->omega, g->trt_magic);
  Sweep s{g->nx, g->ny, g->ld, nullptr, lattice(g, g->inew), g->stream};
  cudaError_t e;
  if (g->storage != PLBM_F64) e = collide_dev(g->storage, g->kind, s, p);
  else if (g->math == PLBM_MATH_STRICT) e = strict::collide_f64(g->kind, s, p);
  else e = fma::collide_f64(g->kind, s, p);
  if (e != cudaSuccess) return cuda_fail(e, "collision kernel");
  return ok();
}

namespace {

// Small grids: one step is a few microseconds of GPU work, less than the
// host's cost of a launch, so a loop of launches leaves the GPU idle.  The
// loop is captured once as a CUDA graph of kGraphSteps (even) fused steps,
// lattice iold -> inew -> iold ..., and replayed; an even count leaves iold
// and inew where they were.
constexpr int kGraphSteps = 16;
constexpr long long kGraphCells = 1ll << 17;

bool graph_key_matches(const plbm_grid_t* g, const void* a, const void* b) {
  const auto& k = g->step_key;
  return g->step_graph && k.a == a && k.b == b && k.stream == g->stream && k.kind == g->kind &&
         k.math == g->math && k.streaming == g->streaming && k.omega == g->omega &&
         k.trt_magic == g->trt_magic && k.dt == g->dt;
}

// Replays the captured loop `reps` times (capturing it first when needed).
// Returns cudaErrorNotSupported when the stream cannot be captured (the
// caller's own capture is in progress, or a stream such as the legacy default
// stream that capture does not take): the caller then launches step by step.
// Nothing has been launched on the stream when it returns that.
cudaError_t replay_step_graph(plbm_grid_t* g, const CollParams& p, int reps) {
  void* a = lattice(g, g->iold);
  void* b = lattice(g, g->inew);
  if (!graph_key_matches(g, a, b)) {
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    cudaError_t e = cudaStreamIsCapturing(g->stream, &cs);
    if (e != cudaSuccess) return e;
    if (cs != cudaStreamCaptureStatusNone) return cudaErrorNotSupported;
    if (g->step_graph) cudaGraphExecDestroy(g->step_graph);
    g->step_graph = nullptr;
    if (cudaStreamBeginCapture(g->stream, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
      cudaGetLastError();
      return cudaErrorNotSupported;
    }
    cudaError_t le = cudaSuccess;
    for (int i = 0; i < kGraphSteps && le == cudaSuccess; i++)
      le = fused_step(g, i % 2 ? b : a, i % 2 ? a : b, p);
    cudaGraph_t graph = nullptr;
    e = cudaStreamEndCapture(g->stream, &graph);
    if (le != cudaSuccess || e != cudaSuccess) {
      if (graph) cudaGraphDestroy(graph);
      return le != cudaSuccess ? le : e;
    }
    e = cudaGraphInstantiate(&g->step_graph, graph, 0);
    cudaGraphDestroy(graph);
    if (e != cudaSuccess) {
      g->step_graph = nullptr;
      return e;
    }
    auto& k = g->step_key;
    k.a = a;
    k.b = b;
    k.stream = g->stream;
    k.kind = g->kind;
    k.math = g->math;
    k.streaming = g->streaming;
    k.omega = g->omega;
    k.trt_magic = g->trt_magic;
    k.dt = g->dt;
  }
  for (int r = 0; r < reps; r++) {
    cudaError_t e = cudaGraphLaunch(g->step_graph, g->stream);
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}

}  // namespace

extern "C" int plbm_perform_lbm_step(plbm_grid_t* g, int nsteps) {
  if (int r = check_grid(g)) return r;
  if (nsteps < 0) return fail(PLBM_E_INVALID, "nsteps = %d < 0", nsteps);
  if (g->storage == PLBM_F64 && g->math == PLBM_MATH_HYBRID && g->kind == PLBM_BGKI)
    return fail(PLBM_E_UNSUPPORTED, "PLBM_MATH_HYBRID is not offered for collide_bgk_improved");
  if (g->storage != PLBM_F64 && (g->math == PLBM_MATH_HYBRID || g->math == PLBM_MATH_DF64) && g->kind != PLBM_BGK)
    return fail(PLBM_E_UNSUPPORTED, "PLBM_MATH_HYBRID / PLBM_MATH_DF64 with deviation storage are offered for collide_bgk only");
  if (int r = check_scheme(g)) return r;
  if (int r = use_device(g)) return r;
  const CollParams p = plbm_make_params(g->omega, g->trt_magic);
  if ((long long)g->nx * g->ny <= kGraphCells && nsteps >= 2 * kGraphSteps) {
    const int reps = nsteps / kGraphSteps;
    cudaError_t e = replay_step_graph(g, p, reps);
    if (e == cudaSuccess) {
      nsteps -= reps * kGraphSteps;  // even: iold, inew unchanged
    } else if (e != cudaErrorNotSupported) {
      return cuda_fail(e, "stream-collide graph");
    }
  }
  for (int i = 0; i < nsteps; i++) {
    cudaError_t e = fused_step(g, lattice(g, g->iold), lattice(g, g->inew), p);
    if (e != cudaSuccess) return cuda_fail(e, "stream-collide kernel");
    const int t = g->iold;  // src/periodic_lbm.f90:22-27
    g->iold = g->inew;
    g->inew = t;
  }
  return ok();
}

// perform_triple_step (src/fvm_bardow.F90:322-340): stream iold -> inew, keep
// the streamed populations in iold, collide inew in place, then rotate
// iold <- inew, inew <- imid, imid <- iold.  Done as one fused kernel that
// writes the pre-collision populations to a spare lattice; the spare then
// takes the place of buffer iold (the buffer-index -> lattice map is
// permuted), so every buffer index holds what the Fortran leaves in it.
extern "C" int plbm_perform_triple_step(plbm_grid_t* g, int nsteps) {
  if (int r = check_grid(g)) return r;
  if (nsteps < 0) return fail(PLBM_E_INVALID, "nsteps = %d < 0", nsteps);
  if (g->imid < 1) return fail(PLBM_E_INVALID, "perform_triple_step needs a third buffer (alloc_grid with nf >= 3)");
  if (g->storage != PLBM_F64)
    return fail(PLBM_E_UNSUPPORTED, "perform_triple_step is offered for PLBM_F64 storage");
  if (g->math != PLBM_MATH_FMA && g->math != PLBM_MATH_STRICT)
    return fail(PLBM_E_UNSUPPORTED, "perform_triple_step runs with PLBM_MATH_FMA or PLBM_MATH_STRICT");
  if (int r = use_device(g)) return r;
  if (!g->spare) {
    CUDA_TRY(cudaMalloc(&g->spare, g->lat_elems * g->elem_bytes), "cudaMalloc(spare lattice)");
    CUDA_TRY(cudaMemsetAsync(g->spare, 0, g->lat_elems * g->elem_bytes, g->stream), "clear spare lattice");
    g->spare_slot = g->nf;
  }
  const CollParams p = plbm_make_params(g->omega, g->trt_magic);
  const bool strict_math = g->math == PLBM_MATH_STRICT;
  for (int i = 0; i < nsteps; i++) {
    void* pre = physical(g, g->spare_slot);
    Sweep s{g->nx, g->ny, g->ld, lattice(g, g->iold), lattice(g, g->inew), g->stream};
    cudaError_t e;
    if (g->streaming != PLBM_STREAM_LBM || (g->kind == PLBM_BGKI && g->ld != g->ny)) {
      // another streaming scheme, or the (ny,nx,0:8) dummy of
      // collide_bgk_improved: the reference's passes
      e = g->streaming != PLBM_STREAM_LBM ? stream_scheme(g, s) : fma::stream_f64(s);
      if (e == cudaSuccess)
        e = cudaMemcpyAsync(pre, s.dst, g->lat_elems * g->elem_bytes, cudaMemcpyDeviceToDevice, g->stream);
      if (e == cudaSuccess) e = strict_math ? strict::collide_f64(g->kind, s, p) : fma::collide_f64(g->kind, s, p);
    } else {
      e = strict_math ? strict::step_pull_pre_f64(g->kind, s, pre, p) : fma::step_pull_pre_f64(g->kind, s, pre, p);
    }
    if (e != cudaSuccess) return cuda_fail(e, "triple-step kernel");
    // the spare now holds f(:,:,:,iold) of the Fortran; the old iold lattice is free
    const int freed = g->slot[g->iold - 1];
    g->slot[g->iold - 1] = g->spare_slot;
    g->spare_slot = freed;
    const int t = g->iold;  // src/fvm_bardow.F90:333-338
    g->iold = g->inew;
    g->inew = g->imid;
    g->imid = t;
  }
  return ok();
}

extern "C" int plbm_equilibrium_device(plbm_grid_t* g, int ibuf, const double* rho, const double* ux,
                                       const double* uy) {
  if (int r = check_grid(g)) return r;
  if (int r = check_buf(g, ibuf)) return r;
  if (!rho || !ux || !uy) return fail(PLBM_E_INVALID, "rho, ux and uy must be non-NULL");
  if (int r = use_device(g)) return r;
  CUDA_TRY(equilibrium(internal_storage(g->storage), 0, g->nx, g->ny, g->ld, rho, ux, uy, 0, lattice(g, ibuf),
                       g->stream, exact_fields(g)),
           "equilibrium kernel");
  return ok();
}

extern "C" int plbm_macros_device(plbm_grid_t* g, int ibuf, double* rho, double* ux, double* uy) {
  if (int r = check_grid(g)) return r;
  if (int r = check_buf(g, ibuf)) return r;
  if (int r = use_device(g)) return r;
  CUDA_TRY(macros(internal_storage(g->storage), 0, g->nx, g->ny, g->ld, lattice(g, ibuf), rho, ux, uy, g->stream,
                  exact_fields(g)),
           "moments kernel");
  return ok();
}

extern "C" int plbm_update_macros(plbm_grid_t* g, double* rho, double* ux, double* uy) {
  if (int r = check_grid(g)) return r;
  if (int r = use_device(g)) return r;
  {
    // page-locked host outputs (every one given): the kernel writes them in place
    void *mr = const_cast<void*>(mapped_host(rho)), *mu = const_cast<void*>(mapped_host(ux)),
         *mv = const_cast<void*>(mapped_host(uy));
    if ((rho || ux || uy) && (!rho || mr) && (!ux || mu) && (!uy || mv)) {
      CUDA_TRY(macros(internal_storage(g->storage), 0, g->nx, g->ny, g->ld, lattice(g, g->inew),
                      static_cast<double*>(mr), static_cast<double*>(mu), static_cast<double*>(mv), g->stream,
                      exact_fields(g)),
               "moments kernel");
      CUDA_TRY(cudaStreamSynchronize(g->stream), "update_macros sync");
      return ok();
    }
  }
  const size_t n = (size_t)g->nx * g->ny;
  if (int r = ensure_scratch(g, 3 * n)) return r;
  double* d = g->scratch;
  // src/fvm_bardow.F90:350-352 reads f(:,:,:,grid%inew)
  const int S = slab_count(g);
  if (S > 1) {
    if (int r = ensure_xfer(g)) return r;
    double* dst[3] = {rho, ux, uy};
    for (int s = 0; s < S; s++) {
      int x0, x1;
      slab_bounds(g, s, S, x0, x1);
      CUDA_TRY(macros_range(internal_storage(g->storage), 0, g->nx, g->ny, g->ld, lattice(g, g->inew), d, d + n,
                            d + 2 * n, x0, x1, g->stream, exact_fields(g)),
               "moments kernel");
      CUDA_TRY(cudaEventRecord(g->slab_ev[s], g->stream), "slab event");
      CUDA_TRY(cudaStreamWaitEvent(g->xfer, g->slab_ev[s], 0), "slab wait");
      const size_t off = (size_t)x0 * g->ny, cnt = (size_t)(x1 - x0) * g->ny;
      for (int k = 0; k < 3; k++)
        if (dst[k])
          CUDA_TRY(cudaMemcpyAsync(dst[k] + off, d + k * n + off, cnt * 8, cudaMemcpyDeviceToHost, g->xfer),
                   "download fields");
    }
    // the last slab's copies wait for every moments kernel before them
    CUDA_TRY(cudaStreamSynchronize(g->xfer), "update_macros sync");
    return ok();
  }
  CUDA_TRY(macros(internal_storage(g->storage), 0, g->nx, g->ny, g->ld, lattice(g, g->inew), d, d + n, d + 2 * n,
                  g->stream, exact_fields(g)),
           "moments kernel");
  if (rho) CUDA_TRY(cudaMemcpyAsync(rho, d, n * 8, cudaMemcpyDeviceToHost, g->stream), "download rho");
  if (ux) CUDA_TRY(cudaMemcpyAsync(ux, d + n, n * 8, cudaMemcpyDeviceToHost, g->stream), "download ux");
  if (uy) CUDA_TRY(cudaMemcpyAsync(uy, d + 2 * n, n * 8, cudaMemcpyDeviceToHost, g->stream), "download uy");
  CUDA_TRY(cudaStreamSynchronize(g->stream), "update_macros sync");
  return ok();
}

extern "C" int plbm_vorticity_device(int order, int nx, int ny, const double* ux, const double* uy, double* w,
                                     void* stream) {
  if (nx < 1 || ny < 1 || nx > PLBM_MAX_EXTENT || ny > PLBM_MAX_EXTENT)
    return fail(PLBM_E_INVALID, "grid size %dx%d", nx, ny);
  if (order != 2 && order != 4 && order != 44) return fail(PLBM_E_INVALID, "vorticity order %d (2, 4 or 44)", order);
  if (!ux || !uy || !w) return fail(PLBM_E_INVALID, "NULL field");
  CUDA_TRY(vorticity(order, nx, ny, ux, uy, w, static_cast<cudaStream_t>(stream)), "vorticity kernel");
  return ok();
}

extern "C" int plbm_vorticity(int order, int nx, int ny, const double* ux, const double* uy, double* w) {
  if (nx < 1 || ny < 1 || nx > PLBM_MAX_EXTENT || ny > PLBM_MAX_EXTENT)
    return fail(PLBM_E_INVALID, "grid size %dx%d", nx, ny);
  if (order != 2 && order != 4 && order != 44) return fail(PLBM_E_INVALID, "vorticity order %d (2, 4 or 44)", order);
  if (!ux || !uy || !w) return fail(PLBM_E_INVALID, "NULL field");
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev < 1) {
    cudaGetLastError();
    return fail(PLBM_E_NODEVICE, "no CUDA device visible");
  }
  const size_t n = (size_t)nx * ny;
  double* d = nullptr;
  CUDA_TRY(cudaMalloc(&d, 3 * n * sizeof(double)), "cudaMalloc(vorticity)");
  cudaError_t e = cudaMemcpy(d, ux, n * 8, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(d + n, uy, n * 8, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = vorticity(order, nx, ny, d, d + n, d + 2 * n, 0);
  if (e == cudaSuccess) e = cudaMemcpy(w, d + 2 * n, n * 8, cudaMemcpyDeviceToHost);
  cudaFree(d);
  if (e != cudaSuccess) return cuda_fail(e, "vorticity");
  return ok();
}

namespace {
int reduce(plbm_grid_t* g, int ibuf, const double* uxa, const double* uya, double out[3]) {
  const size_t n = (size_t)g->nx * g->ny;
  const int nb = reduce_blocks(g->nx, g->ny);
  if (int r = ensure_scratch(g, 3 * n + 3 * (size_t)nb)) return r;
  double* part = g->scratch + 3 * n;
  const double* dua = nullptr;
  const double* dva = nullptr;
  if (uxa) {
    CUDA_TRY(cudaMemcpyAsync(g->scratch, uxa, n * 8, cudaMemcpyHostToDevice, g->stream), "upload uxa");
    CUDA_TRY(cudaMemcpyAsync(g->scratch + n, uya, n * 8, cudaMemcpyHostToDevice, g->stream), "upload uya");
    dua = g->scratch;
    dva = g->scratch + n;
  }
  CUDA_TRY(energy_error_partials(internal_storage(g->storage), 0, g->nx, g->ny, g->ld, lattice(g, ibuf), dua, dva,
                                 part, g->stream),
           "reduction kernel");
  std::vector<double> h(3 * (size_t)nb);
  CUDA_TRY(cudaMemcpyAsync(h.data(), part, h.size() * 8, cudaMemcpyDeviceToHost, g->stream), "download partials");
  CUDA_TRY(cudaStreamSynchronize(g->stream), "reduction sync");
  out[0] = out[1] = out[2] = 0.0;
  for (int b = 0; b < nb; b++)
    for (int k = 0; k < 3; k++) out[k] += h[3 * (size_t)b + k];
  return PLBM_OK;
}
}  // namespace

extern "C" int plbm_kinetic_energy(plbm_grid_t* g, int ibuf, double* energy) {
  if (int r = check_grid(g)) return r;
  if (int r = check_buf(g, ibuf)) return r;
  if (!energy) return fail(PLBM_E_INVALID, "energy is NULL");
  if (int r = use_device(g)) return r;
  double s[3];
  if (int r = reduce(g, ibuf, nullptr, nullptr, s)) return r;
  *energy = s[0];
  return ok();
}

extern "C" int plbm_velocity_l2_error(plbm_grid_t* g, int ibuf, const double* uxa, const double* uya,
                                      double* err) {
  if (int r = check_grid(g)) return r;
  if (int r = check_buf(g, ibuf)) return r;
  if (!uxa || !uya || !err) return fail(PLBM_E_INVALID, "NULL argument");
  if (int r = use_device(g)) return r;
  double s[3];
  if (int r = reduce(g, ibuf, uxa, uya, s)) return r;
  if (!(s[2] > 0.0)) return fail(PLBM_E_INVALID, "reference field has zero norm");
  *err = sqrt(s[1] / s[2]);
  return ok();
}

extern "C" int plbm_synchronize(plbm_grid_t* g) {
  if (int r = check_grid(g)) return r;
  if (int r = use_device(g)) return r;
  CUDA_TRY(cudaStreamSynchronize(g->stream), "synchronize");
  return ok();
}

extern "C" int plbm_hybrid_range_flag(int* flag, int reset) {
  if (!flag) return fail(PLBM_E_INVALID, "flag is NULL");
  CUDA_TRY(cudaDeviceSynchronize(), "synchronize");
  CUDA_TRY(hybrid_range_flag(flag, reset), "read range flag");
  return ok();
}

extern "C" int plbm_launch_step(int storage, int math, int kind, int nx, int ny, int ld, const void* fsrc,
                                void* fdst, double omega, double trt_magic, void* stream) {
  if (nx < 1 || ny < 1 || ld < ny || nx > PLBM_MAX_EXTENT || ld > PLBM_MAX_EXTENT)
    return fail(PLBM_E_INVALID, "bad sizes nx=%d ny=%d ld=%d", nx, ny, ld);
  if (!fsrc || !fdst || fsrc == fdst) return fail(PLBM_E_INVALID, "fsrc and fdst must be distinct device lattices");
  if (kind < PLBM_BGK || kind > PLBM_BGKI) return fail(PLBM_E_INVALID, "unknown collision kind %d", kind);
  const CollParams p = plbm_make_params(omega, trt_magic);
  Sweep s{nx, ny, ld, fsrc, fdst, static_cast<cudaStream_t>(stream)};
  cudaError_t e;
  if (storage == PLBM_F64) {
    if (kind == PLBM_BGKI && ld != ny)
      return fail(PLBM_E_UNSUPPORTED, "fused collide_bgk_improved needs ld == ny");
    if (math == PLBM_MATH_HYBRID && kind == PLBM_BGKI)
      return fail(PLBM_E_UNSUPPORTED, "PLBM_MATH_HYBRID is not offered for collide_bgk_improved");
    if (math == PLBM_MATH_STRICT) e = strict::step_pull_f64(kind, s, p);
    else if (math == PLBM_MATH_HYBRID) e = step_pull_df64(kind, s, p);
    else e = fma::step_pull_f64(kind, s, p);
  } else if (storage == PLBM_F32DEV || storage == PLBM_F16DEV) {
    if (kind == PLBM_BGKI) return fail(PLBM_E_UNSUPPORTED, "collide_bgk_improved needs PLBM_F64 storage");
    e = step_pull_dev(storage, kind, s, p);
  } else {
    return fail(PLBM_E_INVALID, "unknown storage %d", storage);
  }
  if (e != cudaSuccess) return cuda_fail(e, "stream-collide kernel");
  return ok();
}
