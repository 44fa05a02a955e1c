// plugin.cpp -- the simulation-plugin C ABI (sim/lbm.h) on the GPU.
//
// Mirrors sim/sim_slbm.F90: a standard D2Q9 LBM with shifted populations
// (h = f - w), BGK collision and push streaming with periodic wrap.  The
// populations live on the device in the plugin's x-fastest convention
// f(nx,ny,0:8) without halo (ld = nx rounded up to 16); the periodic wrap is
// done by index arithmetic, so the halo and lbm_periodic_bc_push of the
// reference have no counterpart.  The results are those of the reference:
// the push kernel writes every (x,y,q) of the destination exactly once with
// the value the halo copy would bring there.
#include <cuda_runtime.h>
#include <math.h>
#include <string.h>
#include <string>

#include "../../include/plbm_gpu.h"
#include "../../include/plbm_plugin.h"
#include "plbm_launch.h"

using namespace plbm;

namespace plbm_internal {
int fail(int code, const char* fmt, ...);
int cuda_fail(cudaError_t e, const char* what);
}  // namespace plbm_internal
using plbm_internal::cuda_fail;
using plbm_internal::fail;
CollParams plbm_make_params(double omega, double trt_magic);

namespace {

struct PluginSim {
  int nx, ny, ld;
  int kind, storage, math;
  double trt_magic;
  int device;
  size_t elem_bytes, lat_elems;
  void* f[2];
  int cur;  // lattice holding the current state (the reference's f1)
  double* scratch;  // 3*nx*ny doubles
  cudaStream_t stream;
  int status;
  unsigned magic_tag;
  // captured loop of kGraphSteps steps from lattice graph_cur (small grids)
  cudaGraphExec_t graph;
  double graph_omega;
  int graph_cur;
};
constexpr unsigned kTag = 0x504c424du;  // "PLBM"

PluginSim* as_sim(void* p) {
  PluginSim* s = static_cast<PluginSim*>(p);
  if (!s || s->magic_tag != kTag) return nullptr;
  return s;
}

int st_code(int storage) { return storage == PLBM_F64 ? ST_F64SHIFT : storage; }

void destroy(PluginSim* s) {
  if (!s) return;
  cudaSetDevice(s->device);
  if (s->stream) cudaStreamSynchronize(s->stream);
  for (int i = 0; i < 2; i++)
    if (s->f[i]) cudaFree(s->f[i]);
  if (s->scratch) cudaFree(s->scratch);
  if (s->graph) cudaGraphExecDestroy(s->graph);
  if (s->stream) cudaStreamDestroy(s->stream);
  s->magic_tag = 0;
  delete s;
}

// One collide-and-push step from lattice `from` to the other.
cudaError_t push_step(const PluginSim* s, int from, const CollParams& p) {
  Sweep sw{s->nx, s->ny, s->ld, s->f[from], s->f[1 - from], s->stream};
  if (s->storage != PLBM_F64) return step_push_dev(s->storage, s->kind, sw, p);
  if (s->math == PLBM_MATH_STRICT) return strict::step_push_shift_f64(s->kind, sw, p);
  if (s->math == PLBM_MATH_HYBRID) return step_push_hybrid(s->kind, sw, p);
  return fma::step_push_shift_f64(s->kind, sw, p);
}

// Small grids replay a captured loop of kGraphSteps (even) steps instead of
// launching step by step: their steps are shorter than the host's launch.
constexpr int kGraphSteps = 16;
constexpr long long kGraphCells = 1ll << 17;

cudaError_t replay(PluginSim* s, double omega, const CollParams& p, int reps) {
  if (!s->graph || s->graph_omega != omega || s->graph_cur != s->cur) {
    if (s->graph) cudaGraphExecDestroy(s->graph);
    s->graph = nullptr;
    if (cudaStreamBeginCapture(s->stream, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
      cudaGetLastError();
      return cudaErrorNotSupported;  // the caller launches step by step
    }
    cudaError_t le = cudaSuccess;
    cudaError_t e;
    for (int i = 0; i < kGraphSteps && le == cudaSuccess; i++) le = push_step(s, (s->cur + i) & 1, p);
    cudaGraph_t graph = nullptr;
    e = cudaStreamEndCapture(s->stream, &graph);
    if (le != cudaSuccess || e != cudaSuccess) {
      if (graph) cudaGraphDestroy(graph);
      return le != cudaSuccess ? le : e;
    }
    e = cudaGraphInstantiate(&s->graph, graph, 0);
    cudaGraphDestroy(graph);
    if (e != cudaSuccess) {
      s->graph = nullptr;
      return e;
    }
    s->graph_omega = omega;
    s->graph_cur = s->cur;
  }
  for (int r = 0; r < reps; r++) {
    cudaError_t e = cudaGraphLaunch(s->graph, s->stream);
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}

int do_steps(PluginSim* s, double omega, int nsteps) {
  if (s->status) return s->status;
  if (cudaSetDevice(s->device) != cudaSuccess) return s->status = cuda_fail(cudaGetLastError(), "cudaSetDevice");
  const CollParams p = plbm_make_params(omega, s->trt_magic);
  if ((long long)s->nx * s->ny <= kGraphCells && nsteps >= 2 * kGraphSteps) {
    const int reps = nsteps / kGraphSteps;
    cudaError_t e = replay(s, omega, p, reps);
    if (e == cudaSuccess) nsteps -= reps * kGraphSteps;  // even: s->cur unchanged
    else if (e != cudaErrorNotSupported) return s->status = cuda_fail(e, "plugin step graph");
  }
  for (int i = 0; i < nsteps; i++) {
    cudaError_t e = push_step(s, s->cur, p);
    if (e != cudaSuccess) return s->status = cuda_fail(e, "plugin step kernel");
    s->cur = 1 - s->cur;  // move_alloc swap, sim/sim_slbm.F90:91-95
  }
  return PLBM_OK;
}

}  // namespace

extern "C" void* c_plbmgpu_init(int nx, int ny, double dt, const double* rho, const double* u,
                                const double* sigma, void* params) {
  if (nx < 1 || ny < 1 || nx > PLBM_MAX_EXTENT || ny > PLBM_MAX_EXTENT) {
    fail(PLBM_E_INVALID, "grid size %dx%d", nx, ny);
    return nullptr;
  }
  if (dt != 1.0) {  // sim/sim_slbm.F90:48-51
    fail(PLBM_E_INVALID, "Standard LBM only supports dt = 1.0 (got %g)", dt);
    return nullptr;
  }
  if (sigma) {  // sim/sim_slbm.F90:64-70
    fail(PLBM_E_UNSUPPORTED, "non-equilibrium initialisation (sigma) is not implemented");
    return nullptr;
  }
  if (!rho || !u) {
    fail(PLBM_E_INVALID, "rho and u must be non-NULL");
    return nullptr;
  }
  int kind = PLBM_BGK, storage = PLBM_F64, math = PLBM_MATH_FMA;
  double trt_magic = 0.25;
  if (params) {
    const plbm_plugin_params* pp = static_cast<const plbm_plugin_params*>(params);
    if (pp->version != 1 && pp->version != 2) {
      fail(PLBM_E_INVALID, "plbm_plugin_params.version = %d (expected 1 or 2)", pp->version);
      return nullptr;
    }
    kind = pp->kind;
    storage = pp->storage;
    trt_magic = pp->trt_magic;
    if (pp->version >= 2) math = pp->math;
  }
  if (kind != PLBM_BGK && kind != PLBM_TRT && kind != PLBM_RR) {
    fail(PLBM_E_INVALID, "plugin collision kind %d (BGK, TRT or RR)", kind);
    return nullptr;
  }
  if (storage != PLBM_F64 && storage != PLBM_F32DEV && storage != PLBM_F16DEV) {
    fail(PLBM_E_INVALID, "plugin storage %d", storage);
    return nullptr;
  }
  if (math != PLBM_MATH_FMA && math != PLBM_MATH_STRICT && math != PLBM_MATH_HYBRID) {
    fail(PLBM_E_INVALID, "plugin math %d (FMA, STRICT or HYBRID)", math);
    return nullptr;
  }
  if (math == PLBM_MATH_HYBRID && storage != PLBM_F64) {
    fail(PLBM_E_INVALID, "plugin math HYBRID needs PLBM_F64 storage");
    return nullptr;
  }
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev < 1) {
    cudaGetLastError();
    fail(PLBM_E_NODEVICE, "no CUDA device visible");
    return nullptr;
  }
  PluginSim* s = new PluginSim();
  memset(s, 0, sizeof *s);
  s->magic_tag = kTag;
  s->nx = nx;
  s->ny = ny;
  s->ld = (nx % 16) ? nx + (16 - nx % 16) : nx;
  s->kind = kind;
  s->storage = storage;
  s->math = math;
  s->trt_magic = trt_magic;
  cudaGetDevice(&s->device);
  s->elem_bytes = storage == PLBM_F64 ? 8 : (storage == PLBM_F32DEV ? 4 : 2);
  s->lat_elems = (size_t)s->ld * ny * 9;
  const size_t n = (size_t)nx * ny;
  cudaError_t e = cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking);
  for (int i = 0; i < 2 && e == cudaSuccess; i++) e = cudaMalloc(&s->f[i], s->lat_elems * s->elem_bytes);
  if (e == cudaSuccess) e = cudaMalloc(&s->scratch, 3 * n * sizeof(double));
  if (e == cudaSuccess) e = cudaMemsetAsync(s->f[0], 0, s->lat_elems * s->elem_bytes, s->stream);
  // rho slot carries the pressure, u is (nx,ny,2): ux block then uy block
  if (e == cudaSuccess) e = cudaMemcpyAsync(s->scratch, rho, n * 8, cudaMemcpyHostToDevice, s->stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(s->scratch + n, u, 2 * n * 8, cudaMemcpyHostToDevice, s->stream);
  // lbm_eqinit_fields, sim/sim.F90:181-199
  if (e == cudaSuccess)
    e = equilibrium(st_code(storage), 1, nx, ny, s->ld, s->scratch, s->scratch + n, s->scratch + 2 * n, 1, s->f[0],
                    s->stream, math == PLBM_MATH_HYBRID);
  // this%grid%f2 = this%grid%f1, sim/sim_slbm.F90:76
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(s->f[1], s->f[0], s->lat_elems * s->elem_bytes, cudaMemcpyDeviceToDevice, s->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
  if (e != cudaSuccess) {
    cuda_fail(e, "plugin init");
    destroy(s);
    return nullptr;
  }
  s->cur = 0;
  return s;
}

extern "C" void c_plbmgpu_step(void* p, double omega) {
  PluginSim* s = as_sim(p);
  if (!s) {
    fail(PLBM_E_INVALID, "invalid plugin handle");
    return;
  }
  do_steps(s, omega, 1);
}

extern "C" int c_plbmgpu_steps(void* p, double omega, int nsteps) {
  PluginSim* s = as_sim(p);
  if (!s) return fail(PLBM_E_INVALID, "invalid plugin handle");
  if (nsteps < 0) return fail(PLBM_E_INVALID, "nsteps = %d < 0", nsteps);
  return do_steps(s, omega, nsteps);
}

extern "C" void c_plbmgpu_vars(void* p, double* rho, double* u) {
  PluginSim* s = as_sim(p);
  if (!s) {
    fail(PLBM_E_INVALID, "invalid plugin handle");
    return;
  }
  if (s->status) return;
  if (!rho || !u) {
    s->status = fail(PLBM_E_INVALID, "rho and u must be non-NULL");
    return;
  }
  const size_t n = (size_t)s->nx * s->ny;
  cudaError_t e = cudaSetDevice(s->device);
  // lbm_macros of the current state, sim/sim_slbm.F90:112-127
  if (e == cudaSuccess)
    e = macros(st_code(s->storage), 1, s->nx, s->ny, s->ld, s->f[s->cur], s->scratch, s->scratch + n,
               s->scratch + 2 * n, s->stream, s->math == PLBM_MATH_HYBRID);
  if (e == cudaSuccess) e = cudaMemcpyAsync(rho, s->scratch, n * 8, cudaMemcpyDeviceToHost, s->stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(u, s->scratch + n, 2 * n * 8, cudaMemcpyDeviceToHost, s->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
  if (e != cudaSuccess) s->status = cuda_fail(e, "plugin vars");
}

extern "C" void c_plbmgpu_free(void* p) {
  PluginSim* s = as_sim(p);
  if (s) destroy(s);
}

extern "C" int c_plbmgpu_synchronize(void* p) {
  PluginSim* s = as_sim(p);
  if (!s) return fail(PLBM_E_INVALID, "invalid plugin handle");
  if (s->status) return s->status;
  cudaError_t e = cudaSetDevice(s->device);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
  if (e != cudaSuccess) s->status = cuda_fail(e, "plugin synchronize");
  return s->status;
}

extern "C" int c_plbmgpu_status(void* p) {
  PluginSim* s = as_sim(p);
  if (!s) return fail(PLBM_E_INVALID, "invalid plugin handle");
  return s->status;
}

extern "C" double c_plbmgpu_norm(int nx, int ny, const double* u, const double* ua) {
  // norm2(u - ua) / norm2(ua), sim/sim_slbm.F90:198-205
  if (nx < 1 || ny < 1 || !u || !ua) return NAN;
  double a = 0.0, b = 0.0;
  const size_t n = (size_t)nx * ny;
  for (size_t i = 0; i < n; i++) {
    const double d = u[i] - ua[i];
    a += d * d;
    b += ua[i] * ua[i];
  }
  return sqrt(a) / sqrt(b);
}
