// batch.cpp -- plbm_batch_* C ABI: many periodic grids of uneven sizes and
// relaxation times stepped together (see batched.cu for the kernels).
#include <cuda_runtime.h>
#include <string.h>
#include <algorithm>
#include <vector>

#include "../../include/plbm_gpu.h"
#include "plbm_batched.h"
#include "plbm_launch.h"

namespace plbm_internal {
int fail(int code, const char* fmt, ...);
int cuda_fail(cudaError_t e, const char* what);
}  // namespace plbm_internal
using plbm_internal::cuda_fail;
using plbm_internal::fail;
using namespace plbm;
CollParams plbm_make_params(double omega, double trt_magic);

#define CUDA_TRY(expr, what)                            \
  do {                                                  \
    cudaError_t e_ = (expr);                            \
    if (e_ != cudaSuccess) return cuda_fail(e_, what);  \
  } while (0)

struct plbm_batch {
  int ngrids = 0, storage = 0, device = 0, sms = 0, math = PLBM_MATH_FMA;
  std::vector<BatchGrid> grids;   // host copy (off, sizes, params, ty)
  BatchGrid* d_grids = nullptr;
  int2* d_tile_xy = nullptr;    // first cell of each tile (capacity tile_cap)
  int* d_tile_grid = nullptr;   // grid index of each tile (capacity tile_cap)
  size_t tile_cap = 0;
  int small_index = 1;          // every lattice pair has < 2^32 elements
  int ntiles = 0, nt_bgk = 0;
  long long cells = 0;
  size_t elems = 0, elem_bytes = 8;
  void* base = nullptr;
  void* ctrl = nullptr;
  double* scratch = nullptr;
  size_t scratch_elems = 0;
  cudaStream_t own = nullptr, stream = nullptr;
  plbm_batch_schedule sched{};
  int ctas = 0;
  long long steps_done = 0;
  int stall_next = 0;           // next persistent run: unreachable barrier
  cudaGraphExec_t graph[2] = {nullptr, nullptr};
  int graph_steps[2] = {0, 0};
};

namespace {

int pad16(int n) { return n % 16 ? n + (16 - n % 16) : n; }

int bucket_of(int ny) {
  return ny <= 48 ? 0 : ny <= 96 ? 1 : ny <= 192 ? 2 : ny <= 384 ? 3 : 4;
}

int check_schedule(const plbm_batch_schedule& s) {
  if (s.threads < 64 || s.threads > kBatchMaxThreads || (s.threads & 31))
    return fail(PLBM_E_INVALID, "schedule.threads = %d: need a multiple of 32 in [64, %d]", s.threads,
                kBatchMaxThreads);
  if (s.ctas_per_sm < 0 || s.ctas_per_sm > 32) return fail(PLBM_E_INVALID, "schedule.ctas_per_sm = %d", s.ctas_per_sm);
  for (int i = 0; i < PLBM_BATCH_BUCKETS; i++) {
    const int ty = s.ty[i];
    if (ty < 32 || ty > s.threads || (ty & (ty - 1)) || s.threads % ty)
      return fail(PLBM_E_INVALID, "schedule.ty[%d] = %d: need a power of two >= 32 dividing threads=%d", i, ty,
                  s.threads);
  }
  return PLBM_OK;
}

void drop_graphs(plbm_batch_t* b) {
  for (int i = 0; i < 2; i++) {
    if (b->graph[i]) cudaGraphExecDestroy(b->graph[i]);
    b->graph[i] = nullptr;
    b->graph_steps[i] = 0;
  }
}

// Tiles are numbered grid by grid, the BGK grids' first and the TRT grids'
// after them, so that the per-step launch can run each kind with its own
// kernel over a contiguous range; each tile records its grid and first cell.
int apply_schedule(plbm_batch_t* b) {
  std::vector<int> owner;
  std::vector<int2> xy;
  b->nt_bgk = 0;
  for (int pass = 0; pass < 2; pass++) {
    for (int i = 0; i < b->ngrids; i++) {
      BatchGrid& g = b->grids[i];
      if ((g.kind == PLBM_BGK) != (pass == 0)) continue;
      g.ty = b->sched.ty[bucket_of(g.ny)];
      g.lty = 0;
      while ((1 << g.lty) < g.ty) g.lty++;
      const int tx = b->sched.threads / g.ty;
      const int tiles_y = (g.ny + g.ty - 1) / g.ty, tiles_x = (g.nx + tx - 1) / tx;
      if ((long long)owner.size() + (long long)tiles_x * tiles_y > 0x7fffffffLL)
        return fail(PLBM_E_INVALID, "too many tiles");
      for (int a = 0; a < tiles_x; a++)
        for (int c = 0; c < tiles_y; c++) {
          owner.push_back(i);
          xy.push_back(make_int2(a * tx, c * g.ty));
        }
    }
    if (pass == 0) b->nt_bgk = (int)owner.size();
  }
  b->ntiles = (int)owner.size();
  if ((size_t)b->ntiles > b->tile_cap) {
    cudaFree(b->d_tile_grid);
    cudaFree(b->d_tile_xy);
    b->d_tile_grid = nullptr;
    b->d_tile_xy = nullptr;
    b->tile_cap = 0;
    CUDA_TRY(cudaMalloc(&b->d_tile_grid, sizeof(int) * (size_t)b->ntiles), "cudaMalloc(tile table)");
    CUDA_TRY(cudaMalloc(&b->d_tile_xy, sizeof(int2) * (size_t)b->ntiles), "cudaMalloc(tile table)");
    b->tile_cap = (size_t)b->ntiles;
  }
  CUDA_TRY(cudaMemcpy(b->d_grids, b->grids.data(), sizeof(BatchGrid) * b->ngrids, cudaMemcpyHostToDevice),
           "upload batch table");
  CUDA_TRY(cudaMemcpy(b->d_tile_xy, xy.data(), sizeof(int2) * xy.size(), cudaMemcpyHostToDevice),
           "upload tile table");
  CUDA_TRY(cudaMemcpy(b->d_tile_grid, owner.data(), sizeof(int) * owner.size(), cudaMemcpyHostToDevice),
           "upload tile owners");
  int per_sm = 0;
  CUDA_TRY(batch_max_ctas(b->storage, b->sched.threads, b->small_index, &per_sm), "occupancy");
  if (per_sm < 1) return fail(PLBM_E_UNSUPPORTED, "batched kernel does not fit on an SM with %d threads", b->sched.threads);
  const int want = b->sched.ctas_per_sm > 0 ? std::min(b->sched.ctas_per_sm, per_sm) : per_sm;
  b->ctas = std::max(1, std::min(b->ntiles, want * b->sms));
  drop_graphs(b);
  return PLBM_OK;
}

BatchLaunch launch_of(const plbm_batch_t* b) {
  BatchLaunch L;
  L.grids = b->d_grids;
  L.tile_xy = b->d_tile_xy;
  L.tile_grid = b->d_tile_grid;
  L.nt_bgk = b->nt_bgk;
  L.hybrid = b->math == PLBM_MATH_HYBRID;
  L.small_index = b->small_index;
  L.ngrids = b->ngrids;
  L.ntiles = b->ntiles;
  L.threads = b->sched.threads;
  L.ctas = b->ctas;
  L.persistent = b->sched.persistent;
  L.base = b->base;
  L.ctrl = b->ctrl;
  L.stream = b->stream;
  return L;
}

// Queue nsteps (control-block reset + launches) on the batch stream.
cudaError_t enqueue(plbm_batch_t* b, int nsteps) {
  if (b->sched.persistent) {
    cudaError_t e = cudaMemsetAsync(b->ctrl, 0, batch_ctrl_bytes(), b->stream);
    if (e == cudaSuccess && b->stall_next) e = batch_arm_stall(b->ctrl, b->stream);
    b->stall_next = 0;
    if (e != cudaSuccess) return e;
  }
  return batch_run(b->storage, launch_of(b), nsteps, (int)(b->steps_done & 1));
}

void* lattice_of(const plbm_batch_t* b, int gi, int which) {
  const BatchGrid& g = b->grids[gi];
  const size_t lat = (size_t)g.ld * g.nx * 9;
  return static_cast<char*>(b->base) + ((size_t)g.off + (which ? lat : 0)) * b->elem_bytes;
}

int current(const plbm_batch_t* b) { return (int)(b->steps_done & 1); }

int ensure_scratch(plbm_batch_t* b, size_t n) {
  if (b->scratch_elems >= n) return PLBM_OK;
  if (b->scratch) cudaFree(b->scratch);
  b->scratch = nullptr;
  b->scratch_elems = 0;
  CUDA_TRY(cudaMalloc(&b->scratch, n * sizeof(double)), "cudaMalloc(batch scratch)");
  b->scratch_elems = n;
  return PLBM_OK;
}

}  // namespace

extern "C" int plbm_batch_default_schedule(plbm_batch_schedule* s) {
  if (!s) return fail(PLBM_E_INVALID, "NULL schedule");
  s->threads = 256;
  s->ctas_per_sm = 0;
  s->persistent = 1;
  const int ty[PLBM_BATCH_BUCKETS] = {32, 64, 128, 256, 256};
  for (int i = 0; i < PLBM_BATCH_BUCKETS; i++) s->ty[i] = ty[i];
  return PLBM_OK;
}

extern "C" int plbm_batch_create(int ngrids, const int* nx, const int* ny, const int* kind, const double* omega,
                                 const double* trt_magic, int storage, plbm_batch_t** out) {
  if (!out) return fail(PLBM_E_INVALID, "out is NULL");
  *out = nullptr;
  if (ngrids < 1 || !nx || !ny || !kind || !omega) return fail(PLBM_E_INVALID, "bad batch description");
  if (storage != PLBM_F64 && storage != PLBM_F32DEV)
    return fail(PLBM_E_UNSUPPORTED, "batched storage %d (PLBM_F64 or PLBM_F32DEV)", storage);
  for (int i = 0; i < ngrids; i++)
    if (nx[i] < 1 || ny[i] < 1 || nx[i] > PLBM_MAX_EXTENT || ny[i] > PLBM_MAX_EXTENT ||
        (kind[i] != PLBM_BGK && kind[i] != PLBM_TRT) || !(omega[i] > 0 && omega[i] < 2))
      return fail(PLBM_E_INVALID, "grid %d: nx=%d ny=%d kind=%d omega=%g (BGK or TRT, 0<omega<2)", i, nx[i], ny[i],
                  kind[i], omega[i]);
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev < 1) {
    cudaGetLastError();
    return fail(PLBM_E_NODEVICE, "no CUDA device visible");
  }
  plbm_batch_t* b = new plbm_batch_t();
  b->ngrids = ngrids;
  b->storage = storage;
  b->elem_bytes = storage == PLBM_F64 ? 8 : 4;
  cudaGetDevice(&b->device);
  cudaDeviceGetAttribute(&b->sms, cudaDevAttrMultiProcessorCount, b->device);
  b->grids.resize(ngrids);
  size_t off = 0;
  for (int i = 0; i < ngrids; i++) {
    BatchGrid& g = b->grids[i];
    memset(&g, 0, sizeof g);
    g.nx = nx[i];
    g.ny = ny[i];
    g.ld = pad16(ny[i]);
    g.kind = kind[i];
    g.p = plbm_make_params(omega[i], trt_magic ? trt_magic[i] : 0.25);
    g.hp = hybrid_bgk_params(omega[i]);
    g.ht = hybrid_trt_params(g.p);
    g.off = (long long)off;
    off += 2 * (size_t)g.ld * g.nx * 9;
    if (2 * (unsigned long long)g.ld * g.nx * 9 >= (1ull << 32)) b->small_index = 0;
    b->cells += (long long)g.nx * g.ny;
  }
  b->elems = off;
  cudaError_t e = cudaMalloc(&b->base, off * b->elem_bytes);
  if (e == cudaSuccess) e = cudaMemset(b->base, 0, off * b->elem_bytes);
  if (e == cudaSuccess) e = cudaMalloc(&b->d_grids, sizeof(BatchGrid) * ngrids);
  if (e == cudaSuccess) e = cudaMalloc(&b->ctrl, batch_ctrl_bytes());
  if (e == cudaSuccess) e = cudaMemset(b->ctrl, 0, batch_ctrl_bytes());
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&b->own, cudaStreamNonBlocking);
  if (e != cudaSuccess) {
    plbm_batch_destroy(b);
    return cuda_fail(e, "batch allocation");
  }
  b->stream = b->own;
  plbm_batch_default_schedule(&b->sched);
  if (int r = apply_schedule(b)) {
    plbm_batch_destroy(b);
    return r;
  }
  *out = b;
  return PLBM_OK;
}

extern "C" int plbm_batch_destroy(plbm_batch_t* b) {
  if (!b) return PLBM_OK;
  cudaSetDevice(b->device);
  if (b->stream) cudaStreamSynchronize(b->stream);
  drop_graphs(b);
  cudaFree(b->base);
  cudaFree(b->d_grids);
  cudaFree(b->d_tile_xy);
  cudaFree(b->d_tile_grid);
  cudaFree(b->ctrl);
  cudaFree(b->scratch);
  if (b->own) cudaStreamDestroy(b->own);
  delete b;
  return PLBM_OK;
}

extern "C" int plbm_batch_info(const plbm_batch_t* b, int* ngrids, long long* cells, int* ntiles, int* ctas) {
  if (!b) return fail(PLBM_E_INVALID, "NULL batch");
  if (ngrids) *ngrids = b->ngrids;
  if (cells) *cells = b->cells;
  if (ntiles) *ntiles = b->ntiles;
  if (ctas) *ctas = b->ctas;
  return PLBM_OK;
}

extern "C" int plbm_batch_set_schedule(plbm_batch_t* b, const plbm_batch_schedule* s) {
  if (!b || !s) return fail(PLBM_E_INVALID, "NULL argument");
  if (int r = check_schedule(*s)) return r;
  CUDA_TRY(cudaSetDevice(b->device), "cudaSetDevice");
  CUDA_TRY(cudaStreamSynchronize(b->stream), "synchronize");
  b->sched = *s;
  return apply_schedule(b);
}

extern "C" int plbm_batch_get_schedule(const plbm_batch_t* b, plbm_batch_schedule* s) {
  if (!b || !s) return fail(PLBM_E_INVALID, "NULL argument");
  *s = b->sched;
  return PLBM_OK;
}

extern "C" int plbm_batch_set_stream(plbm_batch_t* b, void* stream) {
  if (!b) return fail(PLBM_E_INVALID, "NULL batch");
  b->stream = stream ? static_cast<cudaStream_t>(stream) : b->own;
  drop_graphs(b);
  return PLBM_OK;
}

extern "C" int plbm_batch_set_math(plbm_batch_t* b, int math) {
  if (!b) return fail(PLBM_E_INVALID, "NULL batch");
  if (math != PLBM_MATH_FMA && math != PLBM_MATH_HYBRID)
    return fail(PLBM_E_UNSUPPORTED, "batched math %d (PLBM_MATH_FMA or PLBM_MATH_HYBRID)", math);
  if (math == PLBM_MATH_HYBRID && b->storage != PLBM_F64)
    return fail(PLBM_E_UNSUPPORTED, "PLBM_MATH_HYBRID needs PLBM_F64 storage");
  CUDA_TRY(cudaSetDevice(b->device), "cudaSetDevice");
  CUDA_TRY(cudaStreamSynchronize(b->stream), "synchronize");
  for (BatchGrid& g : b->grids) g.hybrid = math == PLBM_MATH_HYBRID ? 1 : 0;
  b->math = math;
  return apply_schedule(b);
}

extern "C" int plbm_batch_set_equilibrium(plbm_batch_t* b, int grid, const double* rho, const double* ux,
                                          const double* uy) {
  if (!b) return fail(PLBM_E_INVALID, "NULL batch");
  if (grid < 0 || grid >= b->ngrids) return fail(PLBM_E_INVALID, "grid index %d outside 0..%d", grid, b->ngrids - 1);
  if (!rho || !ux || !uy) return fail(PLBM_E_INVALID, "NULL field");
  CUDA_TRY(cudaSetDevice(b->device), "cudaSetDevice");
  const BatchGrid& g = b->grids[grid];
  const size_t n = (size_t)g.nx * g.ny;
  if (int r = ensure_scratch(b, 3 * n)) return r;
  double* d = b->scratch;
  CUDA_TRY(cudaMemcpyAsync(d, rho, n * 8, cudaMemcpyHostToDevice, b->stream), "upload rho");
  CUDA_TRY(cudaMemcpyAsync(d + n, ux, n * 8, cudaMemcpyHostToDevice, b->stream), "upload ux");
  CUDA_TRY(cudaMemcpyAsync(d + 2 * n, uy, n * 8, cudaMemcpyHostToDevice, b->stream), "upload uy");
  const int st = b->storage == PLBM_F64 ? ST_F64 : ST_F32DEV;
  CUDA_TRY(equilibrium(st, 0, g.nx, g.ny, g.ld, d, d + n, d + 2 * n, 0, lattice_of(b, grid, current(b)), b->stream,
                       b->math == PLBM_MATH_HYBRID),
           "equilibrium kernel");
  CUDA_TRY(cudaStreamSynchronize(b->stream), "equilibrium sync");
  return PLBM_OK;
}

extern "C" int plbm_batch_run(plbm_batch_t* b, int nsteps) {
  if (!b) return fail(PLBM_E_INVALID, "NULL batch");
  if (nsteps < 0) return fail(PLBM_E_INVALID, "nsteps = %d < 0", nsteps);
  CUDA_TRY(cudaSetDevice(b->device), "cudaSetDevice");
  CUDA_TRY(enqueue(b, nsteps), "batched step launch");
  b->steps_done += nsteps;
  return PLBM_OK;
}

extern "C" int plbm_batch_capture(plbm_batch_t* b, int nsteps) {
  if (!b) return fail(PLBM_E_INVALID, "NULL batch");
  if (nsteps < 1) return fail(PLBM_E_INVALID, "nsteps = %d < 1", nsteps);
  CUDA_TRY(cudaSetDevice(b->device), "cudaSetDevice");
  const int par = current(b);
  if (b->graph[par]) {
    cudaGraphExecDestroy(b->graph[par]);
    b->graph[par] = nullptr;
  }
  cudaStream_t cap = nullptr;
  CUDA_TRY(cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking), "capture stream");
  cudaStream_t keep = b->stream;
  b->stream = cap;
  cudaGraph_t graph = nullptr;
  cudaError_t e = cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal);
  if (e == cudaSuccess) {
    cudaError_t el = enqueue(b, nsteps);
    e = cudaStreamEndCapture(cap, &graph);
    if (el != cudaSuccess) e = el;
  }
  b->stream = keep;
  cudaStreamDestroy(cap);
  if (e == cudaSuccess) e = cudaGraphInstantiate(&b->graph[par], graph, 0);
  if (graph) cudaGraphDestroy(graph);
  if (e != cudaSuccess) {
    b->graph[par] = nullptr;
    return cuda_fail(e, "graph capture of the batched step");
  }
  b->graph_steps[par] = nsteps;
  return PLBM_OK;
}

extern "C" int plbm_batch_launch_graph(plbm_batch_t* b) {
  if (!b) return fail(PLBM_E_INVALID, "NULL batch");
  const int par = current(b);
  if (!b->graph[par])
    return fail(PLBM_E_INVALID, "no graph captured for the current step parity (call plbm_batch_capture)");
  CUDA_TRY(cudaSetDevice(b->device), "cudaSetDevice");
  CUDA_TRY(cudaGraphLaunch(b->graph[par], b->stream), "cudaGraphLaunch");
  b->steps_done += b->graph_steps[par];
  return PLBM_OK;
}

extern "C" int plbm_batch_inject_stall(plbm_batch_t* b) {
  if (!b) return fail(PLBM_E_INVALID, "NULL batch");
  if (!b->sched.persistent) return fail(PLBM_E_INVALID, "stall injection needs the persistent schedule");
  b->stall_next = 1;
  return PLBM_OK;
}

extern "C" int plbm_batch_synchronize(plbm_batch_t* b) {
  if (!b) return fail(PLBM_E_INVALID, "NULL batch");
  CUDA_TRY(cudaSetDevice(b->device), "cudaSetDevice");
  CUDA_TRY(cudaStreamSynchronize(b->stream), "synchronize");
  if (b->sched.persistent) {
    int err = 0, where = 0;
    CUDA_TRY(batch_read_ctrl(b->ctrl, &err, &where, b->stream), "read control block");
    if (err) return fail(PLBM_E_TIMEOUT, "batched persistent kernel: grid barrier wait expired at step %d", where);
  }
  return PLBM_OK;
}

extern "C" int plbm_batch_steps(const plbm_batch_t* b, long long* steps) {
  if (!b || !steps) return fail(PLBM_E_INVALID, "NULL argument");
  *steps = b->steps_done;
  return PLBM_OK;
}

extern "C" int plbm_batch_macros(plbm_batch_t* b, int grid, double* rho, double* ux, double* uy) {
  if (!b) return fail(PLBM_E_INVALID, "NULL batch");
  if (grid < 0 || grid >= b->ngrids) return fail(PLBM_E_INVALID, "grid index %d outside 0..%d", grid, b->ngrids - 1);
  if (int r = plbm_batch_synchronize(b)) return r;
  const BatchGrid& g = b->grids[grid];
  const size_t n = (size_t)g.nx * g.ny;
  if (int r = ensure_scratch(b, 3 * n)) return r;
  double* d = b->scratch;
  const int st = b->storage == PLBM_F64 ? ST_F64 : ST_F32DEV;
  CUDA_TRY(macros(st, 0, g.nx, g.ny, g.ld, lattice_of(b, grid, current(b)), d, d + n, d + 2 * n, b->stream,
                  b->math == PLBM_MATH_HYBRID),
           "moments kernel");
  if (rho) CUDA_TRY(cudaMemcpyAsync(rho, d, n * 8, cudaMemcpyDeviceToHost, b->stream), "download rho");
  if (ux) CUDA_TRY(cudaMemcpyAsync(ux, d + n, n * 8, cudaMemcpyDeviceToHost, b->stream), "download ux");
  if (uy) CUDA_TRY(cudaMemcpyAsync(uy, d + 2 * n, n * 8, cudaMemcpyDeviceToHost, b->stream), "download uy");
  CUDA_TRY(cudaStreamSynchronize(b->stream), "macros sync");
  return PLBM_OK;
}

extern "C" int plbm_batch_download(plbm_batch_t* b, int grid, double* f) {
  if (!b || !f) return fail(PLBM_E_INVALID, "NULL argument");
  if (grid < 0 || grid >= b->ngrids) return fail(PLBM_E_INVALID, "grid index %d outside 0..%d", grid, b->ngrids - 1);
  if (int r = plbm_batch_synchronize(b)) return r;
  const BatchGrid& g = b->grids[grid];
  const size_t lat = (size_t)g.ld * g.nx * 9;
  if (b->storage == PLBM_F64) {
    CUDA_TRY(cudaMemcpyAsync(f, lattice_of(b, grid, current(b)), lat * 8, cudaMemcpyDeviceToHost, b->stream),
             "download lattice");
  } else {
    if (int r = ensure_scratch(b, lat)) return r;
    CUDA_TRY(cudaMemsetAsync(b->scratch, 0, lat * 8, b->stream), "clear staging");
    CUDA_TRY(dev_to_f64(ST_F32DEV, g.nx, g.ny, g.ld, lattice_of(b, grid, current(b)), b->scratch, b->stream),
             "convert lattice");
    CUDA_TRY(cudaMemcpyAsync(f, b->scratch, lat * 8, cudaMemcpyDeviceToHost, b->stream), "download lattice");
  }
  CUDA_TRY(cudaStreamSynchronize(b->stream), "download sync");
  return PLBM_OK;
}
