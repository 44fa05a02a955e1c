// adjoint.cpp -- plbm_adjoint_* C ABI: forward run with checkpoints and the
// reverse sweep with recomputation (sqrt(T) memory), see adjoint.cu.
//
// Checkpoints hold f_n for n = 0, K, 2K, ... (K = checkpoint_every).  The
// reverse sweep walks the segments [kK, min(kK+K, T)) from the last: the
// segment's states are recomputed from checkpoint k into a K-lattice buffer,
// then the reverse steps n = end-1 .. kK run.  Two segment buffers alternate:
// while the reverse steps of segment k run on the caller's stream, the
// recomputation of segment k-1 runs on a second stream into the other buffer
// (events order each recomputation after the reverse sweep that last read
// its buffer, and each reverse sweep after its recomputation).  The two
// kernels' streams share the SMs and HBM: neither fills the GPU alone at
// 1024^2 (tails of 4096-CTA launches, load latency).  Device memory:
// (ceil(T/K) + 2K + 4) lattices with more than one segment; when the second
// buffer does not fit, one buffer and each recomputation after the previous
// sweep (ceil(T/K) + K + 4).  Each forward
// step is computed twice in all (forward pass + recomputation).
#include <cuda_runtime.h>
#include <stdlib.h>
#include <string.h>
#include <vector>

#include "../../include/plbm_gpu.h"
#include "plbm_adjoint.h"
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

struct plbm_adjoint {
  int nx, ny, ld, storage, nsteps, K, nck, device;
  size_t lat_bytes;
  char* ck = nullptr;    // nck lattices
  char* seg = nullptr;   // nseg x K lattices (nseg = 2 with more than one segment, 1 if 2 do not fit)
  char* work = nullptr;  // 2 lattices
  char* lam = nullptr;   // 2 lattices
  double* u0 = nullptr;  // 2*nx*ny
  double* dom = nullptr; // adjoint_blocks slots
  int nblocks = 0;
  double omega = 1.0;
  const void* fT = nullptr;
  int have_forward = 0;
  int nseg = 1;
  int math = PLBM_MATH_FMA;  // reverse-step arithmetic (plbm_adjoint_set_math)
  cudaStream_t own = nullptr, stream = nullptr;
  cudaStream_t side = nullptr;          // recomputation stream
  cudaEvent_t ev_fork = nullptr, ev_join = nullptr, ev_rec[2] = {nullptr, nullptr}, ev_rev[2] = {nullptr, nullptr};
};

namespace {

int pad16(int n) { return n % 16 ? n + (16 - n % 16) : n; }

void* lat(char* base, const plbm_adjoint_t* a, int i) { return base + (size_t)i * a->lat_bytes; }

cudaError_t fwd_step(const plbm_adjoint_t* a, const void* src, void* dst, const CollParams& p,
                     cudaStream_t stream) {
  Sweep s{a->nx, a->ny, a->ld, src, dst, stream};
  if (a->storage == PLBM_F64) return fma::step_pull_f64(K_BGK, s, p);
  return step_pull_dev(ST_F32DEV, K_BGK, s, p);
}

AdjLaunch base_launch(const plbm_adjoint_t* a) {
  AdjLaunch L;
  memset(&L, 0, sizeof L);
  L.nx = a->nx;
  L.ny = a->ny;
  L.ld = a->ld;
  L.omega = a->omega;
  L.comp = a->storage == PLBM_F32DEV && a->math == PLBM_MATH_HYBRID;
  L.stream = a->stream;
  return L;
}

int st(const plbm_adjoint_t* a) { return a->storage == PLBM_F64 ? ST_F64 : ST_F32DEV; }

}  // namespace

extern "C" int plbm_adjoint_create(int nx, int ny, int storage, int nsteps, int checkpoint_every,
                                   plbm_adjoint_t** out) {
  if (!out) return fail(PLBM_E_INVALID, "out is NULL");
  *out = nullptr;
  if (nx < 1 || ny < 1 || nx > PLBM_MAX_EXTENT || ny > PLBM_MAX_EXTENT || nsteps < 1 || checkpoint_every < 1)
    return fail(PLBM_E_INVALID, "bad adjoint sizes nx=%d ny=%d nsteps=%d checkpoint_every=%d", nx, ny, nsteps,
                checkpoint_every);
  if (storage != PLBM_F64 && storage != PLBM_F32DEV)
    return fail(PLBM_E_UNSUPPORTED, "adjoint storage %d (PLBM_F64 or PLBM_F32DEV)", storage);
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev < 1) {
    cudaGetLastError();
    return fail(PLBM_E_NODEVICE, "no CUDA device visible");
  }
  plbm_adjoint_t* a = new plbm_adjoint_t();
  a->nx = nx;
  a->ny = ny;
  a->ld = pad16(ny);
  a->storage = storage;
  a->nsteps = nsteps;
  a->K = checkpoint_every < nsteps ? checkpoint_every : nsteps;
  a->nck = (nsteps + a->K - 1) / a->K;
  cudaGetDevice(&a->device);
  a->lat_bytes = (size_t)a->ld * nx * 9 * (storage == PLBM_F64 ? 8 : 4);
  a->nblocks = adjoint_blocks(nx, ny);
  // PLBM_ADJOINT_ONE_SEGMENT=1 takes the one-buffer schedule (the fallback
  // below) for tests
  const char* one = getenv("PLBM_ADJOINT_ONE_SEGMENT");
  a->nseg = (a->nck > 1 && !(one && one[0] == '1')) ? 2 : 1;
  cudaError_t e = cudaMalloc(&a->ck, a->lat_bytes * a->nck);
  if (e == cudaSuccess) {
    e = cudaMalloc(&a->seg, a->lat_bytes * a->K * a->nseg);
    if (e == cudaErrorMemoryAllocation && a->nseg == 2) {  // one buffer: recomputation after each sweep
      cudaGetLastError();
      a->nseg = 1;
      e = cudaMalloc(&a->seg, a->lat_bytes * a->K);
    }
  }
  if (e == cudaSuccess) e = cudaMalloc(&a->work, a->lat_bytes * 2);
  if (e == cudaSuccess) e = cudaMalloc(&a->lam, a->lat_bytes * 2);
  if (e == cudaSuccess) e = cudaMalloc(&a->u0, sizeof(double) * 2 * (size_t)nx * ny);
  if (e == cudaSuccess) e = cudaMalloc(&a->dom, sizeof(double) * a->nblocks);
  // padding rows are never written by the kernels: give them a defined value
  if (e == cudaSuccess) e = cudaMemset(a->ck, 0, a->lat_bytes * a->nck);
  if (e == cudaSuccess) e = cudaMemset(a->seg, 0, a->lat_bytes * a->K * a->nseg);
  if (e == cudaSuccess) e = cudaMemset(a->work, 0, a->lat_bytes * 2);
  if (e == cudaSuccess) e = cudaMemset(a->lam, 0, a->lat_bytes * 2);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&a->own, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&a->side, cudaStreamNonBlocking);
  cudaEvent_t* evs[6] = {&a->ev_fork, &a->ev_join, &a->ev_rec[0], &a->ev_rec[1], &a->ev_rev[0], &a->ev_rev[1]};
  for (int i = 0; i < 6 && e == cudaSuccess; i++) e = cudaEventCreateWithFlags(evs[i], cudaEventDisableTiming);
  if (e != cudaSuccess) {
    plbm_adjoint_destroy(a);
    return cuda_fail(e, "adjoint allocation");
  }
  a->stream = a->own;
  *out = a;
  return PLBM_OK;
}

extern "C" int plbm_adjoint_destroy(plbm_adjoint_t* a) {
  if (!a) return PLBM_OK;
  cudaSetDevice(a->device);
  if (a->stream) cudaStreamSynchronize(a->stream);
  if (a->side) cudaStreamSynchronize(a->side);
  cudaFree(a->ck);
  cudaFree(a->seg);
  cudaFree(a->work);
  cudaFree(a->lam);
  cudaFree(a->u0);
  cudaFree(a->dom);
  if (a->own) cudaStreamDestroy(a->own);
  if (a->side) cudaStreamDestroy(a->side);
  cudaEvent_t evs[6] = {a->ev_fork, a->ev_join, a->ev_rec[0], a->ev_rec[1], a->ev_rev[0], a->ev_rev[1]};
  for (cudaEvent_t ev : evs)
    if (ev) cudaEventDestroy(ev);
  delete a;
  return PLBM_OK;
}

extern "C" int plbm_adjoint_set_stream(plbm_adjoint_t* a, void* stream) {
  if (!a) return fail(PLBM_E_INVALID, "NULL adjoint");
  a->stream = stream ? static_cast<cudaStream_t>(stream) : a->own;
  return PLBM_OK;
}

extern "C" int plbm_adjoint_set_math(plbm_adjoint_t* a, int math) {
  if (!a) return fail(PLBM_E_INVALID, "NULL adjoint");
  if (math == PLBM_MATH_FMA || (math == PLBM_MATH_HYBRID && a->storage == PLBM_F32DEV)) {
    a->math = math;
    return PLBM_OK;
  }
  return fail(PLBM_E_UNSUPPORTED, "adjoint math %d with storage %d (PLBM_MATH_FMA, or PLBM_MATH_HYBRID for PLBM_F32DEV)",
              math, a->storage);
}

extern "C" int plbm_adjoint_memory(const plbm_adjoint_t* a, size_t* bytes) {
  if (!a || !bytes) return fail(PLBM_E_INVALID, "NULL argument");
  *bytes = a->lat_bytes * ((size_t)a->nck + (size_t)a->K * a->nseg + 4) +
           sizeof(double) * (2 * (size_t)a->nx * a->ny + a->nblocks);
  return PLBM_OK;
}

extern "C" int plbm_adjoint_forward(plbm_adjoint_t* a, const double* u0, double omega, double* uT) {
  if (!a || !u0) return fail(PLBM_E_INVALID, "NULL argument");
  if (!(omega > 0.0 && omega < 2.0)) return fail(PLBM_E_INVALID, "omega = %g outside (0,2)", omega);
  CUDA_TRY(cudaSetDevice(a->device), "cudaSetDevice");
  const size_t n2 = 2 * (size_t)a->nx * a->ny;
  a->omega = omega;
  CUDA_TRY(cudaMemcpyAsync(a->u0, u0, n2 * sizeof(double), cudaMemcpyDeviceToDevice, a->stream), "copy u0");
  AdjLaunch L = base_launch(a);
  L.u = a->u0;
  L.f = lat(a->ck, a, 0);
  CUDA_TRY(adjoint_launch(st(a), 0, L), "adjoint init kernel");
  const CollParams p = plbm_make_params(omega, 0.25);
  const void* cur = lat(a->ck, a, 0);
  int tog = 0;
  for (int n = 0; n < a->nsteps; n++) {
    void* dst = lat(a->work, a, tog);
    tog ^= 1;
    CUDA_TRY(fwd_step(a, cur, dst, p, a->stream), "forward step");
    cur = dst;
    if ((n + 1) % a->K == 0 && (n + 1) < a->nsteps)
      CUDA_TRY(cudaMemcpyAsync(lat(a->ck, a, (n + 1) / a->K), cur, a->lat_bytes, cudaMemcpyDeviceToDevice, a->stream),
               "checkpoint copy");
  }
  a->fT = cur;
  if (uT) {
    L = base_launch(a);
    L.f = a->fT;
    L.out = uT;
    CUDA_TRY(adjoint_launch(st(a), 1, L), "final moments kernel");
  }
  a->have_forward = 1;
  return PLBM_OK;
}

extern "C" int plbm_adjoint_backward(plbm_adjoint_t* a, const double* grad_uT, double* grad_u0,
                                     double* grad_omega) {
  if (!a || !grad_uT) return fail(PLBM_E_INVALID, "NULL argument");
  if (!a->have_forward) return fail(PLBM_E_INVALID, "plbm_adjoint_backward before plbm_adjoint_forward");
  CUDA_TRY(cudaSetDevice(a->device), "cudaSetDevice");
  AdjLaunch L = base_launch(a);
  L.f = a->fT;
  L.g = grad_uT;
  L.lam_out = lat(a->lam, a, 0);
  CUDA_TRY(adjoint_launch(st(a), 1, L), "lambda_T kernel");
  CUDA_TRY(cudaMemsetAsync(a->dom, 0, sizeof(double) * a->nblocks, a->stream), "clear domega");
  const CollParams p = plbm_make_params(a->omega, 0.25);
  // segment k's states live in buffer k % nseg
  auto seg_lat = [a](int k, int i) { return lat(a->seg, a, (k % a->nseg) * a->K + i); };
  auto seg_end = [a](int k) { return k * a->K + a->K < a->nsteps ? k * a->K + a->K : a->nsteps; };
  // recompute f_{n0+1} .. f_{n1-1} of segment k into its buffer, on the side stream
  auto recompute = [&](int k) -> int {
    const int n0 = k * a->K, n1 = seg_end(k);
    for (int i = 1; i < n1 - n0; i++) {
      const void* src = i == 1 ? lat(a->ck, a, k) : seg_lat(k, i - 1);
      CUDA_TRY(fwd_step(a, src, seg_lat(k, i), p, a->side), "recompute step");
    }
    CUDA_TRY(cudaEventRecord(a->ev_rec[k & 1], a->side), "record recomputation");
    return PLBM_OK;
  };
  // the side stream starts after everything queued on the caller's stream
  CUDA_TRY(cudaEventRecord(a->ev_fork, a->stream), "record fork");
  CUDA_TRY(cudaStreamWaitEvent(a->side, a->ev_fork, 0), "fork");
  int rc = recompute(a->nck - 1);
  if (rc != PLBM_OK) return rc;
  int li = 0;
  for (int k = a->nck - 1; k >= 0; k--) {
    if (k >= 1 && a->nseg == 2) {
      // segment k-1 reuses the buffer of segment k+1: after its reverse sweep
      if (k + 1 < a->nck) CUDA_TRY(cudaStreamWaitEvent(a->side, a->ev_rev[(k + 1) & 1], 0), "wait reverse sweep");
      rc = recompute(k - 1);
      if (rc != PLBM_OK) return rc;
    }
    CUDA_TRY(cudaStreamWaitEvent(a->stream, a->ev_rec[k & 1], 0), "wait recomputation");
    const int n0 = k * a->K;
    for (int n = seg_end(k) - 1; n >= n0; n--) {
      L = base_launch(a);
      L.f = n == n0 ? lat(a->ck, a, k) : seg_lat(k, n - n0);
      L.lam_in = lat(a->lam, a, li);
      L.lam_out = lat(a->lam, a, 1 - li);
      L.dom = a->dom;
      CUDA_TRY(adjoint_launch(st(a), 2, L), "reverse step");
      li = 1 - li;
    }
    CUDA_TRY(cudaEventRecord(a->ev_rev[k & 1], a->stream), "record reverse sweep");
    if (k >= 1 && a->nseg == 1) {  // one buffer: segment k-1 after the sweep of segment k
      CUDA_TRY(cudaStreamWaitEvent(a->side, a->ev_rev[k & 1], 0), "wait reverse sweep");
      rc = recompute(k - 1);
      if (rc != PLBM_OK) return rc;
    }
  }
  // join: nothing of the side stream outlives the call's work on the caller's stream
  CUDA_TRY(cudaEventRecord(a->ev_join, a->side), "record join");
  CUDA_TRY(cudaStreamWaitEvent(a->stream, a->ev_join, 0), "join");
  if (grad_u0) {
    L = base_launch(a);
    L.lam_in = lat(a->lam, a, li);
    L.u = a->u0;
    L.out = grad_u0;
    CUDA_TRY(adjoint_launch(st(a), 3, L), "dL/du0 kernel");
  }
  if (grad_omega) {
    std::vector<double> h(a->nblocks);
    CUDA_TRY(cudaMemcpyAsync(h.data(), a->dom, sizeof(double) * a->nblocks, cudaMemcpyDeviceToHost, a->stream),
             "download domega");
    CUDA_TRY(cudaStreamSynchronize(a->stream), "adjoint sync");
    double s = 0.0;
    for (int b = 0; b < a->nblocks; b++) s += h[b];
    *grad_omega = s;
  }
  return PLBM_OK;
}
