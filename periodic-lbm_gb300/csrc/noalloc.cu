// noalloc.cu -- plbm_velocity_l2_error_noalloc: the velocity L2 error of a
// device lattice against host reference fields, with no device allocation.
//
// Who needs it: callers that cannot call cudaMalloc at the time they want
// the number -- a monitoring hook inside a long batched run whose lattices
// have taken nearly all of HBM (an allocation would fail), a host program
// whose device memory is owned by another allocator (a caching allocator that
// has reserved the free memory), or a time loop that must not pay for, or
// risk the failure of, an allocation per diagnostic.  plbm_velocity_l2_error
// on a grid handle allocates its staging lazily; this entry point stages in a
// file-scope device array instead.
//
// The staging array (g_noalloc_scratch below) holds the two reference fields
// of at most PLBM_NOALLOC_MAX_CELLS cells plus the per-block partial sums:
// 2 * 2^20 + 3 * kReduceBlocks doubles, about 16 MB, reserved on every GPU that
// loads the library until the process exits.
#include <cuda_runtime.h>
#include <math.h>
#include <mutex>

#include "../../include/plbm_gpu.h"
#include "plbm_launch.h"

namespace plbm_internal {
int fail(int code, const char* fmt, ...);
int cuda_fail(cudaError_t e, const char* what);
}  // namespace plbm_internal
using plbm_internal::cuda_fail;
using plbm_internal::fail;

namespace {

constexpr size_t kMaxCells = (size_t)1 << 20;  // PLBM_NOALLOC_MAX_CELLS
constexpr int kMaxPartials = plbm::kReduceBlocks;  // one partial triple per reduction block
constexpr size_t kScratchDoubles = 2 * kMaxCells + 3 * (size_t)kMaxPartials;
static_assert(kMaxCells == (size_t)PLBM_NOALLOC_MAX_CELLS, "staging capacity");
static_assert(3 * kMaxPartials == PLBM_NOALLOC_PARTIAL_DOUBLES, "partial-sum staging, as the header states it");

// Shared by every call on a device; keeps the last call's contents.
static __device__ __align__(256) double g_noalloc_scratch[kScratchDoubles];

constexpr int kMaxDevices = 64;
std::mutex g_mu;
double* g_addr[kMaxDevices] = {};

// Device address of g_noalloc_scratch for the current device, looked up once
// per device with that device current.  In host code the symbol's name is a
// host-side stand-in, never a device address.  The mutex guards this lookup
// only; it does not serialise the calls that use the array.
int scratch_address(double** out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return cuda_fail(e, "cudaGetDevice");
  if (dev < 0 || dev >= kMaxDevices) return fail(PLBM_E_UNSUPPORTED, "device ordinal %d >= %d", dev, kMaxDevices);
  std::lock_guard<std::mutex> lock(g_mu);
  if (!g_addr[dev]) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p) return cuda_fail(e, "cudaGetSymbolAddress(g_noalloc_scratch)");
    g_addr[dev] = static_cast<double*>(p);
  }
  *out = g_addr[dev];
  return PLBM_OK;
}

}  // namespace

extern "C" int plbm_velocity_l2_error_noalloc(int storage, int nx, int ny, int ld, const void* f,
                                              const double* uxa, const double* uya, double* err,
                                              void* cuda_stream) {
  if (nx < 1 || ny < 1 || ld < ny || nx > PLBM_MAX_EXTENT || ld > PLBM_MAX_EXTENT)
    return fail(PLBM_E_INVALID, "bad sizes nx=%d ny=%d ld=%d (extents <= %d)", nx, ny, ld, PLBM_MAX_EXTENT);
  if (storage != PLBM_F64 && storage != PLBM_F32DEV && storage != PLBM_F16DEV)
    return fail(PLBM_E_INVALID, "unknown storage %d", storage);
  if (!f || !uxa || !uya || !err) return fail(PLBM_E_INVALID, "NULL argument");
  const size_t n = (size_t)nx * (size_t)ny;
  if (n > kMaxCells)
    return fail(PLBM_E_INVALID,
                "plbm_velocity_l2_error_noalloc: %dx%d = %zu cells exceeds the fixed staging capacity of "
                "%zu cells (PLBM_NOALLOC_MAX_CELLS); use plbm_velocity_l2_error",
                nx, ny, n, kMaxCells);
  const int nb = plbm::reduce_blocks(nx, ny);
  if (nb > kMaxPartials) return fail(PLBM_E_INVALID, "reduction needs %d partial blocks > %d", nb, kMaxPartials);
  double* base = nullptr;
  if (int r = scratch_address(&base)) return r;
  double* dua = base;
  double* dva = base + kMaxCells;
  double* part = base + 2 * kMaxCells;
  cudaStream_t st = static_cast<cudaStream_t>(cuda_stream);
  double h[3 * kMaxPartials];
  cudaError_t e = cudaMemcpyAsync(dua, uxa, n * sizeof(double), cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(dva, uya, n * sizeof(double), cudaMemcpyHostToDevice, st);
  // every block writes its own partial triple: nothing needs clearing
  if (e == cudaSuccess) e = plbm::energy_error_partials(storage, 0, nx, ny, ld, f, dua, dva, part, st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(h, part, 3 * (size_t)nb * sizeof(double), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return cuda_fail(e, "plbm_velocity_l2_error_noalloc");
  double num = 0.0, den = 0.0;
  for (int b = 0; b < nb; b++) {
    num += h[3 * b + 1];
    den += h[3 * b + 2];
  }
  if (!(den > 0.0)) return fail(PLBM_E_INVALID, "reference field has zero norm");
  *err = sqrt(num / den);
  return PLBM_OK;
}
