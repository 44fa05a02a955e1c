// grid_io.cpp -- .npy output of the moments (the reference's output_npy,
// src/fvm_bardow.F90:930-961 with src/output/npy.f90:13-26) and binary64
// state save / load for restarts.
//
// File format: NumPy .npy version 1.0 as NumPy documents it -- the magic
// "\x93NUMPY", version bytes 1 0, a little-endian uint16 header length, an
// ASCII dict {'descr': '<f8', 'fortran_order': ..., 'shape': (...), } padded
// with spaces and ended by '\n' so that the data starts at a multiple of 64
// bytes, then the raw little-endian binary64 data.  Version 2.0 headers
// (uint32 length) are accepted on read.
#include <cuda_runtime.h>
#include <errno.h>
#include <stdio.h>
#include <string.h>
#include <sys/stat.h>
#include <sys/types.h>

#include <string>
#include <vector>

#include "../../include/plbm_gpu.h"
#include "grid_internal.h"
#include "plbm_launch.h"

using namespace plbm;
using namespace plbm_internal;

namespace {

bool host_little_endian() {
  const unsigned one = 1;
  unsigned char b;
  memcpy(&b, &one, 1);
  return b == 1;
}

std::string npy_header(int ndim, const long long* shape, int fortran_order) {
  std::string d = "{'descr': '<f8', 'fortran_order': ";
  d += fortran_order ? "True" : "False";
  d += ", 'shape': (";
  for (int i = 0; i < ndim; i++) {
    d += std::to_string(shape[i]);
    if (ndim == 1 || i + 1 < ndim) d += ",";
    if (i + 1 < ndim) d += " ";
  }
  d += "), }";
  // magic(6) + version(2) + length(2) + dict + padding + '\n' = multiple of 64
  size_t total = 10 + d.size() + 1;
  const size_t pad = (64 - total % 64) % 64;
  d.append(pad, ' ');
  d += '\n';
  return d;
}

int write_npy(const char* path, const void* data, size_t bytes, int ndim, const long long* shape,
              int fortran_order) {
  if (!host_little_endian()) return fail(PLBM_E_UNSUPPORTED, "big-endian host");
  const std::string h = npy_header(ndim, shape, fortran_order);
  if (h.size() > 65535) return fail(PLBM_E_INVALID, "npy header too long");
  FILE* fp = fopen(path, "wb");
  if (!fp) return fail(PLBM_E_INVALID, "cannot open %s for writing: %s", path, strerror(errno));
  unsigned char pre[10] = {0x93, 'N', 'U', 'M', 'P', 'Y', 1, 0, 0, 0};
  pre[8] = (unsigned char)(h.size() & 0xFF);
  pre[9] = (unsigned char)(h.size() >> 8);
  bool good = fwrite(pre, 1, 10, fp) == 10 && fwrite(h.data(), 1, h.size(), fp) == h.size() &&
              (bytes == 0 || fwrite(data, 1, bytes, fp) == bytes);
  good = (fclose(fp) == 0) && good;
  if (!good) return fail(PLBM_E_INVALID, "short write to %s", path);
  return PLBM_OK;
}

// Value of `key` in the header dict: the text after "'key':" up to the next
// top-level comma (or the closing brace).
std::string dict_value(const std::string& d, const char* key) {
  const std::string k = std::string("'") + key + "'";
  size_t p = d.find(k);
  if (p == std::string::npos) return "";
  p = d.find(':', p + k.size());
  if (p == std::string::npos) return "";
  p++;
  while (p < d.size() && d[p] == ' ') p++;
  size_t e = p;
  int depth = 0;
  for (; e < d.size(); e++) {
    const char c = d[e];
    if (c == '(') depth++;
    else if (c == ')') depth--;
    else if ((c == ',' || c == '}') && depth == 0) break;
  }
  return d.substr(p, e - p);
}

struct NpyInfo {
  int ndim = 0;
  long long shape[8] = {0};
  int fortran_order = 0;
  long long data_offset = 0;
};

int read_npy_header(FILE* fp, const char* path, NpyInfo* info) {
  unsigned char pre[12];
  if (fread(pre, 1, 10, fp) != 10 || memcmp(pre, "\x93NUMPY", 6) != 0)
    return fail(PLBM_E_INVALID, "%s: not an .npy file", path);
  size_t hlen;
  long long off;
  if (pre[6] == 1) {
    hlen = (size_t)pre[8] | ((size_t)pre[9] << 8);
    off = 10;
  } else if (pre[6] == 2 || pre[6] == 3) {
    if (fread(pre + 10, 1, 2, fp) != 2) return fail(PLBM_E_INVALID, "%s: truncated header", path);
    hlen = (size_t)pre[8] | ((size_t)pre[9] << 8) | ((size_t)pre[10] << 16) | ((size_t)pre[11] << 24);
    off = 12;
  } else {
    return fail(PLBM_E_UNSUPPORTED, "%s: npy version %d.%d", path, pre[6], pre[7]);
  }
  if (hlen > (1u << 20)) return fail(PLBM_E_INVALID, "%s: header of %zu bytes", path, hlen);
  std::string d(hlen, '\0');
  if (fread(&d[0], 1, hlen, fp) != hlen) return fail(PLBM_E_INVALID, "%s: truncated header", path);
  const std::string descr = dict_value(d, "descr");
  if (descr != "'<f8'" && descr != "\"<f8\"") return fail(PLBM_E_UNSUPPORTED, "%s: dtype %s (need <f8)", path, descr.c_str());
  const std::string fo = dict_value(d, "fortran_order");
  if (fo != "True" && fo != "False") return fail(PLBM_E_INVALID, "%s: fortran_order %s", path, fo.c_str());
  info->fortran_order = fo == "True";
  const std::string sh = dict_value(d, "shape");
  if (sh.size() < 2 || sh.front() != '(' || sh.back() != ')') return fail(PLBM_E_INVALID, "%s: shape %s", path, sh.c_str());
  info->ndim = 0;
  size_t i = 1;
  while (i < sh.size() - 1) {
    while (i < sh.size() - 1 && (sh[i] == ' ' || sh[i] == ',')) i++;
    if (i >= sh.size() - 1) break;
    long long v = 0;
    bool any = false;
    while (i < sh.size() - 1 && sh[i] >= '0' && sh[i] <= '9') {
      if (v > (1LL << 53)) return fail(PLBM_E_INVALID, "%s: extent too large in shape %s", path, sh.c_str());
      v = v * 10 + (sh[i] - '0');
      any = true;
      i++;
    }
    if (!any || info->ndim >= 8) return fail(PLBM_E_INVALID, "%s: shape %s", path, sh.c_str());
    info->shape[info->ndim++] = v;
  }
  info->data_offset = off + (long long)hlen;
  return PLBM_OK;
}

int mkdir_p(const std::string& dir) {
  if (dir.empty()) return PLBM_OK;
  std::string cur;
  size_t i = 0;
  while (i <= dir.size()) {
    const size_t j = dir.find('/', i);
    cur = dir.substr(0, j == std::string::npos ? dir.size() : j);
    if (!cur.empty() && mkdir(cur.c_str(), 0777) != 0 && errno != EEXIST)
      return fail(PLBM_E_INVALID, "cannot create directory %s: %s", cur.c_str(), strerror(errno));
    if (j == std::string::npos) break;
    i = j + 1;
  }
  return PLBM_OK;
}

}  // namespace

extern "C" int plbm_write_npy(const char* path, const double* data, int ndim, const long long* shape,
                              int fortran_order) {
  if (!path || (!data && ndim > 0) || ndim < 1 || ndim > 8 || !shape)
    return fail(PLBM_E_INVALID, "plbm_write_npy: bad arguments");
  size_t n = 1;
  for (int i = 0; i < ndim; i++) {
    if (shape[i] < 0) return fail(PLBM_E_INVALID, "negative extent");
    n *= (size_t)shape[i];
  }
  return write_npy(path, data, n * sizeof(double), ndim, shape, fortran_order);
}

extern "C" int plbm_read_npy_header(const char* path, int* ndim, long long* shape, int* fortran_order,
                                    long long* data_offset) {
  if (!path) return fail(PLBM_E_INVALID, "NULL path");
  FILE* fp = fopen(path, "rb");
  if (!fp) return fail(PLBM_E_INVALID, "cannot open %s: %s", path, strerror(errno));
  NpyInfo info;
  const int r = read_npy_header(fp, path, &info);
  fclose(fp);
  if (r) return r;
  if (ndim) *ndim = info.ndim;
  if (shape)
    for (int i = 0; i < info.ndim; i++) shape[i] = info.shape[i];
  if (fortran_order) *fortran_order = info.fortran_order;
  if (data_offset) *data_offset = info.data_offset;
  return PLBM_OK;
}

extern "C" int plbm_output_npy(plbm_grid_t* g, const char* path) {
  if (int r = check_grid(g)) return r;
  if (!path) return fail(PLBM_E_INVALID, "NULL path");
  if (int r = use_device(g)) return r;
  const size_t n = (size_t)g->nx * g->ny;
  if (int r = ensure_scratch(g, 3 * n)) return r;
  double* d = g->scratch;  // mf(ny,nx,3): rho, ux, uy planes
  // update_macros reads f(:,:,:,inew) (src/fvm_bardow.F90:350-352)
  PLBM_CUDA_TRY(macros(internal_storage(g->storage), 0, g->nx, g->ny, g->ld, lattice(g, g->inew), d, d + n,
                       d + 2 * n, g->stream, exact_fields(g)),
                "moments kernel");
  std::vector<double> mf(3 * n);
  PLBM_CUDA_TRY(cudaMemcpyAsync(mf.data(), d, 3 * n * sizeof(double), cudaMemcpyDeviceToHost, g->stream),
                "download moments");
  PLBM_CUDA_TRY(cudaStreamSynchronize(g->stream), "moments sync");
  const long long shape[3] = {g->ny, g->nx, 3};
  return write_npy(path, mf.data(), mf.size() * sizeof(double), 3, shape, 1);
}

extern "C" int plbm_output_npy_step(plbm_grid_t* g, const char* folder, const char* filename, int step) {
  if (int r = check_grid(g)) return r;
  if (!filename) return fail(PLBM_E_INVALID, "NULL filename");
  // The reference concatenates folder // '/' // filename, which without a
  // folder names a file in the root directory; here no folder means the
  // working directory.
  std::string full;
  if (folder && folder[0]) {
    if (int r = mkdir_p(folder)) return r;
    full = folder;
    full += "/";
  }
  full += filename;
  if (step >= 0) {
    char num[16];
    snprintf(num, sizeof num, "%09d", step);
    full += num;
  }
  full += ".npy";
  return plbm_output_npy(g, full.c_str());
}

extern "C" int plbm_save_state(plbm_grid_t* g, const char* path) {
  if (int r = check_grid(g)) return r;
  if (!path) return fail(PLBM_E_INVALID, "NULL path");
  std::vector<double> f(g->lat_elems * (size_t)g->nf);
  for (int b = 1; b <= g->nf; b++)
    if (int r = plbm_download(g, f.data() + (size_t)(b - 1) * g->lat_elems, b)) return r;
  const long long shape[4] = {g->ld, g->nx, 9, g->nf};
  return write_npy(path, f.data(), f.size() * sizeof(double), 4, shape, 1);
}

extern "C" int plbm_load_state(plbm_grid_t* g, const char* path) {
  if (int r = check_grid(g)) return r;
  if (!path) return fail(PLBM_E_INVALID, "NULL path");
  FILE* fp = fopen(path, "rb");
  if (!fp) return fail(PLBM_E_INVALID, "cannot open %s: %s", path, strerror(errno));
  NpyInfo info;
  if (int r = read_npy_header(fp, path, &info)) {
    fclose(fp);
    return r;
  }
  const bool shape_ok = info.fortran_order && info.ndim == 4 && info.shape[0] == g->ld && info.shape[1] == g->nx &&
                        info.shape[2] == 9 && info.shape[3] == g->nf;
  if (!shape_ok) {
    fclose(fp);
    return fail(PLBM_E_INVALID, "%s: need a Fortran-order (%d, %d, 9, %d) binary64 array", path, g->ld, g->nx,
                g->nf);
  }
  std::vector<double> f(g->lat_elems * (size_t)g->nf);
  const bool got = fread(f.data(), sizeof(double), f.size(), fp) == f.size();
  fclose(fp);
  if (!got) return fail(PLBM_E_INVALID, "%s: truncated data", path);
  for (int b = 1; b <= g->nf; b++)
    if (int r = plbm_upload(g, f.data() + (size_t)(b - 1) * g->lat_elems, b)) return r;
  return PLBM_OK;
}
