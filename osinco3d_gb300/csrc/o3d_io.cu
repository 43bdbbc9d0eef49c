// o3d_io.cu -- checkpoint and restart: the reference's flow-state file
// (save_fields / read_fields, src/IOfunctions.f90:360-470; reader
// bin/fields_analyser.py:20-31) plus a history file with what an exact
// restart of the time loop also needs (Adams-Bashforth flux history,
// scalar flux history, previous pressure of the extrapolated and learned
// guesses, the dynamic SOR omega).  Host code over the context's own
// download/upload paths, so both methods (FP64 and mixed) restart bit for
// bit.
#include <cstdio>
#include <cstring>
#include <vector>

#include "o3d_internal.cuh"
#include "o3d_kernels.h"

namespace {

// the history file: magic, then int32 nx, ny, nz, nscr, nprev, pairs, then
// double omega, then the FP64 arrays (u, v, w fluxes newest then older, the
// scalar fluxes when nscr = 1), then the pressures: with pairs = 0 the nprev
// previous pressures as FP64 arrays, newest first (one for the linear
// extrapolation and the learned guess, two for the quadratic extrapolation);
// with pairs = 1 (a context that holds its pressures as double-float pairs)
// the current pressure and the nprev previous ones as raw pairs (n FP32 high
// parts, then n low parts each).  A pair need not be representable in FP64
// (its low part may reach more than 29 bits below the high part's last
// bit), so the FP64 pressure of the fields file restores it only to FP64
// precision; loading the history after the fields restores it exactly.
// Files of the first version (magic ...1, no pairs field) load as pairs = 0.
const char HIST_MAGIC[8] = {'O', '3', 'D', 'H', 'I', 'S', 'T', '2'};
const char HIST_MAGIC1[8] = {'O', '3', 'D', 'H', 'I', 'S', 'T', '1'};

struct File {
  FILE* f = nullptr;
  ~File() {
    if (f) fclose(f);
  }
};

bool put(FILE* f, const void* p, size_t bytes) { return fwrite(p, 1, bytes, f) == bytes; }
bool get(FILE* f, void* p, size_t bytes) { return fread(p, 1, bytes, f) == bytes; }

}  // namespace

extern "C" {

int o3d_save_fields(o3d_ctx* c, const char* path, double time) {
  if (!c || !path) return O3D_ERR_BADARG;
  o3d_params P;
  int nx, ny, nz;
  double dx, dy, dz;
  int st = o3d::ctx_geometry(c, &P, &nx, &ny, &nz, &dx, &dy, &dz);
  if (st) return st;
  const size_t n = (size_t)nx * ny * nz;
  std::vector<double> buf(n);
  File F;
  F.f = fopen(path, "wb");
  if (!F.f) {
    o3d::set_error("cannot open %s for writing", path);
    return O3D_ERR_BADARG;
  }
  const int dims[3] = {nx, ny, nz};
  bool ok = put(F.f, &time, 8) && put(F.f, dims, 12);
  // coordinates x(i) = x0 + (i - 1) dx (src/initialization.f90:202-209)
  for (int a = 0; a < 3 && ok; ++a) {
    const int m = dims[a];
    const double o = a == 0 ? P.x0 : a == 1 ? P.y0 : P.z0, h = a == 0 ? dx : a == 1 ? dy : dz;
    std::vector<double> x(m);
    for (int i = 0; i < m; ++i) x[i] = o + i * h;
    ok = put(F.f, x.data(), (size_t)m * 8);
  }
  const int fields[5] = {O3D_FIELD_UX, O3D_FIELD_UY, O3D_FIELD_UZ, O3D_FIELD_PP, O3D_FIELD_PHI};
  for (int q = 0; q < 5 && ok; ++q) {
    if (fields[q] == O3D_FIELD_PHI && !P.nscr) {
      std::fill(buf.begin(), buf.end(), 0.0);  // the reference writes its (unused) phi array
    } else if ((st = o3d_download(c, fields[q], buf.data()))) {
      return st;
    }
    ok = put(F.f, buf.data(), n * 8);
  }
  if (!ok) {
    o3d::set_error("write to %s failed", path);
    return O3D_ERR_BADARG;
  }
  return O3D_OK;
}

int o3d_load_fields(o3d_ctx* c, const char* path, double* time) {
  if (!c || !path) return O3D_ERR_BADARG;
  o3d_params P;
  int nx, ny, nz;
  double dx, dy, dz;
  int st = o3d::ctx_geometry(c, &P, &nx, &ny, &nz, &dx, &dy, &dz);
  if (st) return st;
  File F;
  F.f = fopen(path, "rb");
  if (!F.f) {
    o3d::set_error("cannot open %s", path);
    return O3D_ERR_BADARG;
  }
  double t = 0.0;
  int dims[3];
  if (!get(F.f, &t, 8) || !get(F.f, dims, 12)) {
    o3d::set_error("%s: truncated header", path);
    return O3D_ERR_BADARG;
  }
  if (dims[0] != nx || dims[1] != ny || dims[2] != nz) {
    o3d::set_error("%s holds a %d x %d x %d grid, the context %d x %d x %d", path, dims[0], dims[1], dims[2], nx, ny,
                   nz);
    return O3D_ERR_BADARG;
  }
  if (fseek(F.f, (long)((size_t)(nx + ny + nz) * 8), SEEK_CUR)) {
    o3d::set_error("%s: truncated coordinates", path);
    return O3D_ERR_BADARG;
  }
  const size_t n = (size_t)nx * ny * nz;
  std::vector<double> buf(n);
  const int fields[5] = {O3D_FIELD_UX, O3D_FIELD_UY, O3D_FIELD_UZ, O3D_FIELD_PP, O3D_FIELD_PHI};
  for (int q = 0; q < 5; ++q) {
    if (!get(F.f, buf.data(), n * 8)) {
      o3d::set_error("%s: truncated field %d", path, q);
      return O3D_ERR_BADARG;
    }
    if (fields[q] == O3D_FIELD_PHI && !P.nscr) continue;
    if ((st = o3d_upload(c, fields[q], buf.data()))) return st;
  }
  if (time) *time = t;
  return O3D_OK;
}

int o3d_save_history(o3d_ctx* c, const char* path) {
  if (!c || !path) return O3D_ERR_BADARG;
  o3d_params P;
  int nx, ny, nz;
  double dx, dy, dz;
  int st = o3d::ctx_geometry(c, &P, &nx, &ny, &nz, &dx, &dy, &dz);
  if (st) return st;
  const size_t n = (size_t)nx * ny * nz;
  std::vector<double> buf(n);
  double omega = 0.0;
  int has_prev = 0;
  if ((st = o3d::ctx_history_state(c, &omega, &has_prev, nullptr, 0))) return st;
  File F;
  F.f = fopen(path, "wb");
  if (!F.f) {
    o3d::set_error("cannot open %s for writing", path);
    return O3D_ERR_BADARG;
  }
  const int pairs = o3d::ctx_pressure_pairs(c);
  const int hdr[6] = {nx, ny, nz, P.nscr, has_prev, pairs};
  bool ok = put(F.f, HIST_MAGIC, 8) && put(F.f, hdr, 24) && put(F.f, &omega, 8);
  std::vector<int> ids;
  for (int q = 0; q < 6; ++q) ids.push_back(O3D_FIELD_FU0 + q);
  if (P.nscr)
    for (int h = 0; h < 2; ++h) ids.push_back(O3D_FIELD_FPHI0 + h);
  for (int id : ids) {
    if (!ok) break;
    if ((st = o3d_download(c, id, buf.data()))) return st;
    ok = put(F.f, buf.data(), n * 8);
  }
  for (int q = pairs ? 0 : 1; ok && q <= has_prev; ++q) {
    if (pairs) st = o3d::ctx_pressure_raw(c, q, buf.data(), 0);
    else st = o3d::ctx_history_state(c, nullptr, nullptr, buf.data(), q);
    if (st) return st;
    ok = put(F.f, buf.data(), n * 8);
  }
  if (!ok) {
    o3d::set_error("write to %s failed", path);
    return O3D_ERR_BADARG;
  }
  return O3D_OK;
}

int o3d_load_history(o3d_ctx* c, const char* path) {
  if (!c || !path) return O3D_ERR_BADARG;
  o3d_params P;
  int nx, ny, nz;
  double dx, dy, dz;
  int st = o3d::ctx_geometry(c, &P, &nx, &ny, &nz, &dx, &dy, &dz);
  if (st) return st;
  File F;
  F.f = fopen(path, "rb");
  if (!F.f) {
    o3d::set_error("cannot open %s", path);
    return O3D_ERR_BADARG;
  }
  char magic[8];
  int hdr[6] = {0, 0, 0, 0, 0, 0};
  double omega;
  bool ok = get(F.f, magic, 8);
  const bool v2 = ok && !memcmp(magic, HIST_MAGIC, 8);
  ok = ok && (v2 || !memcmp(magic, HIST_MAGIC1, 8)) && get(F.f, hdr, v2 ? 24 : 20) && get(F.f, &omega, 8);
  if (!ok || hdr[5] < 0 || hdr[5] > 1) {
    o3d::set_error("%s is not a history file", path);
    return O3D_ERR_BADARG;
  }
  if (hdr[0] != nx || hdr[1] != ny || hdr[2] != nz || hdr[3] != P.nscr) {
    o3d::set_error("%s: grid or scalar option differs from the context", path);
    return O3D_ERR_BADARG;
  }
  const size_t n = (size_t)nx * ny * nz;
  std::vector<double> buf(n);
  std::vector<int> ids;
  for (int q = 0; q < 6; ++q) ids.push_back(O3D_FIELD_FU0 + q);
  if (P.nscr)
    for (int h = 0; h < 2; ++h) ids.push_back(O3D_FIELD_FPHI0 + h);
  for (int id : ids) {
    if (!get(F.f, buf.data(), n * 8)) {
      o3d::set_error("%s: truncated", path);
      return O3D_ERR_BADARG;
    }
    if ((st = o3d_upload(c, id, buf.data()))) return st;
  }
  if (hdr[4] < 0 || hdr[4] > 2) {
    o3d::set_error("%s: %d previous pressures (at most 2)", path, hdr[4]);
    return O3D_ERR_BADARG;
  }
  const int pairs = hdr[5], npres = hdr[4] + (pairs ? 1 : 0);
  std::vector<double> pres((size_t)npres * n);
  for (int q = 0; q < npres; ++q)
    if (!get(F.f, pres.data() + (size_t)q * n, n * 8)) {
      o3d::set_error("%s: truncated", path);
      return O3D_ERR_BADARG;
    }
  if (pairs && o3d::ctx_pressure_pairs(c)) {  // exact: the raw pairs back into their buffers
    if ((st = o3d::ctx_restore_history(c, omega, 0, nullptr, nullptr))) return st;
    for (int q = 0; q < npres; ++q)
      if ((st = o3d::ctx_pressure_raw(c, q, pres.data() + (size_t)q * n, 1))) return st;
    return O3D_OK;
  }
  if (pairs) {  // pairs into a context with FP64 pressures: their values hi + lo, rounded to FP64
    std::vector<double> v((size_t)npres * n);
    for (int q = 0; q < npres; ++q) {
      const float* h = reinterpret_cast<const float*>(pres.data() + (size_t)q * n);
      for (size_t i = 0; i < n; ++i) v[(size_t)q * n + i] = (double)h[i] + (double)h[n + i];
    }
    if ((st = o3d_upload(c, O3D_FIELD_PP, v.data()))) return st;
    return o3d::ctx_restore_history(c, omega, hdr[4], hdr[4] >= 1 ? v.data() + n : nullptr,
                                    hdr[4] >= 2 ? v.data() + 2 * n : nullptr);
  }
  return o3d::ctx_restore_history(c, omega, hdr[4], hdr[4] >= 1 ? pres.data() : nullptr,
                                  hdr[4] >= 2 ? pres.data() + n : nullptr);
}

}  // extern "C"
