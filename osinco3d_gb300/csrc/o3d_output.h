// o3d_output.h -- the asynchronous output writer (o3d_output.cu), used by
// o3d_write_output / o3d_output_wait in o3d_api.cu.
#pragma once

#include <string>
#include <vector>

#include <cuda_runtime.h>

namespace o3d {

struct OutWriter;

// what write_xdmf needs to describe one output
struct OutRequest {
  std::string dir;
  int num;
  double time;
  int nx, ny, nz;
  double dx, dy, dz, x0, y0, z0;
};

// Creates the writer on first use, waits for the previous output, and makes
// room for nfields FP64 fields of n points; *snap receives the device
// snapshot (field q at snap + q * n).
int out_prepare(OutWriter** w, long long n, int nfields, double** snap);
// Once the snapshot is complete on `compute`: copies it to pinned host
// memory on the writer's copy stream and writes <dir>/<name>_<num>.bin for
// each field and <dir>/output_<num>.xdmf from a host thread.
int out_submit(OutWriter* w, const OutRequest& r, const char* const* names, int nf, cudaStream_t compute);
// Waits for the writer thread; returns its status.
int out_wait(OutWriter* w);
void out_destroy(OutWriter* w);

}  // namespace o3d
