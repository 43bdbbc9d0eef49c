// o3d_noalloc.cu -- divergence with its statistics for callers that cannot
// allocate device memory.
//
// Some callers of this library cannot call cudaMalloc: a driver that has
// handed all device memory to its own pool allocator at start-up, a time
// loop that must not take the device-wide synchronisation that cudaMalloc
// and cudaFree imply, or code that runs where allocation is forbidden.  The
// entry point below gives them the divergence of a velocity field together
// with its function_stats record without any allocation: the caller passes
// the input and output buffers, and the per-block reduction records live in
// a fixed array in device memory that is part of the library image.
#include <mutex>

#include "o3d_internal.cuh"
#include "o3d_kernels.h"

namespace o3d {

// Most thread blocks the divergence kernel may use.  The kernel tiles the
// grid into columns of 32 x 8 points that march over 28 planes each
// (z_blocks), so a grid needs ceil(nx/32) * ceil(ny/8) * ceil(nz/28) block
// records: 16 * 64 * 19 = 19456 for 512^3, 24 * 48 * 14 = 16128 for
// 768 x 384 x 384.  Both fit.
constexpr long long NOALLOC_MAX_BLOCKS = O3D_NOALLOC_MAX_RECORDS;
static_assert(NOALLOC_MAX_BLOCKS >= 19456, "the scratch must serve a 512^3 grid");

// Scratch of the entry point (768 KiB of 32-byte block records plus the six
// finalized statistics).  Every device that loads the library holds it until
// the process exits.  Each call writes every record it reads, so nothing has
// to start at zero; all calls share it, so calls that overlap on the GPU
// (from different streams or threads) race on it.
static __device__ __align__(256) StatPart g_noalloc_part[NOALLOC_MAX_BLOCKS];
static __device__ __align__(256) double g_noalloc_stats[8];

struct NoallocScratch {
  StatPart* part;
  double* stats;
};

constexpr int NOALLOC_MAX_DEVICES = 64;
static NoallocScratch g_scratch[NOALLOC_MAX_DEVICES];
static bool g_scratch_ready[NOALLOC_MAX_DEVICES];
static std::mutex g_scratch_mu;

// Device addresses of the scratch on the current device, looked up once per
// device (host code cannot use the symbols' names as device addresses).
static int noalloc_scratch(NoallocScratch* out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) {
    set_error("cudaGetDevice failed: %s", cudaGetErrorString(e));
    return O3D_ERR_CUDA;
  }
  if (dev < 0 || dev >= NOALLOC_MAX_DEVICES) {
    set_error("device %d is beyond the %d devices this entry point serves", dev, NOALLOC_MAX_DEVICES);
    return O3D_ERR_BADARG;
  }
  std::lock_guard<std::mutex> lock(g_scratch_mu);
  if (!g_scratch_ready[dev]) {
    NoallocScratch s;
    e = cudaGetSymbolAddress((void**)&s.part, g_noalloc_part);
    if (e != cudaSuccess) {
      set_error("cudaGetSymbolAddress(block records) failed: %s", cudaGetErrorString(e));
      return O3D_ERR_CUDA;
    }
    e = cudaGetSymbolAddress((void**)&s.stats, g_noalloc_stats);
    if (e != cudaSuccess) {
      set_error("cudaGetSymbolAddress(statistics) failed: %s", cudaGetErrorString(e));
      return O3D_ERR_CUDA;
    }
    g_scratch[dev] = s;
    g_scratch_ready[dev] = true;
  }
  *out = g_scratch[dev];
  return O3D_OK;
}

}  // namespace o3d

using namespace o3d;

extern "C" int o3d_divergence_stats_noalloc(const double* d_fx, const double* d_fy, const double* d_fz,
                                            double* d_div, int nx, int ny, int nz, double dx, double dy,
                                            double dz, int bcx, int bcy, int bcz, int odd, void* stream,
                                            double stats[6]) {
  if (!d_fx || !d_fy || !d_fz || !stats) {
    set_error("o3d_divergence_stats_noalloc: null input or statistics pointer");
    return O3D_ERR_BADARG;
  }
  if (nx < 8 || ny < 8 || nz < 8) {
    set_error("o3d_divergence_stats_noalloc: every axis needs at least 8 points (got %d x %d x %d)", nx, ny, nz);
    return O3D_ERR_BADARG;
  }
  const int bcs[3] = {bcx, bcy, bcz};
  for (int a = 0; a < 3; ++a)
    if (bcs[a] != O3D_BC_PERIODIC && bcs[a] != O3D_BC_FREE_SLIP) {
      set_error("o3d_divergence_stats_noalloc: boundary code %d of axis %c is neither periodic nor free-slip",
                bcs[a], "xyz"[a]);
      return O3D_ERR_BADARG;
    }
  if (!(dx > 0.0) || !(dy > 0.0) || !(dz > 0.0)) {
    set_error("o3d_divergence_stats_noalloc: grid spacings must be positive");
    return O3D_ERR_BADARG;
  }
  Grid g;
  g.nx = nx;
  g.ny = ny;
  g.nz = nz;
  g.n = (long long)nx * ny * nz;
  for (int a = 0; a < 3; ++a) g.bc[a] = bcs[a] == O3D_BC_PERIODIC ? AX_PERIODIC : AX_MIRROR;
  const long long blocks = z_blocks(g);
  if (blocks > NOALLOC_MAX_BLOCKS) {
    set_error("o3d_divergence_stats_noalloc: a %d x %d x %d grid needs %lld reduction records "
              "(ceil(nx/32) * ceil(ny/8) * ceil(nz/28)), more than the %lld this entry point holds",
              nx, ny, nz, blocks, NOALLOC_MAX_BLOCKS);
    return O3D_ERR_BADARG;
  }
  NoallocScratch scr;
  int st = noalloc_scratch(&scr);
  if (st) return st;
  Coef3<double> cf;
  make_coef(dx, cf.ax[0]);
  make_coef(dy, cf.ax[1]);
  make_coef(dz, cf.ax[2]);
  cudaStream_t s = (cudaStream_t)stream;
  launch_div<double, double>(d_fx, d_fy, d_fz, d_div, g, cf, odd, 1.0, 0, scr.part, s);
  launch_finalize_stats(scr.part, blocks, g, scr.stats, s);
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaMemcpyAsync(stats, scr.stats, 6 * sizeof(double), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) {
    set_error("o3d_divergence_stats_noalloc: %s", cudaGetErrorString(e));
    return O3D_ERR_CUDA;
  }
  return O3D_OK;
}
