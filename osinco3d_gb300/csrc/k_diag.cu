// k_diag.cu -- output-cadence diagnostics: the curl and the Q-criterion of
// the velocity (src/differential_operators.f90:40-108) and the velocity
// residuals against the previous step (src/utils.f90:93-163).
#include "o3d_internal.cuh"
#include "o3d_kernels.h"

namespace o3d {

// The nine first derivatives of u with the reference's closures: component
// c is odd along axis c ("i" closure), even along the others ("p").  In 2D
// mode the z-derivatives are 0 * f (derz_2dsim, src/derivation.f90:481-495).
template <class T>
__device__ __forceinline__ void grad9(const T* const* u, const Grid& g, const Coef3<T>& cf, int i, int j, int k,
                                      T (&gr)[3][3]) {
#pragma unroll
  for (int c = 0; c < 3; ++c)
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      if (g.bc[a] == AX_ZERO) {
        gr[c][a] = (T)0 * u[c][(long long)i + g.sy() * j + g.sz() * k];
        continue;
      }
      T v[7];
      load_line<3>(u[c], g, a, i, j, k, a == c, v);
      gr[c][a] = d1c(v, cf.ax[a], a == 0 ? xclass(g, i) : 0);
    }
}

// rot = curl u (src/differential_operators.f90:63-74) and
// Q = -1/2 (ux,x^2 + uy,y^2 + uz,z^2) - ux,y uy,x - ux,z uz,x - uy,z uz,y
// (:104-105); any output may be null
template <class T>
__global__ void __launch_bounds__(256) k_vort(const T* __restrict__ u0, const T* __restrict__ u1,
                                              const T* __restrict__ u2, T* __restrict__ rx, T* __restrict__ ry,
                                              T* __restrict__ rz, T* __restrict__ q, Grid g, Coef3<T> cf) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  const int k = blockIdx.z;
  if (i >= g.nx || j >= g.ny) return;
  const T* u[3] = {u0, u1, u2};
  T gr[3][3];
  grad9<T>(u, g, cf, i, j, k, gr);
  const long long p = (long long)i + g.sy() * j + g.sz() * k;
  if (rx) rx[p] = gr[2][1] - gr[1][2];
  if (ry) ry[p] = gr[0][2] - gr[2][0];
  if (rz) rz[p] = gr[1][0] - gr[0][1];
  if (q)
    q[p] = (T)-0.5 * (gr[0][0] * gr[0][0] + gr[1][1] * gr[1][1] + gr[2][2] * gr[2][2]) - gr[0][1] * gr[1][0] -
           gr[0][2] * gr[2][0] - gr[1][2] * gr[2][1];
}

// The output snapshot of write_all_data (src/visualization.f90:242-274) in
// one pass: u, v, w widened to FP64, the vorticity magnitude
// sqrt(rotx^2 + roty^2 + rotz^2) of the curl (src/differential_operators.f90:
// 63-74, the magnitude formed as write_all_data forms it) and the
// Q-criterion (:104-105), computed in the field type T
template <class T>
__global__ void __launch_bounds__(256) k_out_snapshot(const T* __restrict__ u0, const T* __restrict__ u1,
                                                      const T* __restrict__ u2, double* __restrict__ ux,
                                                      double* __restrict__ uy, double* __restrict__ uz,
                                                      double* __restrict__ vort, double* __restrict__ q, Grid g,
                                                      Coef3<T> cf) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  const int k = blockIdx.z;
  if (i >= g.nx || j >= g.ny) return;
  const T* u[3] = {u0, u1, u2};
  T gr[3][3];
  grad9<T>(u, g, cf, i, j, k, gr);
  const long long p = (long long)i + g.sy() * j + g.sz() * k;
  ux[p] = to_t<double>(u0[p]);
  uy[p] = to_t<double>(u1[p]);
  uz[p] = to_t<double>(u2[p]);
  const T rx = gr[2][1] - gr[1][2], ry = gr[0][2] - gr[2][0], rz = gr[1][0] - gr[0][1];
  vort[p] = to_t<double>((T)sqrt(rx * rx + ry * ry + rz * rz));
  q[p] = to_t<double>((T)-0.5 * (gr[0][0] * gr[0][0] + gr[1][1] * gr[1][1] + gr[2][2] * gr[2][2]) -
                      gr[0][1] * gr[1][0] - gr[0][2] * gr[2][0] - gr[1][2] * gr[2][1]);
}

// per block and component: sum of a^2 and max of a, a = |old - u| / (2 dt)
// over the interior points; on equal maxima the larger index (the last in
// the reference's loop order, i fastest) wins
struct ResPart {
  double sum, mx;
  long long imx;
};

__device__ __forceinline__ void res_merge(ResPart& a, double sum, double mx, long long imx) {
  a.sum += sum;
  if (mx > a.mx || (mx == a.mx && imx > a.imx)) { a.mx = mx; a.imx = imx; }
}

template <class T>
__global__ void __launch_bounds__(256) k_vel_resid(const T* __restrict__ u0, const T* __restrict__ u1,
                                                   const T* __restrict__ u2, const T* __restrict__ o0,
                                                   const T* __restrict__ o1, const T* __restrict__ o2, Grid g,
                                                   double dt, ResPart* part) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  const int k = blockIdx.z;
  const T* u[3] = {u0, u1, u2};
  const T* o[3] = {o0, o1, o2};
  ResPart r[3];
  const bool in = i >= 1 && i < g.nx - 1 && j >= 1 && j < g.ny - 1 && k >= 1 && k < g.nz - 1;
  const long long p = (long long)i + g.sy() * j + g.sz() * k;
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    r[c].sum = 0.0; r[c].mx = -1.0; r[c].imx = -1;
    if (in) {
      const double a = fabs((double)o[c][p] - (double)u[c][p]) / (2.0 * dt);
      r[c].sum = a * a;
      r[c].mx = a;
      r[c].imx = p;
    }
  }
  __shared__ ResPart sh[3][8];
  const int t = threadIdx.x + blockDim.x * threadIdx.y, lane = t & 31, w = t >> 5;
#pragma unroll
  for (int c = 0; c < 3; ++c) {
#pragma unroll
    for (int off = 16; off > 0; off >>= 1)
      res_merge(r[c], __shfl_xor_sync(0xffffffffu, r[c].sum, off), __shfl_xor_sync(0xffffffffu, r[c].mx, off),
                __shfl_xor_sync(0xffffffffu, r[c].imx, off));
    if (lane == 0) sh[c][w] = r[c];
  }
  __syncthreads();
  if (t < 3) {
    ResPart a = sh[t][0];
    for (int q = 1; q < (int)(blockDim.x * blockDim.y) / 32; ++q) res_merge(a, sh[t][q].sum, sh[t][q].mx, sh[t][q].imx);
    part[(long long)t * gridDim.x * gridDim.y * gridDim.z + blockIdx.x + gridDim.x * (blockIdx.y + gridDim.y * blockIdx.z)] =
        a;
  }
}

// one block per component folds the block records in a fixed order
__global__ void k_vel_resid_final(const ResPart* __restrict__ part, long long nblk, ResPart* out) {
  __shared__ ResPart sh[32];
  const int c = blockIdx.x, t = threadIdx.x;
  ResPart a;
  a.sum = 0.0; a.mx = -1.0; a.imx = -1;
  for (long long b = t; b < nblk; b += blockDim.x) {
    const ResPart& r = part[c * nblk + b];
    res_merge(a, r.sum, r.mx, r.imx);
  }
#pragma unroll
  for (int off = 16; off > 0; off >>= 1)
    res_merge(a, __shfl_xor_sync(0xffffffffu, a.sum, off), __shfl_xor_sync(0xffffffffu, a.mx, off),
              __shfl_xor_sync(0xffffffffu, a.imx, off));
  if ((t & 31) == 0) sh[t >> 5] = a;
  __syncthreads();
  if (t == 0) {
    ResPart b = sh[0];
    for (int q = 1; q < (int)blockDim.x / 32; ++q) res_merge(b, sh[q].sum, sh[q].mx, sh[q].imx);
    out[c] = b;
  }
}

static inline dim3 dg_grid(const Grid& g) { return dim3((g.nx + 31) / 32, (g.ny + 7) / 8, g.nz); }

template <class T>
void launch_vorticity(const T* const u[3], T* rx, T* ry, T* rz, T* q, const Grid& g, const Coef3<T>& cf,
                      cudaStream_t s) {
  k_vort<T><<<dg_grid(g), dim3(32, 8), 0, s>>>(u[0], u[1], u[2], rx, ry, rz, q, g, cf);
}

template <class T>
void launch_out_snapshot(const T* const u[3], double* const out[5], const Grid& g, const Coef3<T>& cf,
                         cudaStream_t s) {
  k_out_snapshot<T><<<dg_grid(g), dim3(32, 8), 0, s>>>(u[0], u[1], u[2], out[0], out[1], out[2], out[3], out[4], g,
                                                       cf);
}
template void launch_out_snapshot<double>(const double* const*, double* const*, const Grid&, const Coef3<double>&,
                                          cudaStream_t);
template void launch_out_snapshot<float>(const float* const*, double* const*, const Grid&, const Coef3<float>&,
                                         cudaStream_t);

// scratch: 3 * blocks ResPart records, then 3 final records
template <class T>
void launch_vel_residuals(const T* const u[3], const T* const old[3], const Grid& g, double dt, void* scratch,
                          cudaStream_t s) {
  const dim3 gr = dg_grid(g);
  const long long nblk = (long long)gr.x * gr.y * gr.z;
  ResPart* part = (ResPart*)scratch;
  k_vel_resid<T><<<gr, dim3(32, 8), 0, s>>>(u[0], u[1], u[2], old[0], old[1], old[2], g, dt, part);
  k_vel_resid_final<<<3, 256, 0, s>>>(part, nblk, part + 3 * nblk);
}

size_t vel_residual_scratch_bytes(const Grid& g) {
  const dim3 gr = dg_grid(g);
  return (size_t)(3 * (long long)gr.x * gr.y * gr.z + 3) * sizeof(ResPart);
}
size_t vel_residual_result_offset(const Grid& g) {
  const dim3 gr = dg_grid(g);
  return (size_t)(3 * (long long)gr.x * gr.y * gr.z) * sizeof(ResPart);
}

template void launch_vorticity<double>(const double* const*, double*, double*, double*, double*, const Grid&,
                                       const Coef3<double>&, cudaStream_t);
template void launch_vorticity<float>(const float* const*, float*, float*, float*, float*, const Grid&,
                                      const Coef3<float>&, cudaStream_t);
template void launch_vel_residuals<double>(const double* const*, const double* const*, const Grid&, double, void*,
                                           cudaStream_t);
template void launch_vel_residuals<float>(const float* const*, const float* const*, const Grid&, double, void*,
                                          cudaStream_t);

}  // namespace o3d
