// k_stencil.cu -- stencil kernels of the step outside the 2.5D pipeline
// (k_stencil25.cu): single derivatives, standalone nu_t, the scalar
// transport and the flow statistics.  Templated on the arithmetic type T (double for
// the plain method, float for the mixed method).
#include "o3d_internal.cuh"
#include "o3d_kernels.h"

namespace o3d {

// ---------------------------------------------------------------------------
// one derivative (der_type, src/initialization.f90:86-91)
// ---------------------------------------------------------------------------
template <class T>
__global__ void k_der(const T* __restrict__ f, T* __restrict__ df, Grid g, AxisCoef<T> c,
                      int axis, int order, int odd) {
  pdl_enter();
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  const int k = blockIdx.z;
  if (i >= g.nx || j >= g.ny) return;
  const long long q = (long long)i + g.sy() * j + g.sz() * k;
  if (g.bc[axis] == AX_ZERO) {  // derz_2dsim: 0*f*dz, src/derivation.f90:492
    df[q] = (T)0 * f[q];
    return;
  }
  T v[7];
  load_line<3>(f, g, axis, i, j, k, odd != 0, v);
  const int pc = axis == 0 ? xclass(g, i) : 0;
  df[q] = order == 1 ? d1c(v, c, pc) : d2c(v, c, pc);
}

// standalone calculate_nu_t (src/les_turbulence.f90:54-88)
template <class T>
__global__ void k_nu_t(const T* __restrict__ ux, const T* __restrict__ uy, const T* __restrict__ uz,
                       T* __restrict__ nu_t, Grid g, Coef3<T> cf, T csd2) {
  pdl_enter();
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  const int k = blockIdx.z;
  if (i >= g.nx || j >= g.ny) return;
  const long long q = (long long)i + g.sy() * j + g.sz() * k;
  const T* u[3] = {ux, uy, uz};
  T g1[3][3];
#pragma unroll
  for (int c = 0; c < 3; ++c)
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      if (g.bc[a] == AX_ZERO) { g1[c][a] = (T)0; continue; }
      T v[7];
      load_line<3>(u[c], g, a, i, j, k, a == c, v);
      g1[c][a] = d1c(v, cf.ax[a], a == 0 ? xclass(g, i) : 0);
    }
  const T s11 = g1[0][0], s22 = g1[1][1], s33 = g1[2][2];
  const T s12 = (T)0.5 * (g1[0][1] + g1[1][0]);
  const T s13 = (T)0.5 * (g1[0][2] + g1[2][0]);
  const T s23 = (T)0.5 * (g1[1][2] + g1[2][1]);
  nu_t[q] = csd2 * sqrt((T)2 * (s11 * s11 + s22 * s22 + s33 * s33 +
                                (T)2 * (s12 * s12 + s13 * s13 + s23 * s23)));
}

// ---------------------------------------------------------------------------
// statistics_calc (src/utils.f90:277-361): per block partial sums of
// <u^2>,<v^2>,<w^2>, nine <(du_i/dx_j)^2>, E_k, eps, dzeta, eps2 in FP64.
// ---------------------------------------------------------------------------
template <class T>
__global__ void __launch_bounds__(256) k_stats(const T* __restrict__ ux, const T* __restrict__ uy,
                                               const T* __restrict__ uz, Grid g, Coef3<T> cf,
                                               double xnu, double* part) {
  pdl_enter();
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  const int k = blockIdx.z;
  double r[16];
  const int ops[16] = {0};
#pragma unroll
  for (int q = 0; q < 16; ++q) r[q] = 0.0;
  if (i < g.nx && j < g.ny) {
    const T* u[3] = {ux, uy, uz};
    double g1[3][3], g2[3][3], uc[3];
#pragma unroll
    for (int c = 0; c < 3; ++c)
#pragma unroll
      for (int a = 0; a < 3; ++a) {
        if (g.bc[a] == AX_ZERO) { g1[c][a] = 0.0; g2[c][a] = 0.0; continue; }
        T v[7];
        load_line<3>(u[c], g, a, i, j, k, a == c, v);
        const int pc = a == 0 ? xclass(g, i) : 0;
        g1[c][a] = (double)d1c(v, cf.ax[a], pc);
        g2[c][a] = (double)d2c(v, cf.ax[a], pc);
        if (a == 0) uc[c] = (double)v[3];
      }
#pragma unroll
    for (int c = 0; c < 3; ++c) r[c] = uc[c] * uc[c];
#pragma unroll
    for (int c = 0; c < 3; ++c)
#pragma unroll
      for (int a = 0; a < 3; ++a) r[3 + 3 * c + a] = g1[c][a] * g1[c][a];
    r[12] = 0.5 * (uc[0] * uc[0] + uc[1] * uc[1] + uc[2] * uc[2]);
    const double a2 = 2.0 * g1[0][0], b2 = 2.0 * g1[1][1], c2 = 2.0 * g1[2][2];
    const double s12 = g1[0][1] + g1[1][0], s13 = g1[0][2] + g1[2][0], s23 = g1[1][2] + g1[2][1];
    r[13] = 0.5 * xnu * (a2 * a2 + b2 * b2 + c2 * c2 + 2.0 * (s12 * s12) + 2.0 * (s13 * s13) +
                         2.0 * (s23 * s23));
    const double w1 = g1[2][1] - g1[1][2], w2 = g1[0][2] - g1[2][0], w3 = g1[1][0] - g1[0][1];
    r[14] = 0.5 * (w1 * w1 + w2 * w2 + w3 * w3);
    r[15] = (-xnu) * (uc[0] * (g2[0][0] + g2[0][1] + g2[0][2]) +
                      uc[1] * (g2[1][0] + g2[1][1] + g2[1][2]) +
                      uc[2] * (g2[2][0] + g2[2][1] + g2[2][2]));
  }
  block_reduce_store<16>(r, ops, part, block_linear_id());
}

// ---------------------------------------------------------------------------
// transeq (src/integration.f90:405-447): scalar flux, AB update and the
// first clipping pass; partial sums of phi before clipping, after clipping
// and of the weights min(phi, 1-phi).  A thread marches a column of TQ_KZ
// planes: the z-line of phi is a register queue (one new load per plane),
// the x- and y-lines come through the L1 cache, and the three sums are
// accumulated per thread -- in TwoSum-compensated FP32 pairs for the mixed
// method (exact to about 2^-48 over the column), FP64 otherwise -- and
// widened once per thread for the block reduction.
// ---------------------------------------------------------------------------
constexpr int TQ_KZ = 16;
static dim3 tq_grid(const Grid& g) {
  return dim3((g.nx + 31) / 32, (g.ny + 7) / 8, (g.nz + TQ_KZ - 1) / TQ_KZ);
}
static long long tq_blocks(const Grid& g) {
  const dim3 b = tq_grid(g);
  return (long long)b.x * b.y * b.z;
}

template <class T>
__global__ void __launch_bounds__(256) k_transeq(ScalArgs<T> A) {
  pdl_enter();
  const Grid& g = A.g;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  const int k0 = blockIdx.z * TQ_KZ, k1 = min(k0 + TQ_KZ, g.nz);
  constexpr bool F32 = sizeof(T) == 4;
  float s_hi[3] = {0.f, 0.f, 0.f}, s_lo[3] = {0.f, 0.f, 0.f};
  double r[3] = {0.0, 0.0, 0.0};
  const int ops[3] = {RED_SUM, RED_SUM, RED_SUM};
  if (i < g.nx && j < g.ny) {
    const int cls = xclass(g, i);
    const bool zon = g.bc[2] != AX_ZERO;
    const long long xy = (long long)i + g.sy() * j;
    T zq[7];
#pragma unroll
    for (int m = 0; m < 7; ++m) zq[m] = (T)0;
    if (zon) load_line<3>(A.phi, g, 2, i, j, k0, false, zq);  // planes k0 - 3 .. k0 + 3
    for (int k = k0; k < k1; ++k) {
      if (zon && k > k0) {  // the scalar is even: the z ghost planes need no sign
#pragma unroll
        for (int m = 0; m < 6; ++m) zq[m] = zq[m + 1];
        zq[6] = __ldg(A.phi + z_plane(g, k + 3).off + xy);
      }
      const long long q = xy + g.sz() * k;
      T vx[7], vy[7];
      load_line<3>(A.phi, g, 0, i, j, k, false, vx);
      load_line<3>(A.phi, g, 1, i, j, k, false, vy);
      const T pc = vx[3];
      const T s1x = d1c(vx, A.cf.ax[0], cls), s2x = d2c(vx, A.cf.ax[0], cls);
      const T s1y = d1(vy, A.cf.ax[1]), s2y = d2(vy, A.cf.ax[1]);
      const T s1z = zon ? d1(zq, A.cf.ax[2]) : (T)0, s2z = zon ? d2(zq, A.cf.ax[2]) : (T)0;
      T alpha = A.alpha0;
      if (A.les) alpha = alpha + A.nu_t[q] / A.sc;
      const T F = alpha * (s2x + s2y + s2z) - (A.u[0][q] * s1x + A.u[1][q] * s1y + A.u[2][q] * s1z) + A.src[q];
      T ph = pc + A.adu * F;
      if (A.f2) ph = ph + A.bdu * A.f2[q];
      if (A.f3) ph = ph + A.cdu * A.f3[q];
      if (cls == 1) ph = pc;  // open x axis: the inflow value is held
      A.fnew[q] = F;
      const T cl = fmax((T)0, fmin((T)1, ph));
      const T w = cls == 1 ? (T)0 : fmin(cl, (T)1 - cl);  // held inflow nodes take no excess
      A.phi_out[q] = cl;
      if constexpr (F32) {
        two_sum_acc(s_hi[0], s_lo[0], ph);
        two_sum_acc(s_hi[1], s_lo[1], cl);
        two_sum_acc(s_hi[2], s_lo[2], w);
      } else {
        r[0] += (double)ph;
        r[1] += (double)cl;
        r[2] += (double)w;
      }
    }
    if constexpr (F32) {
#pragma unroll
      for (int c = 0; c < 3; ++c) r[c] = to_t<double>(s_hi[c]) + to_t<double>(s_lo[c]);
    }
  }
  block_reduce_store<3>(r, ops, A.part, block_linear_id());
}

// second clipping pass (src/integration.f90:443-450); sums[0..2] are the
// finalized totals of k_transeq.  The FP64 coefficient excess / sum(weight)
// is formed once per block, so no thread divides in FP64; then
// phi <- clip(phi + min(phi, 1 - phi) * coefficient).
template <class T>
__global__ void __launch_bounds__(256) k_scalar_redistribute(T* __restrict__ phi, long long n, const double* sums,
                                                             int nx_inflow) {
  pdl_enter();
  __shared__ double coef;
  if (threadIdx.x == 0) {
    const double wsum = sums[2];
    coef = wsum == 0.0 ? 0.0 : (sums[0] / (double)n - sums[1] / (double)n) / wsum;
  }
  __syncthreads();
  if (sums[2] == 0.0) return;  // nothing to spread the excess over
  const T c = (T)coef;
  for (long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x; q < n; q += (long long)gridDim.x * blockDim.x) {
    if (nx_inflow > 0 && q % nx_inflow == 0) continue;  // open x axis: inflow nodes are held
    const T p = phi[q];
    phi[q] = fmax((T)0, fmin((T)1, p + fmin(p, (T)1 - p) * c));
  }
}

// ---------------------------------------------------------------------------
// fixed-order finalizers
// ---------------------------------------------------------------------------
// G = (warps / M) warps per slot q: lane l of part g folds the records
// g*32 + l, (G + g)*32 + l, ... in order, the lanes fold by a fixed shuffle
// tree and the G parts in order (deterministic).
__global__ void k_finalize(const double* __restrict__ part, long long nblk, int M,
                           unsigned long long opmask, double* out) {
  pdl_enter();
  __shared__ double sh[32];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
  const int G = nw / M > 0 ? nw / M : 1;
  for (int base = 0; base < M; base += nw / G) {
    const int q = base + warp / G, g = warp % G;
    double acc = 0.0;
    int op = 0;
    if (q < M && warp / G < nw / G) {
      op = (int)((opmask >> (2 * q)) & 3ull);
      acc = red_ident(op);
      const double* slot = part + (long long)q * nblk;
      for (long long b = (long long)g * 32 + lane; b < nblk; b += 32LL * G) acc = red_apply(op, acc, slot[b]);
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) acc = red_apply(op, acc, __shfl_xor_sync(0xffffffffu, acc, o));
      if (lane == 0) sh[warp] = acc;
    }
    __syncthreads();
    if (q < M && warp / G < nw / G && g == 0 && lane == 0) {
      double v = sh[warp];
      for (int h = 1; h < G; ++h) v = red_apply(op, v, sh[warp + h]);
      out[q] = v;
    }
    __syncthreads();
  }
}

__global__ void k_finalize_stats(const StatPart* __restrict__ part, long long nblk, Grid g,
                                 double* out6) {
  pdl_enter();
  __shared__ StatPart sh[1024];
  StatPart acc;
  acc.mn = INFINITY; acc.mx = -INFINITY; acc.sum = 0.0; acc.imx = 0x7fffffffffffffffll;
  for (long long b = threadIdx.x; b < nblk; b += blockDim.x) stat_merge(acc, part[b]);
  sh[threadIdx.x] = acc;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if ((int)threadIdx.x < s) stat_merge(sh[threadIdx.x], sh[threadIdx.x + s]);
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    const StatPart r = sh[0];
    out6[0] = r.mn;
    out6[1] = r.mx;
    out6[2] = r.sum / (double)g.n;
    long long im = r.imx < g.n ? r.imx : 0;
    out6[3] = (double)(im % g.nx + 1);
    out6[4] = (double)((im / g.nx) % g.ny + 1);
    out6[5] = (double)(im / ((long long)g.nx * g.ny) + 1);
  }
}

template <class S, class D>
__global__ void k_convert(const S* __restrict__ s, D* __restrict__ d, long long n) {
  pdl_enter();
  const long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (q < n) d[q] = (D)s[q];
}

// ---------------------------------------------------------------------------
// launchers
// ---------------------------------------------------------------------------
static inline dim3 pt_block() { return dim3(32, 8, 1); }
static inline dim3 pt_grid(const Grid& g) { return dim3((g.nx + 31) / 32, (g.ny + 7) / 8, g.nz); }
long long pt_blocks(const Grid& g) { dim3 b = pt_grid(g); return (long long)b.x * b.y * b.z; }

template <class T>
void launch_der(const T* f, T* df, const Grid& g, const AxisCoef<T>& c, int axis, int order,
                int odd, cudaStream_t s) {
  launch_pdl(k_der<T>, pt_grid(g), pt_block(), 0, s, f, df, g, c, axis, order, odd);
}
template <class T>
void launch_nu_t(const T* ux, const T* uy, const T* uz, T* nu, const Grid& g, const Coef3<T>& cf,
                 T csd2, cudaStream_t s) {
  launch_pdl(k_nu_t<T>, pt_grid(g), pt_block(), 0, s, ux, uy, uz, nu, g, cf, csd2);
}
template <class T>
void launch_stats(const T* ux, const T* uy, const T* uz, const Grid& g, const Coef3<T>& cf,
                  double xnu, double* part, cudaStream_t s) {
  launch_pdl(k_stats<T>, pt_grid(g), pt_block(), 0, s, ux, uy, uz, g, cf, xnu, part);
}
template <class T>
void launch_transeq(const ScalArgs<T>& a, const double* sums, cudaStream_t s, long long* nl) {
  long long nblk = tq_blocks(a.g);
  bool two_point = false;
  if constexpr (sizeof(T) == 4) {
    if (stencil_v_ok(a.g)) {
      launch_transeq_v(a, s);
      nblk = transeq_v_blocks(a.g);
      two_point = true;
    }
  }
  if (!two_point) launch_pdl(k_transeq<T>, tq_grid(a.g), dim3(32, 8), 0, s, a);
  launch_finalize(a.part, nblk, 3, 0ull, (double*)sums, s);
  // a grid-stride loop over at most 8 blocks of 256 threads per SM
  const long long want = (a.g.n + 255) / 256;
  launch_pdl(k_scalar_redistribute<T>, (unsigned)(want < 152 * 8 ? want : 152 * 8), 256, 0, s, a.phi_out, a.g.n,
             sums, a.g.bc[0] == AX_OPEN ? a.g.nx : 0);
  *nl += 3;
}
void launch_finalize(const double* part, long long nblk, int M, unsigned long long opmask,
                     double* out, cudaStream_t s) {
  launch_pdl(k_finalize, 1, 1024, 0, s, part, nblk, M, opmask, out);
}
void launch_finalize_stats(const StatPart* part, long long nblk, const Grid& g, double* out6,
                           cudaStream_t s) {
  launch_pdl(k_finalize_stats, 1, 1024, 0, s, part, nblk, g, out6);
}
template <class S, class D>
void launch_convert(const S* s_, D* d, long long n, cudaStream_t s) {
  launch_pdl(k_convert<S, D>, (unsigned)((n + 255) / 256), 256, 0, s, s_, d, n);
}

// FP64 field <-> double-float pair of FP32 planes: hi = RN32(x), lo =
// RN32(x - hi), and back x = hi + lo (exact in FP64).  The conversions are
// the hardware's, subnormals included, so that split(join(pair)) returns
// every normalised pair (a pair hi = RN32(hi + lo)) unchanged at any
// magnitude: a saved and reloaded pressure continues bit for bit.  (These
// run at the API boundary only; the solver's kernels never split.)
__global__ void k_split_pair(const double* __restrict__ x, float* __restrict__ hi, float* __restrict__ lo,
                             long long n) {
  pdl_enter();
  const long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= n) return;
  const double v = x[q];
  const float h = (float)v;
  hi[q] = h;
  lo[q] = (float)(v - (double)h);
}
__global__ void k_join_pair(const float* __restrict__ hi, const float* __restrict__ lo, double* __restrict__ x,
                            long long n) {
  pdl_enter();
  const long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= n) return;
  x[q] = (double)hi[q] + (double)lo[q];
}
void launch_split_pair(const double* x, void* pair, long long n, cudaStream_t s) {
  const PPair p = ppair(pair, n);
  launch_pdl(k_split_pair, (unsigned)((n + 255) / 256), 256, 0, s, x, p.hi, p.lo, n);
}
void launch_join_pair(const void* pair, double* x, long long n, cudaStream_t s) {
  const PPair p = ppair((void*)pair, n);
  launch_pdl(k_join_pair, (unsigned)((n + 255) / 256), 256, 0, s, (const float*)p.hi, (const float*)p.lo, x, n);
}

#define O3D_INST(T)                                                                            \
  template void launch_der<T>(const T*, T*, const Grid&, const AxisCoef<T>&, int, int, int,     \
                              cudaStream_t);                                                   \
  template void launch_nu_t<T>(const T*, const T*, const T*, T*, const Grid&, const Coef3<T>&,  \
                               T, cudaStream_t);                                               \
  template void launch_stats<T>(const T*, const T*, const T*, const Grid&, const Coef3<T>&,     \
                                double, double*, cudaStream_t);                                \
  template void launch_transeq<T>(const ScalArgs<T>&, const double*, cudaStream_t, long long*);
O3D_INST(double)
O3D_INST(float)
template void launch_convert<double, float>(const double*, float*, long long, cudaStream_t);
template void launch_convert<float, double>(const float*, double*, long long, cudaStream_t);

}  // namespace o3d
