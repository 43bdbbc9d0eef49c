// k_poisson.cu -- pressure Poisson solvers on the 7-point operator of
// src/poisson.f90:95-98 (periodic wrap or mirror remap per axis,
// src/poisson.f90:57-92 and :197-206).
//
//  * Red-black SOR with the reference's stop test (max |p_gs - p| < eps),
//    stagnation exit and dynamic omega (src/poisson.f90:100-122), driven by
//    a device-side control block so batches of sweeps run without a host
//    round trip.  Red-black ordering converges to the same fixed point as
//    the reference's lexicographic sweep, not through the same iterates.
//  * Geometric multigrid V(pre,post) cycles (red-black Gauss-Seidel
//    smoother, full-weighting restriction, trilinear prolongation,
//    shared-memory coarse solve) as the inner solver of an FP64 defect-
//    correction loop: r = rhs - A p in FP64 (the rhs's weighted mean
//    removed once per solve), A e = r by V-cycles in T, p += e, stop when
//    max |e| < eps.  Replaces the unusable single V-cycle
//    of src/poisson_multigrid.f90:10-190.
#include "o3d_internal.cuh"
#include "o3d_kernels.h"

namespace o3d {

enum { ST_CONVERGED = 0, ST_STAGNATED = 1, ST_MAXIT = 2 };

// neighbour index of the Poisson remap on one axis
__device__ __forceinline__ int nb_lo(int i, int n, int bc) { return i > 0 ? i - 1 : (bc == AX_PERIODIC ? n - 1 : 1); }
__device__ __forceinline__ int nb_hi(int i, int n, int bc) { return i < n - 1 ? i + 1 : (bc == AX_PERIODIC ? 0 : n - 2); }

// Offsets of the six neighbours of point (i, j, k) with the Poisson remap at
// the ends, in 32-bit arithmetic (a grid holds at most 2^31 points).
struct Nb6 {
  int xm, xp, ym, yp, zm, zp;
};
__device__ __forceinline__ Nb6 nb6(const Grid& g, int i, int j, int k) {
  const int sy = g.nx, sz = g.nx * g.ny;
  Nb6 o;
  o.xm = i > 0 ? -1 : (g.bc[0] == AX_PERIODIC ? g.nx - 1 : 1);
  o.xp = i < g.nx - 1 ? 1 : (g.bc[0] == AX_PERIODIC ? 1 - g.nx : -1);
  o.ym = j > 0 ? -sy : (g.bc[1] == AX_PERIODIC ? (g.ny - 1) * sy : sy);
  o.yp = j < g.ny - 1 ? sy : (g.bc[1] == AX_PERIODIC ? (1 - g.ny) * sy : -sy);
  o.zm = k > 0 ? -sz : (g.bc[2] == AX_PERIODIC ? (g.nz - 1) * sz : sz);
  o.zp = k < g.nz - 1 ? sz : (g.bc[2] == AX_PERIODIC ? (1 - g.nz) * sz : -sz);
  return o;
}
__device__ __forceinline__ int idx3(const Grid& g, int i, int j, int k) { return i + g.nx * (j + g.ny * k); }

// off-diagonal part of A at q: ox (w + e) + oy (s + n) + oz (b + t)
template <class T, class S>
__device__ __forceinline__ T lap6(const S* __restrict__ p, int q, const Nb6& o, const PoiCoef<T>& c) {
  return c.ox * ((T)p[q + o.xm] + (T)p[q + o.xp]) + c.oy * ((T)p[q + o.ym] + (T)p[q + o.yp]) +
         c.oz * ((T)p[q + o.zm] + (T)p[q + o.zp]);
}

template <class T, class S>
__device__ __forceinline__ T lap_nb(const S* __restrict__ p, const Grid& g, int i, int j, int k,
                                    const PoiCoef<T>& c) {
  const long long sy = g.sy(), sz = g.sz();
  const long long rowk = sz * k, rowj = sy * j;
  const int im = nb_lo(i, g.nx, g.bc[0]), ip = nb_hi(i, g.nx, g.bc[0]);
  const int jm = nb_lo(j, g.ny, g.bc[1]), jp = nb_hi(j, g.ny, g.bc[1]);
  const int km = nb_lo(k, g.nz, g.bc[2]), kp = nb_hi(k, g.nz, g.bc[2]);
  const T pw = (T)p[im + rowj + rowk], pe = (T)p[ip + rowj + rowk];
  const T ps = (T)p[i + sy * jm + rowk], pn = (T)p[i + sy * jp + rowk];
  const T pb = (T)p[i + rowj + sz * km], pt = (T)p[i + rowj + sz * kp];
  return c.ox * (pw + pe) + c.oy * (ps + pn) + c.oz * (pb + pt);
}

// ---------------------------------------------------------------------------
// red-black SOR sweep of one colour (FP64, reference semantics)
// ---------------------------------------------------------------------------
// On a periodic axis with an odd point count the wrap joins two points of
// the same colour, so the points of its last plane (n - 1) form separate
// "seam" classes: class bit a is set when coordinate a = n_a - 1 on such an
// axis.  A sweep updates class 0 red, class 0 black, then each seam class
// red and black: within a class and colour no two points are neighbours,
// so this is a Gauss-Seidel ordering (converging to the lexicographic
// sweep's fixed point) for any point counts.
__device__ __forceinline__ int seam_bits(const Grid& g) {
  return (g.bc[0] == AX_PERIODIC && (g.nx & 1) ? 1 : 0) | (g.bc[1] == AX_PERIODIC && (g.ny & 1) ? 2 : 0) |
         (g.bc[2] == AX_PERIODIC && (g.nz & 1) ? 4 : 0);
}

__global__ void __launch_bounds__(256) k_sor_rb(double* __restrict__ p, const double* __restrict__ rhs,
                                                Grid g, PoiCoef<double> c, int color,
                                                SolveCtrl* ctrl, double omega_fixed, int use_ctrl) {
  pdl_enter();
  if (use_ctrl && ctrl->done) return;
  const double om = use_ctrl ? ctrl->omega : omega_fixed;
  const int ih = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  const int k = blockIdx.z;
  const int sb = seam_bits(g);  // class 0 only: the seam planes are left to k_sor_seam
  double d = 0.0;
  if (j < g.ny - ((sb >> 1) & 1) && k < g.nz - ((sb >> 2) & 1)) {
    const int i = 2 * ih + ((j + k + color) & 1);
    if (i < g.nx - (sb & 1)) {
      const int q = idx3(g, i, j, k);
      const double s = lap6<double>(p, q, nb6(g, i, j, k), c);
      const double pc = p[q];
      const double pnew = (rhs[q] - s) * c.invA;
      d = fabs(pnew - pc);
      p[q] = pc + om * (pnew - pc);
    }
  }
  if (ctrl) {
    const double bm = block_max(d);
    if (threadIdx.x == 0 && threadIdx.y == 0 && bm > 0.0)
      atomicMax(&ctrl->dmax_key, (unsigned long long)__double_as_longlong(bm));
  }
}

// the points of seam class cls != 0 and one colour, one thread each
__global__ void __launch_bounds__(256) k_sor_seam(double* __restrict__ p, const double* __restrict__ rhs, Grid g,
                                                  PoiCoef<double> c, int cls, int color, SolveCtrl* ctrl,
                                                  double omega_fixed, int use_ctrl) {
  pdl_enter();
  if (use_ctrl && ctrl->done) return;
  const double om = use_ctrl ? ctrl->omega : omega_fixed;
  const int sb = seam_bits(g);
  // free axes run over 0 .. n - 1, less the seam plane when that axis has one
  const int ex = (cls & 1) ? 1 : g.nx - (sb & 1);
  const int ey = (cls & 2) ? 1 : g.ny - ((sb >> 1) & 1);
  const int ez = (cls & 4) ? 1 : g.nz - ((sb >> 2) & 1);
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  double d = 0.0;
  if (t < (long long)ex * ey * ez) {
    const int a = (int)(t % ex), b = (int)((t / ex) % ey), e3 = (int)(t / ((long long)ex * ey));
    const int i = (cls & 1) ? g.nx - 1 : a, j = (cls & 2) ? g.ny - 1 : b, k = (cls & 4) ? g.nz - 1 : e3;
    if (((i + j + k) & 1) == color) {
      const int q = idx3(g, i, j, k);
      const double s = lap6<double>(p, q, nb6(g, i, j, k), c);
      const double pc = p[q];
      const double pnew = (rhs[q] - s) * c.invA;
      d = fabs(pnew - pc);
      p[q] = pc + om * (pnew - pc);
    }
  }
  if (ctrl) {
    const double bm = block_max(d);
    if (threadIdx.x == 0 && bm > 0.0) atomicMax(&ctrl->dmax_key, (unsigned long long)__double_as_longlong(bm));
  }
}

static int host_seam_bits(const Grid& g) {
  return (g.bc[0] == AX_PERIODIC && (g.nx & 1) ? 1 : 0) | (g.bc[1] == AX_PERIODIC && (g.ny & 1) ? 2 : 0) |
         (g.bc[2] == AX_PERIODIC && (g.nz & 1) ? 4 : 0);
}

// the seam-class passes of one sweep (none when every periodic axis is even)
static int sor_seam_passes(double* p, const double* rhs, const Grid& g, const PoiCoef<double>& c, SolveCtrl* ctrl,
                           double omega, int use_ctrl, cudaStream_t s) {
  const int sb = host_seam_bits(g);
  int nl = 0;
  for (int cls = 1; cls < 8; ++cls) {
    if ((cls & sb) != cls) continue;
    const long long ex = (cls & 1) ? 1 : g.nx - (sb & 1);
    const long long ey = (cls & 2) ? 1 : g.ny - ((sb >> 1) & 1);
    const long long ez = (cls & 4) ? 1 : g.nz - ((sb >> 2) & 1);
    const unsigned blocks = (unsigned)((ex * ey * ez + 255) / 256);
    for (int color = 0; color < 2; ++color) {
      launch_pdl(k_sor_seam, blocks, 256, 0, s, p, rhs, g, c, cls, color, ctrl, omega, use_ctrl);
      ++nl;
    }
  }
  return nl;
}

// stop test and dynamic omega of src/poisson.f90:110-122, once per sweep
__global__ void k_sor_control(SolveCtrl* c) {
  pdl_enter();
  if (c->done) return;
  const double dmax = __longlong_as_double((long long)c->dmax_key);
  c->dmax_key = 0ull;
  c->iter += 1;
  c->dmax = dmax;
  if (dmax < c->eps) { c->done = 1; c->status = ST_CONVERGED; return; }
  if (fabs(c->dmax_old - dmax) < c->eps / 1000.0) { c->done = 1; c->status = ST_STAGNATED; return; }
  if (c->iter > 1 && c->idyn == 1) {
    if (dmax > c->dmax_old) c->omega = c->omega * (2.0 - c->factor);
    else if (dmax < 0.1 * c->dmax_old) c->omega = fmin(c->omega * c->factor, 2.0);
  }
  c->dmax_old = dmax;
  if (c->iter >= c->kmax) { c->done = 1; c->status = ST_MAXIT; }
}

static dim3 rb_grid(const Grid& g) { return dim3((unsigned)((g.nx + 1) / 2 + 31) / 32, (g.ny + 7) / 8, g.nz); }


void launch_sor_control(SolveCtrl* ctrl, cudaStream_t s) { launch_pdl(k_sor_control, 1, 1, 0, s, ctrl); }
void launch_sor_fixed(double* p, const double* rhs, const Grid& g, const PoiCoef<double>& c,
                      double omega, SolveCtrl* ctrl, cudaStream_t s) {
  launch_pdl(k_sor_rb, rb_grid(g), dim3(32, 8), 0, s, p, rhs, g, c, 0, ctrl, omega, 0);
  launch_pdl(k_sor_rb, rb_grid(g), dim3(32, 8), 0, s, p, rhs, g, c, 1, ctrl, omega, 0);
  sor_seam_passes(p, rhs, g, c, ctrl, omega, 0, s);
}

// ---------------------------------------------------------------------------
// multigrid
// ---------------------------------------------------------------------------

// trapezoid weight of the left null vector of the mirror operator (1/2 at
// the end nodes of a mirror axis, 1 elsewhere)
__device__ __forceinline__ double wnode(const Grid& g, int i, int j, int k) {
  double w = 1.0;
  if (g.bc[0] == AX_MIRROR && (i == 0 || i == g.nx - 1)) w *= 0.5;
  if (g.bc[1] == AX_MIRROR && (j == 0 || j == g.ny - 1)) w *= 0.5;
  if (g.bc[2] == AX_MIRROR && (k == 0 || k == g.nz - 1)) w *= 0.5;
  return w;
}

// sum of w*rhs with the trapezoid weights; a thread sums its (i, j) column
// over a chunk of WM_KC planes, a block reduces its 32 x 8 columns
constexpr int WM_KC = 32;
template <class R>
__global__ void __launch_bounds__(256) k_wmean_part(const R* __restrict__ rhs, Grid g, double* part) {
  pdl_enter();
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  const int k0 = blockIdx.z * WM_KC, k1 = min(k0 + WM_KC, g.nz);
  double r[1] = {0.0};
  const int ops[1] = {RED_SUM};
  if (i < g.nx && j < g.ny) {
    double wxy = 1.0;
    if (g.bc[0] == AX_MIRROR && (i == 0 || i == g.nx - 1)) wxy *= 0.5;
    if (g.bc[1] == AX_MIRROR && (j == 0 || j == g.ny - 1)) wxy *= 0.5;
    // the column chunk is summed in the rhs type (at most WM_KC terms, one
    // addition each), the chunks and blocks in FP64; on a mirror z axis the
    // end planes, inside the sum with weight 1, are taken half back out
    R acc = (R)0;
    const R* col = rhs + (long long)i + g.sy() * j;
    for (int k = k0; k < k1; ++k) acc += __ldg(col + g.sz() * k);
    double sum = to_t<double>(acc);
    if (g.bc[2] == AX_MIRROR) {
      if (k0 == 0) sum -= 0.5 * to_t<double>(__ldg(col));
      if (k1 == g.nz) sum -= 0.5 * to_t<double>(__ldg(col + g.sz() * (g.nz - 1)));
    }
    r[0] = wxy * sum;
  }
  block_reduce_store<1>(r, ops, part, block_linear_id());
}

__global__ void k_wmean_final(const double* __restrict__ part, long long nblk, double wsum, SolveCtrl* ctrl) {
  pdl_enter();
  __shared__ double s0[1024];
  double a = 0.0;
  for (long long q = threadIdx.x; q < nblk; q += blockDim.x) a += part[q];
  s0[threadIdx.x] = a;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if ((int)threadIdx.x < s) s0[threadIdx.x] += s0[threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    const double m = s0[0] / wsum;
    ctrl->rhs_mean = m;
    ctrl->rhs_mean_h = (float)m;
    ctrl->rhs_mean_l = (float)(m - (double)ctrl->rhs_mean_h);
  }
}

// rhs <- rhs - mean (the trapezoid-weighted mean of k_wmean_final), in
// place, once per multigrid solve: the residual kernels then read a
// compatible rhs and skip the subtraction.
template <class R>
__global__ void k_rhs_shift(R* __restrict__ rhs, long long n, const SolveCtrl* ctrl) {
  pdl_enter();
  const long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const R mean = to_t<R>(ctrl->rhs_mean);  // subtracted in the rhs type
  if (q < n) rhs[q] = rhs[q] - mean;
}

// ---------------------------------------------------------------------------
// FP64 residual of the defect-correction loop, r0 = rhs - A p, stored in T
// (with MAX, max |r0| of the block into ctrl->res_key).  2.5D: a block owns
// a 32 x 8 column and marches along z over RZ_KC planes; each thread keeps
// p at k-1, k, k+1 of its point in registers, the plane's x/y neighbours
// come from a double-buffered shared tile with a 1-point halo (the halo
// cell of a thread and the next queue head are loaded one plane ahead).
// The neighbour remap is that of src/poisson.f90:57-92 (periodic wrap, or
// mirror about the end node).
// T = double (the FP64 method): one FMA chain,
//   r = fma(-oz, pb+pt, fma(-oy, ps+pn, fma(-ox, pw+pe, fma(-A, pc, rhs)))),
// 7 FP64 operations per point, bound by GB300's 2 FP64 lanes per clock.
// T = float (the mixed method, whose V-cycles take r0 in FP32): every p and
// rhs value is split on the integer pipe into a double-float (hi + lo, 48
// bits) as it is loaded and the operator is evaluated in double-float on
// the FP32 pipe (df_resid7), with no FP64 instruction; its error, about
// 2^-46 of the largest term, is far below what one FP32 V-cycle resolves.
// With shift (T = float only) the rhs is taken less its weighted mean
// (ctrl->rhs_mean), in double-float, instead of a shifted copy.
// ---------------------------------------------------------------------------
constexpr int RZ_TX = 32, RZ_TY = 8, RZ_KC = 32;
static inline dim3 rz_grid(const Grid& g) {
  return dim3((g.nx + RZ_TX - 1) / RZ_TX, (g.ny + RZ_TY - 1) / RZ_TY, (g.nz + RZ_KC - 1) / RZ_KC);
}

static inline PoiDF poi_df(const PoiCoef<double>& c) {
  PoiDF d;
  d.A = df_split_host(c.A);
  d.ox = df_split_host(c.ox);
  d.oy = df_split_host(c.oy);
  d.oz = df_split_host(c.oz);
  return d;
}

template <bool DFP>
struct RzVal {
  using V = double;
  static __device__ __forceinline__ double of(double x) { return x; }
  static __device__ __forceinline__ double of(float x) { return f32_to_f64(x); }
};
template <>
struct RzVal<true> {
  using V = DF;
  static __device__ __forceinline__ DF of(double x) { return split_df(x); }
  static __device__ __forceinline__ DF of(float x) { return DF{x, 0.f}; }
};

// PP: the pressure is the double-float pair pp (the mixed multigrid method's
// layout): its values are loaded as (hi, lo) and need no split.
template <bool PP>
struct RzRaw {
  using type = double;
};
template <>
struct RzRaw<true> {
  using type = float2;
};

template <class T, class R, bool MAX, bool PP>
__global__ void __launch_bounds__(RZ_TX * RZ_TY) k_resid25(const double* __restrict__ p, PPair pp,
                                                           const R* __restrict__ rhs, T* __restrict__ r0, Grid g,
                                                           PoiCoef<double> c, PoiDF cdf, SolveCtrl* ctrl,
                                                           int shift) {
  pdl_enter();
  if (ctrl->done) return;
  constexpr bool DFP = sizeof(T) == 4;
  static_assert(DFP || !PP, "the double-float pressure pair is the mixed method's");
  using Cv = RzVal<DFP>;
  using V = typename Cv::V;
  using Raw = typename RzRaw<PP>::type;
  auto ldr = [&](long long q) -> Raw {
    if constexpr (PP) return make_float2(__ldg(pp.hi + q), __ldg(pp.lo + q));
    else return __ldg(p + q);
  };
  auto cvt = [&](Raw x) -> V {
    if constexpr (PP) return DF{x.x, x.y};
    else return Cv::of(x);
  };
  constexpr int TX = RZ_TX, TY = RZ_TY, SW = TX + 2;
  __shared__ V tile[2][(TY + 2) * SW];
  const int tx = threadIdx.x, ty = threadIdx.y, t = ty * TX + tx;
  const int i0 = blockIdx.x * TX, j0 = blockIdx.y * TY;
  const int i = i0 + tx, j = j0 + ty;
  const bool valid = i < g.nx && j < g.ny;
  const int k0 = blockIdx.z * RZ_KC, k1 = min(k0 + RZ_KC, g.nz);
  const long long sz = g.sz();
  bool f;
  const int cxy = ghost(i, g.nx, g.bc[0], &f) + g.nx * ghost(j, g.ny, g.bc[1], &f);
  // halo cell of this thread (t < 2 (TX + TY)): left, right, below, above
  const bool hon = t < 2 * (TX + TY);
  int hi, hj, hidx;
  if (t < TY) { hi = i0 - 1; hj = j0 + t; hidx = (t + 1) * SW; }
  else if (t < 2 * TY) { hi = i0 + TX; hj = j0 + t - TY; hidx = (t - TY + 1) * SW + TX + 1; }
  else if (t < 2 * TY + TX) { hi = i0 + t - 2 * TY; hj = j0 - 1; hidx = t - 2 * TY + 1; }
  else { const int u = min(t - 2 * TY - TX, TX - 1); hi = i0 + u; hj = j0 + TY; hidx = (TY + 1) * SW + u + 1; }
  const int hxy = ghost(hi, g.nx, g.bc[0], &f) + g.nx * ghost(hj, g.ny, g.bc[1], &f);
  const int sc = (ty + 1) * SW + tx + 1;
  auto zoff = [&](int k) { return sz * ghost(k, g.nz, g.bc[2], &f); };
  const long long out0 = valid ? (long long)i + (long long)g.nx * j : 0;
  DF mean = {0.f, 0.f};
  if (DFP && shift) {
    mean.h = ctrl->rhs_mean_h;
    mean.l = ctrl->rhs_mean_l;
  }

  // loads run one plane ahead and stay raw until they are used, so that the
  // split of a value never waits on a load issued in the same plane step
  V pb = cvt(ldr(zoff(k0 - 1) + cxy)), pc = cvt(ldr(zoff(k0) + cxy));
  Raw ptraw = ldr(zoff(k0 + 1) + cxy);
  Raw hv = hon ? ldr(zoff(k0) + hxy) : Raw{};
  R rr = valid ? __ldg(rhs + out0 + sz * k0) : (R)0;
  float m = 0.f;
  int buf = 0;
  for (int k = k0; k < k1; ++k) {
    const V pt = cvt(ptraw);
    tile[buf][sc] = pc;
    if (hon) tile[buf][hidx] = cvt(hv);
    const R rcur = rr;
    if (k + 1 < k1) {
      ptraw = ldr(zoff(k + 2) + cxy);
      if (hon) hv = ldr(zoff(k + 1) + hxy);
      if (valid) rr = __ldg(rhs + out0 + sz * (k + 1));
    }
    __syncthreads();
    if (valid) {
      const V pw = tile[buf][sc - 1], pe = tile[buf][sc + 1];
      const V ps = tile[buf][sc - SW], pn = tile[buf][sc + SW];
      T rv;
      if constexpr (DFP) {
        DF rh = Cv::of(rcur), rs;  // rhs - mean: exact TwoSum of the high parts, low parts added
        two_sum(rh.h, -mean.h, rs.h, rs.l);
        rs.l += rh.l - mean.l;
        rv = df_resid7(rs, pc, pw, pe, ps, pn, pb, pt, cdf.A, cdf.ox, cdf.oy, cdf.oz);
      } else {
        double r = fma(-c.A, pc, Cv::of(rcur));
        r = fma(-c.ox, pw + pe, r);
        r = fma(-c.oy, ps + pn, r);
        r = fma(-c.oz, pb + pt, r);
        rv = (T)r;
      }
      r0[out0 + sz * k] = rv;
      if (MAX) m = fmaxf(m, fabsf((float)rv));
    }
    pb = pc;
    pc = pt;
    buf ^= 1;
  }
  if (MAX) {
    const float bm = block_max_f(m);
    if (threadIdx.x == 0 && threadIdx.y == 0 && bm > 0.f) {
      // float max as double bits: the max of nonnegative doubles orders like their bits
      atomicMax(&ctrl->res_key, (unsigned long long)__double_as_longlong((double)bm));
    }
  }
}

// The residual of the mixed method's defect correction with two x-adjacent
// points per thread (nx a multiple of 64): a block owns a 64 x 8 column, the pair's
// high and low parts and its FP32 rhs come as float2 loads, the x-y plane
// of the pressure pair lands in a double-buffered shared tile (high and low
// planes, 66 x 10 cells with the 1-cell halo), the z-neighbours stay in
// registers.  Each point's value is df_resid7 of the same operands as in
// k_resid25<float, float, MAX, pair>, so the two give the same bits.
// tile rows: column 1 the left halo, columns 2 .. 2 TX + 1 the pairs (even
// columns, so that a pair is an aligned float2), column 2 TX + 2 the right
// halo; R2_SW even
constexpr int R2_TX = 32, R2_TY = 8, R2_KC = 16, R2_SW = 2 * R2_TX + 4;
static inline dim3 r2_grid(const Grid& g) {
  return dim3((g.nx + 2 * R2_TX - 1) / (2 * R2_TX), (g.ny + R2_TY - 1) / R2_TY, (g.nz + R2_KC - 1) / R2_KC);
}
template <bool MAX>
__global__ void __launch_bounds__(R2_TX * R2_TY) k_resid25p(PPair pp, const float* __restrict__ rhs,
                                                            float* __restrict__ r0, Grid g, PoiDF cdf,
                                                            SolveCtrl* ctrl) {
  pdl_enter();
  if (ctrl->done) return;
  constexpr int TX = R2_TX, TY = R2_TY, SW = R2_SW, PLN = (TY + 2) * SW;
  __shared__ float th[2][PLN], tl[2][PLN];
  const int tx = threadIdx.x, ty = threadIdx.y, t = ty * TX + tx;
  const int i0 = blockIdx.x * 2 * TX, j0 = blockIdx.y * TY;
  const int ia = i0 + 2 * tx, j = j0 + ty;
  const bool valid = j < g.ny;  // nx a multiple of 64: every pair is in the grid
  const int k0 = blockIdx.z * R2_KC, k1 = min(k0 + R2_KC, g.nz);
  const long long sz = g.sz();
  bool f;
  const int jj = ghost(j, g.ny, g.bc[1], &f);
  const int cxy = ia + g.nx * jj;
  // halo cell of this thread (t < 2 (TY + 2 TX)): left and right columns, rows below and above
  const bool hon = t < 2 * (TY + 2 * TX);
  int hi, hj, hidx;
  if (t < TY) { hi = i0 - 1; hj = j0 + t; hidx = (t + 1) * SW + 1; }
  else if (t < 2 * TY) { hi = i0 + 2 * TX; hj = j0 + t - TY; hidx = (t - TY + 1) * SW + 2 * TX + 2; }
  else if (t < 2 * TY + 2 * TX) { hi = i0 + t - 2 * TY; hj = j0 - 1; hidx = t - 2 * TY + 2; }
  else { const int u = min(t - 2 * TY - 2 * TX, 2 * TX - 1); hi = i0 + u; hj = j0 + TY; hidx = (TY + 1) * SW + u + 2; }
  const int hxy = ghost(hi, g.nx, g.bc[0], &f) + g.nx * ghost(hj, g.ny, g.bc[1], &f);
  const int sc = (ty + 1) * SW + 2 * tx + 2;  // the pair's first cell in the tile (even)
  auto zoff = [&](int k) { return sz * ghost(k, g.nz, g.bc[2], &f); };
  const long long out0 = valid ? (long long)ia + (long long)g.nx * j : 0;
  const DF mean = {ctrl->rhs_mean_h, ctrl->rhs_mean_l};
  auto ld2f = [&](const float* b, long long q) { return __ldg(reinterpret_cast<const float2*>(b + q)); };

  float2 bh = ld2f(pp.hi, zoff(k0 - 1) + cxy), bl = ld2f(pp.lo, zoff(k0 - 1) + cxy);
  float2 ch = ld2f(pp.hi, zoff(k0) + cxy), cl = ld2f(pp.lo, zoff(k0) + cxy);
  float2 nh = ld2f(pp.hi, zoff(k0 + 1) + cxy), nl = ld2f(pp.lo, zoff(k0 + 1) + cxy);
  float hvh = hon ? __ldg(pp.hi + zoff(k0) + hxy) : 0.f, hvl = hon ? __ldg(pp.lo + zoff(k0) + hxy) : 0.f;
  float2 rr = valid ? ld2f(rhs, out0 + sz * k0) : make_float2(0.f, 0.f);
  float m = 0.f;
  int buf = 0;
  // (unrolled by two: the tile buffer and the plane queue's registers are
  // fixed in each half)
#pragma unroll 2
  for (int k = k0; k < k1; ++k) {
    const float2 th_ = nh, tl_ = nl;  // plane k + 1
    *reinterpret_cast<float2*>(&th[buf][sc]) = ch;
    *reinterpret_cast<float2*>(&tl[buf][sc]) = cl;
    if (hon) {
      th[buf][hidx] = hvh;
      tl[buf][hidx] = hvl;
    }
    const float2 rcur = rr;
    if (k + 1 < k1) {
      nh = ld2f(pp.hi, zoff(k + 2) + cxy);
      nl = ld2f(pp.lo, zoff(k + 2) + cxy);
      if (hon) {
        hvh = __ldg(pp.hi + zoff(k + 1) + hxy);
        hvl = __ldg(pp.lo + zoff(k + 1) + hxy);
      }
      if (valid) rr = ld2f(rhs, out0 + sz * (k + 1));
    }
    __syncthreads();
    if (valid) {
      const float* H = th[buf];
      const float* L = tl[buf];
      float rv[2];
#pragma unroll
      for (int e = 0; e < 2; ++e) {
        const int q = sc + e;
        const DF pc = e ? DF{ch.y, cl.y} : DF{ch.x, cl.x};
        // the x-neighbour inside the pair from registers, the other from the tile
        const DF pw = e ? DF{ch.x, cl.x} : DF{H[q - 1], L[q - 1]};
        const DF pe = e ? DF{H[q + 1], L[q + 1]} : DF{ch.y, cl.y};
        const DF ps = DF{H[q - SW], L[q - SW]}, pn = DF{H[q + SW], L[q + SW]};
        const DF pb = e ? DF{bh.y, bl.y} : DF{bh.x, bl.x}, pt = e ? DF{th_.y, tl_.y} : DF{th_.x, tl_.x};
        DF rh = DF{e ? rcur.y : rcur.x, 0.f}, rs;  // rhs - mean: exact TwoSum of the high parts, low parts added
        two_sum(rh.h, -mean.h, rs.h, rs.l);
        rs.l += rh.l - mean.l;
        rv[e] = df_resid7(rs, pc, pw, pe, ps, pn, pb, pt, cdf.A, cdf.ox, cdf.oy, cdf.oz);
      }
      *reinterpret_cast<float2*>(r0 + out0 + sz * k) = make_float2(rv[0], rv[1]);
      if (MAX) m = fmaxf(m, fmaxf(fabsf(rv[0]), fabsf(rv[1])));
    }
    bh = ch;
    bl = cl;
    ch = th_;
    cl = tl_;
    buf ^= 1;
  }
  if (MAX) {
    const float bm = block_max_f(m);
    if (threadIdx.x == 0 && threadIdx.y == 0 && bm > 0.f)
      atomicMax(&ctrl->res_key, (unsigned long long)__double_as_longlong((double)bm));
  }
}

// max |rhs - A p| after a solve (less the rhs mean when shift: the mixed
// multigrid solve leaves the rhs unshifted)
template <class R, bool PP>
__global__ void __launch_bounds__(256) k_resid_inf(const double* __restrict__ p, PPair pp, const R* __restrict__ rhs,
                                                   Grid g, PoiCoef<double> c, SolveCtrl* ctrl, int shift) {
  pdl_enter();
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  const int k = blockIdx.z;
  double d = 0.0;
  if (i < g.nx && j < g.ny) {
    const long long q = (long long)i + g.sy() * j + g.sz() * k;
    double ap;
    if constexpr (PP) {  // the pair's value hi + lo, exact in FP64
      auto v = [&](long long o) { return f32_to_f64(pp.hi[o]) + f32_to_f64(pp.lo[o]); };
      const Nb6 o = nb6(g, i, j, k);
      ap = c.ox * (v(q + o.xm) + v(q + o.xp)) + c.oy * (v(q + o.ym) + v(q + o.yp)) +
           c.oz * (v(q + o.zm) + v(q + o.zp)) + c.A * v(q);
    } else {
      ap = lap_nb<double>(p, g, i, j, k, c) + c.A * p[q];
    }
    d = fabs((to_t<double>(rhs[q]) - (shift ? ctrl->rhs_mean : 0.0)) - ap);
  }
  const double bm = block_max(d);
  if (threadIdx.x == 0 && threadIdx.y == 0 && bm > 0.0)
    atomicMax(&ctrl->res_key, (unsigned long long)__double_as_longlong(bm));
}

// first smoothing sweep from e = 0: red points get omega*r/A, black points 0
template <class T>
__global__ void __launch_bounds__(256) k_smooth_zero(T* __restrict__ e, const T* __restrict__ r, Grid g,
                                                     PoiCoef<T> c, T om, const SolveCtrl* ctrl) {
  pdl_enter();
  if (ctrl->done) return;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  const int k = blockIdx.z;
  if (i >= g.nx || j >= g.ny) return;
  const long long q = (long long)i + g.sy() * j + g.sz() * k;
  e[q] = ((i + j + k) & 1) == 0 ? om * (r[q] * c.invA) : (T)0;
}

// first sweep from e = 0 in one pass: red points get omega*r/A, black points
// the relaxed Gauss-Seidel value from those red neighbours,
// omega*(r - omega*lap_nb(r)/A)/A (lap_nb: the off-diagonal part of A)
template <class T>
__global__ void __launch_bounds__(256) k_smooth_first(T* __restrict__ e, const T* __restrict__ r, Grid g,
                                                      PoiCoef<T> c, T om, const SolveCtrl* ctrl) {
  pdl_enter();
  if (ctrl->done) return;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  const int k = blockIdx.z;
  if (i >= g.nx || j >= g.ny) return;
  const int q = idx3(g, i, j, k);
  const T rq = __ldg(r + q);
  if (((i + j + k) & 1) == 0) {
    e[q] = om * (rq * c.invA);
  } else {
    const T sr = lap6<T>(r, q, nb6(g, i, j, k), c);
    e[q] = om * ((rq - om * (sr * c.invA)) * c.invA);
  }
}

// with eout, the colour's updated values and the other colour's old ones go
// to eout (e is left as it was): the first colour pass of a sweep from a
// correction that must end up in another array
// ZP planes per thread (a large level): the loads of all of a thread's
// planes are issued before its updates, which only read the other colour
template <class T, int ZP = 1>
__global__ void __launch_bounds__(256) k_smooth(T* __restrict__ e, const T* __restrict__ r, Grid g,
                                                PoiCoef<T> c, int color, T om, const SolveCtrl* ctrl,
                                                T* __restrict__ eout) {
  pdl_enter();
  if (ctrl->done) return;
  const int ih = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  const int kb = blockIdx.z * ZP;
  if (j >= g.ny) return;
  T s[ZP], ec[ZP], rq[ZP], eo[ZP];
#pragma unroll
  for (int u = 0; u < ZP; ++u) {
    const int k = kb + u;
    if (k >= g.nz) break;
    const int i = 2 * ih + ((j + k + color) & 1);
    if (eout) {  // the other colour's cell of the pair 2 ih, 2 ih + 1
      const int io = 2 * ih + 1 - ((j + k + color) & 1);
      if (io < g.nx) eo[u] = e[idx3(g, io, j, k)];
    }
    if (i < g.nx) {
      const int q = idx3(g, i, j, k);
      s[u] = lap6<T>(e, q, nb6(g, i, j, k), c);
      ec[u] = e[q];
      rq[u] = r[q];
    }
  }
#pragma unroll
  for (int u = 0; u < ZP; ++u) {
    const int k = kb + u;
    if (k >= g.nz) break;
    const int i = 2 * ih + ((j + k + color) & 1);
    if (eout) {
      const int io = 2 * ih + 1 - ((j + k + color) & 1);
      if (io < g.nx) eout[idx3(g, io, j, k)] = eo[u];
    }
    if (i < g.nx) {
      const int q = idx3(g, i, j, k);
      const T en = (rq[u] - s[u]) * c.invA;
      (eout ? eout : e)[q] = ec[u] + om * (en - ec[u]);
    }
  }
}
// planes per thread of a colour pass on a large level
constexpr int SM_ZP = 4;

int launch_sor_sweep_ctrl(double* p, const double* rhs, const Grid& g, const PoiCoef<double>& c,
                          SolveCtrl* ctrl, cudaStream_t s) {
  launch_pdl(k_sor_rb, rb_grid(g), dim3(32, 8), 0, s, p, rhs, g, c, 0, ctrl, 0.0, 1);
  launch_pdl(k_sor_rb, rb_grid(g), dim3(32, 8), 0, s, p, rhs, g, c, 1, ctrl, 0.0, 1);
  return 2 + sor_seam_passes(p, rhs, g, c, ctrl, 0.0, 1, s);
}

// ---------------------------------------------------------------------------
// The one-pass level kernels of a large level as 2.5D marches (FP32): a
// block owns a 32 x 8 column and marches along z over LV_KC planes; the
// stencil field's plane lands in a double-buffered shared tile with a
// 1-cell halo (loaded one plane ahead, as in k_resid25), its z-neighbours
// stay in registers.  OP 0: one colour of a relaxed Gauss-Seidel sweep, in
// place (k_smooth); OP 1: the first sweep from e = 0 (k_smooth_first); OP 2:
// the residual t = r - A e (k_resid).  Each value is the expression of the
// one-pass kernel in the same order, so the results are bit-identical.  In
// place (OP 0) a colour's update reads only the other colour's values and
// its own, which no block writes in that pass.
// ---------------------------------------------------------------------------
constexpr int LV_TX = 32, LV_TY = 8, LV_KC = 16;
static inline dim3 lv_grid(const Grid& g) {
  return dim3((g.nx + LV_TX - 1) / LV_TX, (g.ny + LV_TY - 1) / LV_TY, (g.nz + LV_KC - 1) / LV_KC);
}
// the level kernels take the 2.5D form from this size on
static inline bool lv_big(const Grid& g) { return g.n >= (1LL << 22) && g.nx >= 16 && g.ny >= 8 && g.nz >= 8; }

// one colour pass of the relaxed Gauss-Seidel smoother (k_smooth), SM_ZP
// planes per thread on a large level
template <class T>
static void launch_color(const Grid& g, T* e, const T* r, const PoiCoef<T>& c, int color, T om,
                         const SolveCtrl* ctrl, T* eout, cudaStream_t s) {
  const unsigned gx = (unsigned)(((g.nx + 1) / 2 + 31) / 32), gy = (unsigned)((g.ny + 7) / 8);
  if (lv_big(g))
    launch_pdl(k_smooth<T, SM_ZP>, dim3(gx, gy, (unsigned)((g.nz + SM_ZP - 1) / SM_ZP)), dim3(32, 8), 0, s, e, r, g,
               c, color, om, ctrl, eout);
  else
    launch_pdl(k_smooth<T, 1>, dim3(gx, gy, (unsigned)g.nz), dim3(32, 8), 0, s, e, r, g, c, color, om, ctrl, eout);
}

template <int OP>
__global__ void __launch_bounds__(LV_TX * LV_TY) k_lvl25(float* __restrict__ e, const float* __restrict__ r,
                                                         float* __restrict__ t, Grid g, PoiCoef<float> c, float om,
                                                         int color, const SolveCtrl* ctrl) {
  pdl_enter();
  if (ctrl->done) return;
  constexpr int TX = LV_TX, TY = LV_TY, SW = TX + 2;
  __shared__ float tile[2][(TY + 2) * SW];
  const float* F = OP == 1 ? r : e;  // the field the operator acts on
  const int tx = threadIdx.x, ty = threadIdx.y, th = ty * TX + tx;
  const int i0 = blockIdx.x * TX, j0 = blockIdx.y * TY;
  const int i = i0 + tx, j = j0 + ty;
  const bool valid = i < g.nx && j < g.ny;
  const int k0 = blockIdx.z * LV_KC, k1 = min(k0 + LV_KC, g.nz);
  const long long sz = g.sz();
  bool f;
  const int cxy = ghost(i, g.nx, g.bc[0], &f) + g.nx * ghost(j, g.ny, g.bc[1], &f);
  // halo cell of this thread (th < 2 (TX + TY)): left, right, below, above
  const bool hon = th < 2 * (TX + TY);
  int hi, hj, hidx;
  if (th < TY) { hi = i0 - 1; hj = j0 + th; hidx = (th + 1) * SW; }
  else if (th < 2 * TY) { hi = i0 + TX; hj = j0 + th - TY; hidx = (th - TY + 1) * SW + TX + 1; }
  else if (th < 2 * TY + TX) { hi = i0 + th - 2 * TY; hj = j0 - 1; hidx = th - 2 * TY + 1; }
  else { const int u = min(th - 2 * TY - TX, TX - 1); hi = i0 + u; hj = j0 + TY; hidx = (TY + 1) * SW + u + 1; }
  const int hxy = ghost(hi, g.nx, g.bc[0], &f) + g.nx * ghost(hj, g.ny, g.bc[1], &f);
  const int sc = (ty + 1) * SW + tx + 1;
  auto zoff = [&](int k) { return sz * ghost(k, g.nz, g.bc[2], &f); };
  const long long out0 = valid ? (long long)i + (long long)g.nx * j : 0;

  float pb = __ldg(F + zoff(k0 - 1) + cxy), pc = __ldg(F + zoff(k0) + cxy);
  float ptn = __ldg(F + zoff(k0 + 1) + cxy);
  float hv = hon ? __ldg(F + zoff(k0) + hxy) : 0.f;
  float rr = (OP != 1 && valid) ? __ldg(r + out0 + sz * k0) : 0.f;
  int buf = 0;
  for (int k = k0; k < k1; ++k) {
    const float pt = ptn;
    tile[buf][sc] = pc;
    if (hon) tile[buf][hidx] = hv;
    const float rcur = rr;
    if (k + 1 < k1) {
      ptn = __ldg(F + zoff(k + 2) + cxy);
      if (hon) hv = __ldg(F + zoff(k + 1) + hxy);
      if (OP != 1 && valid) rr = __ldg(r + out0 + sz * (k + 1));
    }
    __syncthreads();
    if (valid) {
      const float* T0 = tile[buf];
      const long long q = out0 + sz * k;
      const bool mine = ((i + j + k + color) & 1) == 0;
      if (OP == 0) {
        if (mine) {
          const float s = c.ox * (T0[sc - 1] + T0[sc + 1]) + c.oy * (T0[sc - SW] + T0[sc + SW]) + c.oz * (pb + pt);
          const float en = (rcur - s) * c.invA;
          e[q] = pc + om * (en - pc);
        }
      } else if (OP == 1) {
        if (((i + j + k) & 1) == 0) {
          e[q] = om * (pc * c.invA);
        } else {
          const float s = c.ox * (T0[sc - 1] + T0[sc + 1]) + c.oy * (T0[sc - SW] + T0[sc + SW]) + c.oz * (pb + pt);
          e[q] = om * ((pc - om * (s * c.invA)) * c.invA);
        }
      } else {
        const float s = c.ox * (T0[sc - 1] + T0[sc + 1]) + c.oy * (T0[sc - SW] + T0[sc + SW]) + c.oz * (pb + pt);
        t[q] = rcur - (s + c.A * pc);
      }
    }
    pb = pc;
    pc = pt;
    buf ^= 1;
  }
}

// OP 1 and 2 of k_lvl25 with two x-adjacent points per thread, for a level
// whose nx is a multiple of 64: a block owns a 64 x 8 column, the pair's
// values come and go as float2, the field's plane lands in a shared tile of
// 68 x 10 cells (column 1 the left halo, the pairs at even columns 2 ..
// 65, column 66 the right halo; the tile of k_resid25p).  The same
// expressions in the same order as k_lvl25: the same bits.
constexpr int LP_TX = 32, LP_TY = 8, LP_KC = 16, LP_SW = 2 * LP_TX + 4;
static inline dim3 lp_grid(const Grid& g) {
  return dim3(g.nx / (2 * LP_TX), (g.ny + LP_TY - 1) / LP_TY, (g.nz + LP_KC - 1) / LP_KC);
}
template <int OP>
__global__ void __launch_bounds__(LP_TX * LP_TY) k_lvl25p(float* __restrict__ e, const float* __restrict__ r,
                                                          float* __restrict__ t, Grid g, PoiCoef<float> c, float om,
                                                          const SolveCtrl* ctrl) {
  pdl_enter();
  if (ctrl->done) return;
  constexpr int TX = LP_TX, TY = LP_TY, SW = LP_SW, PLN = (TY + 2) * SW;
  __shared__ float tile[2][PLN];
  const float* F = OP == 1 ? r : e;
  const int tx = threadIdx.x, ty = threadIdx.y, th = ty * TX + tx;
  const int i0 = blockIdx.x * 2 * TX, j0 = blockIdx.y * TY;
  const int ia = i0 + 2 * tx, j = j0 + ty;
  const bool valid = j < g.ny;  // nx a multiple of 64: every pair is in the grid
  const int k0 = blockIdx.z * LP_KC, k1 = min(k0 + LP_KC, g.nz);
  const long long sz = g.sz();
  bool f;
  const int cxy = ia + g.nx * ghost(j, g.ny, g.bc[1], &f);
  const bool hon = th < 2 * (TY + 2 * TX);
  int hi, hj, hidx;
  if (th < TY) { hi = i0 - 1; hj = j0 + th; hidx = (th + 1) * SW + 1; }
  else if (th < 2 * TY) { hi = i0 + 2 * TX; hj = j0 + th - TY; hidx = (th - TY + 1) * SW + 2 * TX + 2; }
  else if (th < 2 * TY + 2 * TX) { hi = i0 + th - 2 * TY; hj = j0 - 1; hidx = th - 2 * TY + 2; }
  else { const int u = min(th - 2 * TY - 2 * TX, 2 * TX - 1); hi = i0 + u; hj = j0 + TY; hidx = (TY + 1) * SW + u + 2; }
  const int hxy = ghost(hi, g.nx, g.bc[0], &f) + g.nx * ghost(hj, g.ny, g.bc[1], &f);
  const int sc = (ty + 1) * SW + 2 * tx + 2;
  auto zoff = [&](int k) { return sz * ghost(k, g.nz, g.bc[2], &f); };
  const long long out0 = valid ? (long long)ia + (long long)g.nx * j : 0;
  auto ld2f = [&](const float* b, long long q) { return __ldg(reinterpret_cast<const float2*>(b + q)); };

  float2 pb = ld2f(F, zoff(k0 - 1) + cxy), pc = ld2f(F, zoff(k0) + cxy), ptn = ld2f(F, zoff(k0 + 1) + cxy);
  float hv = hon ? __ldg(F + zoff(k0) + hxy) : 0.f;
  float2 rr = (OP == 2 && valid) ? ld2f(r, out0 + sz * k0) : make_float2(0.f, 0.f);
  int buf = 0;
  for (int k = k0; k < k1; ++k) {
    const float2 pt = ptn;
    *reinterpret_cast<float2*>(&tile[buf][sc]) = pc;
    if (hon) tile[buf][hidx] = hv;
    const float2 rcur = rr;
    if (k + 1 < k1) {
      ptn = ld2f(F, zoff(k + 2) + cxy);
      if (hon) hv = __ldg(F + zoff(k + 1) + hxy);
      if (OP == 2 && valid) rr = ld2f(r, out0 + sz * (k + 1));
    }
    __syncthreads();
    if (valid) {
      const float* T0 = tile[buf];
      float o[2];
#pragma unroll
      for (int q2 = 0; q2 < 2; ++q2) {
        const int q = sc + q2;
        const float vc = q2 ? pc.y : pc.x, vb = q2 ? pb.y : pb.x, vt = q2 ? pt.y : pt.x;
        const float s = c.ox * (T0[q - 1] + T0[q + 1]) + c.oy * (T0[q - SW] + T0[q + SW]) + c.oz * (vb + vt);
        if (OP == 1) {
          if (((ia + q2 + j + k) & 1) == 0) o[q2] = om * (vc * c.invA);
          else o[q2] = om * ((vc - om * (s * c.invA)) * c.invA);
        } else {
          o[q2] = (q2 ? rcur.y : rcur.x) - (s + c.A * vc);
        }
      }
      *reinterpret_cast<float2*>((OP == 1 ? e : t) + out0 + sz * k) = make_float2(o[0], o[1]);
    }
    pb = pc;
    pc = pt;
    buf ^= 1;
  }
}

// `n` red-black sweeps of A e = r with relaxation om, in place on e
template <class T>
static void smooth_sweeps(const MGLevel& L, T* e, const T* r, const PoiCoef<T>& c, T om, int n,
                          const SolveCtrl* ctrl, cudaStream_t s, long long* nl) {
  // (a colour pass stays one-pass: its 2.5D form, OP 0 of k_lvl25, loads
  // the whole plane for half its points and measured 85 against 73 us at
  // 512 x 256 x 256)
  for (int q = 0; q < n; ++q)
    for (int color = 0; color < 2; ++color)
      launch_color<T>(L.g, e, r, c, color, om, ctrl, (T*)nullptr, s);
  *nl += 2 * n;
}
// the first sweep from e = 0 and the residual t = r - A e of a level
template <class T>
static void smooth_first(const MGLevel& L, T* e, const T* r, const PoiCoef<T>& c, T om, const SolveCtrl* ctrl,
                         cudaStream_t s) {
  if constexpr (sizeof(T) == 4) {
    if (lv_big(L.g) && !L.plain) {
      if (L.g.nx % (2 * LP_TX) == 0)
        launch_pdl(k_lvl25p<1>, lp_grid(L.g), dim3(LP_TX, LP_TY), 0, s, (float*)e, (const float*)r, (float*)nullptr,
                   L.g, c, (float)om, ctrl);
      else
        launch_pdl(k_lvl25<1>, lv_grid(L.g), dim3(LV_TX, LV_TY), 0, s, (float*)e, (const float*)r, (float*)nullptr,
                   L.g, c, (float)om, 0, ctrl);
      return;
    }
  }
  launch_pdl(k_smooth_first<T>, dim3((L.g.nx + 31) / 32, (L.g.ny + 7) / 8, L.g.nz), dim3(32, 8), 0, s, e, r, L.g, c,
             om, ctrl);
}

template <class T>
__global__ void __launch_bounds__(256) k_resid(const T* __restrict__ e, const T* __restrict__ r,
                                               T* __restrict__ t, Grid g, PoiCoef<T> c,
                                               const SolveCtrl* ctrl) {
  pdl_enter();
  if (ctrl->done) return;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  const int k = blockIdx.z;
  if (i >= g.nx || j >= g.ny) return;
  const int q = idx3(g, i, j, k);
  t[q] = r[q] - (lap6<T>(e, q, nb6(g, i, j, k), c) + c.A * e[q]);
}

template <class T>
static void level_resid(const MGLevel& L, const T* e, const T* r, T* t, const PoiCoef<T>& c, const SolveCtrl* ctrl,
                        cudaStream_t s) {
  if constexpr (sizeof(T) == 4) {
    if (lv_big(L.g) && !L.plain) {
      if (L.g.nx % (2 * LP_TX) == 0)
        launch_pdl(k_lvl25p<2>, lp_grid(L.g), dim3(LP_TX, LP_TY), 0, s, (float*)e, (const float*)r, (float*)t, L.g, c,
                   1.f, ctrl);
      else
        launch_pdl(k_lvl25<2>, lv_grid(L.g), dim3(LV_TX, LV_TY), 0, s, (float*)e, (const float*)r, (float*)t, L.g, c,
                   1.f, 0, ctrl);
      return;
    }
  }
  launch_pdl(k_resid<T>, dim3((L.g.nx + 31) / 32, (L.g.ny + 7) / 8, L.g.nz), dim3(32, 8), 0, s, e, r, t, L.g, c, ctrl);
}

struct Coarsen {
  int c[3];
};

// fine index of coarse index I offset by o along an axis (ghost-mapped)
__device__ __forceinline__ int fine_of(int I, int o, int nf, int bc, int coarsened) {
  if (!coarsened) return I;
  int m = 2 * I + o;
  if (m < 0) m = bc == AX_PERIODIC ? m + nf : -m;
  else if (m >= nf) m = bc == AX_PERIODIC ? m - nf : 2 * (nf - 1) - m;
  return m;
}

// full weighting: tensor product of (1/4, 1/2, 1/4) on every coarsened axis
template <class T>
__global__ void __launch_bounds__(256) k_restrict(const T* __restrict__ tf, T* __restrict__ rc, Grid gf,
                                                  Grid gc, Coarsen cz, const SolveCtrl* ctrl) {
  pdl_enter();
  if (ctrl->done) return;
  const int I = blockIdx.x * blockDim.x + threadIdx.x;
  const int J = blockIdx.y * blockDim.y + threadIdx.y;
  const int K = blockIdx.z;
  if (I >= gc.nx || J >= gc.ny) return;
  T acc = (T)0;
  const int lo0 = cz.c[0] ? -1 : 0, lo1 = cz.c[1] ? -1 : 0, lo2 = cz.c[2] ? -1 : 0;
  for (int oz = lo2; oz <= -lo2; ++oz) {
    const int kf = fine_of(K, oz, gf.nz, gf.bc[2], cz.c[2]);
    const T wz = cz.c[2] ? (oz == 0 ? (T)0.5 : (T)0.25) : (T)1;
    for (int oy = lo1; oy <= -lo1; ++oy) {
      const int jf = fine_of(J, oy, gf.ny, gf.bc[1], cz.c[1]);
      const T wy = cz.c[1] ? (oy == 0 ? (T)0.5 : (T)0.25) : (T)1;
      for (int ox = lo0; ox <= -lo0; ++ox) {
        const int i_f = fine_of(I, ox, gf.nx, gf.bc[0], cz.c[0]);
        const T wx = cz.c[0] ? (ox == 0 ? (T)0.5 : (T)0.25) : (T)1;
        acc += wz * wy * wx * tf[(long long)i_f + gf.sy() * jf + gf.sz() * kf];
      }
    }
  }
  rc[(long long)I + gc.sy() * J + gc.sz() * K] = acc;
}

// full weighting when every axis is coarsened: the 3 x 3 x 3 fine block of
// each coarse point, offsets resolved once per axis, separable weights
// A thread marches KZ coarse planes along z: the fine plane 2K + 1, the
// last of coarse plane K's three, is the first of K + 1's, so its nine
// values stay in registers (18 loads per coarse point instead of 27).  The
// sum of every coarse point still runs over its 27 terms in the same order.
// Large coarse grids take RF_KZ planes per thread; small ones, whose
// restriction is latency-bound, one.
constexpr int RF_KZ = 4;
template <class T, int KZ>
__global__ void __launch_bounds__(256) k_restrict_full(const T* __restrict__ tf, T* __restrict__ rc, Grid gf,
                                                       Grid gc, const SolveCtrl* ctrl) {
  pdl_enter();
  if (ctrl->done) return;
  const int I = blockIdx.x * blockDim.x + threadIdx.x;
  const int J = blockIdx.y * blockDim.y + threadIdx.y;
  const int K0 = blockIdx.z * KZ;
  if (I >= gc.nx || J >= gc.ny) return;
  int xo[3], yo[3];
#pragma unroll
  for (int o = 0; o < 3; ++o) {
    xo[o] = fine_of(I, o - 1, gf.nx, gf.bc[0], 1);
    yo[o] = gf.nx * fine_of(J, o - 1, gf.ny, gf.bc[1], 1);
  }
  const T w[3] = {(T)0.25, (T)0.5, (T)0.25};
  const long long sz = (long long)gf.nx * gf.ny;
  auto plane = [&](int kf, T v[3][3]) {
    const T* base = tf + sz * kf;
#pragma unroll
    for (int oy = 0; oy < 3; ++oy)
#pragma unroll
      for (int ox = 0; ox < 3; ++ox) v[oy][ox] = __ldg(base + yo[oy] + xo[ox]);
  };
  T pl[3][3][3];  // the fine planes 2K - 1, 2K, 2K + 1
  plane(fine_of(K0, -1, gf.nz, gf.bc[2], 1), pl[0]);
  for (int K = K0; K < K0 + KZ && K < gc.nz; ++K) {
    if (K > K0) {
#pragma unroll
      for (int oy = 0; oy < 3; ++oy)
#pragma unroll
        for (int ox = 0; ox < 3; ++ox) pl[0][oy][ox] = pl[2][oy][ox];
    }
    plane(fine_of(K, 0, gf.nz, gf.bc[2], 1), pl[1]);
    plane(fine_of(K, 1, gf.nz, gf.bc[2], 1), pl[2]);
    T acc = (T)0;
#pragma unroll
    for (int oz = 0; oz < 3; ++oz)
#pragma unroll
      for (int oy = 0; oy < 3; ++oy)
#pragma unroll
        for (int ox = 0; ox < 3; ++ox) acc += w[oz] * w[oy] * w[ox] * pl[oz][oy][ox];
    rc[idx3(gc, I, J, K)] = acc;
  }
}

// coarse indices and weights of fine index i along one axis
__device__ __forceinline__ void prol_axis(int i, int nc, int bc, int coarsened, int* c0, int* c1, float* w1) {
  if (!coarsened) { *c0 = i; *c1 = i; *w1 = 0.f; return; }
  if ((i & 1) == 0) { *c0 = i >> 1; *c1 = *c0; *w1 = 0.f; return; }
  *c0 = i >> 1;
  int hi = *c0 + 1;
  if (hi >= nc) hi = bc == AX_PERIODIC ? 0 : nc - 1;
  *c1 = hi;
  *w1 = 0.5f;
}

template <class T>
__global__ void __launch_bounds__(256) k_prolong(T* __restrict__ ef, const T* __restrict__ ec, Grid gf,
                                                 Grid gc, Coarsen cz, const SolveCtrl* ctrl) {
  pdl_enter();
  if (ctrl->done) return;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  const int k = blockIdx.z;
  if (i >= gf.nx || j >= gf.ny) return;
  int x0, x1, y0, y1, z0, z1;
  float wx, wy, wz;
  prol_axis(i, gc.nx, gf.bc[0], cz.c[0], &x0, &x1, &wx);
  prol_axis(j, gc.ny, gf.bc[1], cz.c[1], &y0, &y1, &wy);
  prol_axis(k, gc.nz, gf.bc[2], cz.c[2], &z0, &z1, &wz);
  const T ax0 = (T)(1.f - wx), ax1 = (T)wx, ay0 = (T)(1.f - wy), ay1 = (T)wy, az0 = (T)(1.f - wz), az1 = (T)wz;
  auto at = [&](int a, int b, int c) { return ec[(long long)a + gc.sy() * b + gc.sz() * c]; };
  T v = az0 * (ay0 * (ax0 * at(x0, y0, z0) + ax1 * at(x1, y0, z0)) + ay1 * (ax0 * at(x0, y1, z0) + ax1 * at(x1, y1, z0))) +
        az1 * (ay0 * (ax0 * at(x0, y0, z1) + ax1 * at(x1, y0, z1)) + ay1 * (ax0 * at(x0, y1, z1) + ax1 * at(x1, y1, z1)));
  ef[(long long)i + gf.sy() * j + gf.sz() * k] += v;
}

// Prolongation + add with one thread per coarse cell (I, J, K): its 8 coarse
// corners are read once and the 2 x 2 x 2 fine points (2I+a, 2J+b, 2K+c)
// are updated; used when all three axes are coarsened.
__device__ __forceinline__ int prol_hi(int I, int nc, int bc) {
  return I + 1 < nc ? I + 1 : (bc == AX_PERIODIC ? 0 : nc - 1);
}

template <class T>
__global__ void __launch_bounds__(256) k_prolong_cell(T* __restrict__ ef, const T* __restrict__ ec, Grid gf,
                                                      Grid gc, const SolveCtrl* ctrl) {
  pdl_enter();
  if (ctrl->done) return;
  const int I = blockIdx.x * blockDim.x + threadIdx.x;
  const int J = blockIdx.y * blockDim.y + threadIdx.y;
  const int K = blockIdx.z;
  if (I >= gc.nx || J >= gc.ny) return;
  const int I1 = prol_hi(I, gc.nx, gf.bc[0]), J1 = prol_hi(J, gc.ny, gf.bc[1]), K1 = prol_hi(K, gc.nz, gf.bc[2]);
  auto at = [&](int a, int b, int c) { return __ldg(ec + (long long)a + gc.sy() * b + gc.sz() * c); };
  const T c000 = at(I, J, K), c100 = at(I1, J, K), c010 = at(I, J1, K), c110 = at(I1, J1, K);
  const T c001 = at(I, J, K1), c101 = at(I1, J, K1), c011 = at(I, J1, K1), c111 = at(I1, J1, K1);
  const T h = (T)0.5;
  // values on the 2 x 2 x 2 fine points, x fastest
  const T x00 = h * (c000 + c100), x10 = h * (c010 + c110), x01 = h * (c001 + c101), x11 = h * (c011 + c111);
  const T v[2][2][2] = {{{c000, x00}, {h * (c000 + c010), h * (x00 + x10)}},
                        {{h * (c000 + c001), h * (x00 + x01)},
                         {h * (h * (c000 + c010) + h * (c001 + c011)), h * (h * (x00 + x10) + h * (x01 + x11))}}};
  for (int dc = 0; dc < 2; ++dc) {
    const int kf = 2 * K + dc;
    if (kf >= gf.nz) break;
    for (int db = 0; db < 2; ++db) {
      const int jf = 2 * J + db;
      if (jf >= gf.ny) break;
      const long long row = gf.sy() * jf + gf.sz() * kf;
      const int i0f = 2 * I;
      ef[row + i0f] += v[dc][db][0];
      if (i0f + 1 < gf.nx) ef[row + i0f + 1] += v[dc][db][1];
    }
  }
}

// ---------------------------------------------------------------------------
// Non-nested coarsening (MGLevel::coarsen mode 2) of an axis that cannot be
// halved onto a subset of its nodes: an even free-slip axis (n nodes, the
// ends on the walls) goes to m = (n/2) | 1 nodes spanning the same length,
// an odd periodic axis (period n) to m = ((n+1)/2) & ~1 nodes per period.
// With rho = H/h = (n-1)/(m-1) (free-slip) or n/m (periodic), fine node j
// lies at coarse coordinate s_j = j / rho.  The prolongation interpolates
// linearly there; the restriction is its transpose over the mirror- or
// wrap-extended fine grid, scaled by 1/rho (for rho = 2 that is full
// weighting with the same ghost rule).  Levels below are nested again.
// 1/rho = num/den; rho <= 2.5, so a coarse node takes at most 5 fine nodes.
// ---------------------------------------------------------------------------
constexpr int NN_MAXT = 5;

// Per-axis constants of a non-nested transfer, computed on the host so that
// no kernel divides: the mode of each axis and, for mode 2, the weight scale
// num / den^2 of the restriction and 1 / den of the prolongation.
template <class T>
struct NNXfer {
  int c[3];
  T wsc[3], invden[3];
};

__host__ __device__ __forceinline__ void nn_ratio(int nf, int nc, int bc, int* num, int* den) {
  if (bc == AX_PERIODIC) { *num = nc; *den = nf; }
  else { *num = nc - 1; *den = nf - 1; }
}

__device__ __forceinline__ int floor_div(int a, int b) { return a >= 0 ? a / b : -((-a + b - 1) / b); }

// restriction taps of coarse index J along one axis: NN_MAXT slots of fine
// indices and weights in increasing fine order, unused slots with weight 0
// (and a valid index), so that the sums below run over a fixed, unrolled
// count with the taps in registers: the zero terms add exact zeros
template <class T>
__device__ __forceinline__ void restrict_taps(int J, int nf, int nc, int bc, int mode, T wsc, int (&idx)[NN_MAXT],
                                              T (&w)[NN_MAXT]) {
#pragma unroll
  for (int o = 0; o < NN_MAXT; ++o) {
    idx[o] = 0;
    w[o] = (T)0;
  }
  if (mode == 0) {
    idx[0] = J;
    w[0] = (T)1;
    return;
  }
  if (mode == 1) {
#pragma unroll
    for (int o = 0; o < 3; ++o) {
      idx[o] = fine_of(J, o - 1, nf, bc, 1);
      w[o] = o == 1 ? (T)0.5 : (T)0.25;
    }
    return;
  }
  int num, den;
  nn_ratio(nf, nc, bc, &num, &den);
  // fine je with |je num - J den| < den, weight (den - d) num / den^2,
  // mapped back by the ghost rule
  const int lo = floor_div(J * den - den, num) + 1, hi = floor_div(J * den + den - 1, num);
#pragma unroll
  for (int o = 0; o < NN_MAXT; ++o) {
    const int je = lo + o;
    const int d = abs(je * num - J * den);
    if (je > hi || d >= den) continue;
    int j = je;
    if (bc == AX_PERIODIC) j = j < 0 ? j + nf : (j >= nf ? j - nf : j);
    else if (j < 0) j = -j;
    else if (j > nf - 1) j = 2 * (nf - 1) - j;
    idx[o] = j;
    w[o] = (T)(den - d) * wsc;
  }
}

// One thread per coarse point; the taps are summed along x, then y, then z.
template <class T>
__global__ void __launch_bounds__(256) k_restrict_nn(const T* __restrict__ tf, T* __restrict__ rc, Grid gf, Grid gc,
                                                     NNXfer<T> nn, const SolveCtrl* ctrl) {
  pdl_enter();
  if (ctrl->done) return;
  const int I = blockIdx.x * blockDim.x + threadIdx.x;
  const int J = blockIdx.y * blockDim.y + threadIdx.y;
  const int K = blockIdx.z;
  if (I >= gc.nx || J >= gc.ny) return;
  int xi[NN_MAXT], yi[NN_MAXT], zi[NN_MAXT];
  T xw[NN_MAXT], yw[NN_MAXT], zw[NN_MAXT];
  restrict_taps<T>(I, gf.nx, gc.nx, gf.bc[0], nn.c[0], nn.wsc[0], xi, xw);
  restrict_taps<T>(J, gf.ny, gc.ny, gf.bc[1], nn.c[1], nn.wsc[1], yi, yw);
  restrict_taps<T>(K, gf.nz, gc.nz, gf.bc[2], nn.c[2], nn.wsc[2], zi, zw);
  T acc = (T)0;
#pragma unroll
  for (int a = 0; a < NN_MAXT; ++a) {
    if (zw[a] == (T)0) continue;
    T accy = (T)0;
#pragma unroll
    for (int b = 0; b < NN_MAXT; ++b) {
      if (yw[b] == (T)0) continue;
      const T* row = tf + gf.sz() * zi[a] + gf.sy() * yi[b];
      T accx = (T)0;
#pragma unroll
      for (int q = 0; q < NN_MAXT; ++q)
        if (xw[q] != (T)0) accx += xw[q] * __ldg(row + xi[q]);
      accy += yw[b] * accx;
    }
    acc += zw[a] * accy;
  }
  rc[idx3(gc, I, J, K)] = acc;
}

// The same restriction for a level whose z axis is halved (taps 2K - 1, 2K,
// 2K + 1): a thread marches its (I, J) column over NNZ_KC coarse planes and
// forms the x-y sum of each fine plane once, so that coarse planes K and
// K + 1 share the sum of fine plane 2K + 1.  Each coarse value is the same
// expression in the same order as k_restrict_nn's: the results are identical.
constexpr int NNZ_KC = 8;
template <class T>
__global__ void __launch_bounds__(256) k_restrict_nnz(const T* __restrict__ tf, T* __restrict__ rc, Grid gf,
                                                      Grid gc, NNXfer<T> nn, const SolveCtrl* ctrl) {
  pdl_enter();
  if (ctrl->done) return;
  const int I = blockIdx.x * blockDim.x + threadIdx.x;
  const int J = blockIdx.y * blockDim.y + threadIdx.y;
  const int K0 = blockIdx.z * NNZ_KC, K1 = min(K0 + NNZ_KC, gc.nz);
  if (I >= gc.nx || J >= gc.ny) return;
  int xi[NN_MAXT], yi[NN_MAXT];
  T xw[NN_MAXT], yw[NN_MAXT];
  restrict_taps<T>(I, gf.nx, gc.nx, gf.bc[0], nn.c[0], nn.wsc[0], xi, xw);
  restrict_taps<T>(J, gf.ny, gc.ny, gf.bc[1], nn.c[1], nn.wsc[1], yi, yw);
  auto plane = [&](int k) {
    T accy = (T)0;
#pragma unroll
    for (int b = 0; b < NN_MAXT; ++b) {
      if (yw[b] == (T)0) continue;
      const T* row = tf + gf.sz() * k + gf.sy() * yi[b];
      T accx = (T)0;
#pragma unroll
      for (int q = 0; q < NN_MAXT; ++q)
        if (xw[q] != (T)0) accx += xw[q] * __ldg(row + xi[q]);
      accy += yw[b] * accx;
    }
    return accy;
  };
  T s0 = plane(fine_of(K0, -1, gf.nz, gf.bc[2], 1));
  for (int K = K0; K < K1; ++K) {
    const T s1 = plane(fine_of(K, 0, gf.nz, gf.bc[2], 1));
    const T s2 = plane(fine_of(K, 1, gf.nz, gf.bc[2], 1));
    T acc = (T)0;
    acc += (T)0.25 * s0;
    acc += (T)0.5 * s1;
    acc += (T)0.25 * s2;
    rc[idx3(gc, I, J, K)] = acc;
    s0 = s2;  // fine plane 2K + 1 is the first tap of coarse plane K + 1
  }
}

// Prolongation unit of one axis: a coarse cell (fine 2u and 2u + 1) on a
// halved axis, one fine point otherwise; its two coarse corners and, per
// fine point, the weight of the second corner.
template <class T>
struct PUnit {
  int f0, nf, c0, c1;
  T w[2];
};

template <class T>
__device__ __forceinline__ PUnit<T> prol_unit(int u, int nfine, int nc, int bc, int mode, T invden) {
  PUnit<T> r;
  r.w[0] = r.w[1] = (T)0;
  if (mode == 1) {
    r.f0 = 2 * u;
    r.nf = 2 * u + 1 < nfine ? 2 : 1;
    r.c0 = u;
    r.c1 = prol_hi(u, nc, bc);
    r.w[1] = (T)0.5;
  } else if (mode == 0) {
    r.f0 = u;
    r.nf = 1;
    r.c0 = r.c1 = u;
  } else {
    int num, den;
    nn_ratio(nfine, nc, bc, &num, &den);
    const int q = u * num;  // < 2^31: n^2 / 2 for n < 65536
    r.f0 = u;
    r.nf = 1;
    r.c0 = q / den;
    r.c1 = prol_hi(r.c0, nc, bc);
    r.w[0] = (T)(q - r.c0 * den) * invden;
  }
  return r;
}

__host__ __device__ __forceinline__ int prol_units(int nfine, int nc, int mode) { return mode == 1 ? nc : nfine; }

// One thread per prolongation unit (up to 2 x 2 x 2 fine points): the 8
// coarse corners are read once and interpolated along x, then y, then z.
template <class T>
__global__ void __launch_bounds__(256) k_prolong_nn(T* __restrict__ ef, const T* __restrict__ ec, Grid gf, Grid gc,
                                                    NNXfer<T> nn, const SolveCtrl* ctrl) {
  pdl_enter();
  if (ctrl->done) return;
  const int ux = blockIdx.x * blockDim.x + threadIdx.x;
  const int uy = blockIdx.y * blockDim.y + threadIdx.y;
  const int uz = blockIdx.z;
  if (ux >= prol_units(gf.nx, gc.nx, nn.c[0]) || uy >= prol_units(gf.ny, gc.ny, nn.c[1])) return;
  const PUnit<T> ax = prol_unit<T>(ux, gf.nx, gc.nx, gf.bc[0], nn.c[0], nn.invden[0]);
  const PUnit<T> ay = prol_unit<T>(uy, gf.ny, gc.ny, gf.bc[1], nn.c[1], nn.invden[1]);
  const PUnit<T> az = prol_unit<T>(uz, gf.nz, gc.nz, gf.bc[2], nn.c[2], nn.invden[2]);
  auto at = [&](int a, int b, int c) { return __ldg(ec + (long long)a + gc.sy() * b + gc.sz() * c); };
  T c[2][2][2];  // [z][y][x] corner
#pragma unroll
  for (int zc = 0; zc < 2; ++zc)
#pragma unroll
    for (int yc = 0; yc < 2; ++yc) {
      const int cz = zc ? az.c1 : az.c0, cy = yc ? ay.c1 : ay.c0;
      c[zc][yc][0] = at(ax.c0, cy, cz);
      c[zc][yc][1] = at(ax.c1, cy, cz);
    }
#pragma unroll
  for (int px = 0; px < 2; ++px) {
    if (px >= ax.nf) break;
    T vy[2][2];  // [y point][z corner]
#pragma unroll
    for (int zc = 0; zc < 2; ++zc) {
      const T v0 = c[zc][0][0] + ax.w[px] * (c[zc][0][1] - c[zc][0][0]);
      const T v1 = c[zc][1][0] + ax.w[px] * (c[zc][1][1] - c[zc][1][0]);
#pragma unroll
      for (int py = 0; py < 2; ++py) vy[py][zc] = v0 + ay.w[py] * (v1 - v0);
    }
#pragma unroll
    for (int py = 0; py < 2; ++py) {
      if (py >= ay.nf) break;
#pragma unroll
      for (int pz = 0; pz < 2; ++pz) {
        if (pz >= az.nf) break;
        const T v = vy[py][0] + az.w[pz] * (vy[py][1] - vy[py][0]);
        ef[(long long)(ax.f0 + px) + gf.sy() * (ay.f0 + py) + gf.sz() * (az.f0 + pz)] += v;
      }
    }
  }
}

// Coarsest level: one block, shared memory, weighted mean of r removed,
// `sweeps` red-black Gauss-Seidel sweeps from e = 0.  Each thread resolves
// once the cells it updates in each colour (the colour's cells of a (j, k)
// row are i = 2m + ((colour + j + k) & 1)) and their neighbours' offsets,
// so a sweep is loads, the update and one barrier per colour.
constexpr int COARSE_MAXC = 3;  // cells per thread and colour: 3 x 1024 >= the colour slots of coarse_max()
template <class T>
__global__ void __launch_bounds__(1024) k_coarse(T* __restrict__ e, const T* __restrict__ r, Grid g,
                                                 PoiCoef<T> c, int sweeps, const SolveCtrl* ctrl) {
  pdl_enter();
  if (ctrl->done) return;
  __shared__ T se[coarse_max<T>()];
  __shared__ T sr[coarse_max<T>()];
  __shared__ double red[2][32];
  const int n = (int)g.n;
  const int t = threadIdx.x, nt = blockDim.x;
  double a = 0.0, b = 0.0;
  for (int q = t; q < n; q += nt) {
    const int i = q % g.nx, j = (q / g.nx) % g.ny, k = q / (g.nx * g.ny);
    const double w = wnode(g, i, j, k);
    sr[q] = r[q];
    se[q] = (T)0;
    a += w * (double)r[q];
    b += w;
  }
  a = warp_sum(a);
  b = warp_sum(b);
  if ((t & 31) == 0) { red[0][t >> 5] = a; red[1][t >> 5] = b; }
  __syncthreads();
  if (t < 32) {
    a = t < (nt + 31) / 32 ? red[0][t] : 0.0;
    b = t < (nt + 31) / 32 ? red[1][t] : 0.0;
    a = warp_sum(a);
    b = warp_sum(b);
    if (t == 0) red[0][0] = a / b;
  }
  __syncthreads();
  const T mean = (T)red[0][0];
  for (int q = t; q < n; q += nt) sr[q] -= mean;
  // this thread's cells: centre and the neighbours w, e, s, n, b, t (lap_nb's remap)
  int cell[2][COARSE_MAXC][7];
  const int nxh = (g.nx + 1) / 2;
#pragma unroll
  for (int col = 0; col < 2; ++col)
#pragma unroll
    for (int u = 0; u < COARSE_MAXC; ++u) {
      const int id = t + u * nt, row = id / nxh, m = id - row * nxh;
      const int j = row % g.ny, k = row / g.ny;
      const int i = 2 * m + ((col + j + k) & 1);
      int* cq = cell[col][u];
      cq[0] = -1;
      if (k < g.nz && i < g.nx) {
        const int sy = g.nx, sz = g.nx * g.ny;
        cq[0] = i + sy * j + sz * k;
        cq[1] = nb_lo(i, g.nx, g.bc[0]) + sy * j + sz * k;
        cq[2] = nb_hi(i, g.nx, g.bc[0]) + sy * j + sz * k;
        cq[3] = i + sy * nb_lo(j, g.ny, g.bc[1]) + sz * k;
        cq[4] = i + sy * nb_hi(j, g.ny, g.bc[1]) + sz * k;
        cq[5] = i + sy * j + sz * nb_lo(k, g.nz, g.bc[2]);
        cq[6] = i + sy * j + sz * nb_hi(k, g.nz, g.bc[2]);
      }
    }
  __syncthreads();
  for (int s = 0; s < sweeps; ++s) {
#pragma unroll
    for (int col = 0; col < 2; ++col) {
#pragma unroll
      for (int u = 0; u < COARSE_MAXC; ++u) {
        const int* cq = cell[col][u];
        if (cq[0] < 0) continue;
        const T sn = c.ox * (se[cq[1]] + se[cq[2]]) + c.oy * (se[cq[3]] + se[cq[4]]) + c.oz * (se[cq[5]] + se[cq[6]]);
        se[cq[0]] = (sr[cq[0]] - sn) * c.invA;
      }
      __syncthreads();
    }
  }
  for (int q = t; q < n; q += nt) e[q] = se[q];
}

// whether k_coarse takes a level: it fits shared memory and every colour
// slot has a thread
template <class T>
static inline bool coarse_fits(const Grid& g) {
  return g.n <= coarse_max<T>() && (long long)((g.nx + 1) / 2) * g.ny * g.nz <= 1024LL * COARSE_MAXC;
}
// threads of k_coarse for a level: one per cell of the larger colour, at most 1024
static inline int coarse_threads(const Grid& g) {
  const long long slots = (long long)((g.nx + 1) / 2) * g.ny * g.nz;
  const long long nt = ((slots + 31) / 32) * 32;
  return (int)(nt < 1024 ? (nt < 32 ? 32 : nt) : 1024);
}

// p += e (FP64), max |e| into the control block.  Each thread handles
// UPD_PER consecutive-stride elements and keeps its max in the type of e, so
// the only FP64 work is the addition itself.
constexpr int UPD_PER = 8;

// PP: p is the double-float pair pp, updated by df_add_f (no FP64 operation)
template <class T, bool PP>
__global__ void __launch_bounds__(256) k_update(double* __restrict__ p, PPair pp, const T* __restrict__ e,
                                                long long n, SolveCtrl* ctrl) {
  pdl_enter();
  if (ctrl->done) return;
  const long long base = (long long)blockIdx.x * blockDim.x * UPD_PER + threadIdx.x;
  T m = (T)0;
#pragma unroll
  for (int u = 0; u < UPD_PER; ++u) {
    const long long q = base + (long long)u * blockDim.x;
    if (q < n) {
      const T ev = e[q];
      if constexpr (PP) {
        float h = pp.hi[q], l = pp.lo[q];
        df_add_f(h, l, (float)ev);
        pp.hi[q] = h;
        pp.lo[q] = l;
      } else {
        p[q] += to_t<double>(ev);
      }
      m = fmax(m, fabs(ev));
    }
  }
  double bm;
  if (sizeof(T) == 4) bm = (double)block_max_f((float)m);
  else bm = block_max((double)m);
  if (threadIdx.x == 0 && bm > 0.0) atomicMax(&ctrl->dmax_key, (unsigned long long)__double_as_longlong(bm));
}

// The black pass of the last post-smoothing sweep on the finest level
// fused with the pressure pair's update and max |e| (k_smooth colour 1,
// then k_update): a thread relaxes its black cell as k_smooth does and adds
// the correction of both cells of its pair 2 ih, 2 ih + 1 to the pair as
// k_update does, so the pair and the max are those of the two passes.  The
// black values are not stored: the cycle that updates the pressure is the
// outer iteration's last, and its correction is not read again.
// planes per thread of k_smooth_upd: all loads of a thread's planes are in
// flight together, and a block reduces and publishes its max once for them
constexpr int SU_ZP = 4;
__global__ void __launch_bounds__(256) k_smooth_upd(const float* __restrict__ e, const float* __restrict__ r, Grid g,
                                                    PoiCoef<float> c, float om, PPair pp, SolveCtrl* ctrl) {
  pdl_enter();
  if (ctrl->done) return;
  const int ih = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  const int kb = blockIdx.z * SU_ZP;
  float m = 0.f;
  if (j < g.ny && (g.nx & 1) == 0) {
    // even nx: the pair starts at an even offset, and the correction and
    // both planes of the pressure pair move as float2
    if (2 * ih < g.nx) {
      float2 e2[SU_ZP], h2[SU_ZP], l2[SU_ZP];
      float sl[SU_ZP], rq[SU_ZP];
#pragma unroll
      for (int u = 0; u < SU_ZP; ++u) {
        const int k = kb + u;
        if (k < g.nz) {
          const int par = (j + k + 1) & 1;
          const int q0 = idx3(g, 2 * ih, j, k), q = q0 + par;
          e2[u] = *reinterpret_cast<const float2*>(e + q0);
          sl[u] = lap6<float>(e, q, nb6(g, 2 * ih + par, j, k), c);
          rq[u] = r[q];
          h2[u] = *reinterpret_cast<const float2*>(pp.hi + q0);
          l2[u] = *reinterpret_cast<const float2*>(pp.lo + q0);
        }
      }
#pragma unroll
      for (int u = 0; u < SU_ZP; ++u) {
        const int k = kb + u;
        if (k < g.nz) {
          const int par = (j + k + 1) & 1;
          const int q0 = idx3(g, 2 * ih, j, k);
          const float ec = par ? e2[u].y : e2[u].x;
          const float en = (rq[u] - sl[u]) * c.invA;
          const float ev = ec + om * (en - ec);
          const float v0 = par ? e2[u].x : ev, v1 = par ? ev : e2[u].y;
          df_add_f(h2[u].x, l2[u].x, v0);
          df_add_f(h2[u].y, l2[u].y, v1);
          *reinterpret_cast<float2*>(pp.hi + q0) = h2[u];
          *reinterpret_cast<float2*>(pp.lo + q0) = l2[u];
          m = fmaxf(m, fmaxf(fabsf(v0), fabsf(v1)));
        }
      }
    }
  } else if (j < g.ny) {
    for (int k = kb; k < kb + SU_ZP && k < g.nz; ++k) {
      const int par = (j + k + 1) & 1;
      const int i = 2 * ih + par, io = 2 * ih + 1 - par;  // the black cell and its red partner
      if (io < g.nx) {
        const int qo = idx3(g, io, j, k);
        const float ev = e[qo];
        float h = pp.hi[qo], l = pp.lo[qo];
        df_add_f(h, l, ev);
        pp.hi[qo] = h;
        pp.lo[qo] = l;
        m = fmaxf(m, fabsf(ev));
      }
      if (i < g.nx) {
        const int q = idx3(g, i, j, k);
        const float sl = lap6<float>(e, q, nb6(g, i, j, k), c);
        const float ec = e[q];
        const float en = (r[q] - sl) * c.invA;
        const float ev = ec + om * (en - ec);
        float h = pp.hi[q], l = pp.lo[q];
        df_add_f(h, l, ev);
        pp.hi[q] = h;
        pp.lo[q] = l;
        m = fmaxf(m, fabsf(ev));
      }
    }
  }
  const float bm = block_max_f(m);
  if (threadIdx.x == 0 && threadIdx.y == 0 && bm > 0.f)
    atomicMax(&ctrl->dmax_key, (unsigned long long)__double_as_longlong((double)bm));
}
static dim3 su_grid(const Grid& g) {
  return dim3((unsigned)(((g.nx + 1) / 2 + 31) / 32), (g.ny + 7) / 8, (g.nz + SU_ZP - 1) / SU_ZP);
}

// the last post-smoothing sweep's two colour passes, the black one with the
// pressure pair's update (in place on e; one pass over the level fewer than
// the sweep and k_update: 1.8 % of the 512 x 256 x 256 mixing-layer step)
static void smooth_last_upd(const MGLevel& L, float* e, const float* r, const PoiCoef<float>& c, float om,
                            double* p, SolveCtrl* ctrl, cudaStream_t s, long long* nl) {
  launch_color<float>(L.g, e, r, c, 0, om, ctrl, (float*)nullptr, s);
  launch_pdl(k_smooth_upd, su_grid(L.g), dim3(32, 8), 0, s, (const float*)e, r, L.g, c, om, ppair(p, L.g.n), ctrl);
  *nl += 2;
}

__global__ void k_mg_control(SolveCtrl* c) {
  pdl_enter();
  if (c->done) return;
  const double dmax = __longlong_as_double((long long)c->dmax_key);
  c->dmax_key = 0ull;
  c->iter += 1;
  c->cycles += c->cycles_per_iter;
  c->dmax = dmax;
  // max |r| of this iteration's residual (before its correction was added)
  c->res_inf = __longlong_as_double((long long)c->res_key);
  c->res_key = 0ull;
  if (dmax < c->eps) { c->done = 1; c->status = ST_CONVERGED; return; }
  if (fabs(c->dmax_old - dmax) < c->eps / 1000.0) { c->done = 1; c->status = ST_STAGNATED; return; }
  c->dmax_old = dmax;
  if (c->iter >= c->kmax) { c->done = 1; c->status = ST_MAXIT; }
}

static inline dim3 g3(const Grid& g) { return dim3((g.nx + 31) / 32, (g.ny + 7) / 8, g.nz); }

// the host constants of a level's non-nested transfer
template <class T>
static NNXfer<T> nn_xfer(const MGLevel& L, const MGLevel& C) {
  NNXfer<T> x;
  for (int a = 0; a < 3; ++a) {
    x.c[a] = L.coarsen[a];
    int num = 1, den = 1;
    if (L.coarsen[a] == 2) nn_ratio(L.g.len(a), C.g.len(a), L.g.bc[a], &num, &den);
    x.wsc[a] = (T)((double)num / ((double)den * den));
    x.invden[a] = (T)(1.0 / den);
  }
  return x;
}

// Restriction of the fine level's tf into the coarse level's rc, and
// prolongation of the coarse ec added into the fine ef, with the kernel the
// level's coarsening calls for: every axis halved (one thread per coarse
// point or cell), some axes kept (generic), or a non-nested axis.
template <class T>
static void launch_restrict(const MGLevel& L, const MGLevel& C, const T* tf, T* rc, const SolveCtrl* ctrl,
                            cudaStream_t s) {
  Coarsen cz;
  for (int a = 0; a < 3; ++a) cz.c[a] = L.coarsen[a];
  const dim3 b(32, 8);
  if ((cz.c[0] == 2 || cz.c[1] == 2) && cz.c[2] == 1)
    launch_pdl(k_restrict_nnz<T>, dim3((C.g.nx + 31) / 32, (C.g.ny + 7) / 8, (C.g.nz + NNZ_KC - 1) / NNZ_KC), b, 0,
               s, tf, rc, L.g, C.g, nn_xfer<T>(L, C), ctrl);
  else if (cz.c[0] == 2 || cz.c[1] == 2 || cz.c[2] == 2)
    launch_pdl(k_restrict_nn<T>, g3(C.g), b, 0, s, tf, rc, L.g, C.g, nn_xfer<T>(L, C), ctrl);
  else if (cz.c[0] && cz.c[1] && cz.c[2] && C.g.n >= (1LL << 20))
    launch_pdl(k_restrict_full<T, RF_KZ>, dim3((C.g.nx + 31) / 32, (C.g.ny + 7) / 8, (C.g.nz + RF_KZ - 1) / RF_KZ), b,
               0, s, tf, rc, L.g, C.g, ctrl);
  else if (cz.c[0] && cz.c[1] && cz.c[2])
    launch_pdl(k_restrict_full<T, 1>, g3(C.g), b, 0, s, tf, rc, L.g, C.g, ctrl);
  else
    launch_pdl(k_restrict<T>, g3(C.g), b, 0, s, tf, rc, L.g, C.g, cz, ctrl);
}

template <class T>
static void launch_prolong_add(const MGLevel& L, const MGLevel& C, T* ef, const T* ec, const SolveCtrl* ctrl,
                               cudaStream_t s) {
  Coarsen cz;
  for (int a = 0; a < 3; ++a) cz.c[a] = L.coarsen[a];
  const dim3 b(32, 8);
  if (cz.c[0] == 2 || cz.c[1] == 2 || cz.c[2] == 2) {
    const dim3 gu((unsigned)((prol_units(L.g.nx, C.g.nx, cz.c[0]) + 31) / 32),
                  (unsigned)((prol_units(L.g.ny, C.g.ny, cz.c[1]) + 7) / 8), (unsigned)prol_units(L.g.nz, C.g.nz, cz.c[2]));
    launch_pdl(k_prolong_nn<T>, gu, b, 0, s, ef, ec, L.g, C.g, nn_xfer<T>(L, C), ctrl);
  }
  else if (cz.c[0] && cz.c[1] && cz.c[2])
    launch_pdl(k_prolong_cell<T>, g3(C.g), b, 0, s, ef, ec, L.g, C.g, ctrl);
  else
    launch_pdl(k_prolong<T>, g3(L.g), b, 0, s, ef, ec, L.g, C.g, cz, ctrl);
}

void launch_post_pass(int which, const MGLevel& L, const MGLevel& C, float om, double* p, SolveCtrl* ctrl,
                      cudaStream_t s) {
  const PoiCoef<float> c = make_poi<float>(L.h[0], L.h[1], L.h[2]);
  float* t = (float*)L.t;
  const float* r = (const float*)L.r;
  if (which == 0)
    launch_prolong_add<float>(L, C, t, (const float*)C.e, ctrl, s);
  else if (which == 1)
    launch_color<float>(L.g, t, r, c, 0, om, ctrl, (float*)nullptr, s);
  else
    launch_pdl(k_smooth_upd, su_grid(L.g), dim3(32, 8), 0, s, (const float*)t, r, L.g, c, om, ppair(p, L.g.n),
               ctrl);
}

// One V-cycle on level l for A e = r, from e = 0 (zero_init: the first
// sweep in one pass from r) or from the current e.
// On a fused level (FP32 only) k_mg_down and k_mg_up do the level's work;
// p_upd (finest level, last cycle) asks k_mg_up, or on an unfused level the
// last black pass (k_smooth_upd), for p += e and max |e| as well, and the
// return value tells whether that happened.
template <class T>
static bool vcycle(MGLevel* lv, int l, int nlev, int pre, int post, int coarse_sweeps, T om, SolveCtrl* ctrl,
                   cudaStream_t s, long long* nl, bool zero_init, double* p_upd = nullptr) {
  const MGLevel& L = lv[l];
  if constexpr (sizeof(T) == 4) {
    if (L.fused && l + 1 < nlev) {
      if (!zero_init && pre == 1 && lv_big(L.g) && !L.fuse_all) {
        // from the correction in e: its red pass copied into t (red updated,
        // black kept), the black pass in place on t, then the residual
        // through e and the restriction, as from zero below
        const PoiCoef<float> c = make_poi<float>(L.h[0], L.h[1], L.h[2]);
        launch_color<float>(L.g, (float*)L.e, (const float*)L.r, c, 0, (float)om, ctrl, (float*)L.t, s);
        launch_color<float>(L.g, (float*)L.t, (const float*)L.r, c, 1, (float)om, ctrl, (float*)nullptr, s);
        level_resid<float>(L, (const float*)L.t, (const float*)L.r, (float*)L.e, c, ctrl, s);
        launch_restrict<float>(L, lv[l + 1], (const float*)L.e, (float*)lv[l + 1].r, ctrl, s);
        *nl += 4;
      } else if (zero_init && pre == 1 && lv_big(L.g) && !L.fuse_all) {
        // one sweep from e = 0, the residual and the restriction as 2.5D
        // one-pass kernels: on a large level they move 24.5 B per point at
        // about 70 % of HBM, faster than k_mg_down's issue-bound march over
        // recomputed halos.  The smoothed e goes to t, where k_mg_up reads
        // it; the residual passes through e, which k_mg_up overwrites.
        const PoiCoef<float> c = make_poi<float>(L.h[0], L.h[1], L.h[2]);
        smooth_first<float>(L, (float*)L.t, (const float*)L.r, c, (float)om, ctrl, s);
        level_resid<float>(L, (const float*)L.t, (const float*)L.r, (float*)L.e, c, ctrl, s);
        launch_restrict<float>(L, lv[l + 1], (const float*)L.e, (float*)lv[l + 1].r, ctrl, s);
        *nl += 3;
      } else {
        launch_mg_down(L, lv[l + 1], (float)om, pre, zero_init, ctrl, s);
        *nl += 1;
      }
      vcycle<T>(lv, l + 1, nlev, pre, post, coarse_sweeps, om, ctrl, s, nl, true);
      if (p_upd && post == 1 && lv_big(L.g) && !L.fuse_all) {
        // the cycle that updates the pressure: the prolongation-add into the
        // smoothed e (in t), its red pass and the black pass with the pair's
        // update as one-pass kernels (44.5 B per point near the HBM roofline,
        // 2.7 % of the 256^3 step faster than k_mg_up's 28.5 B per point
        // issue-bound march)
        for (int w = 0; w < 3; ++w) launch_post_pass(w, L, lv[l + 1], (float)om, p_upd, ctrl, s);
        *nl += 3;
        return true;
      }
      launch_mg_up(L, lv[l + 1], (float)om, post, p_upd, ctrl, s);
      *nl += 1;
      return p_upd != nullptr;
    }
  }
  T* e = (T*)L.e;
  T* r = (T*)L.r;
  PoiCoef<T> c = make_poi<T>(L.h[0], L.h[1], L.h[2]);
  const dim3 b(32, 8);
  if (l == nlev - 1) {
    if (coarse_fits<T>(L.g)) {
      launch_pdl(k_coarse<T>, 1, coarse_threads(L.g), 0, s, e, r, L.g, c, coarse_sweeps, ctrl);
      *nl += 1;
    } else {
      smooth_first<T>(L, e, r, c, (T)1, ctrl, s);
      *nl += 1;
      smooth_sweeps<T>(L, e, r, c, (T)1, coarse_sweeps - 1, ctrl, s, nl);
    }
    return false;
  }
  int sweeps = pre;
  if (zero_init) {
    smooth_first<T>(L, e, r, c, om, ctrl, s);
    *nl += 1;
    sweeps -= 1;
  }
  smooth_sweeps<T>(L, e, r, c, om, sweeps, ctrl, s, nl);
  level_resid<T>(L, e, r, (T*)L.t, c, ctrl, s);
  const MGLevel& C = lv[l + 1];
  launch_restrict<T>(L, C, (const T*)L.t, (T*)C.r, ctrl, s);
  *nl += 2;
  vcycle<T>(lv, l + 1, nlev, pre, post, coarse_sweeps, om, ctrl, s, nl, true);
  launch_prolong_add<T>(L, C, e, (const T*)C.e, ctrl, s);
  *nl += 1;
  if constexpr (sizeof(T) == 4) {
    if (p_upd && !L.plain && post >= 1) {  // the last sweep's black pass carries the pressure update
      smooth_sweeps<T>(L, e, r, c, om, post - 1, ctrl, s, nl);
      smooth_last_upd(L, (float*)e, (const float*)r, c, (float)om, p_upd, ctrl, s, nl);
      return true;
    }
  }
  smooth_sweeps<T>(L, e, r, c, om, post, ctrl, s, nl);
  return false;
}

// One outer iteration of the defect-correction loop, in two parts.
// launch_mg_resid: r0 = rhs - mean - A p in FP64 (stored in T) with max |r0|.
// In the mixed method (T = float) p is the double-float pair buffer.
template <class T, class R>
void launch_mg_resid(double* p, const R* rhs, MGLevel* lv, SolveCtrl* ctrl, cudaStream_t s, long long* nl) {
  const MGLevel& L0 = lv[0];
  PoiCoef<double> c64 = make_poi<double>(L0.h[0], L0.h[1], L0.h[2]);
  // the mixed method subtracts the rhs mean here; the FP64 method's rhs was shifted in place
  constexpr bool PP = sizeof(T) == 4;
  if constexpr (sizeof(T) == 4 && sizeof(R) == 4) {
    // two points per thread on whole 64-point x tiles: every thread's pair is
    // in the grid and the x halo is the tile's two edge columns
    if (L0.g.nx % (2 * R2_TX) == 0 && !L0.plain) {
      launch_pdl(k_resid25p<true>, r2_grid(L0.g), dim3(R2_TX, R2_TY), 0, s, ppair(p, L0.g.n), (const float*)rhs,
                 (float*)L0.r, L0.g, poi_df(c64), ctrl);
      *nl += 1;
      return;
    }
  }
  launch_pdl(k_resid25<T, R, true, PP>, rz_grid(L0.g), dim3(RZ_TX, RZ_TY), 0, s, p, ppair(p, L0.g.n), rhs,
             (T*)L0.r, L0.g, c64, poi_df(c64), ctrl, (int)(sizeof(T) == 4));
  *nl += 1;
}

// launch_mg_cycles: `cycles` V-cycles in T on A e = r0 (the first from e = 0,
// or from the correction already in the finest level's e when from_e), then
// p += e in FP64 and the stop test.
template <class T>
void launch_mg_cycles(double* p, MGLevel* lv, int nlev, int pre, int post, int coarse_sweeps, T smooth_omega,
                      int cycles, bool from_e, SolveCtrl* ctrl, cudaStream_t s, long long* nl) {
  const MGLevel& L0 = lv[0];
  bool updated = false;
  for (int q = 0; q < cycles; ++q)
    updated = vcycle<T>(lv, 0, nlev, pre, post, coarse_sweeps, smooth_omega, ctrl, s, nl, q == 0 && !from_e,
                        q == cycles - 1 ? p : nullptr);
  if (!updated) {  // the mixed method's p is the double-float pair
    launch_pdl(k_update<T, sizeof(T) == 4>, (unsigned)((L0.g.n + 256LL * UPD_PER - 1) / (256LL * UPD_PER)), 256, 0,
               s, p, ppair(p, L0.g.n), (const T*)L0.e, L0.g.n, ctrl);
    *nl += 1;
  }
  launch_pdl(k_mg_control, 1, 1, 0, s, ctrl);
  *nl += 1;
}

template <class T, class R>
void launch_mg_outer(double* p, const R* rhs, MGLevel* lv, int nlev, int pre, int post,
                     int coarse_sweeps, T smooth_omega, int cycles, SolveCtrl* ctrl, cudaStream_t s,
                     long long* nl) {
  launch_mg_resid<T, R>(p, rhs, lv, ctrl, s, nl);
  launch_mg_cycles<T>(p, lv, nlev, pre, post, coarse_sweeps, smooth_omega, cycles, false, ctrl, s, nl);
}

// p <- 2 p - p_prev, p_prev <- p (linear extrapolation of the pressure in time)
__global__ void k_extrapolate(double* __restrict__ p, double* __restrict__ pprev, long long n) {
  pdl_enter();
  const long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= n) return;
  const double pc = p[q];
  p[q] = 2.0 * pc - pprev[q];
  pprev[q] = pc;
}
// the same on double-float pairs
__global__ void k_extrapolate_pp(PPair p, PPair pprev, long long n) {
  pdl_enter();
  const long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= n) return;
  const DF pc = pp_load(p, q);
  pp_store(p, q, df_add(df_scale(pc, 2.f), df_neg(pp_load(pprev, q))));
  pp_store(pprev, q, pc);
}
void launch_extrapolate(double* p, double* pprev, long long n, cudaStream_t s, bool pair) {
  if (pair) launch_pdl(k_extrapolate_pp, (unsigned)((n + 255) / 256), 256, 0, s, ppair(p, n), ppair(pprev, n), n);
  else launch_pdl(k_extrapolate, (unsigned)((n + 255) / 256), 256, 0, s, p, pprev, n);
}

// p <- 3 p - 3 p_prev + p_prev2 (quadratic extrapolation in time), and the
// current pressure into pprev2's buffer, which the caller then swaps with
// pprev: the history shifts by one step without a copy
__global__ void k_extrapolate2(double* __restrict__ p, const double* __restrict__ pprev,
                               double* __restrict__ pprev2, long long n) {
  pdl_enter();
  const long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= n) return;
  const double pc = p[q];
  p[q] = 3.0 * (pc - pprev[q]) + pprev2[q];
  pprev2[q] = pc;
}
__global__ void k_extrapolate2_pp(PPair p, PPair pprev, PPair pprev2, long long n) {
  pdl_enter();
  const long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= n) return;
  const DF pc = pp_load(p, q);
  pp_store(p, q, df_add(df_scale(df_add(pc, df_neg(pp_load(pprev, q))), 3.f), pp_load(pprev2, q)));
  pp_store(pprev2, q, pc);
}
void launch_extrapolate2(double* p, const double* pprev, double* pprev2, long long n, cudaStream_t s, bool pair) {
  if (pair)
    launch_pdl(k_extrapolate2_pp, (unsigned)((n + 255) / 256), 256, 0, s, ppair(p, n), ppair((void*)pprev, n),
               ppair(pprev2, n), n);
  else
    launch_pdl(k_extrapolate2, (unsigned)((n + 255) / 256), 256, 0, s, p, pprev, pprev2, n);
}

// the same extrapolation, also writing the last increment d = p - p_prev in T
template <class T>
__global__ void k_extrapolate_d(double* __restrict__ p, double* __restrict__ pprev, T* __restrict__ d, long long n) {
  pdl_enter();
  const long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= n) return;
  const double pc = p[q], pv = pprev[q];
  p[q] = 2.0 * pc - pv;
  pprev[q] = pc;
  d[q] = to_t<T>(pc - pv);
}
__global__ void k_extrapolate_d_pp(PPair p, PPair pprev, float* __restrict__ d, long long n) {
  pdl_enter();
  const long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= n) return;
  const DF pc = pp_load(p, q), pv = pp_load(pprev, q);
  const DF inc = df_add(pc, df_neg(pv));
  pp_store(p, q, df_add(pc, inc));
  pp_store(pprev, q, pc);
  d[q] = inc.h + inc.l;
}

// ---------------------------------------------------------------------------
// learned warm start plumbing.  The network works on multigrid level ll
// (coarsened ll times on every axis).  Its input, for the extrapolated
// pressure p_ex = 2 p^n - p^(n-1): channel 0 = restrict(rhs - mean - A p_ex)
// h_ll^2 / S_r, channel 1 = restrict(p^n - p^(n-1)) / S_d, each scaled by
// its own rms; its output y predicts restrict(p^(n+1) - p_ex) / S_r with
// the mean removed (a constant is in the null space of the periodic and
// mirror operators: the solver leaves it arbitrary).  The correction
// prolong(S_r y) starts the first V-cycle (multigrid) or is added to p
// (SOR).
// ---------------------------------------------------------------------------
// S_r = rms(r h^2), S_d = rms(d) over the coarse grid (one block; the
// scales need no more than FP32 accumulation)
template <class T>
__global__ void k_rms(const T* __restrict__ r, const T* __restrict__ d, long long n, double h2, SolveCtrl* ctrl) {
  pdl_enter();
  __shared__ float sh[2][32];
  float a = 0.f, b = 0.f;
  for (long long q = threadIdx.x; q < n; q += blockDim.x) {
    const float rv = (float)r[q], dv = (float)d[q];
    a = fmaf(rv, rv, a);
    b = fmaf(dv, dv, b);
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    a += __shfl_xor_sync(0xffffffffu, a, o);
    b += __shfl_xor_sync(0xffffffffu, b, o);
  }
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31, nw = blockDim.x >> 5;
  if (l == 0) { sh[0][w] = a; sh[1][w] = b; }
  __syncthreads();
  if (w == 0) {
    a = l < nw ? sh[0][l] : 0.f;
    b = l < nw ? sh[1][l] : 0.f;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      a += __shfl_xor_sync(0xffffffffu, a, o);
      b += __shfl_xor_sync(0xffffffffu, b, o);
    }
    if (l == 0) {
      ctrl->learn_scale = sqrt((double)a / (double)n) * h2 + 1e-300;
      ctrl->learn_scale_d = sqrt((double)b / (double)n) + 1e-300;
    }
  }
}

// network input: channel 0 = r h^2 / S_r, channel 1 = d / S_d (FP32, channel-major)
template <class T>
__global__ void k_features(const T* __restrict__ r, const T* __restrict__ d, long long n, double h2,
                           const SolveCtrl* ctrl, float* __restrict__ feat) {
  pdl_enter();
  const long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= n) return;
  feat[q] = (float)((double)r[q] * h2 / ctrl->learn_scale);
  feat[n + q] = (float)((double)d[q] / ctrl->learn_scale_d);
}

// coarse correction e = S_r * y
template <class T>
__global__ void k_unscale(const float* __restrict__ y, long long n, const SolveCtrl* ctrl, T* __restrict__ e) {
  pdl_enter();
  const long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (q < n) e[q] = (T)((double)y[q] * ctrl->learn_scale);
}

// training target (one block): w = dp - S_d ch1 = restrict(p^(n+1) - p_ex)
// (dp = restrict(p^(n+1) - p^n), ch1 = the increment channel of the input,
// restriction being linear), t = (w - mean w) / S_r
template <class T>
__global__ void k_target(const T* __restrict__ dp, long long n, const SolveCtrl* ctrl, const float* __restrict__ ch1,
                         float* __restrict__ t) {
  pdl_enter();
  __shared__ double sh[1024];
  const double sd = ctrl->learn_scale_d;
  double a = 0.0;
  for (long long q = threadIdx.x; q < n; q += blockDim.x) a += (double)dp[q] - sd * (double)ch1[q];
  sh[threadIdx.x] = a;
  __syncthreads();
  for (int st = blockDim.x / 2; st > 0; st >>= 1) {
    if ((int)threadIdx.x < st) sh[threadIdx.x] += sh[threadIdx.x + st];
    __syncthreads();
  }
  const double mean = sh[0] / (double)n, inv = 1.0 / ctrl->learn_scale;
  for (long long q = threadIdx.x; q < n; q += blockDim.x)
    t[q] = (float)(((double)dp[q] - sd * (double)ch1[q] - mean) * inv);
}

// d = p - pprev in T
template <class T>
__global__ void k_pdiff(const double* __restrict__ p, const double* __restrict__ pprev, T* __restrict__ d, long long n) {
  pdl_enter();
  const long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (q < n) d[q] = to_t<T>(p[q] - pprev[q]);
}
__global__ void k_pdiff_pp(PPair p, PPair pprev, float* __restrict__ d, long long n) {
  pdl_enter();
  const long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= n) return;
  const DF v = df_add(pp_load(p, q), df_neg(pp_load(pprev, q)));
  d[q] = v.h + v.l;
}

// p += e
template <class T>
__global__ void k_padd(double* __restrict__ p, const T* __restrict__ e, long long n) {
  pdl_enter();
  const long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (q < n) p[q] += to_t<double>(e[q]);
}

static inline unsigned b256(long long n) { return (unsigned)((n + 255) / 256); }

// Restricts a level-0 field down to level ll through the levels' scratch
// arrays `which` (0: e, 1: t); returns the level-ll array.
template <class T>
static T* restrict_to(MGLevel* lv, int ll, const T* f0, int which, SolveCtrl* ctrl, cudaStream_t s, long long* nl) {
  const T* src = f0;
  T* dst = nullptr;
  for (int l = 0; l < ll; ++l) {
    dst = (T*)(which ? lv[l + 1].t : lv[l + 1].e);
    launch_restrict<T>(lv[l], lv[l + 1], src, dst, ctrl, s);
    src = dst;
    *nl += 1;
  }
  return dst;
}

// p <- p_ex, p_prev <- p, and the increment into the finest level's t
template <class T>
void launch_learn_extrapolate(double* p, double* pprev, MGLevel* lv, cudaStream_t s, long long* nl, bool pair) {
  const long long n = lv[0].g.n;
  if constexpr (sizeof(T) == 4) {
    if (pair) {
      launch_pdl(k_extrapolate_d_pp, b256(n), 256, 0, s, ppair(p, n), ppair(pprev, n), (float*)lv[0].t, n);
      *nl += 1;
      return;
    }
  }
  launch_pdl(k_extrapolate_d<T>, b256(n), 256, 0, s, p, pprev, (T*)lv[0].t, n);
  *nl += 1;
}

// Network input from the residual of p_ex in the finest level's r (left
// intact) and the increment in its t; uses the e and t arrays of levels
// 1..ll.  ctrl->done must be 0.
template <class T>
void launch_learn_features(MGLevel* lv, int ll, SolveCtrl* ctrl, float* feat, cudaStream_t s, long long* nl) {
  const T* rc = restrict_to<T>(lv, ll, (const T*)lv[0].r, 0, ctrl, s, nl);
  const T* dc = restrict_to<T>(lv, ll, (const T*)lv[0].t, 1, ctrl, s, nl);
  const long long n2 = lv[ll].g.n;
  const double h2 = lv[ll].h[0] * lv[ll].h[0];
  launch_pdl(k_rms<T>, 1, 1024, 0, s, rc, dc, n2, h2, ctrl);
  launch_pdl(k_features<T>, b256(n2), 256, 0, s, rc, dc, n2, h2, ctrl, feat);
  *nl += 2;
}

// Finest level's e <- prolong^ll(S y) (y: network output on level ll); with
// add_to_p, also p += e.
template <class T>
void launch_learn_apply(double* p, const float* y, MGLevel* lv, int ll, bool add_to_p, SolveCtrl* ctrl,
                        cudaStream_t s, long long* nl) {
  const long long n2 = lv[ll].g.n;
  launch_pdl(k_unscale<T>, b256(n2), 256, 0, s, y, n2, ctrl, (T*)lv[ll].e);
  *nl += 1;
  for (int l = ll - 1; l >= 0; --l) {
    cudaMemsetAsync(lv[l].e, 0, (size_t)lv[l].g.n * sizeof(T), s);
    launch_prolong_add<T>(lv[l], lv[l + 1], (T*)lv[l].e, (const T*)lv[l + 1].e, ctrl, s);
    *nl += 1;
  }
  if (add_to_p) {
    launch_pdl(k_padd<T>, b256(lv[0].g.n), 256, 0, s, p, (const T*)lv[0].e, lv[0].g.n);
    *nl += 1;
  }
}

// Training target of the last solve into tgt (FP32); ch1 is the increment
// channel of that solve's network input.
template <class T>
void launch_learn_target(const double* p, const double* pprev, MGLevel* lv, int ll, SolveCtrl* ctrl,
                         const float* ch1, float* tgt, cudaStream_t s, long long* nl) {
  const MGLevel& L0 = lv[0];
  if constexpr (sizeof(T) == 4)  // training samples come from multigrid solves: the pair layout
    launch_pdl(k_pdiff_pp, b256(L0.g.n), 256, 0, s, ppair((void*)p, L0.g.n), ppair((void*)pprev, L0.g.n),
               (float*)L0.t, L0.g.n);
  else
    launch_pdl(k_pdiff<T>, b256(L0.g.n), 256, 0, s, p, pprev, (T*)L0.t, L0.g.n);
  const T* dc = restrict_to<T>(lv, ll, (const T*)L0.t, 1, ctrl, s, nl);
  launch_pdl(k_target<T>, 1, 1024, 0, s, dc, lv[ll].g.n, ctrl, ch1, tgt);
  *nl += 2;
}

#define O3D_LEARN_INST(T)                                                                                      \
  template void launch_learn_extrapolate<T>(double*, double*, MGLevel*, cudaStream_t, long long*, bool);       \
  template void launch_learn_features<T>(MGLevel*, int, SolveCtrl*, float*, cudaStream_t, long long*);         \
  template void launch_learn_apply<T>(double*, const float*, MGLevel*, int, bool, SolveCtrl*, cudaStream_t,    \
                                      long long*);                                                             \
  template void launch_learn_target<T>(const double*, const double*, MGLevel*, int, SolveCtrl*, const float*, \
                                       float*, cudaStream_t, long long*);                                      \
  template void launch_mg_resid<T, double>(double*, const double*, MGLevel*, SolveCtrl*, cudaStream_t,            \
                                           long long*);                                                        \
  template void launch_mg_cycles<T>(double*, MGLevel*, int, int, int, int, T, int, bool, SolveCtrl*,           \
                                    cudaStream_t, long long*);
O3D_LEARN_INST(float)
O3D_LEARN_INST(double)

template <class R>
void launch_rhs_wmean(const R* rhs, const Grid& g, double* part, SolveCtrl* ctrl, cudaStream_t s,
                      long long* nl) {
  const dim3 grid((g.nx + 31) / 32, (g.ny + 7) / 8, (g.nz + WM_KC - 1) / WM_KC);
  launch_pdl(k_wmean_part<R>, grid, dim3(32, 8), 0, s, rhs, g, part);
  *nl += 1;
  launch_rhs_wmean_final(part, (long long)grid.x * grid.y * grid.z, g, ctrl, s, nl);
}

// the mean from per-block weighted sums already in part (nblk records, e.g.
// written by the divergence kernel that produced the rhs)
void launch_rhs_wmean_final(const double* part, long long nblk, const Grid& g, SolveCtrl* ctrl, cudaStream_t s,
                            long long* nl) {
  // sum of the weights: per axis n (periodic) or n - 1 (mirror: halves at both ends)
  double wsum = 1.0;
  for (int a = 0; a < 3; ++a) wsum *= g.bc[a] == AX_MIRROR ? (double)(g.len(a) - 1) : (double)g.len(a);
  launch_pdl(k_wmean_final, 1, 1024, 0, s, part, nblk, wsum, ctrl);
  *nl += 1;
}

template <class R>
void launch_residual_inf(const double* p, const R* rhs, const Grid& g, const PoiCoef<double>& c, SolveCtrl* ctrl,
                         bool shift, cudaStream_t s, bool pair) {
  const PPair pp = ppair((void*)p, g.n);
  if (pair) launch_pdl(k_resid_inf<R, true>, g3(g), dim3(32, 8), 0, s, p, pp, rhs, g, c, ctrl, (int)shift);
  else launch_pdl(k_resid_inf<R, false>, g3(g), dim3(32, 8), 0, s, p, pp, rhs, g, c, ctrl, (int)shift);
}
template <class R>
void launch_rhs_shift(R* rhs, long long n, SolveCtrl* ctrl, cudaStream_t s) {
  launch_pdl(k_rhs_shift<R>, (unsigned)((n + 255) / 256), 256, 0, s, rhs, n, ctrl);
}
template void launch_rhs_shift<float>(float*, long long, SolveCtrl*, cudaStream_t);
template void launch_rhs_shift<double>(double*, long long, SolveCtrl*, cudaStream_t);

template <class T, class R>
void launch_level_kernel(int which, double* p, const R* rhs, const MGLevel& L, SolveCtrl* ctrl,
                         cudaStream_t s, bool pair) {
  PoiCoef<T> c = make_poi<T>(L.h[0], L.h[1], L.h[2]);
  if (which == 0) {
    launch_color<T>(L.g, (T*)L.e, (const T*)L.r, c, 0, (T)1, ctrl, (T*)nullptr, s);
  } else if (which == 2) {  // the first sweep from e = 0 into t, as a large level runs it
    smooth_first<T>(L, (T*)L.t, (const T*)L.r, c, (T)1.25, ctrl, s);
  } else if (which == 3) {  // the level residual from t into e
    level_resid<T>(L, (const T*)L.t, (const T*)L.r, (T*)L.e, c, ctrl, s);
  } else {
    PoiCoef<double> c64 = make_poi<double>(L.h[0], L.h[1], L.h[2]);
    const PPair pp = ppair(p, L.g.n);
    if constexpr (sizeof(T) == 4) {
      if (pair) {
        // the kernel the step runs: two points per thread on whole x tiles
        // with the FP32 rhs (its rhs less the mean, as in the loop)
        if constexpr (sizeof(R) == 4) {
          if (L.g.nx % (2 * R2_TX) == 0 && !L.plain) {
            launch_pdl(k_resid25p<false>, r2_grid(L.g), dim3(R2_TX, R2_TY), 0, s, pp, (const float*)rhs, (float*)L.r,
                       L.g, poi_df(c64), ctrl);
            return;
          }
        }
        launch_pdl(k_resid25<T, R, false, true>, rz_grid(L.g), dim3(RZ_TX, RZ_TY), 0, s, p, pp, rhs, (T*)L.r, L.g,
                   c64, poi_df(c64), ctrl, 0);
        return;
      }
    }
    launch_pdl(k_resid25<T, R, false, false>, rz_grid(L.g), dim3(RZ_TX, RZ_TY), 0, s, p, pp, rhs, (T*)L.r, L.g, c64,
               poi_df(c64), ctrl, 0);
  }
}
template void launch_level_kernel<float, double>(int, double*, const double*, const MGLevel&, SolveCtrl*,
                                                 cudaStream_t, bool);
template void launch_level_kernel<double, double>(int, double*, const double*, const MGLevel&, SolveCtrl*,
                                                  cudaStream_t, bool);
template void launch_level_kernel<float, float>(int, double*, const float*, const MGLevel&, SolveCtrl*,
                                                cudaStream_t, bool);

template void launch_mg_outer<double, double>(double*, const double*, MGLevel*, int, int, int, int,
                                              double, int, SolveCtrl*, cudaStream_t, long long*);
template void launch_mg_outer<float, double>(double*, const double*, MGLevel*, int, int, int, int,
                                             float, int, SolveCtrl*, cudaStream_t, long long*);
template void launch_mg_outer<float, float>(double*, const float*, MGLevel*, int, int, int, int,
                                            float, int, SolveCtrl*, cudaStream_t, long long*);
template void launch_mg_resid<float, float>(double*, const float*, MGLevel*, SolveCtrl*, cudaStream_t, long long*);
template void launch_rhs_wmean<double>(const double*, const Grid&, double*, SolveCtrl*, cudaStream_t, long long*);
template void launch_rhs_wmean<float>(const float*, const Grid&, double*, SolveCtrl*, cudaStream_t, long long*);
template void launch_residual_inf<double>(const double*, const double*, const Grid&, const PoiCoef<double>&,
                                          SolveCtrl*, bool, cudaStream_t, bool);
template void launch_residual_inf<float>(const double*, const float*, const Grid&, const PoiCoef<double>&,
                                         SolveCtrl*, bool, cudaStream_t, bool);

}  // namespace o3d
