// k_stencil25.cu -- the 2.5D stencil kernels of the step: the fused momentum
// predictor (9 first + 9 second derivatives, Smagorinsky nu_t, convection,
// diffusion and the Adams-Bashforth update in one pass), the divergence /
// Poisson right-hand side with its statistics, and the velocity correction
// with its extrema.  Templated on the arithmetic type T (double for the plain
// method, float for the mixed method).
//
// A block owns a TX x TY column of (x, y) points and marches along z over a
// chunk of planes.  Each plane's cells (centres, 3-point x/y halos and the
// per-point inputs) are copied global -> shared by cp.async, several planes
// ahead of the one being computed, into a ring of plane stages: the loads
// need no registers while in flight and the compute of one plane overlaps
// the loads of the next ones.  Each thread keeps the seven z-neighbours of
// its point in a register queue fed from the ring's centre cells.  The ghost
// mapping at the domain ends (periodic wrap, or mirror with the odd-parity
// sign) is resolved once per thread for x and y and once per plane for z;
// a thread negates the mirrored odd cells it copied itself, after its copies
// land and before the block barrier that publishes them.  Points past the
// grid end stage ghost-mapped values, which the lines of the last valid
// points read.
//
// Plane pipeline (local plane lp = k - k0, ring of 4 + P stages, P planes in
// flight beyond the queue head):
//   group(lp)  = copies of plane lp: centres (all planes the queue needs,
//                lp <= np + 2) and halos (lp < np); the per-point inputs of
//                plane lp - 3 (flux history, u*) ride along
//   prologue   : issue group(0 .. P+2)
//   iteration lp: wait until group(lp + 3) landed (P - 1 groups may stay in
//                flight), fix signs of plane lp + 3, __syncthreads, issue
//                group(lp + 3 + P) into the stage of plane lp - 1 (free:
//                every thread passed the barrier after computing it), take
//                the queue head from plane lp + 3, compute plane lp.
#include <atomic>
#include "o3d_internal.cuh"
#include "o3d_kernels.h"

namespace o3d {

// xy part of a ghost-mapped cell: offset within a z-plane and the flips
struct XYCell {
  int off;
  bool fx, fy;
};
__device__ __forceinline__ XYCell xy_cell(const Grid& g, int i, int j) {
  XYCell c;
  c.off = ghost(i, g.nx, g.bc[0], &c.fx) + g.nx * ghost(j, g.ny, g.bc[1], &c.fy);
  return c;
}

// whether a field odd along odd_axis (0/1/2; -1 = even) flips at a cell
__device__ __forceinline__ bool flips(const XYCell& x, bool fz, int odd_axis) {
  return odd_axis == 0 ? x.fx : odd_axis == 1 ? x.fy : odd_axis == 2 ? fz : false;
}

// f at cell (x, z) through the registers, converted to T, sign applied
template <class T, class S>
__device__ __forceinline__ T ldc(const S* __restrict__ f, const XYCell& x, const ZPlane& z, int odd_axis) {
  const T v = to_t<T>(__ldg(f + z.off + x.off));
  return flips(x, z.fz, odd_axis) ? -v : v;
}

// The halo cell a thread stages, by linear thread id t < 6 (TX + TY): the
// left and right 3-column x-halos of the TY rows, then the 3-row y-halos
// below and above the TX columns.  tidx: position in a (TY+6) x (TX+6)
// tile; lidx: position in an x-line array [TY][TX+6] (x-halo cells) or a
// y-line array [TY+6][TX] (y-halo cells).
template <int TX, int TY>
struct Halo {
  XYCell c;
  int tidx, lidx;
  bool on, xh;
};
template <int TX, int TY>
__device__ __forceinline__ Halo<TX, TY> halo_cell(const Grid& g, int i0, int j0, int t) {
  static_assert(6 * (TX + TY) <= TX * TY, "the block must cover its halo cells");
  constexpr int SW = TX + 6;
  Halo<TX, TY> h;
  int hi, hj;
  h.on = t < 6 * (TX + TY);
  h.xh = t < 6 * TY;
  if (t < 3 * TY) {  // left x-halo
    const int col = t % 3, r = t / 3;
    hi = i0 - 3 + col; hj = j0 + r;
    h.tidx = (r + 3) * SW + col; h.lidx = r * SW + col;
  } else if (t < 6 * TY) {  // right x-halo
    const int u = t - 3 * TY, col = u % 3, r = u / 3;
    hi = i0 + TX + col; hj = j0 + r;
    h.tidx = (r + 3) * SW + TX + 3 + col; h.lidx = r * SW + TX + 3 + col;
  } else if (t < 6 * TY + 3 * TX) {  // y-halo below
    const int u = t - 6 * TY, col = u % TX, r = u / TX;
    hi = i0 + col; hj = j0 - 3 + r;
    h.tidx = r * SW + col + 3; h.lidx = r * TX + col;
  } else {  // y-halo above
    const int u = min(t - 6 * TY - 3 * TX, 3 * TX - 1), col = u % TX, r = u / TX;
    hi = i0 + col; hj = j0 + TY + r;
    h.tidx = (TY + 3 + r) * SW + col + 3; h.lidx = (TY + 3 + r) * TX + col;
  }
  h.c = xy_cell(g, hi, hj);
  return h;
}

// Raises a kernel's dynamic shared-memory limit above 48 KB.  The attribute
// belongs to the current device, so it is applied once per device (one flag
// per device and kernel instantiation); devices beyond the table get it on
// every launch.
constexpr int SMEM_MAX_DEVICES = 64;
template <class K>
static void allow_smem(K* kernel, size_t bytes, std::atomic<bool>* done) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) dev = -1;
  if (dev >= 0 && dev < SMEM_MAX_DEVICES && done[dev].load(std::memory_order_acquire)) return;
  if (cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes) == cudaSuccess &&
      dev >= 0 && dev < SMEM_MAX_DEVICES)
    done[dev].store(true, std::memory_order_release);
}

constexpr int TX25 = 32, TY25 = 8, KC25 = 28;  // planes per block: a multiple of the unroll (7)
static inline dim3 grid25(const Grid& g) {
  return dim3((g.nx + TX25 - 1) / TX25, (g.ny + TY25 - 1) / TY25, (g.nz + KC25 - 1) / KC25);
}
long long z_blocks(const Grid& g) {
  const dim3 b = grid25(g);
  return (long long)b.x * b.y * b.z;
}
template <class T>
long long div_blocks(const Grid& g) {
  if (sizeof(T) == 4 && stencil_v_ok(g)) return div_v_blocks(g);
  return z_blocks(g);
}
template <class T>
long long corr_blocks(const Grid& g) {
  if (sizeof(T) == 4 && stencil_v_ok(g)) return corr_v_blocks(g);
  return z_blocks(g);
}
template long long div_blocks<float>(const Grid&);
template long long div_blocks<double>(const Grid&);
template long long corr_blocks<float>(const Grid&);
template long long corr_blocks<double>(const Grid&);

// The plane loop runs in rounds of 7 fully unrolled iterations (the chunk of
// planes is a multiple of 7 and the ring has R = 7 stages, P = 3): the ring
// stage of plane lp and the register slot of each queue plane are then
// compile-time constants.  Slot s of a queue holds the plane whose local
// index is congruent to s - 3 modulo 7, so the seven z-neighbours of plane
// lp = 7 b + u sit in slots (u + m) % 7, m = 0..6, and the head (plane
// lp + 3) replaces plane lp - 4 in slot (u + 6) % 7: no register moves.
constexpr int ZQ = 7;      // z-stencil width = queue length = unroll = ring stages
constexpr int PD = 3;      // planes in flight beyond the queue head
static_assert(4 + PD == ZQ, "the ring must match the unroll");

// ---------------------------------------------------------------------------
// fused predictor, predict_velocity + calculate_nu_t
// (src/integration.f90:106-188, src/les_turbulence.f90:54-88).
// Component c of the velocity is odd along axis c (derxi for ux, deryi for
// uy, derzi for uz).  The flux history of plane lp travels in group(lp + 3),
// issued at iteration lp - PD, into a (PD+1)-stage ring.  Without LES each
// component's six derivatives are used as soon as they are formed; with LES
// the nine first derivatives are kept for the strain rate.
// ---------------------------------------------------------------------------
template <class T, int TX, int TY>
struct PredRing {
  static constexpr int SW = TX + 6, PL = (TY + 6) * SW, NC = TX * TY;
  T tile[ZQ][3][PL];
  T hist[PD + 1][6][NC];  // f2 of u, v, w then f3 of u, v, w at the centre cells
};

template <class T, int TX, int TY, bool LES, bool ZON, bool XO>
__global__ void __launch_bounds__(TX * TY, sizeof(T) == 4 ? 3 : 1) k_predict25(PredArgs<T> A, int kc) {
  pdl_enter();
  using Ring = PredRing<T, TX, TY>;
  constexpr int SW = Ring::SW;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  Ring& sm = *reinterpret_cast<Ring*>(smem_raw);
  const Grid& g = A.g;
  const int tx = threadIdx.x, ty = threadIdx.y, t = ty * TX + tx;
  const int i0 = blockIdx.x * TX, j0 = blockIdx.y * TY;
  const int i = i0 + tx, j = j0 + ty;
  const bool valid = i < g.nx && j < g.ny;
  const int k0 = blockIdx.z * kc;
  const int np = min(kc, g.nz - k0);
  constexpr bool zon = ZON;  // z derivatives (false: 2D, derz_2dsim)
  const bool may_flip = g.bc[0] == AX_MIRROR || g.bc[1] == AX_MIRROR || g.bc[2] == AX_MIRROR;
  const int pcx = XO ? xclass(g, i) : 0;  // open x axis: closure class; 1 = inflow node (held)
  const XYCell cc = xy_cell(g, i, j);
  const Halo<TX, TY> h = halo_cell<TX, TY>(g, i0, j0, t);
  const int sc = (ty + 3) * SW + tx + 3;
  const long long out0 = valid ? (long long)i + (long long)g.nx * j : 0;
  const long long sz = g.sz();
  const int last_centre = zon ? np + 2 : np - 1;

  // group(lp): centre and halo cells of plane lp, history of plane lp - 3
  auto issue = [&](int lp, int st) {
    if (lp <= last_centre) {
      const long long zo = z_plane(g, k0 + lp).off;
#pragma unroll
      for (int c = 0; c < 3; ++c) cp_async<sizeof(T)>(&sm.tile[st][c][sc], A.u[c] + zo + cc.off);
      if (lp < np && h.on) {
#pragma unroll
        for (int c = 0; c < 3; ++c) cp_async<sizeof(T)>(&sm.tile[st][c][h.tidx], A.u[c] + zo + h.c.off);
      }
    }
    const int lh = lp - 3;
    if (lh >= 0 && lh < np && valid) {
      const int hs = lh & PD;
      const long long q = out0 + sz * (k0 + lh);
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        if (A.f2[c]) cp_async<sizeof(T)>(&sm.hist[hs][c][t], A.f2[c] + q);
        if (A.f3[c]) cp_async<sizeof(T)>(&sm.hist[hs][3 + c][t], A.f3[c] + q);
      }
    }
    cp_async_commit();
  };
  // negate the mirrored odd cells this thread copied for plane lp
  auto fix = [&](int lp, int st) {
    if (!may_flip || lp > last_centre) return;
    const bool fz = z_plane(g, k0 + lp).fz;
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      if (flips(cc, fz, c)) sm.tile[st][c][sc] = -sm.tile[st][c][sc];
      if (lp < np && h.on && flips(h.c, fz, c)) sm.tile[st][c][h.tidx] = -sm.tile[st][c][h.tidx];
    }
  };

  T q[3][ZQ];
#pragma unroll
  for (int c = 0; c < 3; ++c)
#pragma unroll
    for (int m = 0; m < ZQ; ++m) q[c][m] = (T)0;
#pragma unroll
  for (int lp = 0; lp < PD + 3; ++lp) issue(lp, lp);
  if constexpr (zon) {  // planes -3..-1 through the registers into slots 0..2
#pragma unroll
    for (int m = 0; m < 3; ++m) {
      const ZPlane z = z_plane(g, k0 - 3 + m);
#pragma unroll
      for (int c = 0; c < 3; ++c) q[c][m] = ldc<T>(A.u[c], cc, z, c);
    }
  }
  cp_async_wait<PD>();  // groups 0..2 landed
#pragma unroll
  for (int m = 0; m < 3; ++m) {
    fix(m, m);
#pragma unroll
    for (int c = 0; c < 3; ++c) q[c][3 + m] = sm.tile[m][c][sc];  // own centre cells, planes 0..2
  }
  for (int lb = 0; lb < np; lb += ZQ) {
#pragma unroll
    for (int u = 0; u < ZQ; ++u) {
      const int lp = lb + u;
      if (lp < np) {
        cp_async_wait<PD - 1>();  // group(lp + 3) landed
        fix(lp + 3, (u + 3) % ZQ);
        __syncthreads();
        issue(lp + 3 + PD, (u + 3 + PD) % ZQ);
        if constexpr (zon) {
#pragma unroll
          for (int c = 0; c < 3; ++c) q[c][(u + 6) % ZQ] = sm.tile[(u + 3) % ZQ][c][sc];
        }
        const int hs = lp & PD;
        const long long p = out0 + sz * (k0 + lp);
        T zc[3][ZQ];  // the z-lines in stencil order (register renaming only)
#pragma unroll
        for (int c = 0; c < 3; ++c)
#pragma unroll
          for (int m = 0; m < ZQ; ++m) zc[c][m] = zon ? q[c][(u + m) % ZQ] : (T)0;
        const T uc0 = sm.tile[u][0][sc], uc1 = sm.tile[u][1][sc], uc2 = sm.tile[u][2][sc];
        if constexpr (!LES) {
#pragma unroll
          for (int c = 0; c < 3; ++c) {
            T v[7];
#pragma unroll
            for (int m = 0; m < 7; ++m) v[m] = sm.tile[u][c][sc - 3 + m];
            const T g1x = d1x<XO>(v, A.cf.ax[0], pcx), g2x = d2x<XO>(v, A.cf.ax[0], pcx);
#pragma unroll
            for (int m = 0; m < 7; ++m) v[m] = sm.tile[u][c][sc + (m - 3) * SW];
            const T g1y = d1(v, A.cf.ax[1]), g2y = d2(v, A.cf.ax[1]);
            const T g1z = zon ? d1(zc[c], A.cf.ax[2]) : (T)0;
            const T g2z = zon ? d2(zc[c], A.cf.ax[2]) : (T)0;
            if (valid) {
              const T nu_eff = A.onere + (T)0;
              const T F = nu_eff * (g2x + g2y + g2z) - (uc0 * g1x + uc1 * g1y + uc2 * g1z);
              T up = v[3] + A.adu * F;
              if (A.f2[c]) up = up + A.bdu * sm.hist[hs][c][t];
              if (A.f3[c]) up = up + A.cdu * sm.hist[hs][3 + c][t];
              A.fnew[c][p] = F;
              A.up[c][p] = pcx == 1 ? v[3] : up;
            }
          }
        } else {
          T g1[3][3], g2[3][3];
#pragma unroll
          for (int c = 0; c < 3; ++c) {
            T v[7];
#pragma unroll
            for (int m = 0; m < 7; ++m) v[m] = sm.tile[u][c][sc - 3 + m];
            g1[c][0] = d1x<XO>(v, A.cf.ax[0], pcx);
            g2[c][0] = d2x<XO>(v, A.cf.ax[0], pcx);
#pragma unroll
            for (int m = 0; m < 7; ++m) v[m] = sm.tile[u][c][sc + (m - 3) * SW];
            g1[c][1] = d1(v, A.cf.ax[1]);
            g2[c][1] = d2(v, A.cf.ax[1]);
            g1[c][2] = zon ? d1(zc[c], A.cf.ax[2]) : (T)0;
            g2[c][2] = zon ? d2(zc[c], A.cf.ax[2]) : (T)0;
          }
          if (valid) {
            const T s11 = g1[0][0], s22 = g1[1][1], s33 = g1[2][2];
            const T s12 = (T)0.5 * (g1[0][1] + g1[1][0]);
            const T s13 = (T)0.5 * (g1[0][2] + g1[2][0]);
            const T s23 = (T)0.5 * (g1[1][2] + g1[2][1]);
            const T smag = sqrt((T)2 * (s11 * s11 + s22 * s22 + s33 * s33 +
                                        (T)2 * (s12 * s12 + s13 * s13 + s23 * s23)));
            const T nut = A.csd2 * smag;
            A.nu_t[p] = nut;
            const T nu_eff = A.onere + nut;
            const T uc[3] = {uc0, uc1, uc2};
#pragma unroll
            for (int c = 0; c < 3; ++c) {
              const T F = nu_eff * (g2[c][0] + g2[c][1] + g2[c][2]) -
                          (uc0 * g1[c][0] + uc1 * g1[c][1] + uc2 * g1[c][2]);
              T up = uc[c] + A.adu * F;
              if (A.f2[c]) up = up + A.bdu * sm.hist[hs][c][t];
              if (A.f3[c]) up = up + A.cdu * sm.hist[hs][3 + c][t];
              A.fnew[c][p] = F;
              A.up[c][p] = pcx == 1 ? uc[c] : up;
            }
          }
        }
      }
    }
  }
  cp_async_wait<0>();
}

// ---------------------------------------------------------------------------
// divergence (src/differential_operators.f90:25-35) -> optional output
// div*scale, with function_stats (src/functions.f90:27-63) accumulated per
// thread over its z-column and reduced once per block.  fx travels as
// x-lines, fy as y-lines, fz as the centre column of the queue.
// ---------------------------------------------------------------------------
template <class T, int TX, int TY>
struct DivRing {
  static constexpr int SW = TX + 6, NC = TX * TY;
  T sx[ZQ][TY * SW];
  T sy[ZQ][(TY + 6) * TX];
  T sz[ZQ][NC];
};

template <class T, class O, int TX, int TY, bool ZON, bool XO>
__global__ void __launch_bounds__(TX * TY) k_div25(const T* __restrict__ fx, const T* __restrict__ fy,
                                                   const T* __restrict__ fz, O* __restrict__ out, Grid g,
                                                   Coef3<T> cf, int odd, T dt, int divide, StatPart* part,
                                                   int kc, double* wpart, int wmask) {
  pdl_enter();
  using Ring = DivRing<T, TX, TY>;
  constexpr int SW = Ring::SW;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  Ring& sm = *reinterpret_cast<Ring*>(smem_raw);
  const int tx = threadIdx.x, ty = threadIdx.y, t = ty * TX + tx;
  const int i0 = blockIdx.x * TX, j0 = blockIdx.y * TY;
  const int i = i0 + tx, j = j0 + ty;
  const bool valid = i < g.nx && j < g.ny;
  const int k0 = blockIdx.z * kc;
  const int np = min(kc, g.nz - k0);
  constexpr bool zon = ZON;  // z derivatives (false: 2D, derz_2dsim)
  const bool may_flip = odd && (g.bc[0] == AX_MIRROR || g.bc[1] == AX_MIRROR || g.bc[2] == AX_MIRROR);
  const int ox = odd ? 0 : -1, oy = odd ? 1 : -1, oz = odd ? 2 : -1;
  const XYCell cc = xy_cell(g, i, j);
  const Halo<TX, TY> h = halo_cell<TX, TY>(g, i0, j0, t);
  const T* __restrict__ hf = h.xh ? fx : fy;  // x-halos belong to the x-lines of fx, y-halos to fy
  const int hodd = h.xh ? ox : oy;
  const int cxi = ty * SW + tx + 3, cyi = (ty + 3) * TX + tx;
  const int pcx = XO ? xclass(g, i) : 0;
  const long long out0 = valid ? (long long)i + (long long)g.nx * j : 0;
  const long long sz = g.sz();

  auto issue = [&](int lp, int st) {
    const long long zo = z_plane(g, k0 + lp).off;
    if (zon && lp <= np + 2) cp_async<sizeof(T)>(&sm.sz[st][t], fz + zo + cc.off);
    if (lp < np) {
      cp_async<sizeof(T)>(&sm.sx[st][cxi], fx + zo + cc.off);
      cp_async<sizeof(T)>(&sm.sy[st][cyi], fy + zo + cc.off);
      if (h.on) cp_async<sizeof(T)>(h.xh ? &sm.sx[st][h.lidx] : &sm.sy[st][h.lidx], hf + zo + h.c.off);
    }
    cp_async_commit();
  };
  auto fix = [&](int lp, int st) {
    if (!may_flip) return;
    const bool fz_ = z_plane(g, k0 + lp).fz;
    if (zon && lp <= np + 2 && flips(cc, fz_, oz)) sm.sz[st][t] = -sm.sz[st][t];
    if (lp < np) {
      if (flips(cc, fz_, ox)) sm.sx[st][cxi] = -sm.sx[st][cxi];
      if (flips(cc, fz_, oy)) sm.sy[st][cyi] = -sm.sy[st][cyi];
      if (h.on && flips(h.c, fz_, hodd)) {
        T* cell = h.xh ? &sm.sx[st][h.lidx] : &sm.sy[st][h.lidx];
        *cell = -*cell;
      }
    }
  };

  T q[ZQ];
#pragma unroll
  for (int m = 0; m < ZQ; ++m) q[m] = (T)0;
#pragma unroll
  for (int lp = 0; lp < PD + 3; ++lp) issue(lp, lp);
  if constexpr (zon) {
#pragma unroll
    for (int m = 0; m < 3; ++m) q[m] = ldc<T>(fz, cc, z_plane(g, k0 - 3 + m), oz);
  }
  cp_async_wait<PD>();
#pragma unroll
  for (int m = 0; m < 3; ++m) {
    fix(m, m);
    if (zon) q[3 + m] = sm.sz[m][t];
  }
  T mn = (T)INFINITY, mx = (T)-INFINITY;
  long long imx = 0x7fffffffffffffffll;
  // column sum: FP64 for T = double; a TwoSum-compensated FP32 pair for
  // T = float (exact to ~2^-48 over the chunk), widened once at the end
  double sum = 0.0;
  float sum_hi = 0.f, sum_lo = 0.f;
  // with wpart (T = float): the trapezoid-weighted sum of the values written,
  // weight 1/2 at each end of an axis whose bit is set in wmask (the mirror
  // axes of the pressure grid), in a TwoSum pair; the weights are powers of
  // two, so each weighted term is exact
  float wsum_hi = 0.f, wsum_lo = 0.f;
  const float wxy = (((wmask & 1) && (i == 0 || i == g.nx - 1)) ? 0.5f : 1.f) *
                    (((wmask & 2) && (j == 0 || j == g.ny - 1)) ? 0.5f : 1.f);
  for (int lb = 0; lb < np; lb += ZQ) {
#pragma unroll
    for (int u = 0; u < ZQ; ++u) {
      const int lp = lb + u;
      if (lp < np) {
        cp_async_wait<PD - 1>();
        fix(lp + 3, (u + 3) % ZQ);
        __syncthreads();
        issue(lp + 3 + PD, (u + 3 + PD) % ZQ);
        if (zon) q[(u + 6) % ZQ] = sm.sz[(u + 3) % ZQ][t];
        T v[7];
#pragma unroll
        for (int m = 0; m < 7; ++m) v[m] = sm.sx[u][cxi - 3 + m];
        const T ddx = d1x<XO>(v, cf.ax[0], pcx);
#pragma unroll
        for (int m = 0; m < 7; ++m) v[m] = sm.sy[u][cyi + (m - 3) * TX];
        const T ddy = d1(v, cf.ax[1]);
#pragma unroll
        for (int m = 0; m < 7; ++m) v[m] = q[(u + m) % ZQ];
        const T ddz = zon ? d1(v, cf.ax[2]) : (T)0;
        const T div = ddx + ddy + ddz;
        if (valid) {
          const long long p = out0 + sz * (k0 + lp);
          const T ov = divide ? div / dt : div;
          if (out) out[p] = to_t<O>(ov);
          if constexpr (sizeof(T) == 4) {
            two_sum_acc(sum_hi, sum_lo, (float)div);
            if (wpart) {
              const int k = k0 + lp;
              const float wz = ((wmask & 4) && (k == 0 || k == g.nz - 1)) ? 0.5f : 1.f;
              two_sum_acc(wsum_hi, wsum_lo, (wxy * wz) * (float)ov);
            }
          } else {
            sum += (double)div;
          }
          if (div < mn) mn = div;
          if (div > mx) { mx = div; imx = p; }  // k ascends: the first max of the column is kept
        }
      }
    }
  }
  cp_async_wait<0>();
  if constexpr (sizeof(T) == 4) sum = to_t<double>(sum_hi) + to_t<double>(sum_lo);
  if (part) {
    if (!(mx >= mn)) { mn = (T)INFINITY; mx = (T)-INFINITY; imx = 0x7fffffffffffffffll; }
    block_stat_t<T>(mn, mx, sum, imx, part, block_linear_id());
  }
  if (wpart) {
    double r[1] = {to_t<double>(wsum_hi) + to_t<double>(wsum_lo)};
    const int ops[1] = {RED_SUM};
    block_reduce_store<1>(r, ops, wpart, block_linear_id());
  }
}

// ---------------------------------------------------------------------------
// correct_velocity (src/integration.f90:297-325) with the per-step extrema of
// the corrected velocity accumulated per thread.  The pressure may be stored
// wider than T (FP64 pressure, FP32 velocity): its cells land in a ring of
// the storage type and each thread converts the cells it copied into the
// T tile before the barrier.  u* of plane lp travels in group(lp + 3),
// issued at iteration lp - PD, into a (PD+1)-stage ring.
// ---------------------------------------------------------------------------
template <class T, class S, int TX, int TY>
struct CorrRing {
  static constexpr int SW = TX + 6, PL = (TY + 6) * SW, NC = TX * TY;
  static constexpr bool CONV = sizeof(S) != sizeof(T);
  S land[CONV ? ZQ : 1][PL];
  T tile[ZQ][PL];
  T up[PD + 1][3][NC];
};

template <class T, class S, int TX, int TY, bool ZON, bool XO>
__global__ void __launch_bounds__(TX * TY) k_correct25(CorrArgs<T, S> A, int kc) {
  pdl_enter();
  using Ring = CorrRing<T, S, TX, TY>;
  constexpr int SW = Ring::SW;
  constexpr bool CONV = Ring::CONV;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  Ring& sm = *reinterpret_cast<Ring*>(smem_raw);
  const Grid& g = A.g;
  const int tx = threadIdx.x, ty = threadIdx.y, t = ty * TX + tx;
  const int i0 = blockIdx.x * TX, j0 = blockIdx.y * TY;
  const int i = i0 + tx, j = j0 + ty;
  const bool valid = i < g.nx && j < g.ny;
  const int k0 = blockIdx.z * kc;
  const int np = min(kc, g.nz - k0);
  constexpr bool zon = ZON;  // z derivatives (false: 2D, derz_2dsim)
  const int pcx = XO ? xclass(g, i) : 0;  // open x axis: closure class; 1 = inflow node (held)
  const XYCell cc = xy_cell(g, i, j);
  const Halo<TX, TY> h = halo_cell<TX, TY>(g, i0, j0, t);
  const int sc = (ty + 3) * SW + tx + 3;
  const long long out0 = valid ? (long long)i + (long long)g.nx * j : 0;
  const long long sz = g.sz();
  const int last_centre = zon ? np + 2 : np - 1;

  auto dst = [&](int st, int idx) -> void* {
    if constexpr (CONV) return &sm.land[st][idx];
    else return &sm.tile[st][idx];
  };
  auto issue = [&](int lp, int st) {
    if (lp <= last_centre) {
      const long long zo = z_plane(g, k0 + lp).off;
      cp_async<sizeof(S)>(dst(st, sc), A.p + zo + cc.off);
      if (lp < np && h.on) cp_async<sizeof(S)>(dst(st, h.tidx), A.p + zo + h.c.off);
    }
    const int lu = lp - 3;
    if (lu >= 0 && lu < np && valid) {
      const long long q = out0 + sz * (k0 + lu);
#pragma unroll
      for (int a = 0; a < 3; ++a) cp_async<sizeof(T)>(&sm.up[lu & PD][a][t], A.up[a] + q);
    }
    cp_async_commit();
  };
  // the pressure is even in every axis: landing cells only need the conversion
  auto fix = [&](int lp, int st) {
    if constexpr (CONV) {
      if (lp > last_centre) return;
      sm.tile[st][sc] = to_t<T>(sm.land[st][sc]);
      if (lp < np && h.on) sm.tile[st][h.tidx] = to_t<T>(sm.land[st][h.tidx]);
    }
  };

  T q[ZQ];
#pragma unroll
  for (int m = 0; m < ZQ; ++m) q[m] = (T)0;
#pragma unroll
  for (int lp = 0; lp < PD + 3; ++lp) issue(lp, lp);
  if constexpr (zon) {
#pragma unroll
    for (int m = 0; m < 3; ++m) q[m] = ldc<T>(A.p, cc, z_plane(g, k0 - 3 + m), -1);
  }
  cp_async_wait<PD>();
#pragma unroll
  for (int m = 0; m < 3; ++m) {
    fix(m, m);
    if (zon) q[3 + m] = sm.tile[m][sc];
  }
  T mn[3], mx[3], am[3];
#pragma unroll
  for (int a = 0; a < 3; ++a) { mn[a] = (T)INFINITY; mx[a] = (T)-INFINITY; am[a] = (T)0; }
  bool nan = false;
  for (int lb = 0; lb < np; lb += ZQ) {
#pragma unroll
    for (int u = 0; u < ZQ; ++u) {
      const int lp = lb + u;
      if (lp < np) {
        cp_async_wait<PD - 1>();
        fix(lp + 3, (u + 3) % ZQ);
        __syncthreads();
        issue(lp + 3 + PD, (u + 3 + PD) % ZQ);
        if (zon) q[(u + 6) % ZQ] = sm.tile[(u + 3) % ZQ][sc];
        T v[7], gp[3];
#pragma unroll
        for (int m = 0; m < 7; ++m) v[m] = sm.tile[u][sc - 3 + m];
        gp[0] = d1x<XO>(v, A.cf.ax[0], pcx);
#pragma unroll
        for (int m = 0; m < 7; ++m) v[m] = sm.tile[u][sc + (m - 3) * SW];
        gp[1] = d1(v, A.cf.ax[1]);
#pragma unroll
        for (int m = 0; m < 7; ++m) v[m] = q[(u + m) % ZQ];
        gp[2] = zon ? d1(v, A.cf.ax[2]) : (T)0;
        if (valid) {
          const long long p = out0 + sz * (k0 + lp);
          const int us = lp & PD;
#pragma unroll
          for (int a = 0; a < 3; ++a) {
            const T un = pcx == 1 ? sm.up[us][a][t] : sm.up[us][a][t] - A.dt * gp[a];  // inflow held
            A.u[a][p] = un;
            if (un != un) nan = true;
            mn[a] = fmin(mn[a], un);
            mx[a] = fmax(mx[a], un);
            am[a] = fmax(am[a], fabs(un));
          }
        }
      }
    }
  }
  cp_async_wait<0>();
  T r[10];
  const int ops[10] = {RED_MIN, RED_MIN, RED_MIN, RED_MAX, RED_MAX, RED_MAX,
                       RED_MAX, RED_MAX, RED_MAX, RED_MAX};
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    r[a] = mn[a];
    r[3 + a] = mx[a];
    r[6 + a] = am[a];
  }
  r[9] = nan ? (T)1 : (T)0;
  block_reduce_store_t<T, 10>(r, ops, A.part, block_linear_id());
}

// ---------------------------------------------------------------------------
// launchers
// ---------------------------------------------------------------------------
template <class T, bool LES, bool ZON, bool XO>
static void predict_launch(const PredArgs<T>& a, cudaStream_t s) {
  constexpr size_t bytes = sizeof(PredRing<T, TX25, TY25>);
  static std::atomic<bool> attr[SMEM_MAX_DEVICES];
  allow_smem(k_predict25<T, TX25, TY25, LES, ZON, XO>, bytes, attr);
  launch_pdl(k_predict25<T, TX25, TY25, LES, ZON, XO>, grid25(a.g), dim3(TX25, TY25), bytes, s, a, KC25);
}
template <class T, bool XO>
static void predict_launch_xo(const PredArgs<T>& a, cudaStream_t s) {
  const bool zon = a.g.bc[2] != AX_ZERO;
  if (a.les) {
    if (zon) predict_launch<T, true, true, XO>(a, s);
    else predict_launch<T, true, false, XO>(a, s);
  } else {
    if (zon) predict_launch<T, false, true, XO>(a, s);
    else predict_launch<T, false, false, XO>(a, s);
  }
}
// the open-x closures are compiled in only for grids with an open x axis
template <class T>
void launch_predict(const PredArgs<T>& a, cudaStream_t s) {
  if constexpr (sizeof(T) == 4) {
    if (stencil_v_ok(a.g)) {
      launch_predict_v(a, s);
      return;
    }
  }
  if (a.g.bc[0] == AX_OPEN) predict_launch_xo<T, true>(a, s);
  else predict_launch_xo<T, false>(a, s);
}

template <class T, class O, bool ZON, bool XO>
static void div_launch(const T* fx, const T* fy, const T* fz, O* out, const Grid& g, const Coef3<T>& cf, int odd,
                       T dt, int divide, StatPart* part, cudaStream_t s, double* wpart, int wmask) {
  constexpr size_t bytes = sizeof(DivRing<T, TX25, TY25>);
  static std::atomic<bool> attr[SMEM_MAX_DEVICES];
  allow_smem(k_div25<T, O, TX25, TY25, ZON, XO>, bytes, attr);
  launch_pdl(k_div25<T, O, TX25, TY25, ZON, XO>, grid25(g), dim3(TX25, TY25), bytes, s, fx, fy, fz, out, g, cf, odd,
             dt, divide, part, KC25, wpart, wmask);
}
template <class T, class O>
void launch_div(const T* fx, const T* fy, const T* fz, O* out, const Grid& g, const Coef3<T>& cf,
                int odd, T dt, int divide, StatPart* part, cudaStream_t s, double* wpart, int wmask) {
  if constexpr (sizeof(T) == 4) {
    if (stencil_v_ok(g)) {
      launch_div_v<O>(fx, fy, fz, out, g, cf, odd, dt, divide, part, s, wpart, wmask);
      return;
    }
  }
  const bool zon = g.bc[2] != AX_ZERO;
  if (g.bc[0] == AX_OPEN) {
    if (zon) div_launch<T, O, true, true>(fx, fy, fz, out, g, cf, odd, dt, divide, part, s, wpart, wmask);
    else div_launch<T, O, false, true>(fx, fy, fz, out, g, cf, odd, dt, divide, part, s, wpart, wmask);
  } else {
    if (zon) div_launch<T, O, true, false>(fx, fy, fz, out, g, cf, odd, dt, divide, part, s, wpart, wmask);
    else div_launch<T, O, false, false>(fx, fy, fz, out, g, cf, odd, dt, divide, part, s, wpart, wmask);
  }
}

template <class T, class S, bool ZON, bool XO>
static void correct_launch(const CorrArgs<T, S>& a, cudaStream_t s) {
  constexpr size_t bytes = sizeof(CorrRing<T, S, TX25, TY25>);
  static std::atomic<bool> attr[SMEM_MAX_DEVICES];
  allow_smem(k_correct25<T, S, TX25, TY25, ZON, XO>, bytes, attr);
  launch_pdl(k_correct25<T, S, TX25, TY25, ZON, XO>, grid25(a.g), dim3(TX25, TY25), bytes, s, a, KC25);
}
template <class T, class S>
void launch_correct(const CorrArgs<T, S>& a, cudaStream_t s) {
  if constexpr (sizeof(T) == 4) {
    if (stencil_v_ok(a.g)) {
      launch_correct_v(a, s);
      return;
    }
  }
  const bool zon = a.g.bc[2] != AX_ZERO;
  if (a.g.bc[0] == AX_OPEN) {
    if (zon) correct_launch<T, S, true, true>(a, s);
    else correct_launch<T, S, false, true>(a, s);
  } else {
    if (zon) correct_launch<T, S, true, false>(a, s);
    else correct_launch<T, S, false, false>(a, s);
  }
}

template void launch_predict<double>(const PredArgs<double>&, cudaStream_t);
template void launch_predict<float>(const PredArgs<float>&, cudaStream_t);
template void launch_div<double, double>(const double*, const double*, const double*, double*, const Grid&,
                                         const Coef3<double>&, int, double, int, StatPart*, cudaStream_t, double*,
                                         int);
template void launch_div<float, float>(const float*, const float*, const float*, float*, const Grid&,
                                       const Coef3<float>&, int, float, int, StatPart*, cudaStream_t, double*, int);
template void launch_div<float, double>(const float*, const float*, const float*, double*, const Grid&,
                                        const Coef3<float>&, int, float, int, StatPart*, cudaStream_t, double*, int);
template void launch_correct<double, double>(const CorrArgs<double, double>&, cudaStream_t);
template void launch_correct<float, double>(const CorrArgs<float, double>&, cudaStream_t);
template void launch_correct<float, float>(const CorrArgs<float, float>&, cudaStream_t);

}  // namespace o3d
