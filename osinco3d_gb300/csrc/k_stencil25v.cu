// k_stencil25v.cu -- FP32 2.5D stencil kernels with two x-adjacent points per
// thread, for the mixed method on grids with nx a multiple of 4 (the
// one-point kernels of k_stencil25.cu serve the other grids and the FP64
// method):
//   k_predict25v   the fused momentum predictor (predict_velocity +
//                  calculate_nu_t, src/integration.f90:106-188,
//                  src/les_turbulence.f90:54-88);
//   k_div25v       divergence (src/differential_operators.f90:25-35) with
//                  function_stats (src/functions.f90:27-63), optionally the
//                  Poisson rhs and its trapezoid-weighted sums;
//   k_correct25v   correct_velocity (src/integration.f90:297-325) with the
//                  extrema of the corrected velocity;
//   k_transeq25v   transeq (src/integration.f90:405-447): the scalar's flux,
//                  AB update, first clipping pass and clipping sums.
//
// A block of 32 x 8 threads owns a 64 x 8 tile of (x, y) points and marches
// along z over a chunk of planes; thread (tx, ty) computes points
// (i0 + 2 tx, j0 + ty) and (i0 + 2 tx + 1, j0 + ty).  Each plane of the
// stencil fields lands in a ring stage of rows with 3 halo rows each side
// where y-lines are needed, and 4 ghost columns each side (3 of them used)
// where x-lines are needed, copied global -> shared by cp.async in 16-byte
// chunks along the rows (the rows are ghost-mapped per row in y and per plane
// in z) and per cell for the x-halo columns and for chunks past the grid end.
// A pair of points then reads its 8-point x-window as 5 aligned float2 loads
// and each row of its y-window as one float2 load, where the one-point
// kernels issue 7 scalar loads per line and point.  The z-neighbours stay in
// a register queue of float2, filled from the ring's centre rows.  Fields
// read once per point (flux history, u*) go through registers, one plane
// ahead of their use, and need no shared memory.
//
// Plane pipeline: a ring of 7 stages, group(lp) copies plane lp and is issued
// PD = 3 planes before the queue head reaches it, as in k_stencil25.cu, but
// the plane loop is not unrolled: with two points per thread an unrolled body
// overflows the instruction cache ("no instruction" was the top warp stall of
// an unrolled version).  Ring stages are runtime indices and the z-queue
// shifts by one slot per plane (slot m holds plane lp - 3 + m).
#include <atomic>

#include "o3d_internal.cuh"
#include "o3d_kernels.h"

namespace o3d {

int v_chunk(const Grid& g, int per_sm);

namespace {

constexpr int ZQ = 7, PD = 3;
constexpr int VX = 64, VY = 8;       // points per tile
constexpr int VTX = 32, VTY = 8;     // threads per block
constexpr int NT = VTX * VTY;
constexpr int VW = VX + 8;           // ring columns: 4 ghost columns each side
constexpr int VR = VY + 6;           // ring rows: 3 halo rows each side
constexpr int NCH = VX / 4;          // 16-byte chunks of a row of floats

__device__ __forceinline__ unsigned smem_u32(const void* p) { return (unsigned)__cvta_generic_to_shared(p); }
__device__ __forceinline__ void cp16(unsigned dst, const void* src) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(dst), "l"(src) : "memory");
}
__device__ __forceinline__ void cp4(unsigned dst, const void* src) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(dst), "l"(src) : "memory");
}
// streaming load of a float pair that is read once (no L1 allocation)
__device__ __forceinline__ float2 ld_stream2(const float* p) {
  float2 v;
  asm volatile("ld.global.nc.L1::no_allocate.v2.f32 {%0, %1}, [%2];\n" : "=f"(v.x), "=f"(v.y) : "l"(p));
  return v;
}
__device__ __forceinline__ float2 lds2(const float* p) { return *reinterpret_cast<const float2*>(p); }

// Raises a kernel's dynamic shared-memory limit above 48 KB, once per device
// (the attribute belongs to the current device).
template <class K>
void allow_smem_v(K* kernel, size_t bytes, std::atomic<bool>* done) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) dev = -1;
  if (dev >= 0 && dev < 64 && done[dev].load(std::memory_order_acquire)) return;
  if (cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes) == cudaSuccess &&
      dev >= 0 && dev < 64)
    done[dev].store(true, std::memory_order_release);
}

// One 16-byte chunk unit of a plane: element offset xy of its first point
// within a plane (the row ghost-mapped), or -1 - row when the chunk lies past
// the x end of the grid (its cells are then copied one by one through the
// ghost map); dst: its float index within a ring stage; x0: the global x of
// its first cell; field: which field it belongs to; flags: 1 = in use, 2 =
// the row is mirrored and the field is odd in y, 4 = needed on every
// plane of the chunk's z-range (z-queue rows; the others only for the planes
// the block computes).
struct Unit {
  int xy, dst, x0;
  unsigned char field, flags;
};

__device__ __forceinline__ Unit unit_of(const Grid& g, int i0, int j0, int rho, int ch, int dst, int field,
                                        bool odd_y, bool zrow) {
  Unit u;
  bool fy;
  const int jj = ghost(j0 + rho - 3, g.ny, g.bc[1], &fy);
  u.x0 = i0 + 4 * ch;
  u.xy = u.x0 < g.nx ? u.x0 + g.nx * jj : -1 - jj;
  u.dst = dst;
  u.field = (unsigned char)field;
  u.flags = 1 | ((fy && odd_y) ? 2 : 0) | (zrow ? 4 : 0);
  return u;
}
__device__ __forceinline__ Unit unit_none() {
  Unit u;
  u.xy = u.dst = u.x0 = 0;
  u.field = 0;
  u.flags = 0;
  return u;
}

// copies one unit of plane z (float fields) into the stage at sbase
__device__ __forceinline__ void issue_unit(const Unit& u, const float* f, const ZPlane& z, const Grid& g,
                                           unsigned sbase) {
  if (u.xy >= 0) {
    cp16(sbase + (unsigned)u.dst * 4u, f + z.off + u.xy);
  } else {  // past the x end: per cell through the ghost map
    const long long row = z.off + (long long)g.nx * (-1 - u.xy);
#pragma unroll
    for (int e = 0; e < 4; ++e) {
      bool fx;
      const int ii = ghost(u.x0 + e, g.nx, g.bc[0], &fx);
      cp4(sbase + (unsigned)(u.dst + e) * 4u, f + row + ii);
    }
  }
}
// negates the cells of a unit this thread copied where the field is odd
// across a mirrored ghost: the row (flag 2), the plane (fz_odd) or, past the
// x end, the column (x_odd)
__device__ __forceinline__ void fix_unit(const Unit& u, float* s, const Grid& g, bool fz_odd, bool x_odd) {
  const bool rowflip = (u.flags & 2) || fz_odd;
  if (u.xy >= 0) {
    if (rowflip) {
#pragma unroll
      for (int e = 0; e < 4; ++e) s[u.dst + e] = -s[u.dst + e];
    }
  } else {
#pragma unroll
    for (int e = 0; e < 4; ++e) {
      bool fx;
      ghost(u.x0 + e, g.nx, g.bc[0], &fx);
      if (rowflip != (fx && x_odd)) s[u.dst + e] = -s[u.dst + e];
    }
  }
}

// One x-halo cell: centre row r (0..7) of the tile, column 1..3 (left) or
// VX + 4 .. VX + 6 (right) of a 72-column row starting at float index base.
struct XCell {
  int xy, dst;
  bool fx, fy;
};
__device__ __forceinline__ XCell xcell_of(const Grid& g, int i0, int j0, int r, int e, int row_base) {
  XCell x;
  const int col = e < 3 ? 1 + e : VX + 4 + (e - 3);
  const int ii = ghost(i0 + col - 4, g.nx, g.bc[0], &x.fx);
  const int jj = ghost(j0 + r, g.ny, g.bc[1], &x.fy);
  x.xy = ii + g.nx * jj;
  x.dst = row_base + col;
  return x;
}

// ---------------------------------------------------------------------------
// predictor.  Ring stage: 14 rows x 3 components x 72 columns; component c
// of the velocity is odd along axis c.
// ---------------------------------------------------------------------------
constexpr int PRS = 3 * VW;         // floats per ring row
constexpr int PS = VR * PRS;        // floats per stage
constexpr int PUNIT = VR * 3 * NCH; // 672 chunk units
constexpr int PUPT = (PUNIT + NT - 1) / NT;
constexpr int PXH = VY * 3 * 6;     // 144 x-halo cells
struct PRing {
  float s[ZQ][PS];
};

template <bool LES, bool ZON, bool XO>
__global__ void __launch_bounds__(NT, 2) k_predict25v(PredArgs<float> A, int kc) {
  pdl_enter();
  extern __shared__ __align__(16) unsigned char smem_raw[];
  PRing& sm = *reinterpret_cast<PRing*>(smem_raw);
  const Grid& g = A.g;
  const int tx = threadIdx.x, ty = threadIdx.y, t = ty * VTX + tx;
  const int i0 = blockIdx.x * VX, j0 = blockIdx.y * VY;
  const int ia = i0 + 2 * tx, j = j0 + ty;
  const bool valid = ia < g.nx && j < g.ny;  // nx is even: both points or neither
  const int k0 = blockIdx.z * kc;
  const int np = min(kc, g.nz - k0);
  constexpr bool zon = ZON;
  const bool may_flip = g.bc[0] == AX_MIRROR || g.bc[1] == AX_MIRROR || g.bc[2] == AX_MIRROR;
  const int pca = XO ? xclass(g, ia) : 0, pcb = XO ? xclass(g, ia + 1) : 0;
  const long long sz = g.sz();
  const long long out0 = valid ? (long long)ia + (long long)g.nx * j : 0;
  const int last_centre = zon ? np + 2 : np - 1;
  const unsigned ring0 = smem_u32(&sm.s[0][0]);

  Unit un[PUPT];
#pragma unroll
  for (int r = 0; r < PUPT; ++r) {
    const int q = t + r * NT;
    if (q < PUNIT) {
      const int rho = q / (3 * NCH), c = (q / NCH) % 3, ch = q % NCH;
      un[r] = unit_of(g, i0, j0, rho, ch, rho * PRS + c * VW + 4 + 4 * ch, c, c == 1, rho >= 3 && rho < 3 + VY);
    } else {
      un[r] = unit_none();
    }
  }
  const bool has_x = t < PXH;
  const int xc_c = (t / 6) % 3;
  const XCell xc = xcell_of(g, i0, j0, has_x ? t / 18 : 0, t % 6, (3 + (has_x ? t / 18 : 0)) * PRS + xc_c * VW);

  // group(lp): plane lp into ring stage st; planes beyond the chunk (the
  // z-queue's last three) only need their centre rows
  auto issue = [&](int lp, int st) {
    if (lp <= last_centre) {
      const ZPlane z = z_plane(g, k0 + lp);
      const unsigned sbase = ring0 + (unsigned)(st * PS) * 4u;
      const bool full = lp < np;
#pragma unroll
      for (int r = 0; r < PUPT; ++r) {
        const Unit& u = un[r];
        if (!(u.flags & 1) || (!full && !(u.flags & 4))) continue;
        issue_unit(u, A.u[u.field], z, g, sbase);
      }
      if (full && has_x) cp4(sbase + (unsigned)xc.dst * 4u, A.u[xc_c] + z.off + xc.xy);
    }
    cp_async_commit();
  };
  auto fix = [&](int lp, int st) {
    if (!may_flip || lp > last_centre) return;
    const bool fz = z_plane(g, k0 + lp).fz;
    float* s = sm.s[st];
    const bool full = lp < np;
#pragma unroll
    for (int r = 0; r < PUPT; ++r) {
      const Unit& u = un[r];
      if (!(u.flags & 1) || (!full && !(u.flags & 4))) continue;
      fix_unit(u, s, g, fz && u.field == 2, u.field == 0);
    }
    if (full && has_x && ((xc_c == 0 && xc.fx) != ((xc_c == 1 && xc.fy) != (xc_c == 2 && fz)))) s[xc.dst] = -s[xc.dst];
  };

  // the pair's own ring position: centre row ty, columns 4 + 2 tx, 5 + 2 tx
  const int own = (ty + 3) * PRS + 4 + 2 * tx;
  float2 q[3][ZQ];
#pragma unroll
  for (int c = 0; c < 3; ++c)
#pragma unroll
    for (int m = 0; m < ZQ; ++m) q[c][m] = make_float2(0.f, 0.f);
#pragma unroll
  for (int lp = 0; lp < PD + 3; ++lp) issue(lp, lp);
  if constexpr (zon) {  // planes -3..-1 through the registers into slots 0..2
    bool fxa, fxb, fyy;
    const int iia = ghost(ia, g.nx, g.bc[0], &fxa), iib = ghost(ia + 1, g.nx, g.bc[0], &fxb);
    const int jj = ghost(j, g.ny, g.bc[1], &fyy);
#pragma unroll
    for (int m = 0; m < 3; ++m) {
      const ZPlane z = z_plane(g, k0 - 3 + m);
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        const float* f = A.u[c] + z.off + (long long)g.nx * jj;
        const bool fl = (c == 1 && fyy) || (c == 2 && z.fz);
        float a = __ldg(f + iia), b = __ldg(f + iib);
        if (fl != (c == 0 && fxa)) a = -a;
        if (fl != (c == 0 && fxb)) b = -b;
        q[c][m] = make_float2(a, b);
      }
    }
  }
  // flux history of plane 0
  float2 h2[3], h3[3];
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    h2[c] = make_float2(0.f, 0.f);
    h3[c] = make_float2(0.f, 0.f);
    if (valid && np > 0) {
      if (A.f2[c]) h2[c] = ld_stream2(A.f2[c] + out0 + sz * k0);
      if (A.f3[c]) h3[c] = ld_stream2(A.f3[c] + out0 + sz * k0);
    }
  }
  cp_async_wait<PD>();  // groups 0..2 landed
#pragma unroll
  for (int m = 0; m < 3; ++m) fix(m, m);
  __syncthreads();  // the queue reads centre cells other threads copied
#pragma unroll
  for (int m = 0; m < 3; ++m)
#pragma unroll
    for (int c = 0; c < 3; ++c) q[c][3 + m] = lds2(&sm.s[m][own + c * VW]);

  // ring slots of planes lp, lp + 3 and lp + 3 + PD, advanced each plane
  int s0 = 0, s3 = 3, s6 = (3 + PD) % ZQ;
#pragma unroll 1
  for (int lp = 0; lp < np; ++lp) {
    cp_async_wait<PD - 1>();  // group(lp + 3) landed
    fix(lp + 3, s3);
    __syncthreads();
    issue(lp + 3 + PD, s6);
    const float* s = sm.s[s0];
    if constexpr (zon) {
#pragma unroll
      for (int c = 0; c < 3; ++c) q[c][6] = lds2(&sm.s[s3][own + c * VW]);
    }
    float2 uc[3];
#pragma unroll
    for (int c = 0; c < 3; ++c) uc[c] = lds2(&s[own + c * VW]);
    const long long p = out0 + sz * (k0 + lp);
    // per component: the pair's x, y, z first derivatives and the sum of its
    // second derivatives
    float g1a[3][3] = {}, g1b[3][3] = {}, lapa[3] = {}, lapb[3] = {};
    auto flux_store = [&](int c, float nua, float nub) {
      const float Fa = nua * lapa[c] - (uc[0].x * g1a[c][0] + uc[1].x * g1a[c][1] + uc[2].x * g1a[c][2]);
      const float Fb = nub * lapb[c] - (uc[0].y * g1b[c][0] + uc[1].y * g1b[c][1] + uc[2].y * g1b[c][2]);
      float upa = uc[c].x + A.adu * Fa, upb = uc[c].y + A.adu * Fb;
      if (A.f2[c]) { upa = upa + A.bdu * h2[c].x; upb = upb + A.bdu * h2[c].y; }
      if (A.f3[c]) { upa = upa + A.cdu * h3[c].x; upb = upb + A.cdu * h3[c].y; }
      if (XO) {  // inflow nodes keep their value
        if (pca == 1) upa = uc[c].x;
        if (pcb == 1) upb = uc[c].y;
      }
      __stcs(reinterpret_cast<float2*>(A.fnew[c] + p), make_float2(Fa, Fb));
      __stcs(reinterpret_cast<float2*>(A.up[c] + p), make_float2(upa, upb));
    };
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      float w[10];  // x-window: columns 2 tx .. 2 tx + 9 of row ty + 3
#pragma unroll
      for (int m = 0; m < 5; ++m) {
        const float2 p2 = lds2(&s[own - 4 + 2 * m + c * VW]);
        w[2 * m] = p2.x;
        w[2 * m + 1] = p2.y;
      }
      g1a[c][0] = d1x<XO>(w + 1, A.cf.ax[0], pca);
      const float g2xa = d2x<XO>(w + 1, A.cf.ax[0], pca);
      g1b[c][0] = d1x<XO>(w + 2, A.cf.ax[0], pcb);
      const float g2xb = d2x<XO>(w + 2, A.cf.ax[0], pcb);
      float va[7], vb[7];
#pragma unroll
      for (int m = 0; m < 7; ++m) {
        const float2 p2 = lds2(&s[own + (m - 3) * PRS + c * VW]);
        va[m] = p2.x;
        vb[m] = p2.y;
      }
      g1a[c][1] = d1(va, A.cf.ax[1]);
      const float g2ya = d2(va, A.cf.ax[1]);
      g1b[c][1] = d1(vb, A.cf.ax[1]);
      const float g2yb = d2(vb, A.cf.ax[1]);
      float g2za = 0.f, g2zb = 0.f;
      if constexpr (zon) {
#pragma unroll
        for (int m = 0; m < 7; ++m) {
          va[m] = q[c][m].x;
          vb[m] = q[c][m].y;
        }
        g1a[c][2] = d1(va, A.cf.ax[2]);
        g2za = d2(va, A.cf.ax[2]);
        g1b[c][2] = d1(vb, A.cf.ax[2]);
        g2zb = d2(vb, A.cf.ax[2]);
      }
      lapa[c] = g2xa + g2ya + g2za;
      lapb[c] = g2xb + g2yb + g2zb;
      if constexpr (!LES) {
        if (valid) flux_store(c, A.onere, A.onere);
      }
    }
    if (valid) {
      if constexpr (LES) {
        auto nut = [&](const float (&g1)[3][3]) {
          const float s11 = g1[0][0], s22 = g1[1][1], s33 = g1[2][2];
          const float s12 = 0.5f * (g1[0][1] + g1[1][0]);
          const float s13 = 0.5f * (g1[0][2] + g1[2][0]);
          const float s23 = 0.5f * (g1[1][2] + g1[2][1]);
          const float smag = sqrtf(2.f * (s11 * s11 + s22 * s22 + s33 * s33 + 2.f * (s12 * s12 + s13 * s13 + s23 * s23)));
          return A.csd2 * smag;
        };
        const float na = nut(g1a), nb = nut(g1b);
        *reinterpret_cast<float2*>(A.nu_t + p) = make_float2(na, nb);
#pragma unroll
        for (int c = 0; c < 3; ++c) flux_store(c, A.onere + na, A.onere + nb);
      }
      // flux history of the next plane, one plane ahead of its use
      if (lp + 1 < np) {
#pragma unroll
        for (int c = 0; c < 3; ++c) {
          if (A.f2[c]) h2[c] = ld_stream2(A.f2[c] + p + sz);
          if (A.f3[c]) h3[c] = ld_stream2(A.f3[c] + p + sz);
        }
      }
    }
    if constexpr (zon) {
#pragma unroll
      for (int c = 0; c < 3; ++c)
#pragma unroll
        for (int m = 0; m < ZQ - 1; ++m) q[c][m] = q[c][m + 1];
    }
    s0 = s0 == ZQ - 1 ? 0 : s0 + 1;
    s3 = s3 == ZQ - 1 ? 0 : s3 + 1;
    s6 = s6 == ZQ - 1 ? 0 : s6 + 1;
  }
  cp_async_wait<0>();
}

// ---------------------------------------------------------------------------
// divergence.  Ring stage: fx as x-lines (8 rows x 72 columns: centre and
// x-halo columns), fy as y-lines (14 rows x 64: centre and 3 halo rows each
// side), fz's centre rows (8 x 64) for the z-queue.  fx, fy, fz are odd along
// x, y, z when `odd` is set.
// ---------------------------------------------------------------------------
constexpr int DX_OFF = 0, DY_OFF = VY * VW, DZ_OFF = DY_OFF + VR * VX;
constexpr int DS = DZ_OFF + VY * VX;          // floats per stage (1984)
constexpr int DUNIT = (VY + VR + VY) * NCH;   // 480 chunk units
constexpr int DUPT = (DUNIT + NT - 1) / NT;
constexpr int DXH = VY * 6;                   // 48 x-halo cells of fx
struct DRing {
  float s[ZQ][DS];
};

template <class O, bool ZON, bool XO>
__global__ void __launch_bounds__(NT, 3) k_div25v(const float* __restrict__ fx, const float* __restrict__ fy,
                                                  const float* __restrict__ fz, O* __restrict__ out, Grid g,
                                                  Coef3<float> cf, int odd, float dt, int divide, StatPart* part,
                                                  int kc, double* wpart, int wmask) {
  pdl_enter();
  extern __shared__ __align__(16) unsigned char smem_raw[];
  DRing& sm = *reinterpret_cast<DRing*>(smem_raw);
  const int tx = threadIdx.x, ty = threadIdx.y, t = ty * VTX + tx;
  const int i0 = blockIdx.x * VX, j0 = blockIdx.y * VY;
  const int ia = i0 + 2 * tx, j = j0 + ty;
  const bool valid = ia < g.nx && j < g.ny;
  const int k0 = blockIdx.z * kc;
  const int np = min(kc, g.nz - k0);
  constexpr bool zon = ZON;
  const bool may_flip = odd && (g.bc[0] == AX_MIRROR || g.bc[1] == AX_MIRROR || g.bc[2] == AX_MIRROR);
  const int pca = XO ? xclass(g, ia) : 0, pcb = XO ? xclass(g, ia + 1) : 0;
  const long long sz = g.sz();
  const long long out0 = valid ? (long long)ia + (long long)g.nx * j : 0;
  const int last_centre = zon ? np + 2 : np - 1;
  const unsigned ring0 = smem_u32(&sm.s[0][0]);

  Unit un[DUPT];
#pragma unroll
  for (int r = 0; r < DUPT; ++r) {
    const int q = t + r * NT;
    const int row = q / NCH, ch = q % NCH;
    if (q >= DUNIT) un[r] = unit_none();
    else if (row < VY)  // fx x-lines: centre rows
      un[r] = unit_of(g, i0, j0, row + 3, ch, DX_OFF + row * VW + 4 + 4 * ch, 0, false, false);
    else if (row < VY + VR)  // fy y-lines: all 14 rows
      un[r] = unit_of(g, i0, j0, row - VY, ch, DY_OFF + (row - VY) * VX + 4 * ch, 1, odd != 0, false);
    else  // fz centre rows, on every plane of the z-queue
      un[r] = unit_of(g, i0, j0, row - VY - VR + 3, ch, DZ_OFF + (row - VY - VR) * VX + 4 * ch, 2, false, true);
  }
  const bool has_x = t < DXH;
  const XCell xc = xcell_of(g, i0, j0, has_x ? t / 6 : 0, t % 6, DX_OFF + (has_x ? t / 6 : 0) * VW);

  auto field = [&](int f) { return f == 0 ? fx : f == 1 ? fy : fz; };
  auto skip = [&](const Unit& u, bool full) {
    return !(u.flags & 1) || (!full && !(u.flags & 4)) || (!zon && (u.flags & 4));
  };
  auto issue = [&](int lp, int st) {
    if (lp <= last_centre) {
      const ZPlane z = z_plane(g, k0 + lp);
      const unsigned sbase = ring0 + (unsigned)(st * DS) * 4u;
      const bool full = lp < np;
#pragma unroll
      for (int r = 0; r < DUPT; ++r) {
        const Unit& u = un[r];
        if (skip(u, full)) continue;
        issue_unit(u, field(u.field), z, g, sbase);
      }
      if (full && has_x) cp4(sbase + (unsigned)xc.dst * 4u, fx + z.off + xc.xy);
    }
    cp_async_commit();
  };
  auto fix = [&](int lp, int st) {
    if (!may_flip || lp > last_centre) return;
    const bool fz_ = z_plane(g, k0 + lp).fz;
    float* s = sm.s[st];
    const bool full = lp < np;
#pragma unroll
    for (int r = 0; r < DUPT; ++r) {
      const Unit& u = un[r];
      if (skip(u, full)) continue;
      fix_unit(u, s, g, fz_ && u.field == 2, u.field == 0);
    }
    if (full && has_x && xc.fx) s[xc.dst] = -s[xc.dst];
  };

  const int ownx = DX_OFF + ty * VW + 4 + 2 * tx;    // the pair in the x-lines
  const int owny = DY_OFF + (ty + 3) * VX + 2 * tx;  // the pair in the y-lines
  const int ownz = DZ_OFF + ty * VX + 2 * tx;        // the pair in the z centres
  float2 q[ZQ];
#pragma unroll
  for (int m = 0; m < ZQ; ++m) q[m] = make_float2(0.f, 0.f);
#pragma unroll
  for (int lp = 0; lp < PD + 3; ++lp) issue(lp, lp);
  if constexpr (zon) {
    bool fxa, fxb, fyy;
    const int iia = ghost(ia, g.nx, g.bc[0], &fxa), iib = ghost(ia + 1, g.nx, g.bc[0], &fxb);
    const int jj = ghost(j, g.ny, g.bc[1], &fyy);
#pragma unroll
    for (int m = 0; m < 3; ++m) {
      const ZPlane z = z_plane(g, k0 - 3 + m);
      const float* f = fz + z.off + (long long)g.nx * jj;
      float a = __ldg(f + iia), b = __ldg(f + iib);
      if (odd && z.fz) { a = -a; b = -b; }
      q[m] = make_float2(a, b);
    }
  }
  cp_async_wait<PD>();
#pragma unroll
  for (int m = 0; m < 3; ++m) fix(m, m);
  __syncthreads();
  if constexpr (zon) {
#pragma unroll
    for (int m = 0; m < 3; ++m) q[3 + m] = lds2(&sm.s[m][ownz]);
  }
  float mn = INFINITY, mx = -INFINITY;
  long long imx = 0x7fffffffffffffffll;
  // the column sum and the trapezoid-weighted sum of the values written, in
  // TwoSum-compensated FP32 pairs (the weights are powers of two, so each
  // weighted term is exact)
  float sum_hi = 0.f, sum_lo = 0.f, wsum_hi = 0.f, wsum_lo = 0.f;
  const float rdt = 1.f / dt;
  const float wyy = ((wmask & 2) && (j == 0 || j == g.ny - 1)) ? 0.5f : 1.f;
  const float wxa = (((wmask & 1) && (ia == 0 || ia == g.nx - 1)) ? 0.5f : 1.f) * wyy;
  const float wxb = (((wmask & 1) && (ia + 1 == 0 || ia + 1 == g.nx - 1)) ? 0.5f : 1.f) * wyy;
  // ring slots of planes lp, lp + 3 and lp + 3 + PD, advanced each plane
  int s0 = 0, s3 = 3, s6 = (3 + PD) % ZQ;
#pragma unroll 1
  for (int lp = 0; lp < np; ++lp) {
    cp_async_wait<PD - 1>();
    fix(lp + 3, s3);
    __syncthreads();
    issue(lp + 3 + PD, s6);
    const float* s = sm.s[s0];
    if constexpr (zon) q[6] = lds2(&sm.s[s3][ownz]);
    float w[10];
#pragma unroll
    for (int m = 0; m < 5; ++m) {
      const float2 p2 = lds2(&s[ownx - 4 + 2 * m]);
      w[2 * m] = p2.x;
      w[2 * m + 1] = p2.y;
    }
    const float ddxa = d1x<XO>(w + 1, cf.ax[0], pca), ddxb = d1x<XO>(w + 2, cf.ax[0], pcb);
    float va[7], vb[7];
#pragma unroll
    for (int m = 0; m < 7; ++m) {
      const float2 p2 = lds2(&s[owny + (m - 3) * VX]);
      va[m] = p2.x;
      vb[m] = p2.y;
    }
    const float ddya = d1(va, cf.ax[1]), ddyb = d1(vb, cf.ax[1]);
    float ddza = 0.f, ddzb = 0.f;
    if constexpr (zon) {
#pragma unroll
      for (int m = 0; m < 7; ++m) {
        va[m] = q[m].x;
        vb[m] = q[m].y;
      }
      ddza = d1(va, cf.ax[2]);
      ddzb = d1(vb, cf.ax[2]);
#pragma unroll
      for (int m = 0; m < ZQ - 1; ++m) q[m] = q[m + 1];
    }
    const float da = ddxa + ddya + ddza, db = ddxb + ddyb + ddzb;
    if (valid) {
      const long long p = out0 + sz * (k0 + lp);
      // div / dt as a product with 1 / dt, formed once: an IEEE division per
      // point costs more than the rest of the pair's arithmetic together
      // (the FP32 rhs then differs from the quotient by at most an ulp)
      const float oa = divide ? da * rdt : da, ob = divide ? db * rdt : db;
      if (out) {
        if constexpr (sizeof(O) == 8)
          __stcs(reinterpret_cast<double2*>(out + p), make_double2(to_t<double>(oa), to_t<double>(ob)));
        else
          __stcs(reinterpret_cast<float2*>(out + p), make_float2(oa, ob));
      }
      two_sum_acc(sum_hi, sum_lo, da);
      two_sum_acc(sum_hi, sum_lo, db);
      if (wpart) {
        const int k = k0 + lp;
        const float wz = ((wmask & 4) && (k == 0 || k == g.nz - 1)) ? 0.5f : 1.f;
        two_sum_acc(wsum_hi, wsum_lo, (wxa * wz) * oa);
        two_sum_acc(wsum_hi, wsum_lo, (wxb * wz) * ob);
      }
      mn = fminf(mn, fminf(da, db));
      if (da > mx) { mx = da; imx = p; }  // k ascends, a before b: the first max is kept
      if (db > mx) { mx = db; imx = p + 1; }
    }
    s0 = s0 == ZQ - 1 ? 0 : s0 + 1;
    s3 = s3 == ZQ - 1 ? 0 : s3 + 1;
    s6 = s6 == ZQ - 1 ? 0 : s6 + 1;
  }
  cp_async_wait<0>();
  if (part) {
    if (!(mx >= mn)) { mn = INFINITY; mx = -INFINITY; imx = 0x7fffffffffffffffll; }
    block_stat_t<float>(mn, mx, to_t<double>(sum_hi) + to_t<double>(sum_lo), imx, part, block_linear_id());
  }
  if (wpart) {
    double r[1] = {to_t<double>(wsum_hi) + to_t<double>(wsum_lo)};
    const int ops[1] = {RED_SUM};
    block_reduce_store<1>(r, ops, wpart, block_linear_id());
  }
}

// ---------------------------------------------------------------------------
// correction, for the mixed method: FP64 pressure, FP32 velocity.  The
// pressure's rows land as FP64 in a ring of 6 stages (16-byte chunks of two
// points; the x-halo cells one by one): the prologue has 6 planes in flight.
// Each thread converts the cells it copied into a ring of 5 FP32 stages (14
// rows x 72 columns) on the integer pipe before the barrier: the planes
// lp - 1 (still read by threads that have not reached the barrier) to lp + 3
// (being converted).  The pressure is even in every axis, so nothing flips.
// ---------------------------------------------------------------------------
constexpr int CL = VR * VW;          // doubles (landing) or floats (tile) per stage
constexpr int CCH = VX / 2;          // 16-byte chunks of a row of doubles (32)
constexpr int CUNIT = VR * CCH;      // 448 chunk units
constexpr int CUPT = (CUNIT + NT - 1) / NT;
constexpr int CLAND = 6;             // FP64 landing stages
constexpr int CTILE = 5;             // FP32 tile stages
struct CRing {
  double land[CLAND][CL];
  float tile[CTILE][CL];
};

template <bool ZON, bool XO>
__global__ void __launch_bounds__(NT, 3) k_correct25v(CorrArgs<float, double> A, int kc) {
  pdl_enter();
  extern __shared__ __align__(16) unsigned char smem_raw[];
  CRing& sm = *reinterpret_cast<CRing*>(smem_raw);
  const Grid& g = A.g;
  const int tx = threadIdx.x, ty = threadIdx.y, t = ty * VTX + tx;
  const int i0 = blockIdx.x * VX, j0 = blockIdx.y * VY;
  const int ia = i0 + 2 * tx, j = j0 + ty;
  const bool valid = ia < g.nx && j < g.ny;
  const int k0 = blockIdx.z * kc;
  const int np = min(kc, g.nz - k0);
  constexpr bool zon = ZON;
  const int pca = XO ? xclass(g, ia) : 0, pcb = XO ? xclass(g, ia + 1) : 0;
  const long long sz = g.sz();
  const long long out0 = valid ? (long long)ia + (long long)g.nx * j : 0;
  const int last_centre = zon ? np + 2 : np - 1;
  const unsigned land0 = smem_u32(&sm.land[0][0]);

  // chunk units: row rho (0..13), chunk ch (points 2 ch, 2 ch + 1); xy < 0:
  // past the x end, per cell through the ghost map (-1 - row)
  int cxy[CUPT], cdst[CUPT], cx0[CUPT];
  bool cuse[CUPT], ccen[CUPT];
#pragma unroll
  for (int r = 0; r < CUPT; ++r) {
    const int q = t + r * NT;
    cuse[r] = q < CUNIT;
    const int rho = cuse[r] ? q / CCH : 0, ch = q % CCH;
    bool fy;
    const int jj = ghost(j0 + rho - 3, g.ny, g.bc[1], &fy);
    cx0[r] = i0 + 2 * ch;
    cxy[r] = cx0[r] < g.nx ? cx0[r] + g.nx * jj : -1 - jj;
    cdst[r] = rho * VW + 4 + 2 * ch;
    ccen[r] = rho >= 3 && rho < 3 + VY;
  }
  const bool has_x = t < VY * 6;
  const XCell xc = xcell_of(g, i0, j0, has_x ? t / 6 : 0, t % 6, (3 + (has_x ? t / 6 : 0)) * VW);

  auto issue = [&](int lp) {
    if (lp <= last_centre) {
      const ZPlane z = z_plane(g, k0 + lp);
      const int ls = lp % CLAND;
      const unsigned sbase = land0 + (unsigned)(ls * CL) * 8u;
      const bool full = lp < np;
      const double* f = A.p + z.off;
#pragma unroll
      for (int r = 0; r < CUPT; ++r) {
        if (!cuse[r] || (!full && !ccen[r])) continue;
        if (cxy[r] >= 0) {
          cp16(sbase + (unsigned)cdst[r] * 8u, f + cxy[r]);
        } else {
          const long long row = (long long)g.nx * (-1 - cxy[r]);
#pragma unroll
          for (int e = 0; e < 2; ++e) {
            bool fxx;
            const int ii = ghost(cx0[r] + e, g.nx, g.bc[0], &fxx);
            cp_async<8>(&sm.land[ls][cdst[r] + e], f + row + ii);
          }
        }
      }
      if (full && has_x) cp_async<8>(&sm.land[ls][xc.dst], f + xc.xy);
    }
    cp_async_commit();
  };
  // convert the cells this thread copied for plane lp into its tile stage
  auto fix = [&](int lp) {
    if (lp > last_centre) return;
    const double* l = sm.land[lp % CLAND];
    float* d = sm.tile[lp % CTILE];
    const bool full = lp < np;
#pragma unroll
    for (int r = 0; r < CUPT; ++r) {
      if (!cuse[r] || (!full && !ccen[r])) continue;
      const double2 v = *reinterpret_cast<const double2*>(&l[cdst[r]]);
      *reinterpret_cast<float2*>(&d[cdst[r]]) = make_float2(f64_to_f32(v.x), f64_to_f32(v.y));
    }
    if (full && has_x) d[xc.dst] = f64_to_f32(l[xc.dst]);
  };

  const int own = (ty + 3) * VW + 4 + 2 * tx;
  float2 q[ZQ];
#pragma unroll
  for (int m = 0; m < ZQ; ++m) q[m] = make_float2(0.f, 0.f);
#pragma unroll
  for (int lp = 0; lp < PD + 3; ++lp) issue(lp);
  if constexpr (zon) {
    bool fxa, fxb, fyy;
    const int iia = ghost(ia, g.nx, g.bc[0], &fxa), iib = ghost(ia + 1, g.nx, g.bc[0], &fxb);
    const int jj = ghost(j, g.ny, g.bc[1], &fyy);
#pragma unroll
    for (int m = 0; m < 3; ++m) {
      const ZPlane z = z_plane(g, k0 - 3 + m);
      const double* f = A.p + z.off + (long long)g.nx * jj;
      q[m] = make_float2(f64_to_f32(__ldg(f + iia)), f64_to_f32(__ldg(f + iib)));
    }
  }
  float2 us[3];
#pragma unroll
  for (int a = 0; a < 3; ++a) us[a] = (valid && np > 0) ? ld_stream2(A.up[a] + out0 + sz * k0) : make_float2(0.f, 0.f);
  cp_async_wait<PD>();
#pragma unroll
  for (int m = 0; m < 3; ++m) fix(m);
  __syncthreads();
  if constexpr (zon) {
#pragma unroll
    for (int m = 0; m < 3; ++m) q[3 + m] = lds2(&sm.tile[m][own]);
  }
  float mn[3], mx[3], am[3];
#pragma unroll
  for (int a = 0; a < 3; ++a) { mn[a] = INFINITY; mx[a] = -INFINITY; am[a] = 0.f; }
  bool nan = false;
#pragma unroll 1
  for (int lp = 0; lp < np; ++lp) {
    cp_async_wait<PD - 1>();
    fix(lp + 3);
    __syncthreads();
    issue(lp + 3 + PD);
    const float* s = sm.tile[lp % CTILE];
    if constexpr (zon) q[6] = lds2(&sm.tile[(lp + 3) % CTILE][own]);
    float w[10];
#pragma unroll
    for (int m = 0; m < 5; ++m) {
      const float2 p2 = lds2(&s[own - 4 + 2 * m]);
      w[2 * m] = p2.x;
      w[2 * m + 1] = p2.y;
    }
    float ga[3], gb[3];
    ga[0] = d1x<XO>(w + 1, A.cf.ax[0], pca);
    gb[0] = d1x<XO>(w + 2, A.cf.ax[0], pcb);
    float va[7], vb[7];
#pragma unroll
    for (int m = 0; m < 7; ++m) {
      const float2 p2 = lds2(&s[own + (m - 3) * VW]);
      va[m] = p2.x;
      vb[m] = p2.y;
    }
    ga[1] = d1(va, A.cf.ax[1]);
    gb[1] = d1(vb, A.cf.ax[1]);
    ga[2] = gb[2] = 0.f;
    if constexpr (zon) {
#pragma unroll
      for (int m = 0; m < 7; ++m) {
        va[m] = q[m].x;
        vb[m] = q[m].y;
      }
      ga[2] = d1(va, A.cf.ax[2]);
      gb[2] = d1(vb, A.cf.ax[2]);
#pragma unroll
      for (int m = 0; m < ZQ - 1; ++m) q[m] = q[m + 1];
    }
    if (valid) {
      const long long p = out0 + sz * (k0 + lp);
#pragma unroll
      for (int a = 0; a < 3; ++a) {
        float na = us[a].x - A.dt * ga[a], nb = us[a].y - A.dt * gb[a];
        if (XO) {  // inflow nodes keep their value
          if (pca == 1) na = us[a].x;
          if (pcb == 1) nb = us[a].y;
        }
        __stcs(reinterpret_cast<float2*>(A.u[a] + p), make_float2(na, nb));
        if (na != na || nb != nb) nan = true;
        mn[a] = fminf(mn[a], fminf(na, nb));
        mx[a] = fmaxf(mx[a], fmaxf(na, nb));
        am[a] = fmaxf(am[a], fmaxf(fabsf(na), fabsf(nb)));
      }
      if (lp + 1 < np) {
#pragma unroll
        for (int a = 0; a < 3; ++a) us[a] = ld_stream2(A.up[a] + p + sz);
      }
    }
  }
  cp_async_wait<0>();
  float r[10];
  const int ops[10] = {RED_MIN, RED_MIN, RED_MIN, RED_MAX, RED_MAX, RED_MAX, RED_MAX, RED_MAX, RED_MAX, RED_MAX};
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    r[a] = mn[a];
    r[3 + a] = mx[a];
    r[6 + a] = am[a];
  }
  r[9] = nan ? 1.f : 0.f;
  block_reduce_store_t<float, 10>(r, ops, A.part, block_linear_id());
}

// ---------------------------------------------------------------------------
// transeq for the mixed method (src/integration.f90:405-447): the scalar flux,
// its AB update and the first clipping pass, with the three clipping sums of
// the reference (phi before clipping, after clipping, and the weights
// min(phi, 1 - phi)) accumulated per thread in TwoSum-compensated FP32 pairs
// and widened once for the block reduction.  The scalar's plane lands in a
// ring stage of 14 rows x 72 columns (it is even in every axis: no sign
// fixes); u, v, w, nu_t, the source and the flux history come through
// registers, one plane ahead.
// ---------------------------------------------------------------------------
constexpr int TS = VR * VW;        // floats per stage
constexpr int TUNIT = VR * NCH;    // 224 chunk units
struct TRing {
  float s[ZQ][TS];
};

template <bool LES, bool ZON, bool XO>
__global__ void __launch_bounds__(NT, 3) k_transeq25v(ScalArgs<float> A, int kc) {
  pdl_enter();
  extern __shared__ __align__(16) unsigned char smem_raw[];
  TRing& sm = *reinterpret_cast<TRing*>(smem_raw);
  const Grid& g = A.g;
  const int tx = threadIdx.x, ty = threadIdx.y, t = ty * VTX + tx;
  const int i0 = blockIdx.x * VX, j0 = blockIdx.y * VY;
  const int ia = i0 + 2 * tx, j = j0 + ty;
  const bool valid = ia < g.nx && j < g.ny;
  const int k0 = blockIdx.z * kc;
  const int np = min(kc, g.nz - k0);
  constexpr bool zon = ZON;
  const int pca = XO ? xclass(g, ia) : 0, pcb = XO ? xclass(g, ia + 1) : 0;
  const long long sz = g.sz();
  const long long out0 = valid ? (long long)ia + (long long)g.nx * j : 0;
  const int last_centre = zon ? np + 2 : np - 1;
  const unsigned ring0 = smem_u32(&sm.s[0][0]);

  const Unit un = t < TUNIT ? unit_of(g, i0, j0, t / NCH, t % NCH, (t / NCH) * VW + 4 + 4 * (t % NCH), 0, false,
                                      t / NCH >= 3 && t / NCH < 3 + VY)
                            : unit_none();
  const bool has_x = t < VY * 6;
  const XCell xc = xcell_of(g, i0, j0, has_x ? t / 6 : 0, t % 6, (3 + (has_x ? t / 6 : 0)) * VW);

  auto issue = [&](int lp, int st) {
    if (lp <= last_centre) {
      const ZPlane z = z_plane(g, k0 + lp);
      const unsigned sbase = ring0 + (unsigned)(st * TS) * 4u;
      const bool full = lp < np;
      if ((un.flags & 1) && (full || (un.flags & 4))) issue_unit(un, A.phi, z, g, sbase);
      if (full && has_x) cp4(sbase + (unsigned)xc.dst * 4u, A.phi + z.off + xc.xy);
    }
    cp_async_commit();
  };

  const int own = (ty + 3) * VW + 4 + 2 * tx;
  const float rsc = 1.f / A.sc;
  float2 q[ZQ];
#pragma unroll
  for (int m = 0; m < ZQ; ++m) q[m] = make_float2(0.f, 0.f);
#pragma unroll
  for (int lp = 0; lp < PD + 3; ++lp) issue(lp, lp);
  if constexpr (zon) {
    bool fxa, fxb, fyy;
    const int iia = ghost(ia, g.nx, g.bc[0], &fxa), iib = ghost(ia + 1, g.nx, g.bc[0], &fxb);
    const int jj = ghost(j, g.ny, g.bc[1], &fyy);
#pragma unroll
    for (int m = 0; m < 3; ++m) {
      const float* f = A.phi + z_plane(g, k0 - 3 + m).off + (long long)g.nx * jj;
      q[m] = make_float2(__ldg(f + iia), __ldg(f + iib));
    }
  }
  // the per-point inputs of a plane: u, v, w, then nu_t, src, f2, f3
  float2 in[7];
  auto load_in = [&](long long p) {
#pragma unroll
    for (int a = 0; a < 3; ++a) in[a] = ld_stream2(A.u[a] + p);
    in[3] = LES ? ld_stream2(A.nu_t + p) : make_float2(0.f, 0.f);
    in[4] = ld_stream2(A.src + p);
    in[5] = A.f2 ? ld_stream2(A.f2 + p) : make_float2(0.f, 0.f);
    in[6] = A.f3 ? ld_stream2(A.f3 + p) : make_float2(0.f, 0.f);
  };
  if (valid && np > 0) load_in(out0 + sz * k0);
  cp_async_wait<PD>();
  __syncthreads();
  if constexpr (zon) {
#pragma unroll
    for (int m = 0; m < 3; ++m) q[3 + m] = lds2(&sm.s[m][own]);
  }
  float s_hi[3] = {0.f, 0.f, 0.f}, s_lo[3] = {0.f, 0.f, 0.f};
  // ring slots of planes lp, lp + 3 and lp + 3 + PD, advanced each plane
  int s0 = 0, s3 = 3, s6 = (3 + PD) % ZQ;
#pragma unroll 1
  for (int lp = 0; lp < np; ++lp) {
    cp_async_wait<PD - 1>();
    __syncthreads();
    issue(lp + 3 + PD, s6);
    const float* s = sm.s[s0];
    if constexpr (zon) q[6] = lds2(&sm.s[s3][own]);
    float w[10];
#pragma unroll
    for (int m = 0; m < 5; ++m) {
      const float2 p2 = lds2(&s[own - 4 + 2 * m]);
      w[2 * m] = p2.x;
      w[2 * m + 1] = p2.y;
    }
    float d1a[3], d1b[3], d2a[3], d2b[3];
    d1a[0] = d1x<XO>(w + 1, A.cf.ax[0], pca);
    d2a[0] = d2x<XO>(w + 1, A.cf.ax[0], pca);
    d1b[0] = d1x<XO>(w + 2, A.cf.ax[0], pcb);
    d2b[0] = d2x<XO>(w + 2, A.cf.ax[0], pcb);
    float va[7], vb[7];
#pragma unroll
    for (int m = 0; m < 7; ++m) {
      const float2 p2 = lds2(&s[own + (m - 3) * VW]);
      va[m] = p2.x;
      vb[m] = p2.y;
    }
    d1a[1] = d1(va, A.cf.ax[1]);
    d2a[1] = d2(va, A.cf.ax[1]);
    d1b[1] = d1(vb, A.cf.ax[1]);
    d2b[1] = d2(vb, A.cf.ax[1]);
    d1a[2] = d2a[2] = d1b[2] = d2b[2] = 0.f;
    if constexpr (zon) {
#pragma unroll
      for (int m = 0; m < 7; ++m) {
        va[m] = q[m].x;
        vb[m] = q[m].y;
      }
      d1a[2] = d1(va, A.cf.ax[2]);
      d2a[2] = d2(va, A.cf.ax[2]);
      d1b[2] = d1(vb, A.cf.ax[2]);
      d2b[2] = d2(vb, A.cf.ax[2]);
#pragma unroll
      for (int m = 0; m < ZQ - 1; ++m) q[m] = q[m + 1];
    }
    if (valid) {
      const long long p = out0 + sz * (k0 + lp);
      const float pc[2] = {w[4], w[5]};
      const int cls[2] = {pca, pcb};
      float Fo[2], co[2];
#pragma unroll
      for (int e = 0; e < 2; ++e) {
        const float* d1v = e ? d1b : d1a;
        const float* d2v = e ? d2b : d2a;
        const float uu = e ? in[0].y : in[0].x, vv = e ? in[1].y : in[1].x, ww = e ? in[2].y : in[2].x;
        float alpha = A.alpha0;
        if (LES) alpha = alpha + (e ? in[3].y : in[3].x) * rsc;  // nu_t / sc as a product (one division per thread)
        const float F = alpha * (d2v[0] + d2v[1] + d2v[2]) - (uu * d1v[0] + vv * d1v[1] + ww * d1v[2]) +
                        (e ? in[4].y : in[4].x);
        float ph = pc[e] + A.adu * F;
        if (A.f2) ph = ph + A.bdu * (e ? in[5].y : in[5].x);
        if (A.f3) ph = ph + A.cdu * (e ? in[6].y : in[6].x);
        if (XO && cls[e] == 1) ph = pc[e];  // open x axis: the inflow value is held
        const float cl = fmaxf(0.f, fminf(1.f, ph));
        const float wt = (XO && cls[e] == 1) ? 0.f : fminf(cl, 1.f - cl);  // held inflow nodes take no excess
        two_sum_acc(s_hi[0], s_lo[0], ph);
        two_sum_acc(s_hi[1], s_lo[1], cl);
        two_sum_acc(s_hi[2], s_lo[2], wt);
        Fo[e] = F;
        co[e] = cl;
      }
      __stcs(reinterpret_cast<float2*>(A.fnew + p), make_float2(Fo[0], Fo[1]));
      __stcs(reinterpret_cast<float2*>(A.phi_out + p), make_float2(co[0], co[1]));
      if (lp + 1 < np) load_in(p + sz);
    }
    s0 = s0 == ZQ - 1 ? 0 : s0 + 1;
    s3 = s3 == ZQ - 1 ? 0 : s3 + 1;
    s6 = s6 == ZQ - 1 ? 0 : s6 + 1;
  }
  cp_async_wait<0>();
  double r[3];
#pragma unroll
  for (int c = 0; c < 3; ++c) r[c] = to_t<double>(s_hi[c]) + to_t<double>(s_lo[c]);
  const int ops[3] = {RED_SUM, RED_SUM, RED_SUM};
  block_reduce_store<3>(r, ops, A.part, block_linear_id());
}

// ---------------------------------------------------------------------------
// correction with an FP32 pressure: the high plane of the mixed multigrid
// method's double-float pair (the FP32 rounding of the FP64 pressure, the
// value the FP64-pressure kernel above converts to).  Its planes land in a
// ring of 7 single-field stages of 14 rows x 72 columns, as the scalar's in
// k_transeq25v, with no conversion pass.
// ---------------------------------------------------------------------------
// u* lands beside the pressure ring: plane L in slot L % UQ, copied with
// the pressure's plane L + 3 (three planes ahead of its use, in flight
// without registers; one plane ahead through registers left the kernel
// waiting on those loads).  Four slots and 64 registers fit four blocks
// per SM (0.102 -> 0.099 ms at 256^3).
constexpr int UQ = 4;
struct TURing {
  float s[ZQ][TS];
  float u[UQ][3][VY * VX];
};
template <bool ZON, bool XO>
__global__ void __launch_bounds__(NT, 4) k_correct25vf(CorrArgs<float, float> A, int kc) {
  pdl_enter();
  extern __shared__ __align__(16) unsigned char smem_raw[];
  TURing& sm = *reinterpret_cast<TURing*>(smem_raw);
  const Grid& g = A.g;
  const int tx = threadIdx.x, ty = threadIdx.y, t = ty * VTX + tx;
  const int i0 = blockIdx.x * VX, j0 = blockIdx.y * VY;
  const int ia = i0 + 2 * tx, j = j0 + ty;
  const bool valid = ia < g.nx && j < g.ny;
  const int k0 = blockIdx.z * kc;
  const int np = min(kc, g.nz - k0);
  constexpr bool zon = ZON;
  const int pca = XO ? xclass(g, ia) : 0, pcb = XO ? xclass(g, ia + 1) : 0;
  const long long sz = g.sz();
  const long long out0 = valid ? (long long)ia + (long long)g.nx * j : 0;
  const int last_centre = zon ? np + 2 : np - 1;
  const unsigned ring0 = smem_u32(&sm.s[0][0]);

  const Unit un = t < TUNIT ? unit_of(g, i0, j0, t / NCH, t % NCH, (t / NCH) * VW + 4 + 4 * (t % NCH), 0, false,
                                      t / NCH >= 3 && t / NCH < 3 + VY)
                            : unit_none();
  const bool has_x = t < VY * 6;
  const XCell xc = xcell_of(g, i0, j0, has_x ? t / 6 : 0, t % 6, (3 + (has_x ? t / 6 : 0)) * VW);

  const int ucol = ty * VX + 2 * tx;  // the pair in a u* plane of the ring
  auto issue = [&](int lp, int st) {
    if (lp <= last_centre) {
      const ZPlane z = z_plane(g, k0 + lp);
      const unsigned sbase = ring0 + (unsigned)(st * TS) * 4u;
      const bool full = lp < np;
      if ((un.flags & 1) && (full || (un.flags & 4))) issue_unit(un, A.p, z, g, sbase);
      if (full && has_x) cp4(sbase + (unsigned)xc.dst * 4u, A.p + z.off + xc.xy);
    }
    const int L = lp - 3;
    if (valid && L >= 0 && L < np) {
      const long long src = out0 + sz * (k0 + L);
#pragma unroll
      for (int a = 0; a < 3; ++a) cp_async<8>(&sm.u[L & (UQ - 1)][a][ucol], A.up[a] + src);
    }
    cp_async_commit();
  };

  const int own = (ty + 3) * VW + 4 + 2 * tx;
  float2 q[ZQ];
#pragma unroll
  for (int m = 0; m < ZQ; ++m) q[m] = make_float2(0.f, 0.f);
#pragma unroll
  for (int lp = 0; lp < PD + 3; ++lp) issue(lp, lp);
  if constexpr (zon) {
    bool fxa, fxb, fyy;
    const int iia = ghost(ia, g.nx, g.bc[0], &fxa), iib = ghost(ia + 1, g.nx, g.bc[0], &fxb);
    const int jj = ghost(j, g.ny, g.bc[1], &fyy);
#pragma unroll
    for (int m = 0; m < 3; ++m) {
      const float* f = A.p + z_plane(g, k0 - 3 + m).off + (long long)g.nx * jj;
      q[m] = make_float2(__ldg(f + iia), __ldg(f + iib));
    }
  }
  cp_async_wait<PD>();
  __syncthreads();
  if constexpr (zon) {
#pragma unroll
    for (int m = 0; m < 3; ++m) q[3 + m] = lds2(&sm.s[m][own]);
  }
  float mn[3], mx[3], am[3];
#pragma unroll
  for (int a = 0; a < 3; ++a) { mn[a] = INFINITY; mx[a] = -INFINITY; am[a] = 0.f; }
  bool nan = false;
  // the plane loop unrolled by the ring's length: every ring stage and
  // z-queue slot index is a constant (plane lp - 3 + m in slot (u + m) % ZQ;
  // 108 -> 102 us at 256^3.  The larger predictor, divergence and scalar
  // bodies ran slower unrolled and keep the rotating queue.)
#pragma unroll 1
  for (int lb = 0; lb < np; lb += ZQ) {
#pragma unroll
    for (int u = 0; u < ZQ; ++u) {
      const int lp = lb + u;
      if (lp >= np) break;
      cp_async_wait<PD - 1>();
      __syncthreads();
      issue(lp + 3 + PD, (u + 3 + PD) % ZQ);
      const float* s = sm.s[u];
      if constexpr (zon) q[(u + 6) % ZQ] = lds2(&sm.s[(u + 3) % ZQ][own]);
      float w[10];
#pragma unroll
      for (int m = 0; m < 5; ++m) {
        const float2 p2 = lds2(&s[own - 4 + 2 * m]);
        w[2 * m] = p2.x;
        w[2 * m + 1] = p2.y;
      }
      float ga[3], gb[3];
      ga[0] = d1x<XO>(w + 1, A.cf.ax[0], pca);
      gb[0] = d1x<XO>(w + 2, A.cf.ax[0], pcb);
      float va[7], vb[7];
#pragma unroll
      for (int m = 0; m < 7; ++m) {
        const float2 p2 = lds2(&s[own + (m - 3) * VW]);
        va[m] = p2.x;
        vb[m] = p2.y;
      }
      ga[1] = d1(va, A.cf.ax[1]);
      gb[1] = d1(vb, A.cf.ax[1]);
      ga[2] = gb[2] = 0.f;
      if constexpr (zon) {
#pragma unroll
        for (int m = 0; m < 7; ++m) {
          va[m] = q[(u + m) % ZQ].x;
          vb[m] = q[(u + m) % ZQ].y;
        }
        ga[2] = d1(va, A.cf.ax[2]);
        gb[2] = d1(vb, A.cf.ax[2]);
      }
      if (valid) {
        const long long p = out0 + sz * (k0 + lp);
        float2 us[3];
#pragma unroll
        for (int a = 0; a < 3; ++a) us[a] = lds2(&sm.u[lp & (UQ - 1)][a][ucol]);
#pragma unroll
        for (int a = 0; a < 3; ++a) {
          float na = us[a].x - A.dt * ga[a], nb = us[a].y - A.dt * gb[a];
          if (XO) {  // inflow nodes keep their value
            if (pca == 1) na = us[a].x;
            if (pcb == 1) nb = us[a].y;
          }
          __stcs(reinterpret_cast<float2*>(A.u[a] + p), make_float2(na, nb));
          if (na != na || nb != nb) nan = true;
          mn[a] = fminf(mn[a], fminf(na, nb));
          mx[a] = fmaxf(mx[a], fmaxf(na, nb));
          am[a] = fmaxf(am[a], fmaxf(fabsf(na), fabsf(nb)));
        }
      }
    }
  }
  cp_async_wait<0>();
  float r[10];
  const int ops[10] = {RED_MIN, RED_MIN, RED_MIN, RED_MAX, RED_MAX, RED_MAX, RED_MAX, RED_MAX, RED_MAX, RED_MAX};
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    r[a] = mn[a];
    r[3 + a] = mx[a];
    r[6 + a] = am[a];
  }
  r[9] = nan ? 1.f : 0.f;
  block_reduce_store_t<float, 10>(r, ops, A.part, block_linear_id());
}

dim3 v_grid(const Grid& g, int kc) {
  return dim3((g.nx + VX - 1) / VX, (g.ny + VY - 1) / VY, (g.nz + kc - 1) / kc);
}

template <bool LES, bool ZON, bool XO>
void predict_v_launch(const PredArgs<float>& a, cudaStream_t s) {
  constexpr size_t bytes = sizeof(PRing);
  static std::atomic<bool> attr[64];
  allow_smem_v(k_predict25v<LES, ZON, XO>, bytes, attr);
  const int kc = v_chunk(a.g, 2);
  launch_pdl(k_predict25v<LES, ZON, XO>, v_grid(a.g, kc), dim3(VTX, VTY), bytes, s, a, kc);
}

template <class O, bool ZON, bool XO>
void div_v_launch(const float* fx, const float* fy, const float* fz, O* out, const Grid& g, const Coef3<float>& cf,
                  int odd, float dt, int divide, StatPart* part, double* wpart, int wmask, cudaStream_t s) {
  constexpr size_t bytes = sizeof(DRing);
  static std::atomic<bool> attr[64];
  allow_smem_v(k_div25v<O, ZON, XO>, bytes, attr);
  const int kc = v_chunk(g, 3);
  launch_pdl(k_div25v<O, ZON, XO>, v_grid(g, kc), dim3(VTX, VTY), bytes, s, fx, fy, fz, out, g, cf, odd, dt,
             divide, part, kc, wpart, wmask);
}

template <bool ZON, bool XO>
void correct_v_launch(const CorrArgs<float, double>& a, cudaStream_t s) {
  constexpr size_t bytes = sizeof(CRing);
  static std::atomic<bool> attr[64];
  allow_smem_v(k_correct25v<ZON, XO>, bytes, attr);
  const int kc = v_chunk(a.g, 3);
  launch_pdl(k_correct25v<ZON, XO>, v_grid(a.g, kc), dim3(VTX, VTY), bytes, s, a, kc);
}

template <bool ZON, bool XO>
void correct_vf_launch(const CorrArgs<float, float>& a, cudaStream_t s) {
  constexpr size_t bytes = sizeof(TURing);
  static std::atomic<bool> attr[64];
  allow_smem_v(k_correct25vf<ZON, XO>, bytes, attr);
  const int kc = v_chunk(a.g, 3);  // the tiling of the FP64-pressure kernel (one record table)
  launch_pdl(k_correct25vf<ZON, XO>, v_grid(a.g, kc), dim3(VTX, VTY), bytes, s, a, kc);
}

template <bool LES, bool ZON, bool XO>
void transeq_v_launch(const ScalArgs<float>& a, cudaStream_t s) {
  constexpr size_t bytes = sizeof(TRing);
  static std::atomic<bool> attr[64];
  allow_smem_v(k_transeq25v<LES, ZON, XO>, bytes, attr);
  const int kc = v_chunk(a.g, 3);
  launch_pdl(k_transeq25v<LES, ZON, XO>, v_grid(a.g, kc), dim3(VTX, VTY), bytes, s, a, kc);
}

}  // namespace

// Planes per block of the two-point kernels: the z chunk count that fills
// whole waves of `per_sm` resident blocks on the 152 SMs best, counting the
// six z-halo planes each chunk re-reads; chunks of at least 14 planes.
int v_chunk(const Grid& g, int per_sm) {
  const long long tiles = (long long)((g.nx + VX - 1) / VX) * ((g.ny + VY - 1) / VY);
  const long long slots = 152LL * per_sm;
  int best = g.nz;
  double best_eff = -1.0;
  for (int nch = 1; nch <= g.nz; ++nch) {
    const int kc = (g.nz + nch - 1) / nch;
    if (kc < 14 && nch > 1) break;
    const long long nb = tiles * ((g.nz + kc - 1) / kc);
    const long long waves = (nb + slots - 1) / slots;
    const double fill = (double)nb / (double)(waves * slots);
    const double eff = fill * (double)kc / (double)(kc + 6);
    if (eff > best_eff + 1e-9) {
      best_eff = eff;
      best = kc;
    }
  }
  return best;
}

bool stencil_v_ok(const Grid& g) { return g.nx % 4 == 0 && g.nx >= 8 && g.ny >= 8 && g.nz >= 8; }

void launch_predict_v(const PredArgs<float>& a, cudaStream_t s) {
  const bool zon = a.g.bc[2] != AX_ZERO, xo = a.g.bc[0] == AX_OPEN;
#define PV(L, Z, X) predict_v_launch<L, Z, X>(a, s)
  if (a.les) {
    if (zon) { if (xo) PV(true, true, true); else PV(true, true, false); }
    else { if (xo) PV(true, false, true); else PV(true, false, false); }
  } else {
    if (zon) { if (xo) PV(false, true, true); else PV(false, true, false); }
    else { if (xo) PV(false, false, true); else PV(false, false, false); }
  }
#undef PV
}

template <class O>
void launch_div_v(const float* fx, const float* fy, const float* fz, O* out, const Grid& g, const Coef3<float>& cf,
                  int odd, float dt, int divide, StatPart* part, cudaStream_t s, double* wpart, int wmask) {
  const bool zon = g.bc[2] != AX_ZERO, xo = g.bc[0] == AX_OPEN;
#define DV(Z, X) div_v_launch<O, Z, X>(fx, fy, fz, out, g, cf, odd, dt, divide, part, wpart, wmask, s)
  if (zon) { if (xo) DV(true, true); else DV(true, false); }
  else { if (xo) DV(false, true); else DV(false, false); }
#undef DV
}
template void launch_div_v<double>(const float*, const float*, const float*, double*, const Grid&,
                                   const Coef3<float>&, int, float, int, StatPart*, cudaStream_t, double*, int);
template void launch_div_v<float>(const float*, const float*, const float*, float*, const Grid&, const Coef3<float>&,
                                  int, float, int, StatPart*, cudaStream_t, double*, int);

void launch_correct_v(const CorrArgs<float, double>& a, cudaStream_t s) {
  const bool zon = a.g.bc[2] != AX_ZERO, xo = a.g.bc[0] == AX_OPEN;
  if (zon) { if (xo) correct_v_launch<true, true>(a, s); else correct_v_launch<true, false>(a, s); }
  else { if (xo) correct_v_launch<false, true>(a, s); else correct_v_launch<false, false>(a, s); }
}

void launch_correct_v(const CorrArgs<float, float>& a, cudaStream_t s) {
  const bool zon = a.g.bc[2] != AX_ZERO, xo = a.g.bc[0] == AX_OPEN;
  if (zon) { if (xo) correct_vf_launch<true, true>(a, s); else correct_vf_launch<true, false>(a, s); }
  else { if (xo) correct_vf_launch<false, true>(a, s); else correct_vf_launch<false, false>(a, s); }
}

// the divergence and the correction run with the same tiling (3 blocks/SM)
long long div_v_blocks(const Grid& g) {
  const int kc = v_chunk(g, 3);
  return (long long)((g.nx + VX - 1) / VX) * ((g.ny + VY - 1) / VY) * ((g.nz + kc - 1) / kc);
}
long long corr_v_blocks(const Grid& g) { return div_v_blocks(g); }

void launch_transeq_v(const ScalArgs<float>& a, cudaStream_t s) {
  const bool zon = a.g.bc[2] != AX_ZERO, xo = a.g.bc[0] == AX_OPEN;
#define TV(L, Z, X) transeq_v_launch<L, Z, X>(a, s)
  if (a.les) {
    if (zon) { if (xo) TV(true, true, true); else TV(true, true, false); }
    else { if (xo) TV(true, false, true); else TV(true, false, false); }
  } else {
    if (zon) { if (xo) TV(false, true, true); else TV(false, true, false); }
    else { if (xo) TV(false, false, true); else TV(false, false, false); }
  }
#undef TV
}
// the transport kernel runs with the divergence's tiling
long long transeq_v_blocks(const Grid& g) { return div_v_blocks(g); }

}  // namespace o3d
