// k_mgfused.cu -- fused level kernels of the FP32 multigrid V-cycle (the
// mixed method's inner solver for the pressure equation, src/poisson.f90:
// 95-98 operator, red-black relaxation).
//
// On a level whose three axes all coarsen, the unfused cycle streams the
// level's arrays through HBM once per smoothing pass: pre-smoothing (first
// sweep from zero, then red and black passes), the residual, the
// full-weighting restriction, the prolongation-add and the post-smoothing
// passes each read and write the level.  Here two kernels do the level's
// work, each in one march along z:
//
//   k_mg_down  pre-smoothing (S = 2 pre colour stages), residual and
//              restriction: reads r (and e when the cycle starts from a
//              correction), writes the smoothed e and the coarse right-hand
//              side;
//   k_mg_up    prolongation-add and post-smoothing (2 post colour stages),
//              and on the finest level p += e (FP64) with max |e|: reads
//              the smoothed e, the coarse correction and r, writes e.
//
// Temporal blocking: a block owns a 32 x 16 column of points and a chunk of
// planes.  Each plane step loads one new plane (cp.async into a ring of
// shared-memory planes, several planes ahead) and advances every stage by
// one plane: stage s works on plane tau - (s - 1), one plane behind the
// stage before it, so that the z-neighbours it reads are final.  In x and y
// every stage also recomputes the halo cells the next stages read (a halo
// of S + 2 cells around the owned column), and the ghost cells beyond a
// domain end hold the mirrored or wrapped values, which the stage updates
// reproduce bit for bit.  A colour stage updates only one colour and reads
// only the other colour and the point itself, so the stages share one
// in-place ring.  Each row of a plane is stored split by x parity, so a
// warp updating one colour of a row reads consecutive words.
//
// Every update uses the expressions of the unfused kernels (k_smooth,
// k_smooth_first, k_resid, k_restrict_full, k_prolong_cell, k_update in
// k_poisson.cu) in the same order, so both paths give the same bits.
#include "o3d_internal.cuh"
#include "o3d_kernels.h"

namespace o3d {

// owned tile 32 x 16, 256 threads (two owned cells each), cp.async D planes ahead
constexpr int MF_FX = 32, MF_FY = 16, MF_OWN = MF_FX * MF_FY, MF_NT = 256, MF_D = 3;

// Extended tile of XW x YW cells.  Each row is split by x parity: the even
// x cells, then the odd ones, XH slots each (XH even, so that two
// consecutive slots form an aligned float2).
template <int XW_, int YW_>
struct Ext {
  static constexpr int XW = XW_, YW = YW_;
  static constexpr int XH = ((XW + 1) / 2 + 1) & ~1;
  static constexpr int NPR = XH / 2;      // slot pairs per half-row
  static constexpr int PL = YW * 2 * XH;  // floats per plane
  static constexpr int NLD = (XW * YW + MF_NT - 1) / MF_NT;
  static __device__ __forceinline__ int at(int lx, int ly) { return (2 * ly + (lx & 1)) * XH + (lx >> 1); }
};

__device__ __forceinline__ float2 ld2(const float* p) { return *reinterpret_cast<const float2*>(p); }
__device__ __forceinline__ void st2(float* p, float2 v) { *reinterpret_cast<float2*>(p) = v; }

// ring slot k planes before the slot s of a ring of N planes
template <int N>
__device__ __forceinline__ int rsub(int s, int k) {
  const int r = s - k;
  return r < 0 ? r + N : r;
}
template <int N>
__device__ __forceinline__ int radd(int s, int k) {
  const int r = s + k;
  return r >= N ? r - N : r;
}

// One work item of a colour stage on the cells [a, XW-1-a] x [a, YW-1-a] of
// a plane: two cells of the stage's colour, slots m0 = 2j and m0 + 1 of the
// colour's half of row ly = a + row (x = 2 m0 + px and x + 2; the colour's
// cells in row ly have x parity (colbase + ly) & 1).  The threads of a block
// take the items in order (Items).
// KIND 0: relaxed Gauss-Seidel update of E (k_smooth); 1: first red value
// from e = 0; 2: first black value from e = 0 (both k_smooth_first, whose
// operator acts on r); 3: the update of KIND 0 whose old value is the first
// red value, recomputed from r (the red cells right after k_smooth_first).
template <class X, int KIND>
__device__ __forceinline__ void rb_item(float* __restrict__ Ec, const float* __restrict__ Em,
                                        const float* __restrict__ Ep, const float* __restrict__ Rc,
                                        const float* __restrict__ Rm, const float* __restrict__ Rp, int a,
                                        int colbase, const PoiCoef<float>& c, float om, int row, int j) {
  constexpr int XH = X::XH;
  if (row >= X::YW - 2 * a) return;
  const int ly = a + row, px = (colbase + ly) & 1;
  const int lx0 = 4 * j + px;
  const bool v0 = lx0 >= a && lx0 <= X::XW - 1 - a;
  const bool v1 = lx0 + 2 >= a && lx0 + 2 <= X::XW - 1 - a;
  if (!v0 && !v1) return;
  const int q = (2 * ly + px) * XH + 2 * j;
  const float2 rq = ld2(Rc + q);
  float2 res;
  if (KIND == 1) {
    res.x = om * (rq.x * c.invA);
    res.y = om * (rq.y * c.invA);
  } else {
    const float* F = KIND == 2 ? Rc : Ec;  // the field the operator acts on
    const float* Fm = KIND == 2 ? Rm : Em;
    const float* Fp = KIND == 2 ? Rp : Ep;
    const int qo = q + (px ? -XH : XH);  // the other parity's half of the row
    const float2 oc = ld2(F + qo);
    const float ox = F[qo + (px ? 2 : -1)];
    const float w0 = px ? oc.x : ox, e0 = px ? oc.y : oc.x;  // x - 1, x + 1 of the first cell
    const float w1 = px ? oc.y : oc.x, e1 = px ? ox : oc.y;  // and of the second
    const float2 sn = ld2(F + q - 2 * XH), nn = ld2(F + q + 2 * XH);
    const float2 bz = ld2(Fm + q), tz = ld2(Fp + q);
    const float s0 = c.ox * (w0 + e0) + c.oy * (sn.x + nn.x) + c.oz * (bz.x + tz.x);
    const float s1 = c.ox * (w1 + e1) + c.oy * (sn.y + nn.y) + c.oz * (bz.y + tz.y);
    if (KIND == 2) {
      res.x = om * ((rq.x - om * (s0 * c.invA)) * c.invA);
      res.y = om * ((rq.y - om * (s1 * c.invA)) * c.invA);
    } else {
      float2 ec;
      if (KIND == 3) {
        ec.x = om * (rq.x * c.invA);
        ec.y = om * (rq.y * c.invA);
      } else {
        ec = ld2(Ec + q);
      }
      const float en0 = (rq.x - s0) * c.invA, en1 = (rq.y - s1) * c.invA;
      res.x = ec.x + om * (en0 - ec.x);
      res.y = ec.y + om * (en1 - ec.y);
    }
  }
  if (v0 && v1) st2(Ec + q, res);
  else if (v0) Ec[q] = res.x;
  else Ec[q + 1] = res.y;
}

// the work items of a thread in a stage whose threads take items id0,
// id0 + stride, ...: row id / NPR, slot pair id % NPR
template <class X, int NI>
struct Items {
  int row[NI], j[NI];
  __device__ __forceinline__ void init(int id0, int stride) {
#pragma unroll
    for (int u = 0; u < NI; ++u) {
      const int id = id0 + u * stride;
      row[u] = id / X::NPR;
      j[u] = id - row[u] * X::NPR;
    }
  }
};
template <class X, int KIND, int NI>
__device__ __forceinline__ void rb_stage(float* Ec, const float* Em, const float* Ep, const float* Rc,
                                         const float* Rm, const float* Rp, int a, int colbase,
                                         const PoiCoef<float>& c, float om, const Items<X, NI>& it) {
#pragma unroll
  for (int u = 0; u < NI; ++u) rb_item<X, KIND>(Ec, Em, Ep, Rc, Rm, Rp, a, colbase, c, om, it.row[u], it.j[u]);
}

// per-thread copy cells of an extended tile with origin (xo, yo)
template <class X>
struct CopyCells {
  int goff[X::NLD], soff[X::NLD];
  __device__ __forceinline__ void init(const Grid& g, int xo, int yo) {
#pragma unroll
    for (int u = 0; u < X::NLD; ++u) {
      const int id = threadIdx.x + u * MF_NT;
      soff[u] = -1;
      goff[u] = 0;
      if (id < X::XW * X::YW) {
        const int lx = id % X::XW, ly = id / X::XW;
        bool f;
        goff[u] = ghost(xo + lx, g.nx, g.bc[0], &f) + g.nx * ghost(yo + ly, g.ny, g.bc[1], &f);
        soff[u] = X::at(lx, ly);
      }
    }
  }
  __device__ __forceinline__ void copy(float* dst, const float* __restrict__ src, long long zo) const {
#pragma unroll
    for (int u = 0; u < X::NLD; ++u)
      if (soff[u] >= 0) cp_async<4>(dst + soff[u], src + zo + goff[u]);
  }
};

__device__ __forceinline__ long long mf_zoff(const Grid& g, int P) {
  bool f;
  return g.sz() * (long long)ghost(P, g.nz, g.bc[2], &f);
}

// ---------------------------------------------------------------------------
// k_mg_down: pre-smoothing (S colour stages), residual, restriction.
// Cells of the extended tile: x in [x0 - S - 2, x0 + 32 + S] (local 0..XW-1);
// stage s covers local [s, XW-1-s], the residual [S+1, XW-S-2] (fine
// x0-1 .. x0+32-1, what the restriction of the owned coarse points reads).
// Planes: the residual runs on [k0-1, k1], stage s on [k0-2-(S-s), k1+1+(S-s)];
// at step tau stage s is at plane tau-s+1 and the residual at tau-S.  From
// e = 0 (ZERO) the first two stages are one pass at plane tau-1 on the cells
// of stage 2, both colours (k_smooth_first's two values).
// ---------------------------------------------------------------------------
// planes in flight: from e = 0, MF_D; from a correction (whose e ring also
// stages the correction's planes) one, so that three blocks fit an SM
template <bool ZERO>
constexpr int down_d() {
  return ZERO ? MF_D : 1;
}

template <int S, bool ZERO>
__global__ void __launch_bounds__(MF_NT, S == 2 ? 4 : 3)
    k_mg_down(const float* __restrict__ r, const float* __restrict__ ein, float* __restrict__ eout,
              float* __restrict__ rc, Grid gf, Grid gc, PoiCoef<float> c, float om, int kc, const SolveCtrl* ctrl) {
  pdl_enter();
  if (ctrl->done) return;
  using X = Ext<MF_FX + 2 * S + 3, MF_FY + 2 * S + 3>;
  constexpr int PL = X::PL, XH = X::XH, D = down_d<ZERO>();
  constexpr int NE = ZERO ? S + 2 : S + 3 + D, NR = S + 1 + D;
  constexpr int TW = MF_FX + 1, TPL = TW * (MF_FY + 1);
  extern __shared__ float4 mf_smem[];
  float* const E = (float*)mf_smem;
  float* const R = E + NE * PL;
  float* const TT = R + NR * PL;
  const int t = threadIdx.x;
  const int x0 = blockIdx.x * MF_FX, y0 = blockIdx.y * MF_FY;
  const int k0 = blockIdx.z * kc, k1 = min(k0 + kc, gf.nz);
  CopyCells<X> cc;
  cc.init(gf, x0 - S - 2, y0 - S - 2);
  // work items of the whole block (itF) or of each half of it (itH)
  constexpr int NIF = ((X::YW - 2) * X::NPR + MF_NT - 1) / MF_NT;
  constexpr int NIH = ((X::YW - 4) * X::NPR + MF_NT / 2 - 1) / (MF_NT / 2);
  Items<X, NIF> itF;
  itF.init(t, MF_NT);
  Items<X, NIH> itH;
  itH.init(t & (MF_NT / 2 - 1), MF_NT / 2);
  const int tau0 = k0 - 1 - S, tau1 = k1 + S;
  // ring slots of plane tau (E, R) and of residual plane tau - S (T)
  int sE = (tau0 - (k0 - S - 8)) % NE, sR = (tau0 - (k0 - S - 8)) % NR, sT = (tau0 - S - (k0 - S - 8)) % 3;
  if (!ZERO) {
    cc.copy(E + rsub<NE>(sE, 1) * PL, ein, mf_zoff(gf, tau0 - 1));
    cc.copy(E + sE * PL, ein, mf_zoff(gf, tau0));
  }
#pragma unroll
  for (int g = 0; g < D; ++g) {  // the inputs of stage 1 at planes tau0 .. tau0 + D - 1
    cc.copy(R + radd<NR>(sR, g) * PL, r, mf_zoff(gf, tau0 + g));
    if (!ZERO) cc.copy(E + radd<NE>(sE, g + 1) * PL, ein, mf_zoff(gf, tau0 + g + 1));
    cp_async_commit();
  }
  for (int tau = tau0; tau <= tau1; ++tau) {
    cp_async_wait<D - 1>();
    __syncthreads();
    if (tau + D <= tau1) {
      cc.copy(R + radd<NR>(sR, D) * PL, r, mf_zoff(gf, tau + D));
      if (!ZERO) cc.copy(E + radd<NE>(sE, D + 1) * PL, ein, mf_zoff(gf, tau + D + 1));
    }
    cp_async_commit();
    if (ZERO) {
      // stages 1 and 2 from e = 0 at plane tau - 1; with S >= 4 the red
      // values are only read by stage 3, which recomputes them (KIND 3)
      const int P = tau - 1;
      if (P >= k0 - S) {
        float* Ec = E + rsub<NE>(sE, 1) * PL;
        const float* Rc = R + rsub<NR>(sR, 1) * PL;
        if (S == 2 && t < MF_NT / 2)
          rb_stage<X, 1>(Ec, nullptr, nullptr, Rc, nullptr, nullptr, 2, P & 1, c, om, itH);
        else if (S == 2)
          rb_stage<X, 2>(Ec, nullptr, nullptr, Rc, R + rsub<NR>(sR, 2) * PL, R + sR * PL, 2, (1 + P) & 1, c, om, itH);
        else
          rb_stage<X, 2>(Ec, nullptr, nullptr, Rc, R + rsub<NR>(sR, 2) * PL, R + sR * PL, 2, (1 + P) & 1, c, om, itF);
      }
    } else {
      rb_stage<X, 0>(E + sE * PL, E + rsub<NE>(sE, 1) * PL, E + radd<NE>(sE, 1) * PL, R + sR * PL, nullptr, nullptr,
                     1, tau & 1, c, om, itF);
    }
    __syncthreads();
#pragma unroll
    for (int s = ZERO ? 3 : 2; s <= S; ++s) {
      const int P = tau - s + 1;
      float* Ec = E + rsub<NE>(sE, s - 1) * PL;
      const float* Em = E + rsub<NE>(sE, s) * PL;
      const float* Ep = E + rsub<NE>(sE, s - 2) * PL;
      const float* Rc = R + rsub<NR>(sR, s - 1) * PL;
      if (P >= k0 - 2 - S + s) {
        if (ZERO && s == 3) rb_stage<X, 3>(Ec, Em, Ep, Rc, nullptr, nullptr, s, ((s - 1) + P) & 1, c, om, itF);
        else rb_stage<X, 0>(Ec, Em, Ep, Rc, nullptr, nullptr, s, ((s - 1) + P) & 1, c, om, itF);
      }
      __syncthreads();
    }
    const int Pt = tau - S;
    if (Pt >= k0 - 1) {  // residual t = r - A e on plane Pt (k_resid), cells 2m and 2m + 1 per item
      const float* Ec = E + rsub<NE>(sE, S) * PL;
      const float* Em = E + rsub<NE>(sE, S + 1) * PL;
      const float* Ep = E + rsub<NE>(sE, S - 1) * PL;
      const float* Rc = R + rsub<NR>(sR, S) * PL;
      float* Tc = TT + sT * TPL;
      constexpr int a = S + 1, mlo = a >> 1, mhi = (X::XW - 1 - a) >> 1, NM = mhi - mlo + 1;
      constexpr int rows = X::YW - 2 * a;
      for (int id = t; id < rows * NM; id += MF_NT) {
        const int row = id / NM, m = mlo + id - row * NM;
        const int ly = a + row;
        const int qe = 2 * ly * XH + m, qo = qe + XH;  // cells 2m (even half) and 2m + 1 (odd half)
        const float ev = Ec[qe], od = Ec[qo];
        const float t0 = Rc[qe] - (c.ox * (Ec[qo - 1] + od) + c.oy * (Ec[qe - 2 * XH] + Ec[qe + 2 * XH]) +
                                   c.oz * (Em[qe] + Ep[qe]) + c.A * ev);
        const float t1 = Rc[qo] - (c.ox * (ev + Ec[qe + 1]) + c.oy * (Ec[qo - 2 * XH] + Ec[qo + 2 * XH]) +
                                   c.oz * (Em[qo] + Ep[qo]) + c.A * od);
        const int lx = 2 * m;
        if (lx >= a) Tc[row * TW + lx - a] = t0;
        if (lx + 1 <= X::XW - 1 - a) Tc[row * TW + lx + 1 - a] = t1;
      }
    }
    {  // the owned cells of plane tau - S + 1 are final
      const int Pe = tau - S + 1;
      if (Pe >= k0 && Pe < k1) {
        const float* Ef = E + rsub<NE>(sE, S - 1) * PL;
#pragma unroll
        for (int o = t; o < MF_OWN; o += MF_NT) {
          const int x = x0 + o % MF_FX, y = y0 + o / MF_FX;
          if (x < gf.nx && y < gf.ny)
            eout[x + (long long)gf.nx * (y + (long long)gf.ny * Pe)] = Ef[X::at(S + 2 + o % MF_FX, S + 2 + o / MF_FX)];
        }
      }
    }
    __syncthreads();
    // full weighting of coarse plane K from residual planes 2K-1 .. 2K+1 (k_restrict_full)
    if ((Pt & 1) && Pt >= k0 + 1 && t < (MF_FX / 2) * (MF_FY / 2)) {
      const int K = (Pt - 1) >> 1;
      const int ci = t % (MF_FX / 2), cj = t / (MF_FX / 2);
      const int I = x0 / 2 + ci, J = y0 / 2 + cj;
      if (K < gc.nz && I < gc.nx && J < gc.ny) {
        const float w[3] = {0.25f, 0.5f, 0.25f};
        const float* Tp[3] = {TT + rsub<3>(sT, 2) * TPL, TT + rsub<3>(sT, 1) * TPL, TT + sT * TPL};
        float acc = 0.f;
#pragma unroll
        for (int oz = 0; oz < 3; ++oz)
#pragma unroll
          for (int oy = 0; oy < 3; ++oy) {
            const float* row = Tp[oz] + (2 * cj + oy) * TW + 2 * ci;
#pragma unroll
            for (int ox = 0; ox < 3; ++ox) acc += w[oz] * w[oy] * w[ox] * row[ox];
          }
        rc[I + (long long)gc.nx * (J + (long long)gc.ny * K)] = acc;
      }
    }
    sE = radd<NE>(sE, 1);
    sR = radd<NR>(sR, 1);
    sT = radd<3>(sT, 1);
  }
  cp_async_wait<0>();
}

// ---------------------------------------------------------------------------
// k_mg_up: prolongation-add (stage 0) and S2 post-smoothing colour stages;
// with UPD also p += e in FP64 and max |e| (k_update).  Cells: x in
// [x0 - S2, x0 + 32 + S2) (local 0..XW-1), stage s on [s, XW-1-s]; planes:
// stage s on [k0-(S2-s), k1-1+(S2-s)], at step tau on plane tau - s.  The
// coarse corrections under the tile (CX x CY cells from coarse x0/2 - S2/2,
// ghost-mapped) and, with UPD, p of the owned cells are staged in shared
// memory with the fine planes.
// ---------------------------------------------------------------------------
template <int S2>
struct UpGeom {
  using X = Ext<MF_FX + 2 * S2, MF_FY + 2 * S2>;
  static constexpr int CX = MF_FX / 2 + S2 + 1, CY = MF_FY / 2 + S2 + 1, CPL = CX * CY;
  // planes in flight: 2 for the 2-stage kernel (its rings then fit 4 blocks per SM)
  static constexpr int D = S2 == 2 ? 2 : MF_D;
  static constexpr int NE = S2 + 2 + D, NR = S2 + 1 + D, NC = 5, NP = D + 1;
  static constexpr size_t floats = (size_t)(NE + NR) * X::PL + NC * CPL + 2;  // + 2: pad before the p ring
  static constexpr size_t bytes = ((floats * 4 + 15) / 16) * 16 + (size_t)NP * MF_OWN * 8;
};

template <int S2, bool UPD>
__global__ void __launch_bounds__(MF_NT, S2 == 2 ? 4 : 3)
    k_mg_up(const float* __restrict__ epre, const float* __restrict__ ecrs, const float* __restrict__ r,
            float* __restrict__ eout, PPair p, Grid gf, Grid gc, PoiCoef<float> c, float om, int kc,
            SolveCtrl* ctrl) {
  pdl_enter();
  if (ctrl->done) return;
  using G = UpGeom<S2>;
  using X = typename G::X;
  constexpr int PL = X::PL, D = G::D, NE = G::NE, NR = G::NR, NC = G::NC, NP = G::NP;
  constexpr int CX = G::CX, CPL = G::CPL;
  extern __shared__ float4 mf_smem[];
  float* const E = (float*)mf_smem;
  float* const R = E + NE * PL;
  float* const CR = R + NR * PL;
  // the pressure ring: NP planes of the owned cells' high parts, then NP of their low parts
  float* const PR = (float*)((char*)mf_smem + ((G::floats * 4 + 15) / 16) * 16);
  const int t = threadIdx.x;
  const int x0 = blockIdx.x * MF_FX, y0 = blockIdx.y * MF_FY;
  const int k0 = blockIdx.z * kc, k1 = min(k0 + kc, gf.nz);
  const int xo = x0 - S2, yo = y0 - S2;
  CopyCells<X> cc;
  cc.init(gf, xo, yo);
  constexpr int NIF = ((X::YW - 2) * X::NPR + MF_NT - 1) / MF_NT;
  Items<X, NIF> itF;
  itF.init(t, MF_NT);
  // the thread's coarse copy cells and, per fine copy cell, its coarse corner
  // (local, in the staged coarse tile) and fine parities
  constexpr int NCC = (CPL + MF_NT - 1) / MF_NT, NOWN = MF_OWN / MF_NT;
  int cgoff[NCC];
#pragma unroll
  for (int u = 0; u < NCC; ++u) {
    const int id = t + u * MF_NT;
    bool f;
    cgoff[u] = id < CPL ? ghost(xo / 2 + id % CX, gc.nx, gc.bc[0], &f) + gc.nx * ghost(yo / 2 + id / CX, gc.ny,
                                                                                          gc.bc[1], &f)
                        : -1;
  }
  // stage 0 items: the coarse cells (ci, cj) under the extended tile, each
  // giving its 2 x 2 fine cells of a plane
  constexpr int PCX = X::XW / 2, PCY = X::YW / 2, NPI = (PCX * PCY + MF_NT - 1) / MF_NT;
  static_assert(X::XW % 2 == 0 && X::YW % 2 == 0, "the extended tile covers whole coarse cells");
  int pco[NPI], pfo[NPI];
#pragma unroll
  for (int u = 0; u < NPI; ++u) {
    const int id = t + u * MF_NT, ci = id % PCX, cj = id / PCX;
    pco[u] = id < PCX * PCY ? cj * CX + ci : -1;
    pfo[u] = 2 * (2 * cj) * X::XH + ci;  // even-x slot of fine cell (2 ci, 2 cj)
  }
  auto copy_coarse = [&](int K) {
    bool f;
    const long long zo = gc.sz() * (long long)ghost(K, gc.nz, gc.bc[2], &f);
#pragma unroll
    for (int u = 0; u < NCC; ++u)
      if (cgoff[u] >= 0) cp_async<4>(CR + ((K - (k0 >> 1) + 8) % NC) * CPL + t + u * MF_NT, ecrs + zo + cgoff[u]);
  };
  // the owned cells o = t + u * MF_NT: in the grid (own), and their xy offset
  bool own[NOWN];
  long long oq[NOWN];
#pragma unroll
  for (int u = 0; u < NOWN; ++u) {
    const int o = t + u * MF_NT, x = x0 + o % MF_FX, y = y0 + o / MF_FX;
    own[u] = x < gf.nx && y < gf.ny;
    oq[u] = x + (long long)gf.nx * y;
  }
  auto copy_p = [&](int P) {
    if (UPD && P >= k0 && P < k1) {
#pragma unroll
      for (int u = 0; u < NOWN; ++u)
        if (own[u]) {
          const int slot = ((P - k0 + 8) % NP) * MF_OWN + t + u * MF_NT;
          cp_async<4>(PR + slot, p.hi + oq[u] + gf.sz() * P);
          cp_async<4>(PR + NP * MF_OWN + slot, p.lo + oq[u] + gf.sz() * P);
        }
    }
  };
  const int tau0 = k0 - S2, tau1 = k1 - 1 + S2;
  int sE = (tau0 - (k0 - S2 - 8)) % NE, sR = (tau0 - (k0 - S2 - 8)) % NR;
  for (int K = tau0 >> 1; K <= ((tau0 + D - 1) >> 1) + 1; ++K) copy_coarse(K);
#pragma unroll
  for (int g = 0; g < D; ++g) {
    const long long zo = mf_zoff(gf, tau0 + g);
    cc.copy(E + radd<NE>(sE, g) * PL, epre, zo);
    cc.copy(R + radd<NR>(sR, g) * PL, r, zo);
    copy_p(tau0 + g - S2);
    cp_async_commit();
  }
  float emax = 0.f;
  const float h = 0.5f;
  for (int tau = tau0; tau <= tau1; ++tau) {
    cp_async_wait<D - 1>();
    __syncthreads();
    if (tau + D <= tau1) {
      const long long zo = mf_zoff(gf, tau + D);
      cc.copy(E + radd<NE>(sE, D) * PL, epre, zo);
      cc.copy(R + radd<NR>(sR, D) * PL, r, zo);
      if (((tau + D) & 1) == 0) copy_coarse(((tau + D) >> 1) + 1);
    }
    copy_p(tau + D - S2);
    cp_async_commit();
    {  // stage 0: e += P ec on plane tau (k_prolong_cell's expressions)
      const int K = tau >> 1, dc = tau & 1;
      const float* C0 = CR + ((K - (k0 >> 1) + 8) % NC) * CPL;
      const float* C1 = CR + ((K + 1 - (k0 >> 1) + 8) % NC) * CPL;
      float* Ec = E + sE * PL;
      constexpr int XH = X::XH;
#pragma unroll
      for (int u = 0; u < NPI; ++u) {
        if (pco[u] < 0) continue;
        const int o = pco[u], f = pfo[u];
        const float c000 = C0[o], c100 = C0[o + 1], c010 = C0[o + CX], c110 = C0[o + CX + 1];
        const float x00 = h * (c000 + c100), x10 = h * (c010 + c110);
        float v00, v10, v01, v11;  // fine (2ci + a, 2cj + b) as v<a><b>
        if (!dc) {
          v00 = c000;
          v10 = x00;
          v01 = h * (c000 + c010);
          v11 = h * (x00 + x10);
        } else {
          const float c001 = C1[o], c101 = C1[o + 1], c011 = C1[o + CX], c111 = C1[o + CX + 1];
          const float x01 = h * (c001 + c101), x11 = h * (c011 + c111);
          v00 = h * (c000 + c001);
          v10 = h * (x00 + x01);
          v01 = h * (h * (c000 + c010) + h * (c001 + c011));
          v11 = h * (h * (x00 + x10) + h * (x01 + x11));
        }
        Ec[f] += v00;
        Ec[f + XH] += v10;
        Ec[f + 2 * XH] += v01;
        Ec[f + 3 * XH] += v11;
      }
    }
    __syncthreads();
#pragma unroll
    for (int s = 1; s <= S2; ++s) {
      const int P = tau - s;
      if (P >= k0 - S2 + s)
        rb_stage<X, 0>(E + rsub<NE>(sE, s) * PL, E + rsub<NE>(sE, s + 1) * PL, E + rsub<NE>(sE, s - 1) * PL,
                       R + rsub<NR>(sR, s) * PL, nullptr, nullptr, s, ((s - 1) + P) & 1, c, om, itF);
      __syncthreads();
    }
    const int Po = tau - S2;
    if (Po >= k0) {
      const float* Ef = E + rsub<NE>(sE, S2) * PL;
      const float* Pf = PR + ((Po - k0 + 8) % NP) * MF_OWN;
#pragma unroll
      for (int u = 0; u < NOWN; ++u) {
        const int o = t + u * MF_NT;
        if (!own[u]) continue;
        const float ev = Ef[X::at(S2 + o % MF_FX, S2 + o / MF_FX)];
        const long long q = oq[u] + gf.sz() * Po;
        eout[q] = ev;
        if (UPD) {  // p += e on the double-float pair, in the order of k_update
          float ph = Pf[o], pl = Pf[NP * MF_OWN + o];
          df_add_f(ph, pl, ev);
          p.hi[q] = ph;
          p.lo[q] = pl;
          emax = fmaxf(emax, fabsf(ev));
        }
      }
    }
    sE = radd<NE>(sE, 1);
    sR = radd<NR>(sR, 1);
  }
  cp_async_wait<0>();
  if (UPD) {
    const float bm = block_max_f(emax);
    if (t == 0 && bm > 0.f) atomicMax(&ctrl->dmax_key, (unsigned long long)__double_as_longlong((double)bm));
  }
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
template <int S, bool ZERO>
static size_t down_smem() {
  using X = Ext<MF_FX + 2 * S + 3, MF_FY + 2 * S + 3>;
  const int D = down_d<ZERO>();
  const int NE = ZERO ? S + 2 : S + 3 + D, NR = S + 1 + D;
  return ((size_t)(NE + NR) * X::PL + 3 * (MF_FX + 1) * (MF_FY + 1)) * sizeof(float);
}
template <int S2>
static size_t up_smem() {
  return UpGeom<S2>::bytes;
}

// planes per block: split z into as many chunks as keep the whole grid
// resident at `per_sm` blocks per SM (152 SMs), at least 32 planes each
static int mf_chunk(const Grid& g, int per_sm = 3) {
  const long long tiles = (long long)((g.nx + MF_FX - 1) / MF_FX) * ((g.ny + MF_FY - 1) / MF_FY);
  long long nch = (per_sm * 152) / (tiles > 0 ? tiles : 1);
  if (nch < 1) nch = 1;
  const long long most = (g.nz + 31) / 32;
  if (nch > most) nch = most;
  int kc = (int)((g.nz + nch - 1) / nch);
  return kc + (kc & 1);
}

template <class K>
static int set_smem(K kern, size_t bytes) {
  return cudaFuncSetAttribute((const void*)kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes) ==
                 cudaSuccess
             ? 0
             : -1;
}

// raises the dynamic shared-memory limit of the fused kernels (call before
// any launch or stream capture)
int mg_fused_setup() {
  int st = 0;
  st |= set_smem(k_mg_down<2, true>, down_smem<2, true>());
  st |= set_smem(k_mg_down<2, false>, down_smem<2, false>());
  st |= set_smem(k_mg_down<4, true>, down_smem<4, true>());
  st |= set_smem(k_mg_down<4, false>, down_smem<4, false>());
  st |= set_smem(k_mg_up<2, true>, up_smem<2>());
  st |= set_smem(k_mg_up<2, false>, up_smem<2>());
  st |= set_smem(k_mg_up<4, true>, up_smem<4>());
  st |= set_smem(k_mg_up<4, false>, up_smem<4>());
  return st;
}

bool mg_fusable(const MGLevel& L, int pre, int post, bool any_size) {
  if (!(L.coarsen[0] == 1 && L.coarsen[1] == 1 && L.coarsen[2] == 1)) return false;
  if (pre < 1 || pre > 2 || post < 1 || post > 2) return false;
  // the ghost cells of the extended tile stay within one wrap or reflection
  if (L.g.nx < 16 || L.g.ny < 16 || L.g.nz < 16) return false;
  // a level too small to give every SM a block runs faster as one-pass
  // kernels (their blocks are short; a fused block is a long chain of
  // dependent plane steps); any_size fuses it all the same
  if (any_size) return true;
  const long long blocks = (long long)((L.g.nx + MF_FX - 1) / MF_FX) * ((L.g.ny + MF_FY - 1) / MF_FY) *
                           ((L.g.nz + mf_chunk(L.g) - 1) / mf_chunk(L.g));
  return blocks >= 152;
}

void launch_mg_down(const MGLevel& L, const MGLevel& C, float om, int pre, bool zero, const SolveCtrl* ctrl,
                    cudaStream_t s) {
  const PoiCoef<float> c = make_poi<float>(L.h[0], L.h[1], L.h[2]);
  const int kc = mf_chunk(L.g, pre == 1 ? 4 : 3);  // the 2-stage kernel fits 4 blocks per SM
  const dim3 grid((L.g.nx + MF_FX - 1) / MF_FX, (L.g.ny + MF_FY - 1) / MF_FY, (L.g.nz + kc - 1) / kc);
  const float* r = (const float*)L.r;
  const float* ein = (const float*)L.e;
  float* eout = (float*)L.t;
  float* rc = (float*)C.r;
#define MF_DOWN(S, Z) \
  launch_pdl(k_mg_down<S, Z>, grid, MF_NT, down_smem<S, Z>(), s, r, ein, eout, rc, L.g, C.g, c, om, kc, ctrl)
  if (pre == 1) {
    if (zero) MF_DOWN(2, true);
    else MF_DOWN(2, false);
  } else {
    if (zero) MF_DOWN(4, true);
    else MF_DOWN(4, false);
  }
#undef MF_DOWN
}

void launch_mg_up(const MGLevel& L, const MGLevel& C, float om, int post, double* p, SolveCtrl* ctrl,
                  cudaStream_t s) {
  const PoiCoef<float> c = make_poi<float>(L.h[0], L.h[1], L.h[2]);
  const int kc = mf_chunk(L.g, post == 1 ? 4 : 3);
  const dim3 grid((L.g.nx + MF_FX - 1) / MF_FX, (L.g.ny + MF_FY - 1) / MF_FY, (L.g.nz + kc - 1) / kc);
  const float* epre = (const float*)L.t;
  const float* ec = (const float*)C.e;
  const float* r = (const float*)L.r;
  float* eout = (float*)L.e;
  const PPair pp = p ? ppair(p, L.g.n) : PPair{nullptr, nullptr};
#define MF_UP(S2, U) \
  launch_pdl(k_mg_up<S2, U>, grid, MF_NT, up_smem<S2>(), s, epre, ec, r, eout, pp, L.g, C.g, c, om, kc, ctrl)
  if (post == 1) {
    if (p) MF_UP(2, true);
    else MF_UP(2, false);
  } else {
    if (p) MF_UP(4, true);
    else MF_UP(4, false);
  }
#undef MF_UP
}

}  // namespace o3d
