// k_stencil.cu -- stencil kernels of the step: single derivatives, the fused
// momentum predictor (9 first + 9 second derivatives, Smagorinsky nu_t,
// convection, diffusion and the Adams-Bashforth update in one pass), the
// divergence/right-hand side, the velocity correction, the scalar transport
// and the flow statistics.  Templated on the arithmetic type T (double for
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
  df[q] = order == 1 ? d1(v, c) : d2(v, c);
}

// ---------------------------------------------------------------------------
// fused predictor, predict_velocity + calculate_nu_t
// (src/integration.f90:106-188, src/les_turbulence.f90:54-88)
// ---------------------------------------------------------------------------
template <class T>
__global__ void __launch_bounds__(256) k_predict(PredArgs<T> A) {
  const Grid& g = A.g;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  const int k = blockIdx.z;
  if (i >= g.nx || j >= g.ny) return;
  const long long q = (long long)i + g.sy() * j + g.sz() * k;

  T uc[3], g1[3][3], g2[3][3];
#pragma unroll
  for (int c = 0; c < 3; ++c) {
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      if (g.bc[a] == AX_ZERO) {
        g1[c][a] = (T)0;
        g2[c][a] = (T)0;
        continue;
      }
      T v[7];
      // component c is odd along its own axis: derxi/derxxi for ux, deryi for uy, derzi for uz
      load_line<3>(A.u[c], g, a, i, j, k, a == c, v);
      g1[c][a] = d1(v, A.cf.ax[a]);
      g2[c][a] = d2(v, A.cf.ax[a]);
      if (a == 0) uc[c] = v[3];
    }
  }
  T nut = (T)0;
  if (A.les) {
    const T s11 = g1[0][0], s22 = g1[1][1], s33 = g1[2][2];
    const T s12 = (T)0.5 * (g1[0][1] + g1[1][0]);
    const T s13 = (T)0.5 * (g1[0][2] + g1[2][0]);
    const T s23 = (T)0.5 * (g1[1][2] + g1[2][1]);
    const T smag = sqrt((T)2 * (s11 * s11 + s22 * s22 + s33 * s33 +
                                (T)2 * (s12 * s12 + s13 * s13 + s23 * s23)));
    nut = A.csd2 * smag;
    A.nu_t[q] = nut;
  }
  const T nu_eff = A.onere + nut;
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    const T F = nu_eff * (g2[c][0] + g2[c][1] + g2[c][2]) -
                (uc[0] * g1[c][0] + uc[1] * g1[c][1] + uc[2] * g1[c][2]);
    T up = uc[c] + A.adu * F;
    if (A.f2[c]) up = up + A.bdu * A.f2[c][q];
    if (A.f3[c]) up = up + A.cdu * A.f3[c][q];
    A.fnew[c][q] = F;
    A.up[c][q] = up;
  }
}

// ---------------------------------------------------------------------------
// 2.5D fused predictor.  A block owns a TX x TY column of (x, y) points and
// marches along z over a chunk of planes.  Each thread keeps the seven
// z-neighbours of its point for the three components in a register queue;
// the current plane's x- and y-lines (with 3-point halos, ghost-mapped at the
// domain ends) are staged in double-buffered shared memory, so every value
// is read from global memory once per plane plus the halos.
// ---------------------------------------------------------------------------
template <class T, class S>
__device__ __forceinline__ T ldg_map(const S* __restrict__ f, const Grid& g, int i, int j, int k,
                                     int odd_axis) {
  bool fx, fy, fz;
  const int ii = ghost(i, g.nx, g.bc[0], &fx);
  const int jj = ghost(j, g.ny, g.bc[1], &fy);
  const int kk = ghost(k, g.nz, g.bc[2] == AX_ZERO ? AX_PERIODIC : g.bc[2], &fz);
  const T v = (T)__ldg(f + ii + g.sy() * jj + g.sz() * kk);
  const bool neg = (fx && odd_axis == 0) || (fy && odd_axis == 1) || (fz && odd_axis == 2);
  return neg ? -v : v;
}

template <class T, int TX, int TY>
__global__ void __launch_bounds__(TX * TY, sizeof(T) == 4 ? 3 : 1) k_predict25(PredArgs<T> A, int kc) {
  const Grid& g = A.g;
  __shared__ T sx[2][3][TY][TX + 6];
  __shared__ T sy[2][3][TY + 6][TX];
  const int tx = threadIdx.x, ty = threadIdx.y;
  const int i0 = blockIdx.x * TX, j0 = blockIdx.y * TY;
  const int i = i0 + tx, j = j0 + ty;
  // points past the grid end still stage ghost-mapped values: the lines of
  // the last valid points read them
  const bool valid = i < g.nx && j < g.ny;
  const int k0 = blockIdx.z * kc;
  const int k1 = min(k0 + kc, g.nz);
  const bool zon = g.bc[2] != AX_ZERO;
  const bool hx = tx < 3, hy = ty < 3;
  const int hxi0 = i0 - 3 + tx, hxi1 = i0 + TX + tx;  // x-halo columns of this thread
  const int hyj0 = j0 - 3 + ty, hyj1 = j0 + TY + ty;  // y-halo rows of this thread

  // register queue: q[c][m] = u_c(i, j, k - 3 + m)
  T q[3][7];
#pragma unroll
  for (int c = 0; c < 3; ++c)
#pragma unroll
    for (int m = 0; m < 6; ++m) q[c][m + 1] = zon || m == 2 ? ldg_map<T>(A.u[c], g, i, j, k0 - 3 + m, c) : (T)0;
  // halos of the first plane
  T hxv[3][2], hyv[3][2];
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    hxv[c][0] = hx ? ldg_map<T>(A.u[c], g, hxi0, j, k0, c) : (T)0;
    hxv[c][1] = hx ? ldg_map<T>(A.u[c], g, hxi1, j, k0, c) : (T)0;
    hyv[c][0] = hy ? ldg_map<T>(A.u[c], g, i, hyj0, k0, c) : (T)0;
    hyv[c][1] = hy ? ldg_map<T>(A.u[c], g, i, hyj1, k0, c) : (T)0;
  }

  int buf = 0;
  for (int k = k0; k < k1; ++k) {
#pragma unroll
    for (int c = 0; c < 3; ++c) {
#pragma unroll
      for (int m = 0; m < 6; ++m) q[c][m] = q[c][m + 1];
      if (!zon) q[c][3] = ldg_map<T>(A.u[c], g, i, j, k, c);
      // stage plane k
      sx[buf][c][ty][tx + 3] = q[c][3];
      sy[buf][c][ty + 3][tx] = q[c][3];
      if (hx) {
        sx[buf][c][ty][tx] = hxv[c][0];
        sx[buf][c][ty][TX + 3 + tx] = hxv[c][1];
      }
      if (hy) {
        sy[buf][c][ty][tx] = hyv[c][0];
        sy[buf][c][TY + 3 + ty][tx] = hyv[c][1];
      }
    }
    // issue the loads of the next plane (queue head and halos) before computing
    const int kn = k + 1;
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      q[c][6] = zon ? ldg_map<T>(A.u[c], g, i, j, k + 3, c) : (T)0;
      if (kn < k1) {
        if (hx) {
          hxv[c][0] = ldg_map<T>(A.u[c], g, hxi0, j, kn, c);
          hxv[c][1] = ldg_map<T>(A.u[c], g, hxi1, j, kn, c);
        }
        if (hy) {
          hyv[c][0] = ldg_map<T>(A.u[c], g, i, hyj0, kn, c);
          hyv[c][1] = ldg_map<T>(A.u[c], g, i, hyj1, kn, c);
        }
      }
    }
    const long long p = (long long)min(i, g.nx - 1) + g.sy() * min(j, g.ny - 1) + g.sz() * k;
    T h2[3], h3[3];
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      h2[c] = A.f2[c] ? __ldg(A.f2[c] + p) : (T)0;
      h3[c] = A.f3[c] ? __ldg(A.f3[c] + p) : (T)0;
    }
    __syncthreads();
    T g1[3][3], g2[3][3];
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      T v[7];
#pragma unroll
      for (int m = 0; m < 7; ++m) v[m] = sx[buf][c][ty][tx + m];
      g1[c][0] = d1(v, A.cf.ax[0]);
      g2[c][0] = d2(v, A.cf.ax[0]);
#pragma unroll
      for (int m = 0; m < 7; ++m) v[m] = sy[buf][c][ty + m][tx];
      g1[c][1] = d1(v, A.cf.ax[1]);
      g2[c][1] = d2(v, A.cf.ax[1]);
      if (zon) {  // q[c][0..6] holds planes k-3 .. k+3
        g1[c][2] = d1(q[c], A.cf.ax[2]);
        g2[c][2] = d2(q[c], A.cf.ax[2]);
      } else {
        g1[c][2] = (T)0;
        g2[c][2] = (T)0;
      }
    }
    if (valid) {
      T nut = (T)0;
      if (A.les) {
        const T s11 = g1[0][0], s22 = g1[1][1], s33 = g1[2][2];
        const T s12 = (T)0.5 * (g1[0][1] + g1[1][0]);
        const T s13 = (T)0.5 * (g1[0][2] + g1[2][0]);
        const T s23 = (T)0.5 * (g1[1][2] + g1[2][1]);
        const T smag = sqrt((T)2 * (s11 * s11 + s22 * s22 + s33 * s33 +
                                    (T)2 * (s12 * s12 + s13 * s13 + s23 * s23)));
        nut = A.csd2 * smag;
        A.nu_t[p] = nut;
      }
      const T nu_eff = A.onere + nut;
      const T uc0 = q[0][3], uc1 = q[1][3], uc2 = q[2][3];
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        const T F = nu_eff * (g2[c][0] + g2[c][1] + g2[c][2]) -
                    (uc0 * g1[c][0] + uc1 * g1[c][1] + uc2 * g1[c][2]);
        T up = q[c][3] + A.adu * F;
        if (A.f2[c]) up = up + A.bdu * h2[c];
        if (A.f3[c]) up = up + A.cdu * h3[c];
        A.fnew[c][p] = F;
        A.up[c][p] = up;
      }
    }
    buf ^= 1;
  }
}

// ---------------------------------------------------------------------------
// 2.5D divergence (src/differential_operators.f90:25-35) -> optional output
// div*scale, with function_stats (src/functions.f90:27-63) accumulated per
// thread over its z-column and reduced once per block.
// ---------------------------------------------------------------------------
template <class T, class O, int TX, int TY>
__global__ void __launch_bounds__(TX * TY) k_div25(const T* __restrict__ fx, const T* __restrict__ fy,
                                                   const T* __restrict__ fz, O* __restrict__ out, Grid g,
                                                   Coef3<T> cf, int odd, T dt, int divide, StatPart* part,
                                                   int kc) {
  __shared__ T sx[2][TY][TX + 6];
  __shared__ T sy[2][TY + 6][TX];
  const int tx = threadIdx.x, ty = threadIdx.y;
  const int i0 = blockIdx.x * TX, j0 = blockIdx.y * TY;
  const int i = i0 + tx, j = j0 + ty;
  const bool valid = i < g.nx && j < g.ny;
  const int k0 = blockIdx.z * kc;
  const int k1 = min(k0 + kc, g.nz);
  const bool zon = g.bc[2] != AX_ZERO;
  const int ox = odd ? 0 : -1, oy = odd ? 1 : -1, oz = odd ? 2 : -1;
  const bool hx = tx < 3, hy = ty < 3;
  T q[7];
#pragma unroll
  for (int m = 0; m < 6; ++m) q[m + 1] = zon ? ldg_map<T>(fz, g, i, j, k0 - 3 + m, oz) : (T)0;
  // values of the next plane to stage: x-line centre and halos, y-line centre and halos
  T cx = ldg_map<T>(fx, g, i, j, k0, ox), cy = ldg_map<T>(fy, g, i, j, k0, oy);
  T hx0 = hx ? ldg_map<T>(fx, g, i0 - 3 + tx, j, k0, ox) : (T)0;
  T hx1 = hx ? ldg_map<T>(fx, g, i0 + TX + tx, j, k0, ox) : (T)0;
  T hy0 = hy ? ldg_map<T>(fy, g, i, j0 - 3 + ty, k0, oy) : (T)0;
  T hy1 = hy ? ldg_map<T>(fy, g, i, j0 + TY + ty, k0, oy) : (T)0;
  T mn = (T)INFINITY, mx = (T)-INFINITY;
  long long imx = 0x7fffffffffffffffll;
  double sum = 0.0;
  int buf = 0;
  for (int k = k0; k < k1; ++k) {
#pragma unroll
    for (int m = 0; m < 6; ++m) q[m] = q[m + 1];
    sx[buf][ty][tx + 3] = cx;
    sy[buf][ty + 3][tx] = cy;
    if (hx) { sx[buf][ty][tx] = hx0; sx[buf][ty][TX + 3 + tx] = hx1; }
    if (hy) { sy[buf][ty][tx] = hy0; sy[buf][TY + 3 + ty][tx] = hy1; }
    q[6] = zon ? ldg_map<T>(fz, g, i, j, k + 3, oz) : (T)0;
    const int kn = k + 1;
    if (kn < k1) {
      cx = ldg_map<T>(fx, g, i, j, kn, ox);
      cy = ldg_map<T>(fy, g, i, j, kn, oy);
      if (hx) { hx0 = ldg_map<T>(fx, g, i0 - 3 + tx, j, kn, ox); hx1 = ldg_map<T>(fx, g, i0 + TX + tx, j, kn, ox); }
      if (hy) { hy0 = ldg_map<T>(fy, g, i, j0 - 3 + ty, kn, oy); hy1 = ldg_map<T>(fy, g, i, j0 + TY + ty, kn, oy); }
    }
    __syncthreads();
    T v[7];
#pragma unroll
    for (int m = 0; m < 7; ++m) v[m] = sx[buf][ty][tx + m];
    const T ddx = d1(v, cf.ax[0]);
#pragma unroll
    for (int m = 0; m < 7; ++m) v[m] = sy[buf][ty + m][tx];
    const T ddy = d1(v, cf.ax[1]);
    const T ddz = zon ? d1(q, cf.ax[2]) : (T)0;
    const T div = ddx + ddy + ddz;
    if (valid) {
      const long long p = (long long)i + g.sy() * j + g.sz() * k;
      if (out) out[p] = (O)(divide ? div / dt : div);
      sum += (double)div;
      if (div < mn) mn = div;
      if (div > mx) { mx = div; imx = p; }  // k ascends: the first max of the column is kept
    }
    buf ^= 1;
  }
  if (part) {
    StatPart st;
    st.mn = (double)mn; st.mx = (double)mx; st.sum = sum; st.imx = imx;
    if (!(mx >= mn)) { st.mn = INFINITY; st.mx = -INFINITY; st.imx = 0x7fffffffffffffffll; }
    block_stat(st, part, block_linear_id());
  }
}

// ---------------------------------------------------------------------------
// 2.5D correct_velocity (src/integration.f90:297-325) with the per-step
// extrema of the corrected velocity accumulated per thread.
// ---------------------------------------------------------------------------
template <class T, class P, int TX, int TY>
__global__ void __launch_bounds__(TX * TY) k_correct25(CorrArgs<T, P> A, int kc) {
  const Grid& g = A.g;
  __shared__ T sx[2][TY][TX + 6];
  __shared__ T sy[2][TY + 6][TX];
  const int tx = threadIdx.x, ty = threadIdx.y;
  const int i0 = blockIdx.x * TX, j0 = blockIdx.y * TY;
  const int i = i0 + tx, j = j0 + ty;
  const bool valid = i < g.nx && j < g.ny;
  const int k0 = blockIdx.z * kc;
  const int k1 = min(k0 + kc, g.nz);
  const bool zon = g.bc[2] != AX_ZERO;
  const bool hx = tx < 3, hy = ty < 3;
  T q[7];
#pragma unroll
  for (int m = 0; m < 6; ++m) q[m + 1] = ldg_map<T>(A.p, g, i, j, k0 - 3 + m, -1);
  T hx0 = hx ? ldg_map<T>(A.p, g, i0 - 3 + tx, j, k0, -1) : (T)0;
  T hx1 = hx ? ldg_map<T>(A.p, g, i0 + TX + tx, j, k0, -1) : (T)0;
  T hy0 = hy ? ldg_map<T>(A.p, g, i, j0 - 3 + ty, k0, -1) : (T)0;
  T hy1 = hy ? ldg_map<T>(A.p, g, i, j0 + TY + ty, k0, -1) : (T)0;
  T mn[3], mx[3], am[3];
#pragma unroll
  for (int a = 0; a < 3; ++a) { mn[a] = (T)INFINITY; mx[a] = (T)-INFINITY; am[a] = (T)0; }
  bool nan = false;
  int buf = 0;
  for (int k = k0; k < k1; ++k) {
#pragma unroll
    for (int m = 0; m < 6; ++m) q[m] = q[m + 1];
    if (!zon) q[3] = ldg_map<T>(A.p, g, i, j, k, -1);
    sx[buf][ty][tx + 3] = q[3];
    sy[buf][ty + 3][tx] = q[3];
    if (hx) { sx[buf][ty][tx] = hx0; sx[buf][ty][TX + 3 + tx] = hx1; }
    if (hy) { sy[buf][ty][tx] = hy0; sy[buf][TY + 3 + ty][tx] = hy1; }
    q[6] = ldg_map<T>(A.p, g, i, j, k + 3, -1);
    const int kn = k + 1;
    if (kn < k1) {
      if (hx) { hx0 = ldg_map<T>(A.p, g, i0 - 3 + tx, j, kn, -1); hx1 = ldg_map<T>(A.p, g, i0 + TX + tx, j, kn, -1); }
      if (hy) { hy0 = ldg_map<T>(A.p, g, i, j0 - 3 + ty, kn, -1); hy1 = ldg_map<T>(A.p, g, i, j0 + TY + ty, kn, -1); }
    }
    const long long p = (long long)min(i, g.nx - 1) + g.sy() * min(j, g.ny - 1) + g.sz() * k;
    T upv[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) upv[a] = __ldg(A.up[a] + p);
    __syncthreads();
    T v[7], gp[3];
#pragma unroll
    for (int m = 0; m < 7; ++m) v[m] = sx[buf][ty][tx + m];
    gp[0] = d1(v, A.cf.ax[0]);
#pragma unroll
    for (int m = 0; m < 7; ++m) v[m] = sy[buf][ty + m][tx];
    gp[1] = d1(v, A.cf.ax[1]);
    gp[2] = zon ? d1(q, A.cf.ax[2]) : (T)0;
    if (valid) {
#pragma unroll
      for (int a = 0; a < 3; ++a) {
        const T un = upv[a] - A.dt * gp[a];
        A.u[a][p] = un;
        if (un != un) nan = true;
        mn[a] = fmin(mn[a], un);
        mx[a] = fmax(mx[a], un);
        am[a] = fmax(am[a], fabs(un));
      }
    }
    buf ^= 1;
  }
  double r[10];
  const int ops[10] = {RED_MIN, RED_MIN, RED_MIN, RED_MAX, RED_MAX, RED_MAX,
                       RED_MAX, RED_MAX, RED_MAX, RED_MAX};
#pragma unroll
  for (int a = 0; a < 3; ++a) { r[a] = (double)mn[a]; r[3 + a] = (double)mx[a]; r[6 + a] = (double)am[a]; }
  r[9] = nan ? 1.0 : 0.0;
  block_reduce_store<10>(r, ops, A.part, block_linear_id());
}

// standalone calculate_nu_t (src/les_turbulence.f90:54-88)
template <class T>
__global__ void k_nu_t(const T* __restrict__ ux, const T* __restrict__ uy, const T* __restrict__ uz,
                       T* __restrict__ nu_t, Grid g, Coef3<T> cf, T csd2) {
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
      g1[c][a] = d1(v, cf.ax[a]);
    }
  const T s11 = g1[0][0], s22 = g1[1][1], s33 = g1[2][2];
  const T s12 = (T)0.5 * (g1[0][1] + g1[1][0]);
  const T s13 = (T)0.5 * (g1[0][2] + g1[2][0]);
  const T s23 = (T)0.5 * (g1[1][2] + g1[2][1]);
  nu_t[q] = csd2 * sqrt((T)2 * (s11 * s11 + s22 * s22 + s33 * s33 +
                                (T)2 * (s12 * s12 + s13 * s13 + s23 * s23)));
}

// ---------------------------------------------------------------------------
// divergence (src/differential_operators.f90:25-35); out = div * scale
// (scale = 1/dt gives the Poisson rhs of correct_pression,
// src/integration.f90:235-239), with function_stats of div.
// ---------------------------------------------------------------------------
template <class T, class O>
__global__ void __launch_bounds__(256) k_div(const T* __restrict__ fx, const T* __restrict__ fy,
                                             const T* __restrict__ fz, O* __restrict__ out,
                                             Grid g, Coef3<T> cf, int odd, T dt, int divide,
                                             StatPart* part) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  const int k = blockIdx.z;
  const bool valid = i < g.nx && j < g.ny;
  double dv = 0.0;
  long long q = 0;
  if (valid) {
    q = (long long)i + g.sy() * j + g.sz() * k;
    const T* f[3] = {fx, fy, fz};
    T d[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      if (g.bc[a] == AX_ZERO) { d[a] = (T)0; continue; }
      T v[7];
      load_line<3>(f[a], g, a, i, j, k, odd != 0, v);
      d[a] = d1(v, cf.ax[a]);
    }
    const T div = d[0] + d[1] + d[2];
    dv = (double)div;
    if (out) out[q] = (O)(divide ? div / dt : div);
  }
  if (part) block_stat(stat_of(dv, q, valid), part, block_linear_id());
}

// ---------------------------------------------------------------------------
// correct_velocity (src/integration.f90:297-325): u = u* - dt dp/dx_i with
// the even ("p") closures, plus the per-step extrema of the corrected field
// (NaN / overflow check, print_velocity_values, compute_cfl).
// ---------------------------------------------------------------------------
template <class T, class P>
__global__ void __launch_bounds__(256) k_correct(CorrArgs<T, P> A) {
  const Grid& g = A.g;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  const int k = blockIdx.z;
  const bool valid = i < g.nx && j < g.ny;
  double r[10];
  const int ops[10] = {RED_MIN, RED_MIN, RED_MIN, RED_MAX, RED_MAX, RED_MAX,
                       RED_MAX, RED_MAX, RED_MAX, RED_MAX};
#pragma unroll
  for (int q = 0; q < 3; ++q) { r[q] = INFINITY; r[3 + q] = -INFINITY; r[6 + q] = 0.0; }
  r[9] = 0.0;
  if (valid) {
    const long long q = (long long)i + g.sy() * j + g.sz() * k;
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      T gp = (T)0;
      if (g.bc[a] != AX_ZERO) {
        T v[7];
        load_line<3>(A.p, g, a, i, j, k, false, v);
        gp = d1(v, A.cf.ax[a]);
      }
      const T un = A.up[a][q] - A.dt * gp;
      A.u[a][q] = un;
      const double d = (double)un;
      if (d != d) r[9] = 1.0;
      else {
        r[a] = d;
        r[3 + a] = d;
        r[6 + a] = fabs(d);
      }
    }
  }
  block_reduce_store<10>(r, ops, A.part, block_linear_id());
}

// ---------------------------------------------------------------------------
// statistics_calc (src/utils.f90:277-361): per block partial sums of
// <u^2>,<v^2>,<w^2>, nine <(du_i/dx_j)^2>, E_k, eps, dzeta, eps2 in FP64.
// ---------------------------------------------------------------------------
template <class T>
__global__ void __launch_bounds__(256) k_stats(const T* __restrict__ ux, const T* __restrict__ uy,
                                               const T* __restrict__ uz, Grid g, Coef3<T> cf,
                                               double xnu, double* part) {
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
        g1[c][a] = (double)d1(v, cf.ax[a]);
        g2[c][a] = (double)d2(v, cf.ax[a]);
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
// and of the weights min(phi, 1-phi).
// ---------------------------------------------------------------------------
template <class T>
__global__ void __launch_bounds__(256) k_transeq(ScalArgs<T> A) {
  const Grid& g = A.g;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  const int k = blockIdx.z;
  double r[3] = {0.0, 0.0, 0.0};
  const int ops[3] = {RED_SUM, RED_SUM, RED_SUM};
  if (i < g.nx && j < g.ny) {
    const long long q = (long long)i + g.sy() * j + g.sz() * k;
    T s1[3], s2[3], pc = (T)0;
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      if (g.bc[a] == AX_ZERO) { s1[a] = (T)0; s2[a] = (T)0; continue; }
      T v[7];
      load_line<3>(A.phi, g, a, i, j, k, false, v);
      s1[a] = d1(v, A.cf.ax[a]);
      s2[a] = d2(v, A.cf.ax[a]);
      if (a == 0) pc = v[3];
    }
    T alpha = A.alpha0;
    if (A.les) alpha = alpha + A.nu_t[q] / A.sc;
    const T F = alpha * (s2[0] + s2[1] + s2[2]) -
                (A.u[0][q] * s1[0] + A.u[1][q] * s1[1] + A.u[2][q] * s1[2]) + A.src[q];
    T ph = pc + A.adu * F;
    if (A.f2) ph = ph + A.bdu * A.f2[q];
    if (A.f3) ph = ph + A.cdu * A.f3[q];
    A.fnew[q] = F;
    r[0] = (double)ph;
    const T cl = fmax((T)0, fmin((T)1, ph));
    r[1] = (double)cl;
    r[2] = (double)fmin(cl, (T)1 - cl);
    A.phi_out[q] = cl;
  }
  block_reduce_store<3>(r, ops, A.part, block_linear_id());
}

// second clipping pass (src/integration.f90:443-450); sums[0..2] are the
// finalized totals of k_transeq.
template <class T>
__global__ void k_scalar_redistribute(T* __restrict__ phi, long long n, const double* sums) {
  const long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= n) return;
  const double wsum = sums[2];
  if (wsum == 0.0) return;  // nothing to spread the excess over
  const double excess = sums[0] / (double)n - sums[1] / (double)n;
  const T p = phi[q];
  const T w = (T)((double)fmin(p, (T)1 - p) / wsum);
  phi[q] = fmax((T)0, fmin((T)1, p + (T)excess * w));
}

// ---------------------------------------------------------------------------
// fixed-order finalizers
// ---------------------------------------------------------------------------
__global__ void k_finalize(const double* __restrict__ part, long long nblk, int M,
                           unsigned long long opmask, double* out) {
  __shared__ double sh[1024];
  for (int q = 0; q < M; ++q) {
    const int op = (int)((opmask >> (2 * q)) & 3ull);
    double acc = red_ident(op);
    const double* slot = part + (long long)q * nblk;
    for (long long b = threadIdx.x; b < nblk; b += blockDim.x) acc = red_apply(op, acc, slot[b]);
    sh[threadIdx.x] = acc;
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1) {
      if ((int)threadIdx.x < s) sh[threadIdx.x] = red_apply(op, sh[threadIdx.x], sh[threadIdx.x + s]);
      __syncthreads();
    }
    if (threadIdx.x == 0) out[q] = sh[0];
    __syncthreads();
  }
}

__global__ void k_finalize_stats(const StatPart* __restrict__ part, long long nblk, Grid g,
                                 double* out6) {
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
  k_der<T><<<pt_grid(g), pt_block(), 0, s>>>(f, df, g, c, axis, order, odd);
}
constexpr int PRED_TX = 32, PRED_TY = 8, PRED_KC = 32;

template <class T>
void launch_predict(const PredArgs<T>& a, cudaStream_t s) {
  const Grid& g = a.g;
  dim3 grid((g.nx + PRED_TX - 1) / PRED_TX, (g.ny + PRED_TY - 1) / PRED_TY, (g.nz + PRED_KC - 1) / PRED_KC);
  k_predict25<T, PRED_TX, PRED_TY><<<grid, dim3(PRED_TX, PRED_TY), 0, s>>>(a, PRED_KC);
}
template <class T>
void launch_nu_t(const T* ux, const T* uy, const T* uz, T* nu, const Grid& g, const Coef3<T>& cf,
                 T csd2, cudaStream_t s) {
  k_nu_t<T><<<pt_grid(g), pt_block(), 0, s>>>(ux, uy, uz, nu, g, cf, csd2);
}
constexpr int Z_TX = 32, Z_TY = 8, Z_KC = 32;
static inline dim3 z_grid(const Grid& g) {
  return dim3((g.nx + Z_TX - 1) / Z_TX, (g.ny + Z_TY - 1) / Z_TY, (g.nz + Z_KC - 1) / Z_KC);
}
long long z_blocks(const Grid& g) { dim3 b = z_grid(g); return (long long)b.x * b.y * b.z; }

template <class T, class O>
void launch_div(const T* fx, const T* fy, const T* fz, O* out, const Grid& g, const Coef3<T>& cf,
                int odd, T dt, int divide, StatPart* part, cudaStream_t s) {
  k_div25<T, O, Z_TX, Z_TY><<<z_grid(g), dim3(Z_TX, Z_TY), 0, s>>>(fx, fy, fz, out, g, cf, odd, dt, divide,
                                                                     part, Z_KC);
}
template <class T, class P>
void launch_correct(const CorrArgs<T, P>& a, cudaStream_t s) {
  k_correct25<T, P, Z_TX, Z_TY><<<z_grid(a.g), dim3(Z_TX, Z_TY), 0, s>>>(a, Z_KC);
}
template <class T>
void launch_stats(const T* ux, const T* uy, const T* uz, const Grid& g, const Coef3<T>& cf,
                  double xnu, double* part, cudaStream_t s) {
  k_stats<T><<<pt_grid(g), pt_block(), 0, s>>>(ux, uy, uz, g, cf, xnu, part);
}
template <class T>
void launch_transeq(const ScalArgs<T>& a, const double* sums, cudaStream_t s, long long* nl) {
  k_transeq<T><<<pt_grid(a.g), pt_block(), 0, s>>>(a);
  launch_finalize(a.part, pt_blocks(a.g), 3, 0ull, (double*)sums, s);
  k_scalar_redistribute<T><<<(unsigned)((a.g.n + 255) / 256), 256, 0, s>>>(a.phi_out, a.g.n, sums);
  *nl += 3;
}
void launch_finalize(const double* part, long long nblk, int M, unsigned long long opmask,
                     double* out, cudaStream_t s) {
  k_finalize<<<1, 1024, 0, s>>>(part, nblk, M, opmask, out);
}
void launch_finalize_stats(const StatPart* part, long long nblk, const Grid& g, double* out6,
                           cudaStream_t s) {
  k_finalize_stats<<<1, 1024, 0, s>>>(part, nblk, g, out6);
}
template <class S, class D>
void launch_convert(const S* s_, D* d, long long n, cudaStream_t s) {
  k_convert<S, D><<<(unsigned)((n + 255) / 256), 256, 0, s>>>(s_, d, n);
}

#define O3D_INST(T)                                                                            \
  template void launch_der<T>(const T*, T*, const Grid&, const AxisCoef<T>&, int, int, int,     \
                              cudaStream_t);                                                   \
  template void launch_predict<T>(const PredArgs<T>&, cudaStream_t);                            \
  template void launch_nu_t<T>(const T*, const T*, const T*, T*, const Grid&, const Coef3<T>&,  \
                               T, cudaStream_t);                                               \
  template void launch_stats<T>(const T*, const T*, const T*, const Grid&, const Coef3<T>&,     \
                                double, double*, cudaStream_t);                                \
  template void launch_transeq<T>(const ScalArgs<T>&, const double*, cudaStream_t, long long*);
O3D_INST(double)
O3D_INST(float)
template void launch_div<double, double>(const double*, const double*, const double*, double*,
                                         const Grid&, const Coef3<double>&, int, double, int,
                                         StatPart*, cudaStream_t);
template void launch_div<float, float>(const float*, const float*, const float*, float*,
                                       const Grid&, const Coef3<float>&, int, float, int,
                                       StatPart*, cudaStream_t);
template void launch_correct<double, double>(const CorrArgs<double, double>&, cudaStream_t);
template void launch_correct<float, double>(const CorrArgs<float, double>&, cudaStream_t);
template void launch_convert<double, float>(const double*, float*, long long, cudaStream_t);
template void launch_convert<float, double>(const float*, double*, long long, cudaStream_t);

}  // namespace o3d
