// o3d_internal.cuh -- shared device/host machinery of libo3d.so.
//
// Grid model: node-inclusive axes of n points (x fastest, column-major like
// the Fortran fields).  Each axis is periodic (wrap with period n points,
// src/derivation.f90:34-56), free-slip (mirror about the end nodes; even
// fields reflect, odd fields reflect with a sign flip, src/derivation.f90:
// 87-159), collapsed (2D mode, every z-derivative is zero,
// src/derivation.f90:481-495) or, on x only, open: inflow at x(1), outflow
// at x(nx), with one-sided closures (d1c / d2c below).
//
// Every boundary row of the reference's explicit closures equals the
// interior stencil applied to ghost values f(-m) = s f(m), f(n-1+m) =
// s f(n-1-m) (s = +1 even, -1 odd) or f(-m) = f(n-m) (periodic), evaluated
// in the same operation order; the kernels use that ghost form, so one
// stencil covers the 18 derivative routines.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>
#include <string.h>

#include "../../include/o3d.h"

namespace o3d {

enum AxisBC { AX_PERIODIC = 0, AX_MIRROR = 1, AX_ZERO = 2, AX_OPEN = 3 };

struct Grid {
  int nx, ny, nz;
  int bc[3];         // AxisBC per axis
  long long n;       // nx*ny*nz
  __host__ __device__ long long sy() const { return nx; }
  __host__ __device__ long long sz() const { return (long long)nx * ny; }
  __host__ __device__ int len(int a) const { return a == 0 ? nx : a == 1 ? ny : nz; }
  __host__ __device__ long long stride(int a) const { return a == 0 ? 1 : a == 1 ? (long long)nx : (long long)nx * ny; }
};

// Stencil coefficients of one axis, computed on the host exactly as the
// reference does (src/derivation.f90:26-30 and :518-522).
template <class T>
struct AxisCoef {
  T a1, b1, c1;   // 1/(60h), 9/(60h), 45/(60h)
  T a2, b2, c2;   // 1/(12h^2), 16/(12h^2), 30/(12h^2)
  T h2, h12, hh;  // 2h, 12h, h^2: the denominators of the open-axis closures
};

template <class T>
struct Coef3 {
  AxisCoef<T> ax[3];
};

inline void make_coef(double h, AxisCoef<double>& c) {
  double sixtyd = 60.0 * h;
  c.a1 = 1.0 / sixtyd; c.b1 = 9.0 / sixtyd; c.c1 = 45.0 / sixtyd;
  double twelved2 = 12.0 * h * h;
  c.a2 = 1.0 / twelved2; c.b2 = 16.0 / twelved2; c.c2 = 30.0 / twelved2;
  c.h2 = 2.0 * h; c.h12 = 12.0 * h; c.hh = h * h;
}
template <class T>
inline Coef3<T> cast_coef(const Coef3<double>& d) {
  Coef3<T> r;
  for (int a = 0; a < 3; ++a) {
    r.ax[a].a1 = (T)d.ax[a].a1; r.ax[a].b1 = (T)d.ax[a].b1; r.ax[a].c1 = (T)d.ax[a].c1;
    r.ax[a].a2 = (T)d.ax[a].a2; r.ax[a].b2 = (T)d.ax[a].b2; r.ax[a].c2 = (T)d.ax[a].c2;
    r.ax[a].h2 = (T)d.ax[a].h2; r.ax[a].h12 = (T)d.ax[a].h12; r.ax[a].hh = (T)d.ax[a].hh;
  }
  return r;
}

// Ghost map of index m in [-3, n+2] onto [0, n-1]; *flip tells whether an odd
// field changes sign there.  Indices farther out (only reached by threads of
// a partial tile, whose results are discarded) are clamped.
__device__ __forceinline__ int ghost(int m, int n, int bc, bool* flip) {
  *flip = false;
  if (m >= 0 && m < n) return m;
  int r;
  if (bc == AX_PERIODIC) {
    r = m < 0 ? m + n : m - n;
  } else {
    *flip = true;
    r = m < 0 ? -m : 2 * (n - 1) - m;
  }
  return r < 0 ? 0 : (r >= n ? n - 1 : r);
}

template <class T>
__device__ __forceinline__ T ld(const T* __restrict__ p, long long i) { return __ldg(p + i); }

// plane k, ghost-mapped along z: element offset of the plane and its flip
struct ZPlane {
  long long off;
  bool fz;
};
__device__ __forceinline__ ZPlane z_plane(const Grid& g, int k) {
  ZPlane z;
  const int kk = ghost(k, g.nz, g.bc[2] == AX_ZERO ? AX_PERIODIC : g.bc[2], &z.fz);
  z.off = g.sz() * kk;
  return z;
}

// block-wide max of nonnegative floats, result valid in thread 0
__device__ __forceinline__ float block_max_f(float v) {
  __shared__ float sh[32];
  const int t = threadIdx.x + blockDim.x * (threadIdx.y + blockDim.y * threadIdx.z);
  const int nt = blockDim.x * blockDim.y * blockDim.z;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
  __syncthreads();
  if ((t & 31) == 0) sh[t >> 5] = v;
  __syncthreads();
  if (t < 32) {
    v = t < (nt + 31) / 32 ? sh[t] : 0.f;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
  }
  return v;
}

// ---- programmatic dependent launch ----------------------------------------
// A kernel launched by launch_pdl may be scheduled while its predecessor in
// the stream is still running; it calls pdl_enter() before anything else:
// let its own dependents be scheduled, then wait until the predecessor has
// completed and its writes are visible.  For a kernel launched without the
// attribute both instructions do nothing.  This overlaps the launch of the
// many short kernels of a V-cycle with the end of the kernel before.
__device__ __forceinline__ void pdl_enter() {
  asm volatile("griddepcontrol.launch_dependents;\n" ::: "memory");
  asm volatile("griddepcontrol.wait;\n" ::: "memory");
}
template <typename... KArgs, typename... Args>
inline cudaError_t launch_pdl(void (*kern)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t s,
                              Args... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  at[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, kern, (KArgs)args...);
}

// ---- cp.async (global -> shared, bypassing the registers) -----------------
template <int B>
__device__ __forceinline__ void cp_async(void* smem, const void* gmem) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.ca.shared.global [%0], [%1], %2;\n" ::"r"(s), "l"(gmem), "n"(B) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory");
}

// ---- binary64 <-> binary32 conversions on the integer pipe ---------------
// GB300 executes FP64 instructions (conversions included) at 2 lanes per
// clock per SM, so a kernel that converts every point is bound by them.
// These convert by the IEEE 754 binary formats themselves: rebias the
// exponent (1023 <-> 127) and move the fraction, rounding the 29 dropped
// fraction bits to nearest, ties to even (roundTiesToEven, IEEE 754-2008
// 4.3.1).  Zeros and normal numbers take the integer path; subnormal,
// infinite, NaN and out-of-range values fall back to the FP64 instruction.
// Results are bit-identical to __double2float_rn and to the exact widening.
// The fallbacks are out of line so that the compiler cannot turn the branch
// into a select that runs the FP64 instruction for every value.
static __device__ __noinline__ float f64_to_f32_rare(double x) { return __double2float_rn(x); }
static __device__ __noinline__ double f32_to_f64_rare(float x) { return (double)x; }

__device__ __forceinline__ float f64_to_f32(double x) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
  const unsigned hi = (unsigned)(b >> 32), lo = (unsigned)b;
  const unsigned e = (hi >> 20) & 0x7ffu;          // biased binary64 exponent
  const unsigned sign = hi & 0x80000000u;
  if (e - 897u <= 253u) {                          // binary32 exponent 1..254
    unsigned f = ((e - 896u) << 23) | ((hi & 0xfffffu) << 3) | (lo >> 29);
    const unsigned rem = lo & 0x1fffffffu;         // the 29 dropped fraction bits
    f += (rem > 0x10000000u || (rem == 0x10000000u && (f & 1u))) ? 1u : 0u;  // carries into the exponent
    return __uint_as_float(sign | f);
  }
  if (((hi << 1) | lo) == 0u) return __uint_as_float(sign);  // +-0
  return f64_to_f32_rare(x);
}

__device__ __forceinline__ double f32_to_f64(float x) {
  const unsigned u = __float_as_uint(x);
  const unsigned e = (u >> 23) & 0xffu;
  if (e - 1u <= 253u)                              // normal: exact widening
    return __hiloint2double((int)((u & 0x80000000u) | ((e + 896u) << 20) | ((u >> 3) & 0xfffffu)), (int)(u << 29));
  if ((u << 1) == 0u) return __hiloint2double((int)(u & 0x80000000u), 0);  // +-0
  return f32_to_f64_rare(x);
}

// Knuth's TwoSum: s + err == a + b exactly (round-to-nearest FP32), six FP32
// operations.  Accumulating (hi, lo) with it keeps a column sum of FP32
// values to about 2^-48 of its magnitude without FP64 arithmetic.
__device__ __forceinline__ void two_sum_acc(float& hi, float& lo, float x) {
  const float s = hi + x;
  const float bp = s - hi;
  const float err = (hi - (s - bp)) + (x - bp);
  hi = s;
  lo += err;
}

// ---- double-float arithmetic (Dekker 1971; Knuth TAOCP vol. 2, 4.2.2) ----
// A value held as hi + lo, two FP32 numbers with |lo| <= ulp(hi) / 2: 48
// significant bits, evaluated on the FP32 pipe (64x the FP64 rate here).
struct __align__(8) DF {
  float h, l;
};

__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
  s = a + b;
  const float bp = s - a;
  e = (a - (s - bp)) + (b - bp);
}

// x = h + l with h = RN32(x) (as f64_to_f32) and l = RN32(x - h), on the
// integer pipe: the 29 fraction bits that h drops (less 2^29 when h rounded
// up) scaled by 2^(e - 1075), e the biased binary64 exponent.  That is exact
// for 2^-74 <= |x| < 2^128 (e in [949, 1150]).  Outside it the split uses no
// FP64 instruction either: below, l = 0 (|x - h| < 2^-98) and h = +-0 under
// 2^-126; above, h = +-inf (NaN for a NaN) and l = 0.
__device__ __forceinline__ DF split_df(double x) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
  const unsigned hi = (unsigned)(b >> 32), lo = (unsigned)b;
  const unsigned e = (hi >> 20) & 0x7ffu;
  const unsigned sign = hi & 0x80000000u;
  unsigned f = ((e - 896u) << 23) | ((hi & 0xfffffu) << 3) | (lo >> 29);
  const unsigned rem = lo & 0x1fffffffu;
  const bool up = rem > 0x10000000u || (rem == 0x10000000u && (f & 1u));
  f += up ? 1u : 0u;
  int ri = up ? (int)rem - (1 << 29) : (int)rem;
  ri = sign ? -ri : ri;                            // a zero remainder stays +0, as x - h does
  DF r;
  r.h = __uint_as_float(sign | f);
  r.l = (float)ri * __uint_as_float((e - 948u) << 23);  // 2^(e - 1075)
  if (e - 949u > 201u) {
    r.l = 0.f;
    if (e < 897u) r.h = __uint_as_float(sign);
    else if (e > 1150u)
      r.h = __uint_as_float(sign | 0x7f800000u | ((e == 2047u && ((hi & 0xfffffu) | lo)) ? 0x400000u : 0u));
  }
  return r;
}

// double-float coefficients of the 7-point operator (hi + lo of A, ox, oy,
// oz), split on the host so that no kernel evaluates FP64 for them
struct PoiDF {
  DF A, ox, oy, oz;
};
inline DF df_split_host(double v) {
  DF r;
  r.h = (float)v;
  r.l = (float)(v - (double)r.h);
  return r;
}

// a * c to about 2^-46 relative, left unnormalised as (p, q): p = RN(a.h c.h)
// and q its exact FMA error plus the cross terms
__device__ __forceinline__ void df_mul(const DF& a, const DF& c, float& p, float& q) {
  p = a.h * c.h;
  q = fmaf(a.h, c.h, -p);
  q = fmaf(a.h, c.l, q);
  q = fmaf(a.l, c.h, q);
}

// rhs - (A pc + ox (pw + pe) + oy (ps + pn) + oz (pb + pt)) with double-float
// operands and coefficients, rounded once to FP32 at the end: the large
// partial sums are carried exactly by TwoSum, so the cancellation between rhs
// and the operator leaves an error of about 2^-46 of the largest term.
__device__ __forceinline__ float df_resid7(const DF& rh, const DF& pc, const DF& pw, const DF& pe, const DF& ps,
                                           const DF& pn, const DF& pb, const DF& pt, const DF& cA, const DF& cx,
                                           const DF& cy, const DF& cz) {
  DF sx, sy, sz;
  two_sum(pw.h, pe.h, sx.h, sx.l);
  sx.l += pw.l + pe.l;
  two_sum(ps.h, pn.h, sy.h, sy.l);
  sy.l += ps.l + pn.l;
  two_sum(pb.h, pt.h, sz.h, sz.l);
  sz.l += pb.l + pt.l;
  float qa, la, qx, lx, qy, ly, qz, lz;
  df_mul(pc, cA, qa, la);
  df_mul(sx, cx, qx, lx);
  df_mul(sy, cy, qy, ly);
  df_mul(sz, cz, qz, lz);
  float s, e1, e2, e3, e4;
  two_sum(rh.h, -qa, s, e1);
  two_sum(s, -qx, s, e2);
  two_sum(s, -qy, s, e3);
  two_sum(s, -qz, s, e4);
  const float l = ((rh.l - la) - (lx + ly + lz)) + ((e1 + e2) + (e3 + e4));
  return s + l;
}

// ---- the pressure of the mixed multigrid method: a double-float pair of
// FP32 planes in one buffer the size of n doubles, hi = RN32(p) at [0, n)
// and lo = RN32(p - hi) at [n, 2n) (floats) ----
struct PPair {
  float* hi;
  float* lo;
};
inline PPair ppair(void* buf, long long n) { return PPair{(float*)buf, (float*)buf + n}; }

// (h, l) <- (h, l) + d for a double-float value and an FP32 increment: the
// exact sum of h and d by TwoSum, the low parts added, and the pair
// renormalised by a second TwoSum (h stays the FP32 rounding of the value)
__device__ __forceinline__ void df_add_f(float& h, float& l, float d) {
  float s, e;
  two_sum(h, d, s, e);
  e += l;
  two_sum(s, e, h, l);
}
// a + b, renormalised
__device__ __forceinline__ DF df_add(const DF& a, const DF& b) {
  float s, e;
  two_sum(a.h, b.h, s, e);
  e += a.l + b.l;
  DF r;
  two_sum(s, e, r.h, r.l);
  return r;
}
// k a for a small integer k (the high product's error recovered by FMA)
__device__ __forceinline__ DF df_scale(const DF& a, float k) {
  const float p = k * a.h;
  float e = fmaf(k, a.h, -p);
  e = fmaf(k, a.l, e);
  DF r;
  two_sum(p, e, r.h, r.l);
  return r;
}
__device__ __forceinline__ DF df_neg(const DF& a) { return DF{-a.h, -a.l}; }
__device__ __forceinline__ DF pp_load(const PPair& p, long long q) { return DF{p.hi[q], p.lo[q]}; }
__device__ __forceinline__ void pp_store(const PPair& p, long long q, const DF& v) {
  p.hi[q] = v.h;
  p.lo[q] = v.l;
}

// conversion of a loaded value to the compute type
template <class T, class S>
__device__ __forceinline__ T to_t(S v) { return (T)v; }
template <>
__device__ __forceinline__ float to_t<float, double>(double v) { return f64_to_f32(v); }
template <>
__device__ __forceinline__ double to_t<double, float>(float v) { return f32_to_f64(v); }

// Loads f at offsets -R..R along axis `a` of point (i,j,k) into v[0..2R].
// Interior points take the fast path; points within R of an end use ghost().
template <int R, class T, class S>
__device__ __forceinline__ void load_line(const S* __restrict__ f, const Grid& g, int a,
                                          int i, int j, int k, bool odd, T* v) {
  const int n = g.len(a);
  const int pos = a == 0 ? i : a == 1 ? j : k;
  const long long st = g.stride(a);
  const long long c = (long long)i + g.sy() * j + g.sz() * k;
  if (pos >= R && pos < n - R) {
#pragma unroll
    for (int o = -R; o <= R; ++o) v[o + R] = (T)ld(f, c + st * o);
  } else {
    const long long base = c - st * pos;
#pragma unroll
    for (int o = -R; o <= R; ++o) {
      bool flip;
      int m = ghost(pos + o, n, g.bc[a], &flip);
      T x = (T)ld(f, base + st * m);
      v[o + R] = (flip && odd) ? -x : x;
    }
  }
}

// 6th-order first derivative a(f3-f-3) - b(f2-f-2) + c(f1-f-1), in the order
// of src/derivation.f90:44-46.
template <class T>
__device__ __forceinline__ T d1(const T* v, const AxisCoef<T>& c) {
  return c.a1 * (v[6] - v[0]) - c.b1 * (v[5] - v[1]) + c.c1 * (v[4] - v[2]);
}
// 4th-order second derivative -a(f-2+f2) + b(f-1+f1) - c f0, in the order of
// src/derivation.f90:530-532; v is the 7-point line (centre v[3]).
template <class T>
__device__ __forceinline__ T d2(const T* v, const AxisCoef<T>& c) {
  return -c.a2 * (v[1] + v[5]) + c.b2 * (v[2] + v[4]) - c.c2 * v[3];
}

// ---- open x axis (nbcx1 = nbcxn = 2) -------------------------------------
// The reference binds no derivative for it (src/initialization.f90:228-242
// stops); this build defines the closure.  First derivative: the one-sided
// scheme of dery1D (src/derivation.f90:950-992) -- 2nd order one-sided at the
// end nodes, 2nd-order central next to them, 4th-order central at the third
// node -- with the 6th-order interior stencil.  Second derivative: 2nd-order
// one-sided at the end nodes, 2nd-order central next to them, the 4th-order
// interior stencil elsewhere.  Position class of index i on an open axis of n
// points: 0 interior, 1..3 the first three nodes, 4..6 the last three.  v is
// the 7-point window f(i-3 .. i+3); the closures read only its in-range values.
__device__ __forceinline__ int open_class(int i, int n) {
  return i < 3 ? i + 1 : (i >= n - 3 ? i - (n - 3) + 4 : 0);
}
__device__ __forceinline__ int xclass(const Grid& g, int i) {
  return g.bc[0] == AX_OPEN ? open_class(i, g.nx) : 0;
}
template <class T>
__device__ __forceinline__ T d1c(const T* v, const AxisCoef<T>& c, int pc) {
  switch (pc) {
    case 0: return d1(v, c);
    case 1: return (-v[5] + (T)4 * v[4] - (T)3 * v[3]) / c.h2;
    case 2:
    case 5: return (v[4] - v[2]) / c.h2;
    case 3:
    case 4: return (-v[5] + (T)8 * v[4] - (T)8 * v[2] + v[1]) / c.h12;
    default: return ((T)3 * v[3] - (T)4 * v[2] + v[1]) / c.h2;
  }
}
template <class T>
__device__ __forceinline__ T d2c(const T* v, const AxisCoef<T>& c, int pc) {
  switch (pc) {
    case 1: return ((T)2 * v[3] - (T)5 * v[4] + (T)4 * v[5] - v[6]) / c.hh;
    case 2:
    case 5: return (v[2] - (T)2 * v[3] + v[4]) / c.hh;
    case 6: return ((T)2 * v[3] - (T)5 * v[2] + (T)4 * v[1] - v[0]) / c.hh;
    default: return d2(v, c);
  }
}
// x-derivatives of a kernel compiled with (XO) or without the open-axis
// closures: without them the plain stencil, no class test
template <bool XO, class T>
__device__ __forceinline__ T d1x(const T* v, const AxisCoef<T>& c, int pc) {
  if constexpr (XO) return d1c(v, c, pc);
  else return d1(v, c);
}
template <bool XO, class T>
__device__ __forceinline__ T d2x(const T* v, const AxisCoef<T>& c, int pc) {
  if constexpr (XO) return d2c(v, c, pc);
  else return d2(v, c);
}

// ---- order-preserving keys for atomic min/max of doubles ----------------
__device__ __forceinline__ unsigned long long dkey(double x) {
  unsigned long long u = (unsigned long long)__double_as_longlong(x);
  return (u >> 63) ? ~u : (u | 0x8000000000000000ull);
}
__host__ __device__ inline double dkey_inv(unsigned long long k) {
  unsigned long long u = (k >> 63) ? (k & 0x7fffffffffffffffull) : ~k;
  double d;
  memcpy(&d, &u, 8);
  return d;
}
constexpr unsigned long long KEY_MIN = 0ull;             // below every double
constexpr unsigned long long KEY_MAX = ~0ull;            // above every double

// ---- warp/block reductions ------------------------------------------------
__device__ __forceinline__ double warp_max(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}
__device__ __forceinline__ double warp_min(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmin(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}
__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Block-wide max, result valid in thread 0.  blockDim.x*y*z <= 1024.
__device__ inline double block_max(double v) {
  __shared__ double sh[32];
  const int t = threadIdx.x + blockDim.x * (threadIdx.y + blockDim.y * threadIdx.z);
  const int nt = blockDim.x * blockDim.y * blockDim.z;
  v = warp_max(v);
  __syncthreads();
  if ((t & 31) == 0) sh[t >> 5] = v;
  __syncthreads();
  if (t < 32) {
    v = t < (nt + 31) / 32 ? sh[t] : -INFINITY;
    v = warp_max(v);
  }
  return v;
}
__device__ inline double block_sum(double v) {
  __shared__ double sh[32];
  const int t = threadIdx.x + blockDim.x * (threadIdx.y + blockDim.y * threadIdx.z);
  const int nt = blockDim.x * blockDim.y * blockDim.z;
  v = warp_sum(v);
  __syncthreads();
  if ((t & 31) == 0) sh[t >> 5] = v;
  __syncthreads();
  if (t < 32) {
    v = t < (nt + 31) / 32 ? sh[t] : 0.0;
    v = warp_sum(v);
  }
  return v;
}

// Field statistics of function_stats (src/functions.f90:27-63): min, max,
// sum and the first linear index of the max.  One record per block, reduced
// in a fixed order by finalize_stats so the sums are deterministic.
struct StatPart {
  double mn, mx, sum;
  long long imx;
};

__device__ inline void stat_merge(StatPart& a, const StatPart& b) {
  a.mn = fmin(a.mn, b.mn);
  if (b.mx > a.mx || (b.mx == a.mx && b.imx < a.imx)) { a.mx = b.mx; a.imx = b.imx; }
  a.sum += b.sum;
}

__device__ inline StatPart stat_shfl(const StatPart& s, int o) {
  StatPart r;
  r.mn = __shfl_xor_sync(0xffffffffu, s.mn, o);
  r.mx = __shfl_xor_sync(0xffffffffu, s.mx, o);
  r.sum = __shfl_xor_sync(0xffffffffu, s.sum, o);
  r.imx = __shfl_xor_sync(0xffffffffu, s.imx, o);
  return r;
}

// Reduces s over the block and stores the block's record at part[blk].
__device__ inline void block_stat(StatPart s, StatPart* part, long long blk) {
  __shared__ StatPart sh[32];
  const int t = threadIdx.x + blockDim.x * (threadIdx.y + blockDim.y * threadIdx.z);
  const int nt = blockDim.x * blockDim.y * blockDim.z;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) stat_merge(s, stat_shfl(s, o));
  __syncthreads();
  if ((t & 31) == 0) sh[t >> 5] = s;
  __syncthreads();
  if (t < 32) {
    if (t < (nt + 31) / 32) s = sh[t];
    else { s.mn = INFINITY; s.mx = -INFINITY; s.sum = 0; s.imx = 0x7fffffffffffffffll; }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) stat_merge(s, stat_shfl(s, o));
    if (t == 0) part[blk] = s;
  }
}

// The same record reduced with the extrema in the field type T (min/max in
// FP32 are exact and stay off the FP64 pipe, which GB300 runs at 2 lanes
// per clock) and the sum in FP64; the block record is stored as StatPart.
template <class T>
__device__ inline void block_stat_t(T mn, T mx, double sum, long long imx, StatPart* part, long long blk) {
  __shared__ T shm[2][32];
  __shared__ double shs[32];
  __shared__ long long shi[32];
  const int t = threadIdx.x + blockDim.x * (threadIdx.y + blockDim.y * threadIdx.z);
  const int nt = blockDim.x * blockDim.y * blockDim.z;
  auto merge = [&](T omn, T omx, double osum, long long oimx) {
    mn = omn < mn ? omn : mn;
    if (omx > mx || (omx == mx && oimx < imx)) { mx = omx; imx = oimx; }
    sum += osum;
  };
#pragma unroll
  for (int o = 16; o > 0; o >>= 1)
    merge(__shfl_xor_sync(0xffffffffu, mn, o), __shfl_xor_sync(0xffffffffu, mx, o),
          __shfl_xor_sync(0xffffffffu, sum, o), __shfl_xor_sync(0xffffffffu, imx, o));
  __syncthreads();
  if ((t & 31) == 0) { shm[0][t >> 5] = mn; shm[1][t >> 5] = mx; shs[t >> 5] = sum; shi[t >> 5] = imx; }
  __syncthreads();
  if (t < 32) {
    if (t < (nt + 31) / 32) { mn = shm[0][t]; mx = shm[1][t]; sum = shs[t]; imx = shi[t]; }
    else { mn = (T)INFINITY; mx = (T)-INFINITY; sum = 0.0; imx = 0x7fffffffffffffffll; }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
      merge(__shfl_xor_sync(0xffffffffu, mn, o), __shfl_xor_sync(0xffffffffu, mx, o),
            __shfl_xor_sync(0xffffffffu, sum, o), __shfl_xor_sync(0xffffffffu, imx, o));
    if (t == 0) {
      StatPart r;
      r.mn = to_t<double>(mn); r.mx = to_t<double>(mx); r.sum = sum; r.imx = imx;
      part[blk] = r;
    }
  }
}

__device__ __forceinline__ StatPart stat_of(double v, long long idx, bool valid) {
  StatPart s;
  if (valid && !(v != v)) { s.mn = v; s.mx = v; s.sum = v; s.imx = idx; }
  else { s.mn = INFINITY; s.mx = -INFINITY; s.sum = valid ? v : 0.0; s.imx = 0x7fffffffffffffffll; }
  return s;
}

// ---- M-slot block reductions with per-slot operator -----------------------
// ops is a compile-time list of RED_SUM / RED_MIN / RED_MAX; slot q of block
// blk goes to part[q*nblk + blk] (slot-major, so the finalizer reads each
// slot coalesced); k_finalize reduces the records in a fixed order
// (deterministic sums).
enum RedOp { RED_SUM = 0, RED_MIN = 1, RED_MAX = 2 };

__device__ __forceinline__ double red_apply(int op, double a, double b) {
  return op == RED_SUM ? a + b : op == RED_MIN ? fmin(a, b) : fmax(a, b);
}
__device__ __forceinline__ double red_ident(int op) {
  return op == RED_SUM ? 0.0 : op == RED_MIN ? INFINITY : -INFINITY;
}

template <int M>
__device__ inline void block_reduce_store(double (&v)[M], const int (&ops)[M], double* part,
                                          long long blk) {
  const long long nblk = (long long)gridDim.x * gridDim.y * gridDim.z;
  __shared__ double sh[M][32];
  const int t = threadIdx.x + blockDim.x * (threadIdx.y + blockDim.y * threadIdx.z);
  const int nt = blockDim.x * blockDim.y * blockDim.z;
  const int nw = (nt + 31) / 32;
#pragma unroll
  for (int q = 0; q < M; ++q) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v[q] = red_apply(ops[q], v[q], __shfl_xor_sync(0xffffffffu, v[q], o));
  }
  __syncthreads();
  if ((t & 31) == 0) {
#pragma unroll
    for (int q = 0; q < M; ++q) sh[q][t >> 5] = v[q];
  }
  __syncthreads();
  if (t < 32) {
#pragma unroll
    for (int q = 0; q < M; ++q) {
      double x = t < nw ? sh[q][t] : red_ident(ops[q]);
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) x = red_apply(ops[q], x, __shfl_xor_sync(0xffffffffu, x, o));
      if (t == 0) part[(long long)q * nblk + blk] = x;
    }
  }
}

// The same reduction carried out in T (slots with RED_MIN / RED_MAX only
// need T's exact min/max), the block's records widened to FP64 on store.
template <class T>
__device__ __forceinline__ T red_apply_t(int op, T a, T b) {
  return op == RED_SUM ? a + b : op == RED_MIN ? (b < a ? b : a) : (b > a ? b : a);
}
template <class T>
__device__ __forceinline__ T red_ident_t(int op) {
  return op == RED_SUM ? (T)0 : op == RED_MIN ? (T)INFINITY : (T)-INFINITY;
}
template <class T, int M>
__device__ inline void block_reduce_store_t(T (&v)[M], const int (&ops)[M], double* part, long long blk) {
  const long long nblk = (long long)gridDim.x * gridDim.y * gridDim.z;
  __shared__ T sh[M][32];
  const int t = threadIdx.x + blockDim.x * (threadIdx.y + blockDim.y * threadIdx.z);
  const int nt = blockDim.x * blockDim.y * blockDim.z;
  const int nw = (nt + 31) / 32;
#pragma unroll
  for (int q = 0; q < M; ++q) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v[q] = red_apply_t<T>(ops[q], v[q], __shfl_xor_sync(0xffffffffu, v[q], o));
  }
  __syncthreads();
  if ((t & 31) == 0) {
#pragma unroll
    for (int q = 0; q < M; ++q) sh[q][t >> 5] = v[q];
  }
  __syncthreads();
  if (t < 32) {
#pragma unroll
    for (int q = 0; q < M; ++q) {
      T x = t < nw ? sh[q][t] : red_ident_t<T>(ops[q]);
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) x = red_apply_t<T>(ops[q], x, __shfl_xor_sync(0xffffffffu, x, o));
      if (t == 0) part[(long long)q * nblk + blk] = to_t<double>(x);
    }
  }
}

__device__ __forceinline__ long long block_linear_id() {
  return (long long)blockIdx.x + (long long)gridDim.x * ((long long)blockIdx.y + (long long)gridDim.y * blockIdx.z);
}

// ---- per-step device diagnostics ------------------------------------------
struct DevDiag {
  unsigned long long umin[3], umax[3], uabs[3];  // ordered keys
  int nan_flag;
  int pad;
  double divp[6], divu[6];                       // function_stats of div(u*), div(u)
  double sums[32];                               // finalized sums (statistics, scalar clipping)
};

// Device-side state of a pressure solve.  Every Poisson kernel returns at
// once when `done` is set, so batches of sweeps/cycles can be queued (and
// captured in a CUDA graph) without a host round trip per iteration.
struct SolveCtrl {
  unsigned long long dmax_key;   // max |update| of the current sweep/cycle (raw bits, >= 0)
  unsigned long long res_key;    // max |residual|
  double omega;                  // SOR relaxation (dynamic update of src/poisson.f90:115-121)
  double dmax_old;               // starts at 1609 (src/poisson.f90:52)
  double dmax;                   // last completed sweep
  double eps, factor;
  double rhs_mean;               // weighted mean removed from the rhs (multigrid)
  float rhs_mean_h, rhs_mean_l;  // the same as a double-float (hi + lo)
  double res_inf;
  int iter, kmax, idyn, done, status;
  int cycles;            // V-cycles run so far
  int cycles_per_iter;   // V-cycles per outer iteration (multigrid)
  double learn_scale;    // learned warm start: rms of the restricted residual x h^2 (input 0 and output scale)
  double learn_scale_d;  // learned warm start: rms of the restricted increment (input 1 scale)
};

}  // namespace o3d
