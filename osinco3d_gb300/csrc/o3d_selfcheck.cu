// o3d_selfcheck.cu -- device self-check of the integer-pipe binary64 <->
// binary32 conversions (f64_to_f32, f32_to_f64 in o3d_internal.cuh) and of
// the double-float split (split_df) against the FP64 instructions.
#include <cstdio>

#include "o3d_internal.cuh"
#include "o3d_kernels.h"

namespace o3d {

__device__ __forceinline__ unsigned long long mix64(unsigned long long x) {
  x += 0x9e3779b97f4a7c15ull;
  x = (x ^ (x >> 30)) * 0xbf58476d1ce4e5b9ull;
  x = (x ^ (x >> 27)) * 0x94d049bb133111ebull;
  return x ^ (x >> 31);
}

// case q % 4: 0 raw 64-bit pattern; 1 a binary32 value widened and nudged;
// 2 a pattern whose dropped 29 bits are exactly half (a tie); 3 a value
// around the binary32 normal range limits
__global__ void k_check_conversions(long long n, unsigned long long seed, unsigned long long* bad) {
  unsigned long long local = 0;
  for (long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x; q < n; q += (long long)gridDim.x * blockDim.x) {
    const unsigned long long r = mix64(seed ^ (unsigned long long)q);
    unsigned long long b = r;
    switch ((int)(q & 3)) {
      case 1: {
        const double w = (double)__uint_as_float((unsigned)r);
        b = (unsigned long long)__double_as_longlong(w) + ((r >> 40) & 7) - 3;
        break;
      }
      case 2: b = (r & ~0x1fffffffull) | 0x10000000ull; break;
      case 3: {
        const unsigned e = (unsigned)((r >> 52) % 80) + (((r >> 60) & 1) ? 860u : 1110u);  // near 897 and 1150
        b = (r & 0x800fffffffffffffull) | ((unsigned long long)e << 52);
        break;
      }
      default: break;
    }
    const double x = __longlong_as_double((long long)b);
    if (x == x) {
      const float a = f64_to_f32(x), c = __double2float_rn(x);
      if (__float_as_uint(a) != __float_as_uint(c)) ++local;
      // split: h = RN32(x), l = RN32(x - h) (x - h is exact in binary64) for
      // 2^-74 <= |x| < 2^128; below, h = RN32(x) flushed to 0 under 2^-126
      // and l = 0; above, h = +-inf and l = 0
      const DF s = split_df(x);
      const double ax = fabs(x);
      DF w;
      if (ax >= 0x1p-74 && ax < 0x1p128) {
        w.h = c;
        w.l = __double2float_rn(x - (double)c);
      } else {
        w.h = ax < 0x1p-126 ? copysignf(0.f, c) : c;
        w.l = 0.f;
      }
      const bool edge = isinf(c) && ax < 0x1p128;  // rounds up to inf: l is left unspecified
      if (!edge && (__float_as_uint(s.h) != __float_as_uint(w.h) || __float_as_uint(s.l) != __float_as_uint(w.l)))
        ++local;
    }
    const float f = __uint_as_float((unsigned)(r >> 17));
    if (f == f) {
      const double a = f32_to_f64(f), c = (double)f;
      if (__double_as_longlong(a) != __double_as_longlong(c)) ++local;
    }
  }
  if (local) atomicAdd(bad, local);
}

}  // namespace o3d

extern "C" int o3d_check_conversions(long long n, unsigned long long seed, long long* mismatches) {
  if (n < 0 || !mismatches) return O3D_ERR_BADARG;
  unsigned long long* d = nullptr;
  if (cudaMalloc(&d, sizeof *d) != cudaSuccess) return O3D_ERR_NOMEM;
  cudaMemset(d, 0, sizeof *d);
  o3d::k_check_conversions<<<1216, 256>>>(n, seed, d);
  unsigned long long h = 0;
  const cudaError_t e = cudaMemcpy(&h, d, sizeof h, cudaMemcpyDeviceToHost);
  cudaFree(d);
  if (e != cudaSuccess) {
    o3d::set_error("o3d_check_conversions: %s", cudaGetErrorString(e));
    return O3D_ERR_CUDA;
  }
  *mismatches = (long long)h;
  return O3D_OK;
}
