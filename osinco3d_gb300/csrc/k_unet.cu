// k_unet.cu -- kernels of the learned Poisson warm start: 3x3x3 convolutions
// as implicit GEMMs on the BF16 tensor cores (FP32 accumulation), their
// data and weight gradients, pooling, upsampling, the 1x1 output head, the
// loss and the Adam update.
//
// Activations are BF16, channels-last: element (i, j, k, c) of a tensor with
// channel stride cs lives at ((k*ny + j)*nx + i)*cs + c0 + c, so a channel
// slice [c0, c0 + C) of a wider buffer is a tensor too (concatenation costs
// nothing).  Spatial axes either wrap (periodic) or read zeros outside.
//
// GEMM mapping of the forward convolution: M = voxels, N = output channels,
// K = 27 taps x input channels; mma.sync.m16n8k16 with BF16 operands.  On
// the deep levels' small grids the reduction is split into slices over the
// (tap, 16-channel step) sequence, each block writing FP32 partials that a
// second kernel sums in slice order (deterministic) before the epilogue.
#include <atomic>

#include <cuda_bf16.h>

#include "o3d_internal.cuh"
#include "o3d_unet.h"

namespace o3d {

__device__ __forceinline__ int wrapc(int m, int n, int per, bool* ok) {
  if (m >= 0 && m < n) { *ok = true; return m; }
  if (per) { *ok = true; return m < 0 ? m + n : m - n; }
  *ok = false;
  return 0;
}

__device__ __forceinline__ uint32_t ldpair(const __nv_bfloat16* p) {
  return *reinterpret_cast<const uint32_t*>(p);
}

__device__ __forceinline__ void mma_bf16(float (&d)[4], const uint32_t (&a)[4], const uint32_t (&b)[2]) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};\n"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

// ---------------------------------------------------------------------------
// forward convolution (also the data gradient, with the flipped, transposed
// weights): Y[p, n] = act( sum_t sum_k X[p + o_t, k] W[t, n, k] + bias[n] )
// W is BF16 [27][N][K] with K (input channels) innermost.
// Block: 4 warps, 64 voxels (16 per warp) x NT*8 output channels; blockIdx.z
// is the reduction slice (gridDim.z slices; 1 = no split, fused epilogue).
// ---------------------------------------------------------------------------
__device__ __forceinline__ void conv_epilogue(const ConvArgs& A, long long p, int n, float v0, float v1) {
  __nv_bfloat16* yrow = A.y + p * A.ycs + A.yc0;
  if (A.bias) { v0 += A.bias[n]; v1 += A.bias[n + 1]; }
  if (A.relu) { v0 = fmaxf(v0, 0.f); v1 = fmaxf(v1, 0.f); }
  if (A.mask) {  // data gradient through the ReLU of the layer below
    const __nv_bfloat16* mrow = A.mask + p * A.mcs + A.mc0;
    if (!(__bfloat162float(mrow[n]) > 0.f)) v0 = 0.f;
    if (!(__bfloat162float(mrow[n + 1]) > 0.f)) v1 = 0.f;
  }
  if (A.accumulate) {
    v0 += __bfloat162float(yrow[n]);
    v1 += __bfloat162float(yrow[n + 1]);
  }
  __nv_bfloat162 o;
  o.x = __float2bfloat16(v0);
  o.y = __float2bfloat16(v1);
  *reinterpret_cast<__nv_bfloat162*>(yrow + n) = o;
}

template <int NT>
__global__ void __launch_bounds__(128) k_conv3(ConvArgs A) {
  pdl_enter();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int g = lane >> 2, tq = lane & 3;
  const long long nvox = (long long)A.v.nx * A.v.ny * A.v.nz;
  const long long pbase = (long long)blockIdx.x * 64 + warp * 16;
  const int n0 = blockIdx.y * NT * 8;
  // this block's slice [q0, q1) of the (tap, 16-channel step) sequence
  const int kpt = A.K / 16, nq = 27 * kpt, S = gridDim.z;
  const int q0 = (int)((long long)nq * blockIdx.z / S), q1 = (int)((long long)nq * (blockIdx.z + 1) / S);
  // the two voxels whose rows this thread holds
  int ci[2], cj[2], ck[2];
  bool live[2];
#pragma unroll
  for (int r = 0; r < 2; ++r) {
    const long long p = pbase + g + 8 * r;
    live[r] = p < nvox;
    const long long pc = live[r] ? p : 0;
    ci[r] = (int)(pc % A.v.nx);
    cj[r] = (int)((pc / A.v.nx) % A.v.ny);
    ck[r] = (int)(pc / ((long long)A.v.nx * A.v.ny));
  }
  float acc[NT][4];
#pragma unroll
  for (int t = 0; t < NT; ++t)
#pragma unroll
    for (int q = 0; q < 4; ++q) acc[t][q] = 0.f;

  for (int tap = q0 / kpt; tap * kpt < q1; ++tap) {
    const int dx = tap % 3 - 1, dy = (tap / 3) % 3 - 1, dz = tap / 9 - 1;
    const __nv_bfloat16* row[2];
    bool ok[2];
#pragma unroll
    for (int r = 0; r < 2; ++r) {
      bool ox, oy, oz;
      const int ii = wrapc(ci[r] + dx, A.v.nx, A.v.per[0], &ox);
      const int jj = wrapc(cj[r] + dy, A.v.ny, A.v.per[1], &oy);
      const int kk = wrapc(ck[r] + dz, A.v.nz, A.v.per[2], &oz);
      ok[r] = live[r] && ox && oy && oz;
      row[r] = A.x + (((long long)kk * A.v.ny + jj) * A.v.nx + ii) * A.xcs + A.xc0;
    }
    const __nv_bfloat16* wt = A.w + (long long)tap * A.N * A.K;
    const int ka = max(q0 - tap * kpt, 0) * 16, kb = min(q1 - tap * kpt, kpt) * 16;
    for (int k0 = ka; k0 < kb; k0 += 16) {
      uint32_t a[4];
      const int kc = k0 + 2 * tq;
      a[0] = ok[0] ? ldpair(row[0] + kc) : 0u;
      a[1] = ok[1] ? ldpair(row[1] + kc) : 0u;
      a[2] = ok[0] ? ldpair(row[0] + kc + 8) : 0u;
      a[3] = ok[1] ? ldpair(row[1] + kc + 8) : 0u;
#pragma unroll
      for (int t = 0; t < NT; ++t) {
        const int n = n0 + t * 8 + g;
        uint32_t b[2];
        if (n < A.N) {
          const __nv_bfloat16* wn = wt + (long long)n * A.K + kc;
          b[0] = ldpair(wn);
          b[1] = ldpair(wn + 8);
        } else {
          b[0] = 0u;
          b[1] = 0u;
        }
        mma_bf16(acc[t], a, b);
      }
    }
  }
  // epilogue (pairs of channels): bias, activation, BF16 store; or the FP32
  // partial of this slice, ws[(z * nvox + p) * N + n]
#pragma unroll
  for (int r = 0; r < 2; ++r) {
    const long long p = pbase + g + 8 * r;
    if (p >= nvox) continue;
#pragma unroll
    for (int t = 0; t < NT; ++t) {
      const int n = n0 + t * 8 + 2 * tq;
      if (n >= A.N) continue;
      if (S == 1) {
        conv_epilogue(A, p, n, acc[t][2 * r], acc[t][2 * r + 1]);
      } else {
        float2 v;
        v.x = acc[t][2 * r];
        v.y = acc[t][2 * r + 1];
        *reinterpret_cast<float2*>(A.ws + ((long long)blockIdx.z * nvox + p) * A.N + n) = v;
      }
    }
  }
}

// sum of the S slices' partials in slice order, then the epilogue
__global__ void k_conv3_reduce(ConvArgs A, int S) {
  pdl_enter();
  const long long nvox = (long long)A.v.nx * A.v.ny * A.v.nz;
  const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;  // channel pair index
  const int half = A.N / 2;
  if (e >= nvox * half) return;
  const long long p = e / half;
  const int n = 2 * (int)(e % half);
  float v0 = 0.f, v1 = 0.f;
  for (int z = 0; z < S; ++z) {
    const float2 v = *reinterpret_cast<const float2*>(A.ws + ((long long)z * nvox + p) * A.N + n);
    v0 += v.x;
    v1 += v.y;
  }
  conv_epilogue(A, p, n, v0, v1);
}

// ---------------------------------------------------------------------------
// weight gradient: dW[t, k, n] += sum_p X[p + o_t, k] dY[p, n]   (FP32)
// GEMM with M = input channels (16 per block row), N = output channels,
// K = voxels.  Grid: (27 taps, K/16, voxel chunks); 4 warps split the chunk.
// ---------------------------------------------------------------------------
template <int NT>
__global__ void __launch_bounds__(128) k_conv3_wgrad(WgradArgs A) {
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int g = lane >> 2, tq = lane & 3;
  const int tap = blockIdx.x;
  const int k0 = blockIdx.y * 16;
  const long long nvox = (long long)A.v.nx * A.v.ny * A.v.nz;
  const long long c0 = (long long)blockIdx.z * A.chunk;
  const long long c1 = min(c0 + A.chunk, nvox);
  const int dx = tap % 3 - 1, dy = (tap / 3) % 3 - 1, dz = tap / 9 - 1;
  float acc[NT][4];
#pragma unroll
  for (int t = 0; t < NT; ++t)
#pragma unroll
    for (int q = 0; q < 4; ++q) acc[t][q] = 0.f;
  for (long long pb = c0 + warp * 16; pb < c1; pb += 64) {
    // A[m = k, kk = p]: rows k0+g, k0+g+8; cols p = pb + 2tq + {0,1}, +8
    uint32_t a[4];
    __nv_bfloat16 av[2][4];
    const __nv_bfloat16 zero = __float2bfloat16(0.f);
#pragma unroll
    for (int cq = 0; cq < 4; ++cq) {
      const long long p = pb + 2 * tq + (cq & 1) + ((cq >> 1) ? 8 : 0);
      bool ok = p < c1;
      const __nv_bfloat16* xr = nullptr;
      if (ok) {
        const int i = (int)(p % A.v.nx), j = (int)((p / A.v.nx) % A.v.ny), k = (int)(p / ((long long)A.v.nx * A.v.ny));
        bool ox, oy, oz;
        const int ii = wrapc(i + dx, A.v.nx, A.v.per[0], &ox);
        const int jj = wrapc(j + dy, A.v.ny, A.v.per[1], &oy);
        const int kk = wrapc(k + dz, A.v.nz, A.v.per[2], &oz);
        ok = ox && oy && oz;
        xr = A.x + (((long long)kk * A.v.ny + jj) * A.v.nx + ii) * A.xcs + A.xc0 + k0;
      }
      av[0][cq] = ok ? xr[g] : zero;
      av[1][cq] = ok ? xr[g + 8] : zero;
    }
    // pack: a0 (row g, cols 2tq..2tq+1), a1 (row g+8), a2 (row g, cols +8), a3 (row g+8, cols +8)
    __nv_bfloat162 t2;
    t2.x = av[0][0]; t2.y = av[0][1]; a[0] = *reinterpret_cast<uint32_t*>(&t2);
    t2.x = av[1][0]; t2.y = av[1][1]; a[1] = *reinterpret_cast<uint32_t*>(&t2);
    t2.x = av[0][2]; t2.y = av[0][3]; a[2] = *reinterpret_cast<uint32_t*>(&t2);
    t2.x = av[1][2]; t2.y = av[1][3]; a[3] = *reinterpret_cast<uint32_t*>(&t2);
    // B[kk = p][n]: rows p = pb + 2tq + {0,1} (b0), +8 (b1); col n = g
#pragma unroll
    for (int t = 0; t < NT; ++t) {
      const int n = t * 8 + g;
      uint32_t b[2];
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        __nv_bfloat162 bb;
        const long long p0 = pb + 2 * tq + 8 * h;
        bb.x = (p0 < c1 && n < A.N) ? A.dy[p0 * A.dycs + A.dyc0 + n] : zero;
        bb.y = (p0 + 1 < c1 && n < A.N) ? A.dy[(p0 + 1) * A.dycs + A.dyc0 + n] : zero;
        b[h] = *reinterpret_cast<uint32_t*>(&bb);
      }
      mma_bf16(acc[t], a, b);
    }
  }
  // reduce the 4 warps in shared memory, then one atomic add per element
  __shared__ float red[4][16][NT * 8];
#pragma unroll
  for (int t = 0; t < NT; ++t) {
    red[warp][g][t * 8 + 2 * tq] = acc[t][0];
    red[warp][g][t * 8 + 2 * tq + 1] = acc[t][1];
    red[warp][g + 8][t * 8 + 2 * tq] = acc[t][2];
    red[warp][g + 8][t * 8 + 2 * tq + 1] = acc[t][3];
  }
  __syncthreads();
  for (int e = threadIdx.x; e < 16 * NT * 8; e += blockDim.x) {
    const int m = e / (NT * 8), n = e % (NT * 8);
    if (n >= A.N || k0 + m >= A.K) continue;
    const float s = red[0][m][n] + red[1][m][n] + red[2][m][n] + red[3][m][n];
    atomicAdd(A.dw + ((long long)tap * A.K + k0 + m) * A.N + n, s);
  }
}

// bias gradient: db[n] += sum_p dY[p, n]
__global__ void k_bias_grad(const __nv_bfloat16* __restrict__ dy, int dycs, int dyc0, long long nvox, int N,
                            float* __restrict__ db) {
  const int n = blockIdx.y;
  float s = 0.f;
  for (long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x; p < nvox; p += (long long)gridDim.x * blockDim.x)
    s += __bfloat162float(dy[p * dycs + dyc0 + n]);
  s = warp_sum(s);
  __shared__ float sh[32];
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x < 32) {
    s = threadIdx.x < blockDim.x / 32 ? sh[threadIdx.x] : 0.f;
    s = warp_sum(s);
    if (threadIdx.x == 0) atomicAdd(db + n, s);
  }
}

// ---------------------------------------------------------------------------
// average pooling 2x2x2 and nearest upsampling x2 (and their adjoints)
// ---------------------------------------------------------------------------
__global__ void k_pool(const __nv_bfloat16* __restrict__ x, int xcs, int xc0, Vol vf, __nv_bfloat16* __restrict__ y,
                       int ycs, int yc0, Vol vc, int C) {
  pdl_enter();
  const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const long long nc = (long long)vc.nx * vc.ny * vc.nz * C;
  if (e >= nc) return;
  const int c = (int)(e % C);
  const long long P = e / C;
  const int I = (int)(P % vc.nx), J = (int)((P / vc.nx) % vc.ny), K = (int)(P / ((long long)vc.nx * vc.ny));
  float s = 0.f;
  for (int d = 0; d < 8; ++d) {
    const int i = 2 * I + (d & 1), j = 2 * J + ((d >> 1) & 1), k = 2 * K + (d >> 2);
    s += __bfloat162float(x[(((long long)k * vf.ny + j) * vf.nx + i) * xcs + xc0 + c]);
  }
  y[P * ycs + yc0 + c] = __float2bfloat16(0.125f * s);
}

// dX (fine) = dY (coarse) / 8 on each child
__global__ void k_pool_back(const __nv_bfloat16* __restrict__ dy, int dycs, int dyc0, Vol vc,
                            __nv_bfloat16* __restrict__ dx, int dxcs, int dxc0, Vol vf, int C, int accumulate) {
  const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const long long nf = (long long)vf.nx * vf.ny * vf.nz * C;
  if (e >= nf) return;
  const int c = (int)(e % C);
  const long long p = e / C;
  const int i = (int)(p % vf.nx), j = (int)((p / vf.nx) % vf.ny), k = (int)(p / ((long long)vf.nx * vf.ny));
  const long long P = ((long long)(k >> 1) * vc.ny + (j >> 1)) * vc.nx + (i >> 1);
  float v = 0.125f * __bfloat162float(dy[P * dycs + dyc0 + c]);
  if (accumulate) v += __bfloat162float(dx[p * dxcs + dxc0 + c]);
  dx[p * dxcs + dxc0 + c] = __float2bfloat16(v);
}

// nearest upsampling: Y[p] = X[p / 2]
__global__ void k_upsample(const __nv_bfloat16* __restrict__ x, int xcs, int xc0, Vol vc,
                           __nv_bfloat16* __restrict__ y, int ycs, int yc0, Vol vf, int C) {
  pdl_enter();
  const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const long long nf = (long long)vf.nx * vf.ny * vf.nz * C;
  if (e >= nf) return;
  const int c = (int)(e % C);
  const long long p = e / C;
  const int i = (int)(p % vf.nx), j = (int)((p / vf.nx) % vf.ny), k = (int)(p / ((long long)vf.nx * vf.ny));
  const long long P = ((long long)(k >> 1) * vc.ny + (j >> 1)) * vc.nx + (i >> 1);
  y[p * ycs + yc0 + c] = x[P * xcs + xc0 + c];
}

// adjoint of nearest upsampling: dX[P] = sum of the 8 children of dY
__global__ void k_upsample_back(const __nv_bfloat16* __restrict__ dy, int dycs, int dyc0, Vol vf,
                                __nv_bfloat16* __restrict__ dx, int dxcs, int dxc0, Vol vc, int C,
                                const __nv_bfloat16* __restrict__ mask, int mcs, int mc0) {
  const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const long long nc = (long long)vc.nx * vc.ny * vc.nz * C;
  if (e >= nc) return;
  const int c = (int)(e % C);
  const long long P = e / C;
  const int I = (int)(P % vc.nx), J = (int)((P / vc.nx) % vc.ny), K = (int)(P / ((long long)vc.nx * vc.ny));
  float s = 0.f;
  for (int d = 0; d < 8; ++d) {
    const int i = 2 * I + (d & 1), j = 2 * J + ((d >> 1) & 1), k = 2 * K + (d >> 2);
    s += __bfloat162float(dy[(((long long)k * vf.ny + j) * vf.nx + i) * dycs + dyc0 + c]);
  }
  if (mask && !(__bfloat162float(mask[P * mcs + mc0 + c]) > 0.f)) s = 0.f;
  dx[P * dxcs + dxc0 + c] = __float2bfloat16(s);
}

// ---------------------------------------------------------------------------
// 1x1 head (FP32 out): out[p] = sum_c wh[c] X[p, c] + bh
// ---------------------------------------------------------------------------
__global__ void k_head(const __nv_bfloat16* __restrict__ x, int xcs, int C, long long nvox, const float* __restrict__ wh,
                       const float* __restrict__ bh, float* __restrict__ out) {
  pdl_enter();
  const long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= nvox) return;
  float s = bh[0];
  for (int c = 0; c < C; ++c) s += wh[c] * __bfloat162float(x[p * xcs + c]);
  out[p] = s;
}

// loss = mean (out - tgt)^2; dout = 2 (out - tgt) / n; loss partial sums per block
__global__ void k_mse(const float* __restrict__ out, const float* __restrict__ tgt, long long n, float* __restrict__ dout,
                      float* __restrict__ loss) {
  const long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  float d = 0.f;
  if (p < n) {
    d = out[p] - tgt[p];
    dout[p] = 2.f * d / (float)n;
  }
  float s = warp_sum(d * d);
  __shared__ float sh[32];
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x < 32) {
    s = threadIdx.x < blockDim.x / 32 ? sh[threadIdx.x] : 0.f;
    s = warp_sum(s);
    if (threadIdx.x == 0) atomicAdd(loss, s / (float)n);
  }
}

// head backward: dX[p, c] = dout[p] wh[c] (masked by ReLU of X); dwh, dbh by atomics
__global__ void k_head_back(const __nv_bfloat16* __restrict__ x, int xcs, int C, long long nvox,
                            const float* __restrict__ wh, const float* __restrict__ dout,
                            __nv_bfloat16* __restrict__ dx, float* __restrict__ dwh, float* __restrict__ dbh) {
  const long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  __shared__ float sw[64];
  __shared__ float sb;
  if (threadIdx.x < 64) sw[threadIdx.x] = 0.f;
  if (threadIdx.x == 0) sb = 0.f;
  __syncthreads();
  if (p < nvox) {
    const float g = dout[p];
    atomicAdd(&sb, g);
    for (int c = 0; c < C; ++c) {
      const float xv = __bfloat162float(x[p * xcs + c]);
      atomicAdd(&sw[c], g * xv);
      dx[p * xcs + c] = __float2bfloat16(xv > 0.f ? g * wh[c] : 0.f);
    }
  }
  __syncthreads();
  if (threadIdx.x < C) atomicAdd(dwh + threadIdx.x, sw[threadIdx.x]);
  if (threadIdx.x == 0) atomicAdd(dbh, sb);
}

// ---------------------------------------------------------------------------
// weights: FP32 master [27][K][N] -> BF16 forward copy [27][N][K] and
// data-gradient copy [27][K][N] with the taps mirrored (o_{26-t} = -o_t)
// ---------------------------------------------------------------------------
__global__ void k_pack_weights(const float* __restrict__ w, int K, int N, __nv_bfloat16* __restrict__ wf,
                               __nv_bfloat16* __restrict__ wb) {
  const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const long long tot = 27LL * K * N;
  if (e >= tot) return;
  const int n = (int)(e % N);
  const int k = (int)((e / N) % K);
  const int t = (int)(e / ((long long)K * N));
  const __nv_bfloat16 v = __float2bfloat16(w[e]);
  wf[((long long)t * N + n) * K + k] = v;
  wb[((long long)(26 - t) * K + k) * N + n] = v;
}

// Adam (decoupled from the layer structure: one flat parameter vector)
__global__ void k_adam(float* __restrict__ w, const float* __restrict__ g, float* __restrict__ m, float* __restrict__ v,
                       long long n, float lr, float b1, float b2, float eps, float c1, float c2) {
  const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= n) return;
  const float gi = g[e];
  const float mi = b1 * m[e] + (1.f - b1) * gi;
  const float vi = b2 * v[e] + (1.f - b2) * gi * gi;
  m[e] = mi;
  v[e] = vi;
  w[e] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
}

// FP32 (n, ny, nz) x `nch` inputs -> BF16 channels-last, padded to cs channels with zeros
__global__ void k_pack_input(const float* __restrict__ in, int nch, long long nvox, __nv_bfloat16* __restrict__ x, int cs) {
  pdl_enter();
  const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= nvox * cs) return;
  const int c = (int)(e % cs);
  const long long p = e / cs;
  x[e] = __float2bfloat16(c < nch ? in[(long long)c * nvox + p] : 0.f);
}

// ---------------------------------------------------------------------------
// The same convolution on the fifth-generation tensor cores: one CTA of 4
// warps computes 128 voxels x all N output channels as a chain of
// tcgen05.mma (kind::f16, BF16 operands, M = 128, N, K = 16 per instruction)
// accumulating in tensor memory (TMEM, 128 lanes x N FP32 columns).  Each
// K-step is one (tap, 16-channel) pair: its A tile (the 128 voxels' shifted
// input rows, zeros outside the volume) and B tile (W[tap][n][k0..k0+15])
// are gathered by cp.async into one of TC_STAGES shared-memory stages in the
// canonical K-major layout without swizzle (8-row x 16-byte core matrices,
// the two K halves 128 B apart, row groups 256 B apart).  Thread 0 issues
// the MMA of a stage once all threads' copies landed (cp.async.wait_group,
// fence.proxy.async, barrier) and commits it to the stage's mbarrier; a
// stage is refilled after that mbarrier fired.  The epilogue reads the
// accumulator back with tcgen05.ld (warp w: lanes 32w .. 32w + 31, its
// voxels) and applies conv_epilogue, or stores the FP32 partial of a split
// slice as k_conv3 does.  Every mbarrier wait is bounded (about a second
// of clock); a wait that runs out sets g_tc_timeout and the CTA finishes
// without further waits.
// ---------------------------------------------------------------------------
// TC_STAGES stages, copies started TC_LA steps ahead: a stage is refilled
// TC_STAGES - TC_LA steps after the MMA that read it was issued, so the
// wait for that MMA rarely stalls (with 4 stages and 3 ahead every step
// waited for the previous step's MMA)
constexpr int TC_M = 128, TC_THREADS = 128, TC_STAGES = 8, TC_LA = 4;
constexpr int TC_A_BYTES = TC_M * 32;  // 128 rows x 16 BF16

__device__ int g_tc_timeout;

__device__ __forceinline__ uint32_t tc_smem(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }
// byte offset of row r, K half h (BF16 k 0..7 or 8..15) in a K-major tile
__device__ __forceinline__ uint32_t tc_off(int r, int h) {
  return (uint32_t)(((r >> 3) * 2 + h) * 128 + (r & 7) * 16);
}
// shared-memory matrix descriptor: start address, leading byte offset (K
// direction) 128, stride byte offset (row groups) 256, descriptor version 1,
// no swizzle
__device__ __forceinline__ uint64_t tc_desc(uint32_t saddr) {
  return (uint64_t)((saddr >> 4) & 0x3fffu) | ((uint64_t)(128u >> 4) << 16) | ((uint64_t)(256u >> 4) << 32) |
         ((uint64_t)1 << 46);
}
// instruction descriptor of kind::f16: FP32 accumulator, BF16 A and B, both
// K-major, N >> 3 and M >> 4
__device__ __forceinline__ uint32_t tc_idesc(int n) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(TC_M >> 4) << 24);
}
__device__ __forceinline__ void tc_cp16(uint32_t dst, const void* src, bool ok) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(dst), "l"(src), "r"(ok ? 16 : 0) : "memory");
}
__device__ __forceinline__ void tc_mbar_init(uint32_t a) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(a) : "memory");
}
// waits for the completion of the phase of parity `par`; false after about
// 2^31 clocks without it
__device__ __forceinline__ bool tc_mbar_wait(uint32_t a, uint32_t par) {
  const long long t0 = clock64();
  for (;;) {
    uint32_t done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(a), "r"(par)
        : "memory");
    if (done) return true;
    if (clock64() - t0 > (1LL << 31)) return false;
  }
}
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory"); }
__device__ __forceinline__ void tc_mma(uint32_t tmem, uint64_t ad, uint64_t bd, uint32_t idesc, int accum) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.u32 p, %4, 0;\n tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(
          tmem),
      "l"(ad), "l"(bd), "r"(idesc), "r"(accum)
      : "memory");
}
__device__ __forceinline__ void tc_commit(uint32_t mbar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(mbar) : "memory");
}
// 16 consecutive FP32 columns of the warp's 32 TMEM lanes (one lane per thread)
__device__ __forceinline__ void tc_ld16(uint32_t taddr, float (&v)[16]) {
  uint32_t r[16];
  asm volatile("tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];\n"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
               : "r"(taddr)
               : "memory");
  asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
#pragma unroll
  for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

__global__ void __launch_bounds__(TC_THREADS) k_conv3_tc(ConvArgs A, int ncols) {
  pdl_enter();
  extern __shared__ __align__(128) unsigned char tc_sm[];
  const int t = threadIdx.x, warp = t >> 5;
  const int N = A.N;
  const int stage_bytes = TC_A_BYTES + N * 32;
  const uint32_t sbase = tc_smem(tc_sm);
  const uint32_t mbar0 = sbase + TC_STAGES * stage_bytes;  // TC_STAGES mbarriers, 8 B each
  volatile uint32_t* tslot = reinterpret_cast<volatile uint32_t*>(tc_sm + TC_STAGES * stage_bytes + 8 * TC_STAGES);
  const long long nvox = (long long)A.v.nx * A.v.ny * A.v.nz;
  const long long p = (long long)blockIdx.x * TC_M + t;  // this thread's voxel row
  const bool live = p < nvox;
  const long long pc = live ? p : 0;
  const int ci = (int)(pc % A.v.nx), cj = (int)((pc / A.v.nx) % A.v.ny), ck = (int)(pc / ((long long)A.v.nx * A.v.ny));
  const int kpt = A.K / 16, nq = 27 * kpt, S = gridDim.z;
  const int q0 = (int)((long long)nq * blockIdx.z / S), q1 = (int)((long long)nq * (blockIdx.z + 1) / S);
  const int nsteps = q1 - q0;

  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(
                     tc_smem((const void*)tslot)),
                 "r"(ncols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::: "memory");
  }
  if (t == 0) {
    for (int s = 0; s < TC_STAGES; ++s) tc_mbar_init(mbar0 + 8 * s);
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tslot;
  const uint32_t idesc = tc_idesc(N);

  auto load = [&](int q, int st) {
    const int tap = q / kpt, k0 = (q - tap * kpt) * 16;
    bool ox, oy, oz;
    const int ii = wrapc(ci + tap % 3 - 1, A.v.nx, A.v.per[0], &ox);
    const int jj = wrapc(cj + (tap / 3) % 3 - 1, A.v.ny, A.v.per[1], &oy);
    const int kk = wrapc(ck + tap / 9 - 1, A.v.nz, A.v.per[2], &oz);
    const bool ok = live && ox && oy && oz;
    const __nv_bfloat16* row = A.x + (((long long)kk * A.v.ny + jj) * A.v.nx + ii) * A.xcs + A.xc0 + k0;
    const uint32_t a = sbase + st * stage_bytes;
    tc_cp16(a + tc_off(t, 0), ok ? (const void*)row : (const void*)A.x, ok);
    tc_cp16(a + tc_off(t, 1), ok ? (const void*)(row + 8) : (const void*)A.x, ok);
    const uint32_t b = a + TC_A_BYTES;
    const __nv_bfloat16* wt = A.w + (long long)tap * N * A.K + k0;
    for (int c = t; c < 2 * N; c += TC_THREADS) {
      const int n = c >> 1, h = c & 1;
      tc_cp16(b + tc_off(n, h), wt + (long long)n * A.K + 8 * h, true);
    }
  };

  bool ok_all = true;
#pragma unroll 1
  for (int i = 0; i < TC_LA; ++i) {
    if (i < nsteps) load(q0 + i, i);
    cp_async_commit();
  }
#pragma unroll 1
  for (int i = 0; i < nsteps; ++i) {
    const int st = i % TC_STAGES;
    const int nx = i + TC_LA;  // the step whose copies start now
    if (nx < nsteps) {
      const int sn = nx % TC_STAGES;
      // its stage was last read by the MMA of step nx - TC_STAGES
      if (nx >= TC_STAGES && ok_all) ok_all = tc_mbar_wait(mbar0 + 8 * sn, (uint32_t)((nx / TC_STAGES - 1) & 1));
      load(q0 + nx, sn);
    }
    cp_async_commit();
    cp_async_wait<TC_LA>();  // step i's copies landed
    asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
    ok_all = __syncthreads_and(ok_all) != 0;  // one verdict for the CTA: after a timeout nobody waits again
    if (t == 0 && ok_all) {
      tc_fence_after();
      const uint32_t a = sbase + st * stage_bytes;
      tc_mma(tmem, tc_desc(a), tc_desc(a + TC_A_BYTES), idesc, i > 0 ? 1 : 0);
      tc_commit(mbar0 + 8 * st);
    }
  }
  cp_async_wait<0>();
  // every thread waits for the last MMA (its commit covers all earlier ones)
  if (nsteps > 0 && ok_all) {
    const int st = (nsteps - 1) % TC_STAGES;
    ok_all = tc_mbar_wait(mbar0 + 8 * st, (uint32_t)(((nsteps - 1) / TC_STAGES) & 1));
  }
  ok_all = __syncthreads_and(ok_all) != 0;
  tc_fence_after();
  if (!ok_all) atomicExch(&g_tc_timeout, 1);
  if (nsteps > 0 && ok_all) {
    const uint32_t lane_base = tmem + ((uint32_t)(32 * warp) << 16);
    for (int c0 = 0; c0 < N; c0 += 16) {
      float v[16];
      tc_ld16(lane_base + (uint32_t)c0, v);
      if (live) {
#pragma unroll
        for (int j = 0; j < 16; j += 2) {
          const int n = c0 + j;
          if (S == 1) {
            conv_epilogue(A, p, n, v[j], v[j + 1]);
          } else {
            *reinterpret_cast<float2*>(A.ws + ((long long)blockIdx.z * nvox + p) * N + n) = make_float2(v[j], v[j + 1]);
          }
        }
      }
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem), "r"(ncols) : "memory");
}

// ---------------------------------------------------------------------------
// launchers
// ---------------------------------------------------------------------------
// blocks of a convolution before splitting: 64 voxels x (16 or 32) channels
static long long conv_tiles(long long nvox, int N) {
  return ((nvox + 63) / 64) * (N <= 16 ? (N + 15) / 16 : (N + 31) / 32);
}

int conv_splits(long long nvox, int K, int N) {
  const long long tiles = conv_tiles(nvox, N);
  const int nq = 27 * (K / 16);
  const long long want = (2LL * 152 + tiles - 1) / tiles;  // two waves of blocks on 152 SMs
  long long S = want < nq / 4 ? want : nq / 4;             // at least 4 channel steps per slice
  if (S > 27) S = 27;
  return S < 1 ? 1 : (int)S;
}

// the tensor-core kernel takes 16-byte aligned rows (channel stride and
// offset multiples of 8) and N a multiple of 16 up to 256
static bool conv_tc_ok(const ConvArgs& a) {
  return a.xcs % 8 == 0 && a.xc0 % 8 == 0 && a.K % 16 == 0 && a.N % 16 == 0 && a.N >= 16 && a.N <= 256 &&
         ((uintptr_t)a.x % 16) == 0 && ((uintptr_t)a.w % 16) == 0;
}
static int conv_tc_splits(long long nvox, int K) {
  const long long tiles = (nvox + TC_M - 1) / TC_M;
  const int nq = 27 * (K / 16);
  const long long want = (2LL * 152 + tiles - 1) / tiles;  // two CTAs per SM
  long long S = want < nq / 4 ? want : nq / 4;             // at least 4 K-steps per slice
  if (S > 27) S = 27;
  return S < 1 ? 1 : (int)S;
}

// whether a tensor-core convolution gave up on a wait since the last call
// (the flag is cleared); call with no kernel of the network in flight
int conv_tc_timed_out() {
  int v = 0;
  if (cudaMemcpyFromSymbol(&v, g_tc_timeout, sizeof v) != cudaSuccess) return -1;
  if (v) {
    const int z = 0;
    cudaMemcpyToSymbol(g_tc_timeout, &z, sizeof z);
  }
  return v;
}

int launch_conv3(const ConvArgs& a, cudaStream_t s) {
  const long long nvox = (long long)a.v.nx * a.v.ny * a.v.nz;
  if (conv_tc_ok(a)) {
    int S = a.ws ? conv_tc_splits(nvox, a.K) : 1;
    while (S > 1 && (long long)S * nvox * a.N > a.ws_cap) --S;
    int ncols = 32;
    while (ncols < a.N) ncols *= 2;
    const size_t smem = (size_t)TC_STAGES * (TC_A_BYTES + a.N * 32) + 8 * TC_STAGES + 16;
    // the shared-memory opt-in belongs to the current device: set it per device
    static std::atomic<bool> attr_done[64];
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) dev = -1;
    if (!(dev >= 0 && dev < 64 && attr_done[dev].load())) {
      if (cudaFuncSetAttribute(k_conv3_tc, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               (int)((size_t)TC_STAGES * (TC_A_BYTES + 256 * 32) + 8 * TC_STAGES + 16)) ==
              cudaSuccess &&
          dev >= 0 && dev < 64)
        attr_done[dev].store(true);
    }
    launch_pdl(k_conv3_tc, dim3((unsigned)((nvox + TC_M - 1) / TC_M), 1, S), TC_THREADS, smem, s, a, ncols);
    if (S > 1) launch_pdl(k_conv3_reduce, (unsigned)((nvox * (a.N / 2) + 255) / 256), 256, 0, s, a, S);
    return S > 1 ? 2 : 1;
  }
  const unsigned gx = (unsigned)((nvox + 63) / 64);
  int S = a.ws ? conv_splits(nvox, a.K, a.N) : 1;
  while (S > 1 && (long long)S * nvox * a.N > a.ws_cap) --S;
  if (a.N <= 16) {
    launch_pdl(k_conv3<2>, dim3(gx, (a.N + 15) / 16, S), 128, 0, s, a);
  } else {
    launch_pdl(k_conv3<4>, dim3(gx, (a.N + 31) / 32, S), 128, 0, s, a);
  }
  if (S > 1) launch_pdl(k_conv3_reduce, (unsigned)((nvox * (a.N / 2) + 255) / 256), 256, 0, s, a, S);
  return S > 1 ? 2 : 1;
}

void launch_wgrad(const WgradArgs& a0, cudaStream_t s) {
  WgradArgs a = a0;
  const long long nvox = (long long)a.v.nx * a.v.ny * a.v.nz;
  if (a.chunk <= 0) a.chunk = 4096;
  const unsigned gz = (unsigned)((nvox + a.chunk - 1) / a.chunk);
  const dim3 grid(27, (a.K + 15) / 16, gz);
  if (a.N <= 16) k_conv3_wgrad<2><<<grid, 128, 0, s>>>(a);
  else if (a.N <= 32) k_conv3_wgrad<4><<<grid, 128, 0, s>>>(a);
  else if (a.N <= 64) k_conv3_wgrad<8><<<grid, 128, 0, s>>>(a);
  else k_conv3_wgrad<16><<<grid, 128, 0, s>>>(a);
}

void launch_bias_grad(const __nv_bfloat16* dy, int dycs, int dyc0, long long nvox, int N, float* db, cudaStream_t s) {
  const long long nbx = (nvox + 255) / 256;
  const unsigned gx = (unsigned)(nbx < 256 ? nbx : 256);
  k_bias_grad<<<dim3(gx, N), 256, 0, s>>>(dy, dycs, dyc0, nvox, N, db);
}

static inline unsigned nb256(long long n) { return (unsigned)((n + 255) / 256); }

void launch_pool(const __nv_bfloat16* x, int xcs, int xc0, const Vol& vf, __nv_bfloat16* y, int ycs, int yc0,
                 const Vol& vc, int C, cudaStream_t s) {
  launch_pdl(k_pool, nb256((long long)vc.nx * vc.ny * vc.nz * C), 256, 0, s, x, xcs, xc0, vf, y, ycs, yc0, vc, C);
}
void launch_pool_back(const __nv_bfloat16* dy, int dycs, int dyc0, const Vol& vc, __nv_bfloat16* dx, int dxcs,
                      int dxc0, const Vol& vf, int C, int accumulate, cudaStream_t s) {
  k_pool_back<<<nb256((long long)vf.nx * vf.ny * vf.nz * C), 256, 0, s>>>(dy, dycs, dyc0, vc, dx, dxcs, dxc0, vf, C,
                                                                             accumulate);
}
void launch_upsample(const __nv_bfloat16* x, int xcs, int xc0, const Vol& vc, __nv_bfloat16* y, int ycs, int yc0,
                     const Vol& vf, int C, cudaStream_t s) {
  launch_pdl(k_upsample, nb256((long long)vf.nx * vf.ny * vf.nz * C), 256, 0, s, x, xcs, xc0, vc, y, ycs, yc0, vf, C);
}
void launch_upsample_back(const __nv_bfloat16* dy, int dycs, int dyc0, const Vol& vf, __nv_bfloat16* dx, int dxcs,
                          int dxc0, const Vol& vc, int C, const __nv_bfloat16* mask, int mcs, int mc0,
                          cudaStream_t s) {
  k_upsample_back<<<nb256((long long)vc.nx * vc.ny * vc.nz * C), 256, 0, s>>>(dy, dycs, dyc0, vf, dx, dxcs, dxc0, vc,
                                                                                C, mask, mcs, mc0);
}
void launch_head(const __nv_bfloat16* x, int xcs, int C, long long nvox, const float* wh, const float* bh, float* out,
                 cudaStream_t s) {
  launch_pdl(k_head, nb256(nvox), 256, 0, s, x, xcs, C, nvox, wh, bh, out);
}
void launch_head_back(const __nv_bfloat16* x, int xcs, int C, long long nvox, const float* wh, const float* dout,
                      __nv_bfloat16* dx, float* dwh, float* dbh, cudaStream_t s) {
  k_head_back<<<nb256(nvox), 256, 0, s>>>(x, xcs, C, nvox, wh, dout, dx, dwh, dbh);
}
void launch_mse(const float* out, const float* tgt, long long n, float* dout, float* loss, cudaStream_t s) {
  k_mse<<<nb256(n), 256, 0, s>>>(out, tgt, n, dout, loss);
}
void launch_pack_weights(const float* w, int K, int N, __nv_bfloat16* wf, __nv_bfloat16* wb, cudaStream_t s) {
  k_pack_weights<<<nb256(27LL * K * N), 256, 0, s>>>(w, K, N, wf, wb);
}
void launch_adam(float* w, const float* g, float* m, float* v, long long n, float lr, float b1, float b2, float eps,
                 float c1, float c2, cudaStream_t s) {
  k_adam<<<nb256(n), 256, 0, s>>>(w, g, m, v, n, lr, b1, b2, eps, c1, c2);
}
void launch_pack_input(const float* in, int nch, long long nvox, __nv_bfloat16* x, int cs, cudaStream_t s) {
  launch_pdl(k_pack_input, nb256(nvox * cs), 256, 0, s, in, nch, nvox, x, cs);
}

}  // namespace o3d

namespace o3d {
// d *= (m > 0): ReLU mask on a channel slice
__global__ void k_mask(__nv_bfloat16* __restrict__ d, int dcs, int dc0, const __nv_bfloat16* __restrict__ m, int mcs,
                       int mc0, long long nvox, int C) {
  const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= nvox * C) return;
  const int c = (int)(e % C);
  const long long p = e / C;
  if (!(__bfloat162float(m[p * mcs + mc0 + c]) > 0.f)) d[p * dcs + dc0 + c] = __float2bfloat16(0.f);
}
void launch_mask(__nv_bfloat16* d, int dcs, int dc0, const __nv_bfloat16* m, int mcs, int mc0, long long nvox, int C,
                 cudaStream_t s) {
  k_mask<<<(unsigned)((nvox * C + 255) / 256), 256, 0, s>>>(d, dcs, dc0, m, mcs, mc0, nvox, C);
}
}  // namespace o3d
