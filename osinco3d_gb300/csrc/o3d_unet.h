// o3d_unet.h -- argument blocks and launchers of the learned warm start.
#pragma once

#include <cuda_bf16.h>
#include <cuda_runtime.h>

namespace o3d {

// A 3D grid of voxels; per axis, neighbours past the end wrap (per = 1) or read zero.
struct Vol {
  int nx, ny, nz;
  int per[3];
};

struct ConvArgs {
  const __nv_bfloat16* x;   // input tensor
  int xcs, xc0;             // its channel stride and offset
  const __nv_bfloat16* w;   // BF16 [27][N][K]
  const float* bias;        // N or nullptr
  __nv_bfloat16* y;         // output tensor
  int ycs, yc0;
  const __nv_bfloat16* mask;  // zero the output where mask <= 0 (ReLU backward), or nullptr
  int mcs, mc0;
  Vol v;
  int K, N;                 // input / output channels (K multiple of 16, N even)
  int relu;
  int accumulate;           // add to the existing output
  float* ws;                // FP32 split-K partials (ws_cap floats), or nullptr
  long long ws_cap;
};

struct WgradArgs {
  const __nv_bfloat16* x;   // layer input
  int xcs, xc0;
  const __nv_bfloat16* dy;  // gradient at the layer's pre-activation output
  int dycs, dyc0;
  float* dw;                // FP32 [27][K][N], accumulated
  Vol v;
  int K, N;
  long long chunk;          // voxels per block
};

// Number of slices the (tap, channel) reduction of a convolution over nvox
// voxels with K inputs and N outputs is split into: 1 on grids that fill the
// GPU, up to 27 * K / 64 on the small grids of the deep levels.
int conv_splits(long long nvox, int K, int N);
int launch_conv3(const ConvArgs& a, cudaStream_t s);  // returns the kernels launched
// 1 if a tensor-core convolution gave up on a bounded wait since the last
// call (then its output is not valid), 0 if not, -1 if the flag is unreadable
int conv_tc_timed_out();
void launch_wgrad(const WgradArgs& a, cudaStream_t s);
void launch_bias_grad(const __nv_bfloat16* dy, int dycs, int dyc0, long long nvox, int N, float* db, cudaStream_t s);
void launch_pool(const __nv_bfloat16* x, int xcs, int xc0, const Vol& vf, __nv_bfloat16* y, int ycs, int yc0,
                 const Vol& vc, int C, cudaStream_t s);
void launch_pool_back(const __nv_bfloat16* dy, int dycs, int dyc0, const Vol& vc, __nv_bfloat16* dx, int dxcs,
                      int dxc0, const Vol& vf, int C, int accumulate, cudaStream_t s);
void launch_upsample(const __nv_bfloat16* x, int xcs, int xc0, const Vol& vc, __nv_bfloat16* y, int ycs, int yc0,
                     const Vol& vf, int C, cudaStream_t s);
void launch_upsample_back(const __nv_bfloat16* dy, int dycs, int dyc0, const Vol& vf, __nv_bfloat16* dx, int dxcs,
                          int dxc0, const Vol& vc, int C, const __nv_bfloat16* mask, int mcs, int mc0,
                          cudaStream_t s);
void launch_head(const __nv_bfloat16* x, int xcs, int C, long long nvox, const float* wh, const float* bh, float* out,
                 cudaStream_t s);
void launch_head_back(const __nv_bfloat16* x, int xcs, int C, long long nvox, const float* wh, const float* dout,
                      __nv_bfloat16* dx, float* dwh, float* dbh, cudaStream_t s);
void launch_mse(const float* out, const float* tgt, long long n, float* dout, float* loss, cudaStream_t s);
void launch_pack_weights(const float* w, int K, int N, __nv_bfloat16* wf, __nv_bfloat16* wb, cudaStream_t s);
void launch_adam(float* w, const float* g, float* m, float* v, long long n, float lr, float b1, float b2, float eps,
                 float c1, float c2, cudaStream_t s);
void launch_pack_input(const float* in, int nch, long long nvox, __nv_bfloat16* x, int cs, cudaStream_t s);
void launch_mask(__nv_bfloat16* d, int dcs, int dc0, const __nv_bfloat16* m, int mcs, int mc0, long long nvox, int C,
                 cudaStream_t s);

}  // namespace o3d
