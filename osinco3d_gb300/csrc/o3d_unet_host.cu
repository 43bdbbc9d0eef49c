// o3d_unet_host.cu -- the 3D U-Net of the learned Poisson warm start:
// parameters, activations, forward pass, backward pass, Adam, and the C ABI
// (o3d_unet_*).
//
// Architecture (L levels, base width c): level l works at resolution n/2^l
// with C_l = c 2^l channels.  Encoder: two 3x3x3 conv+ReLU per level, 2x2x2
// average pooling between levels.  Decoder: nearest upsampling x2, channel
// concatenation with the encoder output of the level (the concat buffer is
// written in place by both producers), two 3x3x3 conv+ReLU.  Head: 1x1 conv
// to one FP32 channel.  BF16 weights and activations, FP32 accumulation,
// FP32 master weights and Adam moments.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <new>
#include <random>
#include <vector>

#include "o3d_internal.cuh"
#include "o3d_kernels.h"
#include "o3d_unet.h"

namespace o3d {

struct ConvLayer {
  int K, N;                 // input (padded to 16) / output channels
  long long w_off, b_off;   // offsets in the flat parameter vector
  __nv_bfloat16* wf;        // [27][N][K]
  __nv_bfloat16* wb;        // [27][K][N], taps mirrored (data gradient)
};

struct Tensor {
  __nv_bfloat16* p = nullptr;
  int cs = 0, c0 = 0, C = 0;
  Vol v;
};

struct UNet {
  int levels, base, in_ch;
  Vol vol[8];
  std::vector<ConvLayer> enc_a, enc_b, dec_a, dec_b;
  long long head_w, head_b, nparam;
  float *w = nullptr, *g = nullptr, *m = nullptr, *v = nullptr;  // FP32 parameters, gradients, Adam moments
  long long step = 0;
  // activations
  Tensor xin;                         // packed input, 16 channels
  std::vector<Tensor> ea, cat, pool, da, d, dbot;
  // gradients
  std::vector<Tensor> g_ea, g_cat, g_pool, g_da, g_d;
  float* out = nullptr;               // head output (FP32)
  float* dout = nullptr;
  float* loss = nullptr;
  float* ws = nullptr;                // split-K partials of the convolutions
  long long ws_cap = 0;
  cudaStream_t s = nullptr;
  cudaEvent_t ev = nullptr;           // orders the forward pass after / before a caller's stream
  cudaGraphExec_t fwd_exec = nullptr; // the forward pass as one graph (inference)
  long long launches = 0;             // kernels launched by forward/backward so far
  std::vector<void*> allocs;
};

static int ch(const UNet& u, int l) { return u.base << l; }

static int ualloc(UNet& u, void** p, size_t bytes) {
  if (cudaMalloc(p, bytes) != cudaSuccess) {
    cudaGetLastError();
    set_error("cudaMalloc of %zu bytes for the U-Net failed", bytes);
    return O3D_ERR_NOMEM;
  }
  u.allocs.push_back(*p);
  if (cudaMemsetAsync(*p, 0, bytes, u.s) != cudaSuccess) return O3D_ERR_CUDA;
  return O3D_OK;
}

static long long nvox(const Vol& v) { return (long long)v.nx * v.ny * v.nz; }

static int tensor(UNet& u, Tensor* t, const Vol& v, int C) {
  t->v = v;
  t->cs = C;
  t->c0 = 0;
  t->C = C;
  return ualloc(u, (void**)&t->p, (size_t)nvox(v) * C * sizeof(__nv_bfloat16));
}

static Tensor slice(const Tensor& t, int c0, int C) {
  Tensor r = t;
  r.c0 = t.c0 + c0;
  r.C = C;
  return r;
}

static void add_layer(UNet& u, std::vector<ConvLayer>& list, int K, int N, long long* off) {
  ConvLayer L;
  L.K = K;
  L.N = N;
  L.w_off = *off;
  *off += 27LL * K * N;
  L.b_off = *off;
  *off += N;
  L.wf = L.wb = nullptr;
  list.push_back(L);
}

static void conv(UNet& u, const ConvLayer& L, const Tensor& x, const Tensor& y, bool relu) {
  ConvArgs a;
  a.x = x.p; a.xcs = x.cs; a.xc0 = x.c0;
  a.w = L.wf;
  a.bias = u.w + L.b_off;
  a.y = y.p; a.ycs = y.cs; a.yc0 = y.c0;
  a.mask = nullptr; a.mcs = 0; a.mc0 = 0;
  a.v = x.v;
  a.K = L.K; a.N = L.N;
  a.relu = relu;
  a.accumulate = 0;
  a.ws = u.ws;
  a.ws_cap = u.ws_cap;
  u.launches += launch_conv3(a, u.s);
}

// dX = conv(dY, mirrored W^T), masked by (mask > 0) when given
static void conv_dgrad(UNet& u, const ConvLayer& L, const Tensor& dy, const Tensor& dx, const Tensor* mask) {
  ConvArgs a;
  a.x = dy.p; a.xcs = dy.cs; a.xc0 = dy.c0;
  a.w = L.wb;
  a.bias = nullptr;
  a.y = dx.p; a.ycs = dx.cs; a.yc0 = dx.c0;
  a.mask = mask ? mask->p : nullptr;
  a.mcs = mask ? mask->cs : 0;
  a.mc0 = mask ? mask->c0 : 0;
  a.v = dy.v;
  a.K = L.N; a.N = L.K;
  a.relu = 0;
  a.accumulate = 0;
  a.ws = u.ws;
  a.ws_cap = u.ws_cap;
  u.launches += launch_conv3(a, u.s);
}

static void conv_wgrad(UNet& u, const ConvLayer& L, const Tensor& x, const Tensor& dy) {
  WgradArgs a;
  a.x = x.p; a.xcs = x.cs; a.xc0 = x.c0;
  a.dy = dy.p; a.dycs = dy.cs; a.dyc0 = dy.c0;
  a.dw = u.g + L.w_off;
  a.v = x.v;
  a.K = L.K; a.N = L.N;
  a.chunk = 4096;
  launch_wgrad(a, u.s);
  launch_bias_grad(dy.p, dy.cs, dy.c0, nvox(dy.v), L.N, u.g + L.b_off, u.s);
}

static void pack_all(UNet& u) {
  auto pack = [&](std::vector<ConvLayer>& list) {
    for (auto& L : list) launch_pack_weights(u.w + L.w_off, L.K, L.N, L.wf, L.wb, u.s);
  };
  pack(u.enc_a); pack(u.enc_b); pack(u.dec_a); pack(u.dec_b);
}

static void forward(UNet& u) {
  const int Lv = u.levels;
  for (int l = 0; l < Lv; ++l) {
    const Tensor& in = l == 0 ? u.xin : u.pool[l];
    conv(u, u.enc_a[l], in, u.ea[l], true);
    const Tensor skip = l < Lv - 1 ? slice(u.cat[l], 2 * ch(u, l), ch(u, l)) : u.dbot[0];
    conv(u, u.enc_b[l], u.ea[l], skip, true);
    if (l < Lv - 1) {
      launch_pool(skip.p, skip.cs, skip.c0, skip.v, u.pool[l + 1].p, u.pool[l + 1].cs, 0, u.vol[l + 1], ch(u, l),
                  u.s);
      u.launches += 1;
    }
  }
  for (int l = Lv - 2; l >= 0; --l) {
    const Tensor& below = l == Lv - 2 ? u.dbot[0] : u.d[l + 1];
    launch_upsample(below.p, below.cs, below.c0, u.vol[l + 1], u.cat[l].p, u.cat[l].cs, 0, u.vol[l], ch(u, l + 1),
                    u.s);
    u.launches += 1;
    conv(u, u.dec_a[l], u.cat[l], u.da[l], true);
    conv(u, u.dec_b[l], u.da[l], u.d[l], true);
  }
  launch_head(u.d[0].p, u.d[0].cs, ch(u, 0), nvox(u.vol[0]), u.w + u.head_w, u.w + u.head_b, u.out, u.s);
  u.launches += 1;
}

// the forward pass replayed from a graph captured on first use (the
// buffers and weights keep their addresses; o3d_unet_set_params repacks in
// place), which removes the launch gaps between its ~30 small kernels
static int forward_graph(UNet& u) {
  if (!u.fwd_exec) {
    cudaGraph_t g;
    if (cudaStreamBeginCapture(u.s, cudaStreamCaptureModeThreadLocal) != cudaSuccess) return O3D_ERR_CUDA;
    forward(u);
    if (cudaStreamEndCapture(u.s, &g) != cudaSuccess) return O3D_ERR_CUDA;
    const cudaError_t e = cudaGraphInstantiate(&u.fwd_exec, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) {
      u.fwd_exec = nullptr;
      return O3D_ERR_CUDA;
    }
  }
  return cudaGraphLaunch(u.fwd_exec, u.s) == cudaSuccess ? O3D_OK : O3D_ERR_CUDA;
}

// gradients of the loss in u.dout with respect to every parameter, into u.g
static void backward(UNet& u) {
  const int Lv = u.levels;
  cudaMemsetAsync(u.g, 0, (size_t)u.nparam * sizeof(float), u.s);
  // head; dD0 is masked by D0 > 0 inside
  launch_head_back(u.d[0].p, u.d[0].cs, ch(u, 0), nvox(u.vol[0]), u.w + u.head_w, u.dout, u.g_d[0].p,
                   u.g + u.head_w, u.g + u.head_b, u.s);
  for (int l = 0; l <= Lv - 2; ++l) {
    // decoder level l: g_d[l] is the gradient at dec_b's pre-activation
    conv_wgrad(u, u.dec_b[l], u.da[l], u.g_d[l]);
    conv_dgrad(u, u.dec_b[l], u.g_d[l], u.g_da[l], &u.da[l]);
    conv_wgrad(u, u.dec_a[l], u.cat[l], u.g_da[l]);
    conv_dgrad(u, u.dec_a[l], u.g_da[l], u.g_cat[l], &u.cat[l]);
    // the upsampled part of the concat feeds the level below in the decoder
    const Tensor gup = slice(u.g_cat[l], 0, ch(u, l + 1));
    Tensor& gnext = u.g_d[l + 1];
    launch_upsample_back(gup.p, gup.cs, gup.c0, u.vol[l], gnext.p, gnext.cs, 0, u.vol[l + 1], ch(u, l + 1), nullptr,
                         0, 0, u.s);
  }
  // bottom level (its output is dbot = the source of the top-most upsample)
  for (int l = Lv - 1; l >= 0; --l) {
    const Tensor& gskip = l == Lv - 1 ? u.g_d[Lv - 1] : u.g_cat[l];
    const Tensor gs = l == Lv - 1 ? gskip : slice(gskip, 2 * ch(u, l), ch(u, l));
    const Tensor skip = l == Lv - 1 ? u.dbot[0] : slice(u.cat[l], 2 * ch(u, l), ch(u, l));
    if (l < Lv - 1) {
      // add the pooling path's gradient, then the ReLU mask of the skip output
      launch_pool_back(u.g_pool[l + 1].p, u.g_pool[l + 1].cs, 0, u.vol[l + 1], gs.p, gs.cs, gs.c0, u.vol[l], ch(u, l),
                       1, u.s);
      launch_mask(gs.p, gs.cs, gs.c0, skip.p, skip.cs, skip.c0, nvox(u.vol[l]), ch(u, l), u.s);
    }
    conv_wgrad(u, u.enc_b[l], u.ea[l], gs);
    conv_dgrad(u, u.enc_b[l], gs, u.g_ea[l], &u.ea[l]);
    const Tensor& in = l == 0 ? u.xin : u.pool[l];
    conv_wgrad(u, u.enc_a[l], in, u.g_ea[l]);
    if (l > 0) conv_dgrad(u, u.enc_a[l], u.g_ea[l], u.g_pool[l], nullptr);
  }
}

static int build(UNet& u, int nx, int ny, int nz, const int per[3], int base, int levels, int in_ch,
                 unsigned long long seed) {
  u.levels = levels;
  u.base = base;
  u.in_ch = in_ch;
  for (int l = 0; l < levels; ++l) {
    u.vol[l].nx = nx >> l;
    u.vol[l].ny = ny >> l;
    u.vol[l].nz = nz >> l;
    for (int a = 0; a < 3; ++a) u.vol[l].per[a] = per[a];
  }
  long long off = 0;
  for (int l = 0; l < levels; ++l) {
    const int K = l == 0 ? 16 : ch(u, l - 1);
    add_layer(u, u.enc_a, K, ch(u, l), &off);
    add_layer(u, u.enc_b, ch(u, l), ch(u, l), &off);
  }
  u.dec_a.resize(0);
  u.dec_b.resize(0);
  for (int l = 0; l < levels - 1; ++l) {
    add_layer(u, u.dec_a, 3 * ch(u, l), ch(u, l), &off);
    add_layer(u, u.dec_b, ch(u, l), ch(u, l), &off);
  }
  u.head_w = off;
  off += ch(u, 0);
  u.head_b = off;
  off += 1;
  u.nparam = off;
  int st;
  if ((st = ualloc(u, (void**)&u.w, off * 4)) || (st = ualloc(u, (void**)&u.g, off * 4)) ||
      (st = ualloc(u, (void**)&u.m, off * 4)) || (st = ualloc(u, (void**)&u.v, off * 4)))
    return st;
  auto wbufs = [&](std::vector<ConvLayer>& list) -> int {
    for (auto& L : list) {
      const size_t b = 27ull * L.K * L.N * sizeof(__nv_bfloat16);
      int s2 = ualloc(u, (void**)&L.wf, b);
      if (s2) return s2;
      s2 = ualloc(u, (void**)&L.wb, b);
      if (s2) return s2;
    }
    return 0;
  };
  if ((st = wbufs(u.enc_a)) || (st = wbufs(u.enc_b)) || (st = wbufs(u.dec_a)) || (st = wbufs(u.dec_b))) return st;
  // He-normal initialisation (fan-in over the real input channels), zero biases
  std::vector<float> h(off, 0.f);
  std::mt19937_64 rng(seed);
  auto init = [&](const ConvLayer& L, int kreal) {
    std::normal_distribution<float> nd(0.f, std::sqrt(2.f / (27.f * (float)kreal)));
    for (int t = 0; t < 27; ++t)
      for (int k = 0; k < L.K; ++k)
        for (int n = 0; n < L.N; ++n) h[L.w_off + ((long long)t * L.K + k) * L.N + n] = k < kreal ? nd(rng) : 0.f;
  };
  for (int l = 0; l < levels; ++l) {
    init(u.enc_a[l], l == 0 ? in_ch : u.enc_a[l].K);
    init(u.enc_b[l], u.enc_b[l].K);
  }
  for (int l = 0; l < levels - 1; ++l) {
    init(u.dec_a[l], u.dec_a[l].K);
    init(u.dec_b[l], u.dec_b[l].K);
  }
  {
    std::normal_distribution<float> nd(0.f, std::sqrt(1.f / (float)ch(u, 0)));
    for (int c = 0; c < ch(u, 0); ++c) h[u.head_w + c] = 0.1f * nd(rng);
  }
  if (cudaMemcpyAsync(u.w, h.data(), off * 4, cudaMemcpyHostToDevice, u.s) != cudaSuccess) return O3D_ERR_CUDA;
  // activations and their gradients
  u.ea.resize(levels); u.g_ea.resize(levels);
  u.cat.resize(levels); u.g_cat.resize(levels);
  u.pool.resize(levels); u.g_pool.resize(levels);
  u.da.resize(levels); u.g_da.resize(levels);
  u.d.resize(levels); u.g_d.resize(levels);
  u.dbot.resize(1);
  if ((st = tensor(u, &u.xin, u.vol[0], 16))) return st;
  for (int l = 0; l < levels; ++l) {
    const int C = ch(u, l);
    if ((st = tensor(u, &u.ea[l], u.vol[l], C)) || (st = tensor(u, &u.g_ea[l], u.vol[l], C))) return st;
    if (l > 0 && ((st = tensor(u, &u.pool[l], u.vol[l], ch(u, l - 1))) ||
                  (st = tensor(u, &u.g_pool[l], u.vol[l], ch(u, l - 1)))))
      return st;
    if (l < levels - 1) {
      if ((st = tensor(u, &u.cat[l], u.vol[l], 3 * C)) || (st = tensor(u, &u.g_cat[l], u.vol[l], 3 * C)) ||
          (st = tensor(u, &u.da[l], u.vol[l], C)) || (st = tensor(u, &u.g_da[l], u.vol[l], C)) ||
          (st = tensor(u, &u.d[l], u.vol[l], C)))
        return st;
    }
    if ((st = tensor(u, &u.g_d[l], u.vol[l], C))) return st;
  }
  if ((st = tensor(u, &u.dbot[0], u.vol[levels - 1], ch(u, levels - 1)))) return st;
  const long long n0 = nvox(u.vol[0]);
  if ((st = ualloc(u, (void**)&u.out, n0 * 4)) || (st = ualloc(u, (void**)&u.dout, n0 * 4)) ||
      (st = ualloc(u, (void**)&u.loss, 16)))
    return st;
  // split-K workspace: the largest slices x voxels x outputs over the forward
  // and data-gradient convolutions
  long long cap = 0;
  auto need = [&](const std::vector<ConvLayer>& list, int first_level) {
    for (size_t i = 0; i < list.size(); ++i) {
      const long long nv = nvox(u.vol[first_level + (int)i]);
      const ConvLayer& L = list[i];
      const long long f = conv_splits(nv, L.K, L.N) * nv * L.N;
      const long long b = conv_splits(nv, L.N, L.K) * nv * L.K;
      cap = std::max(cap, std::max(f, b));
    }
  };
  need(u.enc_a, 0); need(u.enc_b, 0); need(u.dec_a, 0); need(u.dec_b, 0);
  u.ws_cap = cap;
  if ((st = ualloc(u, (void**)&u.ws, (size_t)cap * 4))) return st;
  pack_all(u);
  return cudaStreamSynchronize(u.s) == cudaSuccess ? O3D_OK : O3D_ERR_CUDA;
}

}  // namespace o3d

using namespace o3d;

struct o3d_unet {
  UNet u;
};

static int check_last(const char* what) {
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    set_error("%s: %s", what, cudaGetErrorString(e));
    return O3D_ERR_CUDA;
  }
  return O3D_OK;
}

extern "C" {

int o3d_unet_create(int nx, int ny, int nz, const int periodic[3], int base_channels, int levels, int in_channels,
                    unsigned long long seed, o3d_unet** out) {
  if (!out || !periodic) return O3D_ERR_BADARG;
  *out = nullptr;
  if (levels < 2 || levels > 6 || base_channels < 16 || base_channels % 16 || base_channels > 64 || in_channels < 1 ||
      in_channels > 16) {
    set_error("U-Net: levels must be 2..6, base channels a multiple of 16 up to 64, inputs 1..16");
    return O3D_ERR_BADARG;
  }
  const int div = 1 << (levels - 1);
  if (nx % div || ny % div || nz % div || nx / div < 2 || ny / div < 2 || nz / div < 2) {
    set_error("U-Net: grid %d x %d x %d must be divisible by 2^(levels-1) = %d with at least 2 points left", nx, ny,
              nz, div);
    return O3D_ERR_BADARG;
  }
  if ((base_channels << (levels - 1)) * 8 > 1024) {
    set_error("U-Net: the bottom level would have more than 128 channels");
    return O3D_ERR_BADARG;
  }
  o3d_unet* n = new (std::nothrow) o3d_unet();
  if (!n) return O3D_ERR_NOMEM;
  if (cudaStreamCreateWithFlags(&n->u.s, cudaStreamNonBlocking) != cudaSuccess ||
      cudaEventCreateWithFlags(&n->u.ev, cudaEventDisableTiming) != cudaSuccess) {
    if (n->u.s) cudaStreamDestroy(n->u.s);
    delete n;
    set_error("U-Net: stream or event creation failed");
    return O3D_ERR_CUDA;
  }
  int st = o3d::build(n->u, nx, ny, nz, periodic, base_channels, levels, in_channels, seed);
  if (!st) st = check_last("U-Net build");
  if (st) {
    o3d_unet_destroy(n);
    return st;
  }
  *out = n;
  return O3D_OK;
}

int o3d_unet_destroy(o3d_unet* n) {
  if (!n) return O3D_OK;
  if (n->u.s) cudaStreamSynchronize(n->u.s);
  if (n->u.fwd_exec) cudaGraphExecDestroy(n->u.fwd_exec);
  if (n->u.ev) cudaEventDestroy(n->u.ev);
  for (void* p : n->u.allocs) cudaFree(p);
  if (n->u.s) cudaStreamDestroy(n->u.s);
  delete n;
  return O3D_OK;
}

long long o3d_unet_num_params(const o3d_unet* n) { return n ? n->u.nparam : 0; }

int o3d_unet_get_params(o3d_unet* n, float* host) {
  if (!n || !host) return O3D_ERR_BADARG;
  if (cudaMemcpyAsync(host, n->u.w, n->u.nparam * 4, cudaMemcpyDeviceToHost, n->u.s) != cudaSuccess ||
      cudaStreamSynchronize(n->u.s) != cudaSuccess)
    return O3D_ERR_CUDA;
  return O3D_OK;
}

int o3d_unet_set_params(o3d_unet* n, const float* host) {
  if (!n || !host) return O3D_ERR_BADARG;
  if (cudaMemcpyAsync(n->u.w, host, n->u.nparam * 4, cudaMemcpyHostToDevice, n->u.s) != cudaSuccess)
    return O3D_ERR_CUDA;
  pack_all(n->u);
  if (cudaStreamSynchronize(n->u.s) != cudaSuccess) return O3D_ERR_CUDA;
  return check_last("U-Net set_params");
}

// d_in: in_channels x nvox FP32 (channel-major, each channel x fastest);
// d_out: nvox FP32.  Runs on the network's stream after `wait` (a cudaStream_t
// whose prior work the network must see; NULL = none).
int o3d_unet_forward_dev(o3d_unet* n, const float* d_in, float* d_out, void* wait) {
  if (!n || !d_in || !d_out) return O3D_ERR_BADARG;
  UNet& u = n->u;
  if (wait) {
    cudaEventRecord(u.ev, (cudaStream_t)wait);
    cudaStreamWaitEvent(u.s, u.ev, 0);
  }
  launch_pack_input(d_in, u.in_ch, nvox(u.vol[0]), u.xin.p, 16, u.s);
  int st = forward_graph(u);
  if (st) {
    set_error("U-Net forward graph: %s", cudaGetErrorString(cudaGetLastError()));
    return st;
  }
  cudaMemcpyAsync(d_out, u.out, nvox(u.vol[0]) * 4, cudaMemcpyDeviceToDevice, u.s);
  if (wait) {
    cudaEventRecord(u.ev, u.s);
    cudaStreamWaitEvent((cudaStream_t)wait, u.ev, 0);
  }
  return check_last("U-Net forward");
}

// Loss and gradients of one sample (no update); grads to host when given.
int o3d_unet_gradients(o3d_unet* n, const float* d_in, const float* d_target, float* loss, float* host_grad) {
  if (!n || !d_in || !d_target) return O3D_ERR_BADARG;
  UNet& u = n->u;
  launch_pack_input(d_in, u.in_ch, nvox(u.vol[0]), u.xin.p, 16, u.s);
  forward(u);
  cudaMemsetAsync(u.loss, 0, 4, u.s);
  launch_mse(u.out, d_target, nvox(u.vol[0]), u.dout, u.loss, u.s);
  backward(u);
  int st = check_last("U-Net gradients");
  if (st) return st;
  if (loss && cudaMemcpyAsync(loss, u.loss, 4, cudaMemcpyDeviceToHost, u.s) != cudaSuccess) return O3D_ERR_CUDA;
  if (host_grad && cudaMemcpyAsync(host_grad, u.g, u.nparam * 4, cudaMemcpyDeviceToHost, u.s) != cudaSuccess)
    return O3D_ERR_CUDA;
  if (cudaStreamSynchronize(u.s) != cudaSuccess) return O3D_ERR_CUDA;
  return O3D_OK;
}

// One Adam step on one sample (MSE loss against d_target).
int o3d_unet_train_step(o3d_unet* n, const float* d_in, const float* d_target, float lr, float* loss) {
  if (!n) return O3D_ERR_BADARG;
  UNet& u = n->u;
  int st = o3d_unet_gradients(n, d_in, d_target, loss, nullptr);
  if (st) return st;
  u.step += 1;
  const float b1 = 0.9f, b2 = 0.999f;
  const float c1 = 1.f - std::pow(b1, (float)u.step), c2 = 1.f - std::pow(b2, (float)u.step);
  launch_adam(u.w, u.g, u.m, u.v, u.nparam, lr, b1, b2, 1e-8f, c1, c2, u.s);
  pack_all(u);
  return check_last("U-Net train step");
}

}  // extern "C"

// used by the solver context (o3d_api.cu)
namespace o3d {
// The forward pass enqueued on the caller's stream s (so that a solver can
// capture it in its own CUDA graph); the network's buffers are shared, so
// the network must not run elsewhere meanwhile.
int unet_enqueue_forward(o3d_unet* n, const float* d_in, float* d_out, cudaStream_t s, long long* nl) {
  UNet& u = n->u;
  const cudaStream_t own = u.s;
  u.s = s;
  const long long l0 = u.launches;
  launch_pack_input(d_in, u.in_ch, nvox(u.vol[0]), u.xin.p, 16, u.s);
  forward(u);
  *nl += 1 + (u.launches - l0);
  const cudaError_t e = cudaMemcpyAsync(d_out, u.out, nvox(u.vol[0]) * 4, cudaMemcpyDeviceToDevice, u.s);
  u.s = own;
  return e == cudaSuccess ? O3D_OK : O3D_ERR_CUDA;
}
// waits for the network's own queued work (weight packing after training)
int unet_sync(o3d_unet* n) {
  if (cudaStreamSynchronize(n->u.s) != cudaSuccess) return O3D_ERR_CUDA;
  if (conv_tc_timed_out() != 0) {
    set_error("a tensor-core convolution of the network timed out on a wait; its output is invalid");
    return O3D_ERR_CUDA;
  }
  return O3D_OK;
}
int unet_grid(const o3d_unet* n, int* nx, int* ny, int* nz, int* in_ch) {
  *nx = n->u.vol[0].nx;
  *ny = n->u.vol[0].ny;
  *nz = n->u.vol[0].nz;
  *in_ch = n->u.in_ch;
  return 0;
}
}  // namespace o3d
