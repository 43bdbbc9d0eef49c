// o3d_api.cu -- context management and host orchestration of the step,
// behind the extern "C" entry points declared in include/o3d.h.
//
// One context = one grid, one CUDA stream, device-resident fields.  Field
// storage is FP64 for the plain method and FP32 for the mixed method; the
// pressure is FP64 in both (it is the unknown of the FP64 defect-correction
// loop).  The Adams-Bashforth flux history is a ring of three buffers per
// component, so the history shift of src/integration.f90:176-188 costs no
// copy.
#include <utility>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <new>
#include <vector>

#include "o3d_internal.cuh"
#include "o3d_output.h"
#include "o3d_kernels.h"

using namespace o3d;

static thread_local char g_err[512] = "";

static void errf(const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_err, sizeof g_err, fmt, ap);
  va_end(ap);
}

namespace o3d {
// error text for o3d_last_error(), for the entry points of other files
void set_error(const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_err, sizeof g_err, fmt, ap);
  va_end(ap);
}
}  // namespace o3d

static double bits_to_double(unsigned long long k) {
  double d;
  memcpy(&d, &k, 8);
  return d;
}

#define CK(call)                                                                       \
  do {                                                                                 \
    cudaError_t e_ = (call);                                                           \
    if (e_ != cudaSuccess) {                                                           \
      snprintf(g_err, sizeof g_err, "%s failed: %s (%s:%d)", #call, cudaGetErrorString(e_), \
               __FILE__, __LINE__);                                                    \
      return O3D_ERR_CUDA;                                                             \
    }                                                                                  \
  } while (0)

#define CKL()                                                                          \
  do {                                                                                 \
    cudaError_t e_ = cudaGetLastError();                                               \
    if (e_ != cudaSuccess) {                                                           \
      snprintf(g_err, sizeof g_err, "kernel launch failed: %s (%s:%d)",               \
               cudaGetErrorString(e_), __FILE__, __LINE__);                            \
      return O3D_ERR_CUDA;                                                             \
    }                                                                                  \
  } while (0)

struct o3d_ctx {
  o3d_params P;
  Grid g;        // stencil grid: per-axis closure of the derivative routines
  Grid gp;       // Poisson grid: remap of the chosen poisson_solver_* routine
  Coef3<double> cf;
  double dx, dy, dz, delta;
  double adt[3], bdt[3], cdt[3];
  double omega;
  int mixed;
  size_t esz;
  cudaStream_t s;

  void* u[3];
  void* up[3];
  void* fu[3][3];    // ring: [0] newest flux, [1] one older, [2] free
  void* nu_t;
  void* phi;
  void* phi2;
  void* src;
  void* fphi[3];
  void* rhs;
  float* rhs32;      // the mixed multigrid step's rhs, FP32 (its values are FP32 numbers)
  int rhs_f32;       // the current rhs is rhs32, not rhs
  // the pressure and its history; with pdf (the mixed multigrid method) each
  // of these buffers holds a double-float pair of FP32 planes (PPair: hi =
  // RN32(p), then lo = RN32(p - hi)), converted to FP64 at the API
  double* pp;
  int pdf;
  double* pp_prev;   // previous step's pressure (extrapolated and learned guesses, lazy)
  int pp_prev_valid;
  double* pp_prev2;  // the one before (quadratic extrapolation, lazy)
  int pp_prev2_valid;
  o3d_unet* unet;    // network of the learned guess (not owned)
  float* feat;       // its input on the network grid (2 channels)
  float* ynet;       // its output
  float* sample_feat;  // caller's buffers for training samples (features, target)
  float* sample_tgt;
  int sample_ready;
  int learn_level;     // multigrid level of the network grid
  double* stage[4];  // FP64 staging buffers for host transfers (lazy)
  void* uold[3];     // velocity kept by o3d_save_old_velocity (lazy)
  void* vout[4];     // curl and Q-criterion outputs (lazy)
  void* rscratch;    // velocity residual block records (lazy)
  OutWriter* out;    // asynchronous output writer (lazy)

  double* part;      // per-block reduction records
  StatPart* spart;
  double* wpart;     // weighted rhs sums per divergence block (mixed method)
  int rhs_wsum;      // wpart holds the sums of the current rhs
  DevDiag* diag;
  DevDiag* diag_h;   // pinned
  SolveCtrl* ctrl;
  SolveCtrl* ctrl_h; // pinned

  std::vector<MGLevel> mg;
  int mg_ok;
  cudaGraphExec_t sor_exec;
  int sor_batch;
  long long sor_nodes;
  cudaGraphExec_t mg_exec;
  int mg_batch;
  long long mg_nodes;
  cudaGraphExec_t learn_exec;  // first outer iteration with the learned guess (multigrid)
  cudaGraphExec_t mg_exec32;    // the same two graphs for the FP32 rhs
  long long mg_nodes32;
  cudaGraphExec_t learn_exec32;
  long long learn_nodes32;
  long long learn_nodes;

  cudaEvent_t ev[4];
  // host transfers of o3d_step_host: a copy stream beside the context's, so
  // that the FP64 <-> FP32 conversions overlap the copies of other fields
  cudaStream_t xs;
  cudaEvent_t xev[8];
  cudaEvent_t p_in_wait;  // set by o3d_step_host: the pressure's upload, awaited when the solve starts
  double* p_out_host;     // set by o3d_step_host: the pressure's host copy, issued when the solve ends
  long long launches;
};

namespace {

// Allocates and zero-fills on the context's stream.  The stream is
// non-blocking, so a plain cudaMemset (legacy default stream) could land
// after later uploads on the context's stream.
int dalloc(cudaStream_t s, void** p, size_t bytes) {
  if (cudaMalloc(p, bytes) != cudaSuccess) {
    cudaGetLastError();
    snprintf(g_err, sizeof g_err, "cudaMalloc of %zu bytes failed", bytes);
    *p = nullptr;
    return O3D_ERR_NOMEM;
  }
  if (cudaMemsetAsync(*p, 0, bytes, s) != cudaSuccess) return O3D_ERR_CUDA;
  return O3D_OK;
}

size_t fbytes(const o3d_ctx* c) { return (size_t)c->g.n * c->esz; }

int stage_ready(o3d_ctx* c, int k) {
  for (int q = 0; q <= k; ++q)
    if (!c->stage[q]) {
      int st = dalloc(c->s, (void**)&c->stage[q], (size_t)c->g.n * sizeof(double));
      if (st) return st;
    }
  return O3D_OK;
}

// host double buffer -> device field of the context's storage type
int put_field(o3d_ctx* c, void* dst, const double* host) {
  if (!c->mixed) {
    CK(cudaMemcpyAsync(dst, host, (size_t)c->g.n * 8, cudaMemcpyHostToDevice, c->s));
    return O3D_OK;
  }
  int st = stage_ready(c, 0);
  if (st) return st;
  CK(cudaMemcpyAsync(c->stage[0], host, (size_t)c->g.n * 8, cudaMemcpyHostToDevice, c->s));
  launch_convert<double, float>(c->stage[0], (float*)dst, c->g.n, c->s);
  c->launches++;
  CKL();
  return O3D_OK;
}

int get_field(o3d_ctx* c, const void* src, double* host) {
  if (!c->mixed) {
    CK(cudaMemcpyAsync(host, src, (size_t)c->g.n * 8, cudaMemcpyDeviceToHost, c->s));
    return O3D_OK;
  }
  int st = stage_ready(c, 0);
  if (st) return st;
  launch_convert<float, double>((const float*)src, c->stage[0], c->g.n, c->s);
  c->launches++;
  CKL();
  CK(cudaMemcpyAsync(host, c->stage[0], (size_t)c->g.n * 8, cudaMemcpyDeviceToHost, c->s));
  return O3D_OK;
}

// host FP64 pressure <-> a pressure buffer of the context (pp or its
// history): a plain copy, or through stage[0] and the pair split / join
// when the context holds its pressure as double-float pairs
int put_pressure(o3d_ctx* c, double* dev, const double* host) {
  const size_t bytes = (size_t)c->g.n * 8;
  if (!c->pdf) {
    CK(cudaMemcpyAsync(dev, host, bytes, cudaMemcpyHostToDevice, c->s));
    return O3D_OK;
  }
  int st = stage_ready(c, 0);
  if (st) return st;
  CK(cudaMemcpyAsync(c->stage[0], host, bytes, cudaMemcpyHostToDevice, c->s));
  launch_split_pair(c->stage[0], dev, c->g.n, c->s);
  c->launches++;
  CKL();
  return O3D_OK;
}
int get_pressure(o3d_ctx* c, const double* dev, double* host) {
  const size_t bytes = (size_t)c->g.n * 8;
  if (!c->pdf) {
    CK(cudaMemcpyAsync(host, dev, bytes, cudaMemcpyDeviceToHost, c->s));
    return O3D_OK;
  }
  int st = stage_ready(c, 0);
  if (st) return st;
  launch_join_pair(dev, c->stage[0], c->g.n, c->s);
  c->launches++;
  CKL();
  CK(cudaMemcpyAsync(host, c->stage[0], bytes, cudaMemcpyDeviceToHost, c->s));
  return O3D_OK;
}

void* field_ptr(o3d_ctx* c, int f, bool* is_pp) {
  *is_pp = false;
  switch (f) {
    case O3D_FIELD_UX: return c->u[0];
    case O3D_FIELD_UY: return c->u[1];
    case O3D_FIELD_UZ: return c->u[2];
    case O3D_FIELD_PP: *is_pp = true; return c->pp;
    case O3D_FIELD_UX_PRED: return c->up[0];
    case O3D_FIELD_UY_PRED: return c->up[1];
    case O3D_FIELD_UZ_PRED: return c->up[2];
    case O3D_FIELD_PHI: return c->phi;
    case O3D_FIELD_SRC: return c->src;
    case O3D_FIELD_NU_T: return c->nu_t;
    case O3D_FIELD_RHS: *is_pp = true; return c->rhs;  // FP64 in both methods
    default: break;
  }
  if (f >= O3D_FIELD_FU0 && f < O3D_FIELD_FU0 + 6) {
    int q = f - O3D_FIELD_FU0;
    return c->fu[q / 2][q % 2];
  }
  if (f >= O3D_FIELD_FPHI0 && f < O3D_FIELD_FPHI0 + 2) return c->fphi[f - O3D_FIELD_FPHI0];
  return nullptr;
}

// AB coefficients of the step, src/integration.f90:84-98
void ab_coefs(const o3d_ctx* c, int itime, double* a, double* b, double* cc) {
  int s = (c->P.itscheme == 1 || itime == 1) ? 0 : (c->P.itscheme == 2 || itime == 2) ? 1 : 2;
  *a = c->adt[s];
  *b = c->bdt[s];
  *cc = c->cdt[s];
}

void rotate_ring(void* r[3]) {
  void* a = r[0];
  void* b = r[1];
  void* f = r[2];
  r[0] = f;  // the new flux becomes the newest history
  r[1] = a;  // the previous newest ages by one
  r[2] = b;  // the oldest buffer is free for the next step
}

template <class T>
int predict_t(o3d_ctx* c, int itime) {
  double a, b, cc;
  ab_coefs(c, itime, &a, &b, &cc);
  PredArgs<T> A;
  for (int q = 0; q < 3; ++q) {
    A.u[q] = (const T*)c->u[q];
    A.up[q] = (T*)c->up[q];
    A.fnew[q] = (T*)c->fu[q][2];
    A.f2[q] = b != 0.0 ? (const T*)c->fu[q][0] : nullptr;
    A.f3[q] = cc != 0.0 ? (const T*)c->fu[q][1] : nullptr;
  }
  A.nu_t = (T*)c->nu_t;
  A.g = c->g;
  A.cf = cast_coef<T>(c->cf);
  A.adu = (T)a;
  A.bdu = (T)b;
  A.cdu = (T)cc;
  A.onere = (T)(1.0 / c->P.re);
  const double csd = c->P.cs * c->delta;
  A.csd2 = (T)(csd * csd);
  A.les = c->P.iles == 1;
  launch_predict<T>(A, c->s);
  c->launches++;
  CKL();
  // history shift (src/integration.f90:176-188) as a ring rotation; with
  // Euler (itscheme 1) the history is never read, so rotating is harmless
  for (int q = 0; q < 3; ++q) {
    if (c->P.itscheme == 2) {
      void* t = c->fu[q][0];
      c->fu[q][0] = c->fu[q][2];
      c->fu[q][2] = t;
    } else {
      rotate_ring(c->fu[q]);
    }
  }
  return O3D_OK;
}

template <class T>
int rhs_t(o3d_ctx* c) {
  Coef3<T> cf = cast_coef<T>(c->cf);
  // the Poisson rhs is FP64 in both methods (the mixed method's FP32
  // divergence widened exactly), so that removing its weighted mean leaves a
  // compatible problem to FP64 rounding
  // the mixed method's kernel also sums the rhs with the trapezoid weights of
  // the pressure grid, for the compatibility mean of the solve
  const bool fuse_wsum = sizeof(T) == 4;
  int wmask = 0;
  for (int a = 0; a < 3; ++a)
    if (c->gp.bc[a] == AX_MIRROR) wmask |= 1 << a;
  // the mixed multigrid solve reads the rhs as it is computed, in FP32: its
  // residual kernel takes the value exactly (no FP64 load, no split) and
  // subtracts the mean in double-float arithmetic
  const bool f32 = sizeof(T) == 4 && c->P.solver == O3D_SOLVER_MG;
  if (f32)
    launch_div<T, T>((const T*)c->up[0], (const T*)c->up[1], (const T*)c->up[2], (T*)c->rhs32, c->g, cf, 1,
                     (T)c->P.dt, 1, c->spart, c->s, c->wpart, wmask);
  else
    launch_div<T, double>((const T*)c->up[0], (const T*)c->up[1], (const T*)c->up[2], (double*)c->rhs, c->g, cf,
                          1, (T)c->P.dt, 1, c->spart, c->s, fuse_wsum ? c->wpart : nullptr, wmask);
  c->rhs_f32 = f32 ? 1 : 0;
  c->rhs_wsum = fuse_wsum ? 1 : 0;
  launch_finalize_stats(c->spart, div_blocks<T>(c->g), c->g, c->diag->divp, c->s);
  c->launches += 2;
  CKL();
  return O3D_OK;
}

template <class T, class P>
void correct_args(o3d_ctx* c, const P* p, CorrArgs<T, P>& A) {
  A.p = p;
  for (int q = 0; q < 3; ++q) {
    A.up[q] = (const T*)c->up[q];
    A.u[q] = (T*)c->u[q];
  }
  A.g = c->g;
  A.cf = cast_coef<T>(c->cf);
  A.dt = (T)c->P.dt;
  A.part = c->part;
}

template <class T>
int correct_t(o3d_ctx* c) {
  if (sizeof(T) == 4 && c->pdf) {
    // the gradient of the FP32 pressure: the high plane of the pair (the
    // FP32 rounding of the FP64 value, as the FP64-pressure kernels convert)
    CorrArgs<float, float> A;
    correct_args<float, float>(c, (const float*)c->pp, A);
    launch_correct<float, float>(A, c->s);
  } else {
    CorrArgs<T, double> A;
    correct_args<T, double>(c, c->pp, A);
    launch_correct<T, double>(A, c->s);
  }
  // min x3, max x3, |max| x3, nan flag
  unsigned long long ops = 0;
  for (int q = 0; q < 10; ++q) ops |= (unsigned long long)(q < 3 ? RED_MIN : RED_MAX) << (2 * q);
  launch_finalize(c->part, corr_blocks<T>(c->g), 10, ops, c->diag->sums, c->s);
  c->launches += 2;
  CKL();
  return O3D_OK;
}

template <class T>
int divu_diag_t(o3d_ctx* c) {
  Coef3<T> cf = cast_coef<T>(c->cf);
  launch_div<T, T>((const T*)c->u[0], (const T*)c->u[1], (const T*)c->u[2], (T*)nullptr, c->g, cf, 1,
                   (T)c->P.dt, 0, c->spart, c->s);
  launch_finalize_stats(c->spart, div_blocks<T>(c->g), c->g, c->diag->divu, c->s);
  c->launches += 2;
  CKL();
  return O3D_OK;
}

template <class T>
int transeq_t(o3d_ctx* c, int itime) {
  double a, b, cc;
  ab_coefs(c, itime, &a, &b, &cc);
  ScalArgs<T> A;
  A.phi = (const T*)c->phi;
  A.phi_out = (T*)c->phi2;
  for (int q = 0; q < 3; ++q) A.u[q] = (const T*)c->u[q];
  A.src = (const T*)c->src;
  A.nu_t = (const T*)c->nu_t;
  A.fnew = (T*)c->fphi[2];
  A.f2 = b != 0.0 ? (const T*)c->fphi[0] : nullptr;
  A.f3 = cc != 0.0 ? (const T*)c->fphi[1] : nullptr;
  A.g = c->g;
  A.cf = cast_coef<T>(c->cf);
  A.adu = (T)a;
  A.bdu = (T)b;
  A.cdu = (T)cc;
  A.alpha0 = (T)(1.0 / (c->P.re * c->P.sc));
  A.sc = (T)c->P.sc;
  A.les = c->P.iles == 1;
  A.part = c->part;
  launch_transeq<T>(A, c->diag->sums + 16, c->s, &c->launches);
  CKL();
  std::swap(c->phi, c->phi2);
  if (c->P.itscheme == 2) std::swap(c->fphi[0], c->fphi[2]);
  else rotate_ring(c->fphi);
  return O3D_OK;
}

// ---- pressure solve --------------------------------------------------------

int mg_smooth_cfg(const o3d_ctx* c, int* pre, int* post);

int build_mg(o3d_ctx* c) {
  const int maxlev = c->P.mg_levels > 0 ? c->P.mg_levels : 32;
  Grid g = c->gp;
  double h[3] = {c->dx, c->dy, c->dz};
  c->mg.clear();
  for (;;) {
    MGLevel L;
    memset(&L, 0, sizeof L);
    L.g = g;
    for (int a = 0; a < 3; ++a) L.h[a] = h[a];
    int any = 0;
    Grid ng = g;
    double nh[3] = {h[0], h[1], h[2]};
    for (int a = 0; a < 3; ++a) {
      const int n = g.len(a);
      int cn = 0, mode = 0;
      // halved onto every other node: even periodic, odd free-slip
      if (g.bc[a] == AX_PERIODIC && n % 2 == 0 && n / 2 >= 4) { cn = n / 2; mode = 1; }
      if (g.bc[a] == AX_MIRROR && n % 2 == 1 && (n + 1) / 2 >= 3) { cn = (n + 1) / 2; mode = 1; }
      // non-nested onto about half the nodes (k_restrict_nn / k_prolong_nn):
      // even free-slip to an odd count, odd periodic to an even count, so
      // that the next level is nested again; H/h stays <= 2.5
      if (!mode && g.bc[a] == AX_MIRROR && n >= 6 && n % 2 == 0) { cn = (n / 2) | 1; mode = 2; }
      if (!mode && g.bc[a] == AX_PERIODIC && n >= 9 && n % 2 == 1) { cn = ((n + 1) / 2) & ~1; mode = 2; }
      L.coarsen[a] = mode;
      if (mode) {
        any = 1;
        if (a == 0) ng.nx = cn;
        if (a == 1) ng.ny = cn;
        if (a == 2) ng.nz = cn;
        if (mode == 1) nh[a] = 2.0 * h[a];
        else nh[a] = g.bc[a] == AX_PERIODIC ? h[a] * n / cn : h[a] * (n - 1) / (cn - 1);
      }
    }
    ng.n = (long long)ng.nx * ng.ny * ng.nz;
    const bool last = !any || (int)c->mg.size() + 1 >= maxlev || g.n <= 512;
    if (last) for (int a = 0; a < 3; ++a) L.coarsen[a] = 0;
    c->mg.push_back(L);
    if (last) break;
    for (int a = 0; a < 3; ++a) h[a] = nh[a];
    g = ng;
  }
  // fused level kernels (FP32): every level that coarsens on all axes and is
  // large enough, unless the caller asked for one kernel per pass
  int pre, post;
  mg_smooth_cfg(c, &pre, &post);
  const bool fuse = c->mixed && c->P.mg_kernels != 1;
  if (fuse && mg_fused_setup()) {
    errf("fused multigrid kernels: %s", cudaGetErrorString(cudaGetLastError()));
    return O3D_ERR_CUDA;
  }
  for (size_t l = 0; l < c->mg.size(); ++l) {
    MGLevel& L = c->mg[l];
    L.fused = l + 1 < c->mg.size() && fuse && mg_fusable(L, pre, post, c->P.mg_kernels == 2);
    L.fuse_all = c->P.mg_kernels == 2;
    L.plain = c->P.mg_kernels == 1;
  }
  const size_t tsz = c->mixed ? 4 : 8;
  for (auto& L : c->mg) {
    int st;
    if ((st = dalloc(c->s, &L.e, (size_t)L.g.n * tsz))) return st;
    if ((st = dalloc(c->s, &L.r, (size_t)L.g.n * tsz))) return st;
    if ((st = dalloc(c->s, &L.t, (size_t)L.g.n * tsz))) return st;
  }
  c->mg_ok = 1;
  return O3D_OK;
}

int mg_cycles_of(const o3d_ctx* c) {
  if (c->P.solver != O3D_SOLVER_MG) return 0;
  return c->P.mg_cycles > 0 ? c->P.mg_cycles : 1;
}

int reset_ctrl(o3d_ctx* c, double omega, double eps, int kmax, int idyn) {
  SolveCtrl* h = c->ctrl_h;
  memset(h, 0, sizeof *h);
  h->omega = omega;
  h->dmax_old = 1609.0;  // src/poisson.f90:52
  h->eps = eps;
  // factor of the dynamic omega rule: 1.01 for the x-periodic/y-free-slip
  // solver, 1.05 otherwise (src/poisson.f90:35,162,288)
  h->factor = (c->gp.bc[0] == AX_PERIODIC && c->gp.bc[1] == AX_MIRROR) ? 1.01 : 1.05;
  h->kmax = kmax;
  h->idyn = idyn;
  h->cycles_per_iter = mg_cycles_of(c);
  CK(cudaMemcpyAsync(c->ctrl, h, sizeof *h, cudaMemcpyHostToDevice, c->s));
  return O3D_OK;
}

int read_ctrl(o3d_ctx* c) {
  CK(cudaMemcpyAsync(c->ctrl_h, c->ctrl, sizeof(SolveCtrl), cudaMemcpyDeviceToHost, c->s));
  CK(cudaStreamSynchronize(c->s));
  return O3D_OK;
}

int capture_sor(o3d_ctx* c) {
  if (c->sor_exec) return O3D_OK;
  c->sor_batch = 16;
  PoiCoef<double> pc = make_poi<double>(c->dx, c->dy, c->dz);
  cudaGraph_t graph;
  CK(cudaStreamBeginCapture(c->s, cudaStreamCaptureModeThreadLocal));
  long long nodes = 0;
  for (int q = 0; q < c->sor_batch; ++q) {
    nodes += launch_sor_sweep_ctrl(c->pp, (const double*)c->rhs, c->gp, pc, c->ctrl, c->s);
    launch_sor_control(c->ctrl, c->s);
    nodes += 1;
  }
  CK(cudaStreamEndCapture(c->s, &graph));
  CK(cudaGraphInstantiate(&c->sor_exec, graph, 0));
  CK(cudaGraphDestroy(graph));
  c->sor_nodes = nodes;
  return O3D_OK;
}

// red-black sweeps of the coarsest multigrid level when it is too large
// for the one-block shared-memory solve
constexpr int MG_COARSE_SWEEPS = 16;

int mg_smooth_cfg(const o3d_ctx* c, int* pre, int* post) {
  // the plain FP64 method is the V(2,2) Gauss-Seidel cycle; the mixed one
  // defaults to V(1,1) over-relaxed: with omega 1.25 it needs no more cycles
  // per step than V(2,1) or V(2,2) at 256^3 and each cycle is cheaper
  *pre = c->P.mg_pre > 0 ? c->P.mg_pre : (c->mixed ? 1 : 2);
  *post = c->P.mg_post > 0 ? c->P.mg_post : (c->mixed ? 1 : 2);
  return 0;
}

double mg_omega_of(const o3d_ctx* c) {
  if (c->P.mg_omega > 0.0) return c->P.mg_omega;
  return c->mixed ? 1.25 : 1.0;
}

int capture_mg(o3d_ctx* c) {
  const bool f32 = c->rhs_f32;
  cudaGraphExec_t* exec = f32 ? &c->mg_exec32 : &c->mg_exec;
  if (*exec) return O3D_OK;
  if (!c->mg_ok) {
    int st = build_mg(c);
    if (st) return st;
  }
  c->mg_batch = 2;
  int pre, post;
  mg_smooth_cfg(c, &pre, &post);
  const int coarse_sweeps = MG_COARSE_SWEEPS;
  long long nl = 0;
  cudaGraph_t graph;
  CK(cudaStreamBeginCapture(c->s, cudaStreamCaptureModeThreadLocal));
  for (int q = 0; q < c->mg_batch; ++q) {
    const int cyc = mg_cycles_of(c);
    const double om = mg_omega_of(c);
    if (c->mixed && f32)
      launch_mg_outer<float, float>(c->pp, c->rhs32, c->mg.data(), (int)c->mg.size(), pre, post, coarse_sweeps,
                                    (float)om, cyc, c->ctrl, c->s, &nl);
    else if (c->mixed)
      launch_mg_outer<float, double>(c->pp, (const double*)c->rhs, c->mg.data(), (int)c->mg.size(), pre,
                                    post, coarse_sweeps, (float)om, cyc, c->ctrl, c->s, &nl);
    else
      launch_mg_outer<double, double>(c->pp, (const double*)c->rhs, c->mg.data(), (int)c->mg.size(),
                                      pre, post, coarse_sweeps, om, cyc, c->ctrl, c->s, &nl);
  }
  CK(cudaStreamEndCapture(c->s, &graph));
  CK(cudaGraphInstantiate(exec, graph, 0));
  CK(cudaGraphDestroy(graph));
  (f32 ? c->mg_nodes32 : c->mg_nodes) = nl;
  return O3D_OK;
}

// Sets up the learned-guess machinery: multigrid scratch levels, the level
// the network works on, and its buffers.  The level is the deepest one
// reached by coarsening every axis each time, with at most three
// coarsenings and at least 16 points on every axis (256^3 -> 32^3,
// 128^3 -> 16^3, 32^3 -> 16^3).
int learn_ready(o3d_ctx* c) {
  if (!c->mg_ok) {
    int st = build_mg(c);
    if (st) return st;
  }
  int ll = 0;
  while (ll < 3 && ll + 1 < (int)c->mg.size()) {
    const MGLevel& L = c->mg[ll];
    if (!(L.coarsen[0] == 1 && L.coarsen[1] == 1 && L.coarsen[2] == 1)) break;
    const Grid& g = c->mg[ll + 1].g;
    if (g.nx < 16 || g.ny < 16 || g.nz < 16) break;
    ++ll;
  }
  if (ll < 1) {
    errf("the learned warm start needs a grid that coarsens at least once on every axis to 16+ points");
    return O3D_ERR_BADARG;
  }
  c->learn_level = ll;
  const long long n2 = c->mg[ll].g.n;
  if (!c->feat) {
    int st = dalloc(c->s, (void**)&c->feat, (size_t)n2 * 2 * sizeof(float));
    if (!st) st = dalloc(c->s, (void**)&c->ynet, (size_t)n2 * sizeof(float));
    if (st) return st;
  }
  return O3D_OK;
}

// The start of a solve with the learned guess (or with training samples):
// p <- p_ex = 2 p(n) - p(n-1), p(n-1) <- p(n), the increment into the finest
// level's t; the FP64 residual of p_ex (the first outer iteration's, for
// multigrid) and the increment, restricted, form the network's input; the
// network's correction starts the first V-cycle (multigrid) or is added to p
// (SOR).  Everything is enqueued on the context's stream.
int enqueue_learned_first(o3d_ctx* c, bool learned, bool sampling, bool use_mg, int pre, int post,
                          long long* nl) {
  const int ll = c->learn_level;
  MGLevel* lv = c->mg.data();
  if (c->mixed) launch_learn_extrapolate<float>(c->pp, c->pp_prev, lv, c->s, nl, c->pdf);
  else launch_learn_extrapolate<double>(c->pp, c->pp_prev, lv, c->s, nl, false);
  if (use_mg) {
    if (c->mixed && c->rhs_f32) launch_mg_resid<float, float>(c->pp, c->rhs32, lv, c->ctrl, c->s, nl);
    else if (c->mixed) launch_mg_resid<float, double>(c->pp, (const double*)c->rhs, lv, c->ctrl, c->s, nl);
    else launch_mg_resid<double, double>(c->pp, (const double*)c->rhs, lv, c->ctrl, c->s, nl);
  } else {
    if (c->mixed) launch_level_kernel<float, double>(1, c->pp, (const double*)c->rhs, lv[0], c->ctrl, c->s, false);
    else launch_level_kernel<double, double>(1, c->pp, (const double*)c->rhs, lv[0], c->ctrl, c->s, false);
    *nl += 1;
  }
  if (c->mixed) launch_learn_features<float>(lv, ll, c->ctrl, c->feat, c->s, nl);
  else launch_learn_features<double>(lv, ll, c->ctrl, c->feat, c->s, nl);
  CKL();
  if (sampling) {
    CK(cudaMemcpyAsync(c->sample_feat, c->feat, (size_t)c->mg[ll].g.n * 2 * sizeof(float), cudaMemcpyDeviceToDevice,
                       c->s));
    c->sample_ready = 1;
  }
  if (learned) {
    int st = unet_enqueue_forward(c->unet, c->feat, c->ynet, c->s, nl);
    if (st) {
      errf("U-Net forward: %s", cudaGetErrorString(cudaGetLastError()));
      return st;
    }
    if (c->mixed) launch_learn_apply<float>(c->pp, c->ynet, lv, ll, !use_mg, c->ctrl, c->s, nl);
    else launch_learn_apply<double>(c->pp, c->ynet, lv, ll, !use_mg, c->ctrl, c->s, nl);
    CKL();
  }
  if (use_mg) {  // the rest of the first outer iteration, from the network's correction when learned
    const int cyc = mg_cycles_of(c);
    const double om = mg_omega_of(c);
    if (c->mixed)
      launch_mg_cycles<float>(c->pp, lv, (int)c->mg.size(), pre, post, MG_COARSE_SWEEPS, (float)om, cyc, learned,
                              c->ctrl, c->s, nl);
    else
      launch_mg_cycles<double>(c->pp, lv, (int)c->mg.size(), pre, post, MG_COARSE_SWEEPS, om, cyc, learned, c->ctrl,
                               c->s, nl);
    CKL();
  }
  return O3D_OK;
}

// Solves A pp = rhs with the context's solver; pp holds the initial guess.
int solve(o3d_ctx* c, double* omega_io, double eps, int kmax, int idyn, o3d_step_info* info) {
  if (c->p_in_wait) {  // o3d_step_host: the pressure upload overlapped the predictor and the rhs
    CK(cudaStreamWaitEvent(c->s, c->p_in_wait, 0));
    c->p_in_wait = nullptr;
    if (c->pdf) {
      launch_split_pair(c->stage[3], c->pp, c->g.n, c->s);
      c->launches++;
      CKL();
    }
  }
  const int guess = c->P.guess;
  const bool learned = guess == O3D_GUESS_LEARNED;
  const bool sampling = c->sample_feat != nullptr;
  const bool quad = guess == O3D_GUESS_EXTRAPOLATED2;
  const bool need_hist = guess == O3D_GUESS_EXTRAPOLATED || quad || learned || sampling;
  if (learned && !c->unet) {
    errf("the learned initial guess needs a network (o3d_attach_unet)");
    return O3D_ERR_NOT_BUILT;
  }
  if (need_hist && !c->pp_prev) {
    int st0 = dalloc(c->s, (void**)&c->pp_prev, (size_t)c->g.n * 8);
    if (st0) return st0;
  }
  if (quad && !c->pp_prev2) {
    int st0 = dalloc(c->s, (void**)&c->pp_prev2, (size_t)c->g.n * 8);
    if (st0) return st0;
  }
  if (sampling && (c->P.solver != O3D_SOLVER_MG || (guess != O3D_GUESS_EXTRAPOLATED && !learned))) {
    errf("training samples come from multigrid solves with the extrapolated or learned guess");
    return O3D_ERR_BADARG;
  }
  if ((learned || sampling)) {
    int st0 = learn_ready(c);
    if (st0) return st0;
  }
  if (guess == O3D_GUESS_ZERO) CK(cudaMemsetAsync(c->pp, 0, (size_t)c->g.n * 8, c->s));
  int st = reset_ctrl(c, *omega_io, eps, kmax, idyn);
  if (st) return st;
  CK(cudaEventRecord(c->ev[2], c->s));
  const bool use_mg = c->P.solver == O3D_SOLVER_MG;
  // an open x axis makes the all-Neumann problem incompatible (net flux
  // through inflow and outflow): every solver then takes the rhs less its mean
  const bool open_x = c->g.bc[0] == AX_OPEN;
  if (use_mg || learned || sampling || open_x) {
    // the weighted mean of the rhs (compatibility of the singular problem):
    // removed in place, except for the mixed multigrid solve, whose FP64
    // residual kernel subtracts it as it reads the rhs
    // (from the divergence kernel's sums once per rhs: a later solve of the
    // same, possibly shifted, rhs sums it again)
    if (c->rhs_wsum) launch_rhs_wmean_final(c->wpart, div_blocks<float>(c->g), c->gp, c->ctrl, c->s, &c->launches);
    else if (c->rhs_f32) launch_rhs_wmean<float>(c->rhs32, c->gp, c->part, c->ctrl, c->s, &c->launches);
    else launch_rhs_wmean<double>((const double*)c->rhs, c->gp, c->part, c->ctrl, c->s, &c->launches);
    c->rhs_wsum = 0;
    if (!(c->mixed && use_mg)) {
      launch_rhs_shift<double>((double*)c->rhs, c->g.n, c->ctrl, c->s);
      c->launches++;
    }
    CKL();
  }
  c->sample_ready = 0;
  int pre = 2, post = 2;
  mg_smooth_cfg(c, &pre, &post);
  if (use_mg) {
    if ((st = capture_mg(c))) return st;
  } else {
    if ((st = capture_sor(c))) return st;
  }
  if (need_hist) {
    if (c->pp_prev_valid && (learned || sampling)) {
      if (learned && use_mg && !sampling) {
        // replayed from a graph captured on first use
        cudaGraphExec_t& lexec = c->rhs_f32 ? c->learn_exec32 : c->learn_exec;
        long long& lnodes = c->rhs_f32 ? c->learn_nodes32 : c->learn_nodes;
        if (!lexec) {
          long long nl = 0;
          cudaGraph_t graph;
          CK(cudaStreamBeginCapture(c->s, cudaStreamCaptureModeThreadLocal));
          const int st1 = enqueue_learned_first(c, true, false, true, pre, post, &nl);
          const cudaError_t e1 = cudaStreamEndCapture(c->s, &graph);
          if (st1) {
            if (e1 == cudaSuccess) cudaGraphDestroy(graph);
            return st1;
          }
          CK(e1);
          const cudaError_t e2 = cudaGraphInstantiate(&lexec, graph, 0);
          cudaGraphDestroy(graph);
          CK(e2);
          lnodes = nl;
        }
        CK(cudaGraphLaunch(lexec, c->s));
        c->launches += lnodes;
      } else {
        if ((st = enqueue_learned_first(c, learned, sampling, use_mg, pre, post, &c->launches))) return st;
      }
    } else if (quad && c->pp_prev_valid && c->pp_prev2_valid) {
      // 3 p(n) - 3 p(n-1) + p(n-2); p(n) lands in pp_prev2's buffer, which
      // becomes pp_prev (the history shifts by a pointer swap, no copy)
      launch_extrapolate2(c->pp, c->pp_prev, c->pp_prev2, c->g.n, c->s, c->pdf);
      std::swap(c->pp_prev, c->pp_prev2);
      c->launches++;
      CKL();
    } else if (c->pp_prev_valid && (guess == O3D_GUESS_EXTRAPOLATED || quad)) {
      if (quad) {  // second solve: keep p(n-1) for the quadratic guess of the next one
        CK(cudaMemcpyAsync(c->pp_prev2, c->pp_prev, (size_t)c->g.n * 8, cudaMemcpyDeviceToDevice, c->s));
        c->pp_prev2_valid = 1;
      }
      launch_extrapolate(c->pp, c->pp_prev, c->g.n, c->s, c->pdf);
      c->launches++;
      CKL();
    } else {
      // first solve: no history yet, start from the previous pressure
      CK(cudaMemcpyAsync(c->pp_prev, c->pp, (size_t)c->g.n * 8, cudaMemcpyDeviceToDevice, c->s));
      c->pp_prev_valid = 1;
    }
  }
  for (;;) {
    if (use_mg) {
      CK(cudaGraphLaunch(c->rhs_f32 ? c->mg_exec32 : c->mg_exec, c->s));
      c->launches += c->rhs_f32 ? c->mg_nodes32 : c->mg_nodes;
    } else {
      CK(cudaGraphLaunch(c->sor_exec, c->s));
      c->launches += c->sor_nodes;
    }
    if ((st = read_ctrl(c))) return st;
    if (c->ctrl_h->done) break;
  }
  if (c->sample_ready && c->sample_tgt) {
    CK(cudaMemsetAsync(&c->ctrl->done, 0, sizeof(int), c->s));
    const long long n2 = c->mg[c->learn_level].g.n;
    if (c->mixed)
      launch_learn_target<float>(c->pp, c->pp_prev, c->mg.data(), c->learn_level, c->ctrl, c->feat + n2,
                                 c->sample_tgt, c->s, &c->launches);
    else
      launch_learn_target<double>(c->pp, c->pp_prev, c->mg.data(), c->learn_level, c->ctrl, c->feat + n2,
                                  c->sample_tgt, c->s, &c->launches);
    CKL();
    CK(cudaMemsetAsync(&c->ctrl->done, 0xff, sizeof(int), c->s));
  }
  // SOR: max |rhs - A p| of the final pressure; multigrid: max |r| of the
  // last outer iteration's residual, recorded by the loop itself (a second
  // FP64 pass would cost as much as a fifth of a cycle)
  if (!use_mg || c->P.diagnostics >= 2) {
    PoiCoef<double> pc = make_poi<double>(c->dx, c->dy, c->dz);
    CK(cudaMemsetAsync(&c->ctrl->res_key, 0, sizeof(unsigned long long), c->s));
    if (c->rhs_f32)
      launch_residual_inf<float>(c->pp, c->rhs32, c->gp, pc, c->ctrl, c->mixed && use_mg, c->s, c->pdf);
    else
      launch_residual_inf<double>(c->pp, (const double*)c->rhs, c->gp, pc, c->ctrl, c->mixed && use_mg, c->s,
                                  c->pdf);
    c->launches++;
    CKL();
  }
  CK(cudaEventRecord(c->ev[3], c->s));
  if ((st = read_ctrl(c))) return st;
  const SolveCtrl* h = c->ctrl_h;
  *omega_io = h->omega;
  if (info) {
    info->poisson_iters = h->iter;
    info->poisson_cycles = h->cycles;
    info->poisson_dmax = h->dmax;
    info->poisson_res_inf = (!use_mg || c->P.diagnostics >= 2) ? bits_to_double(h->res_key) : h->res_inf;
    info->omega = h->omega;
    float ms = 0.f;
    cudaEventElapsedTime(&ms, c->ev[2], c->ev[3]);
    info->poisson_ms = ms;
    info->poisson_status = h->status == 0 ? O3D_OK : h->status == 1 ? O3D_WARN_STAGNATION : O3D_WARN_POISSON_MAXIT;
  }
  return h->status == 0 ? O3D_OK : h->status == 1 ? O3D_WARN_STAGNATION : O3D_WARN_POISSON_MAXIT;
}

int check_params(const o3d_params* p) {
  if (p->nx < 8 || p->ny < 8 || p->nz < 8) {
    errf("grid too small: every axis needs at least 8 points (got %d x %d x %d)", p->nx, p->ny, p->nz);
    return O3D_ERR_BADARG;
  }
  if ((long long)p->nx * p->ny * p->nz > (1LL << 31)) {
    errf("grid of %lld points exceeds 2^31", (long long)p->nx * p->ny * p->nz);
    return O3D_ERR_BADARG;
  }
  auto bc_ok = [](int a, int b) { return (a == 0 && b == 0) || (a == 1 && b == 1); };
  const bool xopen = p->nbcx1 == 2 && p->nbcxn == 2;
  if (!xopen && !bc_ok(p->nbcx1, p->nbcxn)) { errf("unrecognized x boundary types nbcx1=%d nbcxn=%d", p->nbcx1, p->nbcxn); return O3D_ERR_BADARG; }
  if (xopen && !(p->nbcy1 == 1 && p->nbcyn == 1 && (p->sim2d || (p->nbcz1 == 1 && p->nbczn == 1)))) {
    errf("an open x axis (nbcx 2) needs free-slip y and z: its pressure problem is Neumann on every face");
    return O3D_ERR_BADARG;
  }
  if (!bc_ok(p->nbcy1, p->nbcyn)) { errf("unrecognized y boundary types nbcy1=%d nbcyn=%d", p->nbcy1, p->nbcyn); return O3D_ERR_BADARG; }
  if (!p->sim2d && !bc_ok(p->nbcz1, p->nbczn)) { errf("unrecognized z boundary types nbcz1=%d nbczn=%d", p->nbcz1, p->nbczn); return O3D_ERR_BADARG; }
  if (p->nbcx1 == 1 && p->nbcy1 == 0) {
    errf("no Poisson solver for free-slip x with periodic y");
    return O3D_ERR_BADARG;
  }
  if (p->itscheme < 1 || p->itscheme > 3) { errf("itscheme %d unrecognized", p->itscheme); return O3D_ERR_BADARG; }
  if (p->precision != O3D_PREC_FP64 && p->precision != O3D_PREC_MIXED) { errf("precision %d unknown", p->precision); return O3D_ERR_BADARG; }
  if (p->solver != O3D_SOLVER_SOR && p->solver != O3D_SOLVER_MG) { errf("solver %d unknown", p->solver); return O3D_ERR_BADARG; }
  if (p->mg_omega < 0.0 || p->mg_omega >= 2.0 || p->mg_pre < 0 || p->mg_post < 0 || p->mg_cycles < 0 ||
      p->mg_kernels < 0 || p->mg_kernels > 2) {
    errf("multigrid options out of range (mg_omega in [0, 2), sweep and cycle counts >= 0, mg_kernels 0..2)");
    return O3D_ERR_BADARG;
  }
  if (!(p->dt > 0.0) || !(p->re > 0.0) || !(p->xlx > 0.0) || !(p->yly > 0.0) || !(p->zlz > 0.0)) {
    errf("dt, re and the domain lengths must be positive");
    return O3D_ERR_BADARG;
  }
  return O3D_OK;
}

}  // namespace

// ===========================================================================
// C ABI
// ===========================================================================
extern "C" {

const char* o3d_last_error(void) { return g_err; }

void o3d_default_params(o3d_params* p) {
  memset(p, 0, sizeof *p);
  const double twopi = 2.0 * 3.14159265358979323846;
  p->nx = p->ny = p->nz = 64;
  p->xlx = p->yly = p->zlz = twopi * 63.0 / 64.0;  // dx = 2 pi / 64 on the node-inclusive grid
  p->itscheme = 3;
  p->dt = 0.2 * twopi / 64.0;
  p->re = 1600.0;
  p->omega = 2.0 / (1.0 + sin(3.14159265358979323846 * twopi / 64.0));
  p->eps = 1e-8;
  p->kmax = 2000;
  p->sc = 1.0;
  p->cs = 0.17;
  p->precision = O3D_PREC_FP64;
  p->solver = O3D_SOLVER_SOR;
  p->guess = O3D_GUESS_PREVIOUS;
  p->diagnostics = 1;
}

int o3d_create(const o3d_params* p, o3d_ctx** out) {
  if (!p || !out) { errf("null argument"); return O3D_ERR_BADARG; }
  *out = nullptr;
  int st = check_params(p);
  if (st) return st;
  o3d_ctx* c = new (std::nothrow) o3d_ctx();
  if (!c) return O3D_ERR_NOMEM;
  c->P = *p;
  c->mixed = p->precision == O3D_PREC_MIXED;
  c->pdf = c->mixed && p->solver == O3D_SOLVER_MG;
  c->esz = c->mixed ? 4 : 8;
  c->g.nx = p->nx; c->g.ny = p->ny; c->g.nz = p->nz;
  c->g.n = (long long)p->nx * p->ny * p->nz;
  c->g.bc[0] = p->nbcx1 == 0 ? AX_PERIODIC : p->nbcx1 == 1 ? AX_MIRROR : AX_OPEN;
  c->g.bc[1] = p->nbcy1 == 0 ? AX_PERIODIC : AX_MIRROR;
  c->g.bc[2] = p->sim2d ? AX_ZERO : (p->nbcz1 == 0 ? AX_PERIODIC : AX_MIRROR);
  // Poisson variant chosen from the x and y types (src/initialization.f90:283-301):
  // 0000 all periodic, 0011 y mirror, 111111 x, y and z mirror; an open x
  // axis takes dp/dx = 0 at inflow and outflow, the mirror remap
  c->gp = c->g;
  if (p->nbcx1 == 0 && p->nbcy1 == 0) { c->gp.bc[0] = c->gp.bc[1] = c->gp.bc[2] = AX_PERIODIC; }
  else if (p->nbcx1 == 0) { c->gp.bc[0] = AX_PERIODIC; c->gp.bc[1] = AX_MIRROR; c->gp.bc[2] = AX_PERIODIC; }
  else { c->gp.bc[0] = c->gp.bc[1] = c->gp.bc[2] = AX_MIRROR; }
  // src/initialization.f90:182-202
  c->dx = p->xlx / (double)(p->nx - 1);
  c->dy = p->yly / (double)(p->ny - 1);
  c->dz = p->zlz / (double)(p->nz - 1);
  c->delta = std::pow(c->dx * c->dy * c->dz, 1.0 / 3.0);
  const double dt = p->dt;
  c->adt[0] = dt; c->bdt[0] = 0.0; c->cdt[0] = 0.0;
  c->adt[1] = 3.0 * dt / 2.0; c->bdt[1] = -1.0 * dt / 2.0; c->cdt[1] = 0.0;
  c->adt[2] = 23.0 * dt / 12.0; c->bdt[2] = -16.0 * dt / 12.0; c->cdt[2] = 5.0 * dt / 12.0;
  c->omega = p->omega;
  make_coef(c->dx, c->cf.ax[0]);
  make_coef(c->dy, c->cf.ax[1]);
  make_coef(c->dz, c->cf.ax[2]);

  if (cudaStreamCreateWithFlags(&c->s, cudaStreamNonBlocking) != cudaSuccess) {
    snprintf(g_err, sizeof g_err, "cudaStreamCreate failed: %s", cudaGetErrorString(cudaGetLastError()));
    delete c;
    return O3D_ERR_CUDA;
  }
  for (int q = 0; q < 4; ++q) cudaEventCreate(&c->ev[q]);
  const size_t fb = fbytes(c);
  st = 0;
  for (int q = 0; q < 3 && !st; ++q) {
    st = st ? st : dalloc(c->s, &c->u[q], fb);
    st = st ? st : dalloc(c->s, &c->up[q], fb);
    for (int h = 0; h < 3 && !st; ++h) st = dalloc(c->s, &c->fu[q][h], fb);
  }
  st = st ? st : dalloc(c->s, &c->nu_t, fb);
  st = st ? st : dalloc(c->s, &c->rhs, (size_t)c->g.n * 8);
  if (p->precision == O3D_PREC_MIXED && p->solver == O3D_SOLVER_MG)
    st = st ? st : dalloc(c->s, (void**)&c->rhs32, (size_t)c->g.n * 4);
  st = st ? st : dalloc(c->s, (void**)&c->pp, (size_t)c->g.n * 8);
  if (!st && p->nscr) {
    st = st ? st : dalloc(c->s, &c->phi, fb);
    st = st ? st : dalloc(c->s, &c->phi2, fb);
    st = st ? st : dalloc(c->s, &c->src, fb);
    for (int h = 0; h < 3 && !st; ++h) st = dalloc(c->s, &c->fphi[h], fb);
  }
  const long long nb = pt_blocks(c->g) + 1;
  st = st ? st : dalloc(c->s, (void**)&c->part, (size_t)nb * 16 * sizeof(double));
  st = st ? st : dalloc(c->s, (void**)&c->spart, (size_t)nb * sizeof(StatPart));
  st = st ? st : dalloc(c->s, (void**)&c->wpart,
                        (size_t)std::max(z_blocks(c->g), div_blocks<float>(c->g)) * sizeof(double));
  st = st ? st : dalloc(c->s, (void**)&c->diag, sizeof(DevDiag));
  st = st ? st : dalloc(c->s, (void**)&c->ctrl, sizeof(SolveCtrl));
  if (!st && cudaMallocHost((void**)&c->diag_h, sizeof(DevDiag)) != cudaSuccess) st = O3D_ERR_NOMEM;
  if (!st && cudaMallocHost((void**)&c->ctrl_h, sizeof(SolveCtrl)) != cudaSuccess) st = O3D_ERR_NOMEM;
  if (!st && cudaStreamSynchronize(c->s) != cudaSuccess) st = O3D_ERR_CUDA;
  if (st) {
    o3d_destroy(c);
    return st;
  }
  *out = c;
  return O3D_OK;
}

int o3d_destroy(o3d_ctx* c) {
  if (!c) return O3D_OK;
  out_destroy(c->out);
  if (c->s) cudaStreamSynchronize(c->s);
  for (int q = 0; q < 3; ++q) {
    cudaFree(c->u[q]);
    cudaFree(c->up[q]);
    for (int h = 0; h < 3; ++h) cudaFree(c->fu[q][h]);
    cudaFree(c->fphi[q]);
  }
  cudaFree(c->nu_t); cudaFree(c->rhs); cudaFree(c->rhs32); cudaFree(c->pp); cudaFree(c->pp_prev);
  cudaFree(c->pp_prev2);
  cudaFree(c->feat); cudaFree(c->ynet);
  cudaFree(c->phi); cudaFree(c->phi2); cudaFree(c->src);
  for (int q = 0; q < 4; ++q) cudaFree(c->stage[q]);
  for (int q = 0; q < 3; ++q) cudaFree(c->uold[q]);
  for (int q = 0; q < 4; ++q) cudaFree(c->vout[q]);
  cudaFree(c->rscratch);
  cudaFree(c->part); cudaFree(c->spart); cudaFree(c->wpart); cudaFree(c->diag); cudaFree(c->ctrl);
  if (c->diag_h) cudaFreeHost(c->diag_h);
  if (c->ctrl_h) cudaFreeHost(c->ctrl_h);
  for (auto& L : c->mg) { cudaFree(L.e); cudaFree(L.r); cudaFree(L.t); }
  if (c->sor_exec) cudaGraphExecDestroy(c->sor_exec);
  if (c->mg_exec) cudaGraphExecDestroy(c->mg_exec);
  if (c->learn_exec) cudaGraphExecDestroy(c->learn_exec);
  if (c->mg_exec32) cudaGraphExecDestroy(c->mg_exec32);
  if (c->learn_exec32) cudaGraphExecDestroy(c->learn_exec32);
  for (int q = 0; q < 4; ++q) if (c->ev[q]) cudaEventDestroy(c->ev[q]);
  for (int q = 0; q < 8; ++q) if (c->xev[q]) cudaEventDestroy(c->xev[q]);
  if (c->xs) cudaStreamDestroy(c->xs);
  if (c->s) cudaStreamDestroy(c->s);
  delete c;
  return O3D_OK;
}

long long o3d_launch_count(const o3d_ctx* c) { return c ? c->launches : 0; }
void* o3d_stream(o3d_ctx* c) { return c ? (void*)c->s : nullptr; }

int o3d_upload(o3d_ctx* c, int field, const double* host) {
  if (!c || !host) return O3D_ERR_BADARG;
  bool is_pp;
  void* d = field_ptr(c, field, &is_pp);
  if (!d) { errf("field %d not allocated or unknown", field); return O3D_ERR_BADARG; }
  if (field == O3D_FIELD_RHS) {
    c->rhs_wsum = 0;
    c->rhs_f32 = 0;
  }
  if (field == O3D_FIELD_PP) {
    int st = put_pressure(c, c->pp, host);
    if (st) return st;
  } else if (is_pp) {
    CK(cudaMemcpyAsync(d, host, (size_t)c->g.n * 8, cudaMemcpyHostToDevice, c->s));
  } else {
    int st = put_field(c, d, host);
    if (st) return st;
  }
  CK(cudaStreamSynchronize(c->s));
  return O3D_OK;
}

int o3d_download(o3d_ctx* c, int field, double* host) {
  if (!c || !host) return O3D_ERR_BADARG;
  bool is_pp;
  void* d = field_ptr(c, field, &is_pp);
  if (!d) { errf("field %d not allocated or unknown", field); return O3D_ERR_BADARG; }
  if (field == O3D_FIELD_RHS && c->rhs_f32) {  // the step's FP32 rhs, widened exactly
    int st = get_field(c, c->rhs32, host);
    if (st) return st;
  } else if (field == O3D_FIELD_PP) {
    int st = get_pressure(c, c->pp, host);
    if (st) return st;
  } else if (is_pp) {
    CK(cudaMemcpyAsync(host, d, (size_t)c->g.n * 8, cudaMemcpyDeviceToHost, c->s));
  } else {
    int st = get_field(c, d, host);
    if (st) return st;
  }
  CK(cudaStreamSynchronize(c->s));
  return O3D_OK;
}

int o3d_der_dev(o3d_ctx* c, int axis, int order, int odd, const double* d_f, double* d_df) {
  if (!c || axis < 0 || axis > 2 || (order != 1 && order != 2)) { errf("bad derivative request"); return O3D_ERR_BADARG; }
  launch_der<double>(d_f, d_df, c->g, c->cf.ax[axis], axis, order, odd, c->s);
  c->launches++;
  CKL();
  return O3D_OK;
}

int o3d_der(o3d_ctx* c, int axis, int order, int odd, const double* f, double* df) {
  if (!c || !f || !df) return O3D_ERR_BADARG;
  int st = stage_ready(c, 1);
  if (st) return st;
  const size_t b = (size_t)c->g.n * 8;
  CK(cudaMemcpyAsync(c->stage[0], f, b, cudaMemcpyHostToDevice, c->s));
  if ((st = o3d_der_dev(c, axis, order, odd, c->stage[0], c->stage[1]))) return st;
  CK(cudaMemcpyAsync(df, c->stage[1], b, cudaMemcpyDeviceToHost, c->s));
  CK(cudaStreamSynchronize(c->s));
  return O3D_OK;
}

int o3d_divergence(o3d_ctx* c, const double* fx, const double* fy, const double* fz, int odd,
                   double* divf) {
  if (!c || !fx || !fy || !fz || !divf) return O3D_ERR_BADARG;
  int st = stage_ready(c, 3);
  if (st) return st;
  const size_t b = (size_t)c->g.n * 8;
  CK(cudaMemcpyAsync(c->stage[0], fx, b, cudaMemcpyHostToDevice, c->s));
  CK(cudaMemcpyAsync(c->stage[1], fy, b, cudaMemcpyHostToDevice, c->s));
  CK(cudaMemcpyAsync(c->stage[2], fz, b, cudaMemcpyHostToDevice, c->s));
  launch_div<double, double>(c->stage[0], c->stage[1], c->stage[2], c->stage[3], c->g, c->cf, odd, 1.0,
                             0, c->spart, c->s);
  c->launches++;
  CKL();
  CK(cudaMemcpyAsync(divf, c->stage[3], b, cudaMemcpyDeviceToHost, c->s));
  CK(cudaStreamSynchronize(c->s));
  return O3D_OK;
}

int o3d_calculate_nu_t(o3d_ctx* c) {
  if (!c) return O3D_ERR_BADARG;
  const double csd = c->P.cs * c->delta;
  if (c->mixed)
    launch_nu_t<float>((const float*)c->u[0], (const float*)c->u[1], (const float*)c->u[2], (float*)c->nu_t,
                       c->g, cast_coef<float>(c->cf), (float)(csd * csd), c->s);
  else
    launch_nu_t<double>((const double*)c->u[0], (const double*)c->u[1], (const double*)c->u[2],
                        (double*)c->nu_t, c->g, c->cf, csd * csd, c->s);
  c->launches++;
  CKL();
  CK(cudaStreamSynchronize(c->s));
  return O3D_OK;
}

int o3d_predict_velocity(o3d_ctx* c, int itime) {
  if (!c) return O3D_ERR_BADARG;
  int st = c->mixed ? predict_t<float>(c, itime) : predict_t<double>(c, itime);
  if (st) return st;
  CK(cudaStreamSynchronize(c->s));
  return O3D_OK;
}

int o3d_correct_pression(o3d_ctx* c, double* omega, o3d_step_info* info) {
  if (!c || !omega) return O3D_ERR_BADARG;
  int st = c->mixed ? rhs_t<float>(c) : rhs_t<double>(c);
  if (st) return st;
  return solve(c, omega, c->P.eps, c->P.kmax, c->P.idyn, info);
}

int o3d_correct_velocity(o3d_ctx* c) {
  if (!c) return O3D_ERR_BADARG;
  int st = c->mixed ? correct_t<float>(c) : correct_t<double>(c);
  if (st) return st;
  CK(cudaMemcpyAsync(c->diag_h, c->diag, sizeof(DevDiag), cudaMemcpyDeviceToHost, c->s));
  CK(cudaStreamSynchronize(c->s));
  const double* r = c->diag_h->sums;
  if (r[9] != 0.0 || r[3] > 1000.0 || r[4] > 1000.0 || r[5] > 1000.0) {
    errf("velocity diverged (NaN or max > 1000)");
    return O3D_ERR_NONFINITE;
  }
  return O3D_OK;
}

int o3d_transeq(o3d_ctx* c, int itime) {
  if (!c) return O3D_ERR_BADARG;
  if (!c->phi) { errf("scalar transport needs nscr = 1 at creation"); return O3D_ERR_BADARG; }
  int st = c->mixed ? transeq_t<float>(c, itime) : transeq_t<double>(c, itime);
  if (st) return st;
  CK(cudaStreamSynchronize(c->s));
  return O3D_OK;
}

int o3d_poisson_solve(o3d_ctx* c, double* pp, const double* rhs, double* omega, double eps, int kmax,
                      int idyn, int* iters, double* dmax) {
  if (!c || !pp || !rhs || !omega) return O3D_ERR_BADARG;
  int pst = put_pressure(c, c->pp, pp);
  if (pst) return pst;
  CK(cudaMemcpyAsync(c->rhs, rhs, (size_t)c->g.n * 8, cudaMemcpyHostToDevice, c->s));
  c->rhs_wsum = 0;  // a caller's rhs: its mean takes the separate pass
  c->rhs_f32 = 0;
  int st = O3D_OK;
  o3d_step_info info;
  memset(&info, 0, sizeof info);
  const int guess = c->P.guess;
  c->P.guess = O3D_GUESS_PREVIOUS;  // pp is the caller's initial guess
  int rs = solve(c, omega, eps, kmax, idyn, &info);
  c->P.guess = guess;
  if (rs < 0) return rs;
  if ((pst = get_pressure(c, c->pp, pp))) return pst;
  CK(cudaStreamSynchronize(c->s));
  if (iters) *iters = info.poisson_iters;
  if (dmax) *dmax = info.poisson_dmax;
  return rs;
}

int o3d_step(o3d_ctx* c, int itime, o3d_step_info* info) {
  if (!c) return O3D_ERR_BADARG;
  o3d_step_info loc;
  if (!info) info = &loc;
  memset(info, 0, sizeof *info);
  CK(cudaEventRecord(c->ev[0], c->s));
  int st = c->mixed ? predict_t<float>(c, itime) : predict_t<double>(c, itime);
  if (st) return st;
  st = c->mixed ? rhs_t<float>(c) : rhs_t<double>(c);
  if (st) return st;
  const int ps = solve(c, &c->omega, c->P.eps, c->P.kmax, c->P.idyn, info);
  if (ps < 0) return ps;
  if (c->p_out_host) {  // o3d_step_host: the final pressure goes out while the step finishes
    const double* src = c->pp;
    if (c->pdf) {  // joined to FP64 in stage 3 first
      launch_join_pair(c->pp, c->stage[3], c->g.n, c->s);
      c->launches++;
      CKL();
      src = c->stage[3];
    }
    CK(cudaEventRecord(c->xev[5], c->s));
    CK(cudaStreamWaitEvent(c->xs, c->xev[5], 0));
    CK(cudaMemcpyAsync(c->p_out_host, src, (size_t)c->g.n * 8, cudaMemcpyDeviceToHost, c->xs));
    c->p_out_host = nullptr;
  }
  st = c->mixed ? correct_t<float>(c) : correct_t<double>(c);
  if (st) return st;
  if (c->P.nscr) {
    st = c->mixed ? transeq_t<float>(c, itime) : transeq_t<double>(c, itime);
    if (st) return st;
  }
  if (c->P.diagnostics) {
    st = c->mixed ? divu_diag_t<float>(c) : divu_diag_t<double>(c);
    if (st) return st;
  }
  CK(cudaEventRecord(c->ev[1], c->s));
  CK(cudaMemcpyAsync(c->diag_h, c->diag, sizeof(DevDiag), cudaMemcpyDeviceToHost, c->s));
  CK(cudaStreamSynchronize(c->s));
  const DevDiag* d = c->diag_h;
  for (int q = 0; q < 6; ++q) {
    info->divu_pred_stats[q] = d->divp[q];
    info->divu_stats[q] = d->divu[q];
  }
  const double h[3] = {c->dx, c->dy, c->dz};
  for (int a = 0; a < 3; ++a) {
    info->umin[a] = d->sums[a];
    info->umax[a] = d->sums[3 + a];
    info->cfl[a] = d->sums[6 + a] * c->P.dt / h[a];
  }
  info->diverged = d->sums[9] != 0.0 || d->sums[3] > 1000.0 || d->sums[4] > 1000.0 || d->sums[5] > 1000.0;
  float ms = 0.f;
  cudaEventElapsedTime(&ms, c->ev[0], c->ev[1]);
  info->step_ms = ms;
  if (info->diverged) {
    errf("velocity diverged at step %d (NaN or max > 1000)", itime);
    return O3D_ERR_NONFINITE;
  }
  return ps;
}

int o3d_step_host(o3d_ctx* c, int itime, double* ux, double* uy, double* uz, double* pp,
                  o3d_step_info* info) {
  if (!c || !ux || !uy || !uz || !pp) return O3D_ERR_BADARG;
  int st;
  if (!c->xs) {
    CK(cudaStreamCreateWithFlags(&c->xs, cudaStreamNonBlocking));
    for (int q = 0; q < 8; ++q) CK(cudaEventCreateWithFlags(&c->xev[q], cudaEventDisableTiming));
  }
  if (c->mixed && (st = stage_ready(c, c->pdf ? 3 : 2))) return st;
  double* const hu[3] = {ux, uy, uz};
  const size_t bytes = (size_t)c->g.n * 8;
  // inputs: copied on the copy stream (after earlier work of the context
  // stream), each velocity converted on the context stream once it landed
  CK(cudaEventRecord(c->xev[7], c->s));
  CK(cudaStreamWaitEvent(c->xs, c->xev[7], 0));
  for (int k = 0; k < 3; ++k) {
    if (c->mixed) {
      CK(cudaMemcpyAsync(c->stage[k], hu[k], bytes, cudaMemcpyHostToDevice, c->xs));
      CK(cudaEventRecord(c->xev[k], c->xs));
      CK(cudaStreamWaitEvent(c->s, c->xev[k], 0));
      launch_convert<double, float>(c->stage[k], (float*)c->u[k], c->g.n, c->s);
      c->launches++;
    } else {
      CK(cudaMemcpyAsync(c->u[k], hu[k], bytes, cudaMemcpyHostToDevice, c->xs));
    }
  }
  if (!c->mixed) {
    CK(cudaEventRecord(c->xev[2], c->xs));
    CK(cudaStreamWaitEvent(c->s, c->xev[2], 0));
  }
  // the pressure lands while the predictor and the rhs run (the solve waits
  // for it) and leaves as soon as the solve ends (o3d_step issues the copy)
  // (with pdf into stage 3, split into the pair by solve() once it landed)
  CK(cudaMemcpyAsync(c->pdf ? (void*)c->stage[3] : (void*)c->pp, pp, bytes, cudaMemcpyHostToDevice, c->xs));
  CK(cudaEventRecord(c->xev[3], c->xs));
  c->p_in_wait = c->xev[3];
  c->p_out_host = pp;
  CKL();
  const int rs = o3d_step(c, itime, info);
  c->p_in_wait = nullptr;
  c->p_out_host = nullptr;
  if (rs < 0) {
    cudaStreamSynchronize(c->xs);
    return rs;
  }
  // outputs: each velocity as soon as it is converted
  CK(cudaEventRecord(c->xev[4], c->s));
  CK(cudaStreamWaitEvent(c->xs, c->xev[4], 0));
  for (int k = 0; k < 3; ++k) {
    if (c->mixed) {
      launch_convert<float, double>((const float*)c->u[k], c->stage[k], c->g.n, c->s);
      c->launches++;
      CK(cudaEventRecord(c->xev[k], c->s));
      CK(cudaStreamWaitEvent(c->xs, c->xev[k], 0));
      CK(cudaMemcpyAsync(hu[k], c->stage[k], bytes, cudaMemcpyDeviceToHost, c->xs));
    } else {
      CK(cudaMemcpyAsync(hu[k], c->u[k], bytes, cudaMemcpyDeviceToHost, c->xs));
    }
  }
  CKL();
  CK(cudaStreamSynchronize(c->xs));
  return rs;
}

int o3d_statistics_calc(o3d_ctx* c, double t, double out[17]) {
  if (!c || !out) return O3D_ERR_BADARG;
  const double xnu = 1.0 / c->P.re;
  if (c->mixed)
    launch_stats<float>((const float*)c->u[0], (const float*)c->u[1], (const float*)c->u[2], c->g,
                        cast_coef<float>(c->cf), xnu, c->part, c->s);
  else
    launch_stats<double>((const double*)c->u[0], (const double*)c->u[1], (const double*)c->u[2], c->g,
                         c->cf, xnu, c->part, c->s);
  launch_finalize(c->part, pt_blocks(c->g), 16, 0ull, c->diag->sums, c->s);
  c->launches += 2;
  CKL();
  CK(cudaMemcpyAsync(c->diag_h, c->diag, sizeof(DevDiag), cudaMemcpyDeviceToHost, c->s));
  CK(cudaStreamSynchronize(c->s));
  const double* S = c->diag_h->sums;
  const double N = (double)c->g.n;
  out[0] = t;
  out[1] = S[12] / N;
  out[2] = S[13] / N;
  out[3] = S[15] / N;
  out[4] = S[14] / N;
  for (int q = 0; q < 3; ++q) out[5 + q] = S[q] / N;
  for (int q = 0; q < 9; ++q) out[8 + q] = S[3 + q] / N;
  return O3D_OK;
}

}  // extern "C"

namespace o3d {
int ctx_geometry(o3d_ctx* c, o3d_params* p, int* nx, int* ny, int* nz, double* dx, double* dy, double* dz) {
  *p = c->P;
  *nx = c->g.nx; *ny = c->g.ny; *nz = c->g.nz;
  *dx = c->dx; *dy = c->dy; *dz = c->dz;
  return O3D_OK;
}

int ctx_history_state(o3d_ctx* c, double* omega, int* nprev, double* prev_host, int which) {
  if (omega) *omega = c->omega;
  const int n = !(c->pp_prev && c->pp_prev_valid) ? 0 : (c->pp_prev2 && c->pp_prev2_valid ? 2 : 1);
  if (nprev) *nprev = n;
  if (prev_host && which >= 1 && which <= n) {
    int st = get_pressure(c, which == 1 ? c->pp_prev : c->pp_prev2, prev_host);
    if (st) return st;
    CK(cudaStreamSynchronize(c->s));
  }
  return O3D_OK;
}

int ctx_pressure_pairs(const o3d_ctx* c) { return c->pdf; }

int ctx_pressure_raw(o3d_ctx* c, int which, void* host, int to_device) {
  double** buf = which == 0 ? &c->pp : which == 1 ? &c->pp_prev : &c->pp_prev2;
  const size_t bytes = (size_t)c->g.n * 8;
  if (to_device) {
    if (!*buf) {
      int st = dalloc(c->s, (void**)buf, bytes);
      if (st) return st;
    }
    CK(cudaMemcpyAsync(*buf, host, bytes, cudaMemcpyHostToDevice, c->s));
    if (which == 1) c->pp_prev_valid = 1;
    if (which == 2) c->pp_prev2_valid = 1;
  } else {
    if (!*buf) {
      errf("no pressure buffer %d to read", which);
      return O3D_ERR_BADARG;
    }
    CK(cudaMemcpyAsync(host, *buf, bytes, cudaMemcpyDeviceToHost, c->s));
  }
  CK(cudaStreamSynchronize(c->s));
  return O3D_OK;
}

int ctx_restore_history(o3d_ctx* c, double omega, int nprev, const double* prev1, const double* prev2) {
  c->omega = omega;
  c->pp_prev_valid = 0;
  c->pp_prev2_valid = 0;
  const double* host[2] = {prev1, prev2};
  double** dev[2] = {&c->pp_prev, &c->pp_prev2};
  for (int q = 0; q < nprev && q < 2; ++q) {
    if (!*dev[q]) {
      int st = dalloc(c->s, (void**)dev[q], (size_t)c->g.n * 8);
      if (st) return st;
    }
    int st = put_pressure(c, *dev[q], host[q]);
    if (st) return st;
  }
  CK(cudaStreamSynchronize(c->s));
  c->pp_prev_valid = nprev >= 1;
  c->pp_prev2_valid = nprev >= 2;
  return O3D_OK;
}
}  // namespace o3d

extern "C" {

int o3d_vorticity(o3d_ctx* c, double* rotx, double* roty, double* rotz, double* q) {
  if (!c) return O3D_ERR_BADARG;
  double* host[4] = {rotx, roty, rotz, q};
  const size_t tsz = c->mixed ? 4 : 8;
  for (int k = 0; k < 4; ++k)
    if (host[k] && !c->vout[k]) {
      int st = dalloc(c->s, &c->vout[k], (size_t)c->g.n * tsz);
      if (st) return st;
    }
  void* out[4];
  for (int k = 0; k < 4; ++k) out[k] = host[k] ? c->vout[k] : nullptr;
  if (c->mixed) {
    const float* u[3] = {(const float*)c->u[0], (const float*)c->u[1], (const float*)c->u[2]};
    launch_vorticity<float>(u, (float*)out[0], (float*)out[1], (float*)out[2], (float*)out[3], c->g,
                            cast_coef<float>(c->cf), c->s);
  } else {
    const double* u[3] = {(const double*)c->u[0], (const double*)c->u[1], (const double*)c->u[2]};
    launch_vorticity<double>(u, (double*)out[0], (double*)out[1], (double*)out[2], (double*)out[3], c->g, c->cf,
                             c->s);
  }
  c->launches++;
  CKL();
  for (int k = 0; k < 4; ++k)
    if (host[k]) {
      int st = get_field(c, out[k], host[k]);
      if (st) return st;
    }
  CK(cudaStreamSynchronize(c->s));
  return O3D_OK;
}

int o3d_save_old_velocity(o3d_ctx* c) {
  if (!c) return O3D_ERR_BADARG;
  const size_t bytes = (size_t)c->g.n * (c->mixed ? 4 : 8);
  for (int a = 0; a < 3; ++a) {
    if (!c->uold[a]) {
      int st = dalloc(c->s, &c->uold[a], bytes);
      if (st) return st;
    }
    CK(cudaMemcpyAsync(c->uold[a], c->u[a], bytes, cudaMemcpyDeviceToDevice, c->s));
  }
  return O3D_OK;
}

int o3d_velocity_residuals(o3d_ctx* c, double t_ref, double u_ref, double out[15]) {
  if (!c || !out) return O3D_ERR_BADARG;
  if (!c->uold[0]) {
    errf("o3d_velocity_residuals needs o3d_save_old_velocity first");
    return O3D_ERR_BADARG;
  }
  if (!c->rscratch) {
    int st = dalloc(c->s, &c->rscratch, vel_residual_scratch_bytes(c->g));
    if (st) return st;
  }
  if (c->mixed) {
    const float* u[3] = {(const float*)c->u[0], (const float*)c->u[1], (const float*)c->u[2]};
    const float* o[3] = {(const float*)c->uold[0], (const float*)c->uold[1], (const float*)c->uold[2]};
    launch_vel_residuals<float>(u, o, c->g, c->P.dt, c->rscratch, c->s);
  } else {
    const double* u[3] = {(const double*)c->u[0], (const double*)c->u[1], (const double*)c->u[2]};
    const double* o[3] = {(const double*)c->uold[0], (const double*)c->uold[1], (const double*)c->uold[2]};
    launch_vel_residuals<double>(u, o, c->g, c->P.dt, c->rscratch, c->s);
  }
  c->launches += 2;
  CKL();
  struct { double sum, mx; long long imx; } r[3];
  CK(cudaMemcpyAsync(r, (const char*)c->rscratch + vel_residual_result_offset(c->g), sizeof r,
                     cudaMemcpyDeviceToHost, c->s));
  CK(cudaStreamSynchronize(c->s));
  const double scale = t_ref / u_ref, N = (double)c->g.n;
  for (int a = 0; a < 3; ++a) {
    out[a] = scale * std::sqrt((1.0 / N) * r[a].sum);
    out[3 + a] = scale * (r[a].mx > 0.0 ? r[a].mx : 0.0);
    const long long p = r[a].imx < 0 ? 0 : r[a].imx;
    out[6 + 3 * a] = (double)(p % c->g.nx + 1);
    out[7 + 3 * a] = (double)((p / c->g.nx) % c->g.ny + 1);
    out[8 + 3 * a] = (double)(p / ((long long)c->g.nx * c->g.ny) + 1);
  }
  return O3D_OK;
}

int o3d_rbsor_sweeps_dev(o3d_ctx* c, double* d_pp, const double* d_rhs, double omega, int nsweeps,
                         double* dmax_last) {
  if (!c || !d_pp || !d_rhs || nsweeps < 1) return O3D_ERR_BADARG;
  PoiCoef<double> pc = make_poi<double>(c->dx, c->dy, c->dz);
  int st = reset_ctrl(c, omega, 0.0, 1 << 30, 0);
  if (st) return st;
  for (int q = 0; q < nsweeps; ++q) {
    if (q == nsweeps - 1) CK(cudaMemsetAsync(&c->ctrl->dmax_key, 0, 8, c->s));
    launch_sor_fixed(d_pp, d_rhs, c->gp, pc, omega, c->ctrl, c->s);
    c->launches += 2;
  }
  CKL();
  if ((st = read_ctrl(c))) return st;
  if (dmax_last) *dmax_last = bits_to_double(c->ctrl_h->dmax_key);
  return O3D_OK;
}

int o3d_attach_unet(o3d_ctx* c, o3d_unet* net) {
  if (!c) return O3D_ERR_BADARG;
  if (c->learn_exec || c->learn_exec32) {
    CK(cudaStreamSynchronize(c->s));
    if (c->learn_exec) cudaGraphExecDestroy(c->learn_exec);
    if (c->learn_exec32) cudaGraphExecDestroy(c->learn_exec32);
    c->learn_exec = nullptr;
    c->learn_exec32 = nullptr;
  }
  c->unet = net;
  if (!net) return O3D_OK;
  if (unet_sync(net)) {
    errf("the network's queued work failed");
    return O3D_ERR_CUDA;
  }
  int st = learn_ready(c);
  if (st) return st;
  int nx, ny, nz, nin;
  unet_grid(net, &nx, &ny, &nz, &nin);
  const Grid& g2 = c->mg[c->learn_level].g;
  if (nx != g2.nx || ny != g2.ny || nz != g2.nz || nin != 2) {
    c->unet = nullptr;
    errf("network grid %d x %d x %d (%d inputs) differs from the guess grid %d x %d x %d (2 inputs)", nx, ny, nz, nin,
         g2.nx, g2.ny, g2.nz);
    return O3D_ERR_BADARG;
  }
  CK(cudaStreamSynchronize(c->s));
  return O3D_OK;
}

int o3d_guess_grid(o3d_ctx* c, int dims[3]) {
  if (!c || !dims) return O3D_ERR_BADARG;
  int st = learn_ready(c);
  if (st) return st;
  dims[0] = c->mg[c->learn_level].g.nx;
  dims[1] = c->mg[c->learn_level].g.ny;
  dims[2] = c->mg[c->learn_level].g.nz;
  CK(cudaStreamSynchronize(c->s));
  return O3D_OK;
}

int o3d_set_sample_buffers(o3d_ctx* c, float* d_feat, float* d_tgt) {
  if (!c) return O3D_ERR_BADARG;
  if ((d_feat == nullptr) != (d_tgt == nullptr)) {
    errf("sample buffers: give both the feature and the target buffer, or neither");
    return O3D_ERR_BADARG;
  }
  if (d_feat) {
    int st = learn_ready(c);
    if (st) return st;
  }
  c->sample_feat = d_feat;
  c->sample_tgt = d_tgt;
  c->sample_ready = 0;
  return O3D_OK;
}

int o3d_sample_ready(const o3d_ctx* c) { return c ? c->sample_ready : 0; }

int o3d_time_kernel(o3d_ctx* c, int kernel, int reps, double* ms_per_launch) {
  if (!c || reps < 1 || !ms_per_launch || kernel < 0 || kernel > 11) {
    errf("bad o3d_time_kernel request");
    return O3D_ERR_BADARG;
  }
  double* p_scratch = nullptr;
  if (kernel >= 3) {
    if (!c->mg_ok) {
      int st = build_mg(c);
      if (st) return st;
    }
    if (kernel >= 5 && kernel != 7 && kernel != 8 && !(c->mg.size() > 1 && c->mg[0].fused)) {
      errf("o3d_time_kernel: the finest level does not run the fused multigrid kernels");
      return O3D_ERR_BADARG;
    }
    if (kernel == 6 || kernel == 11) {
      CK(cudaMalloc(&p_scratch, (size_t)c->g.n * 8));
      CK(cudaMemcpyAsync(p_scratch, c->pp, (size_t)c->g.n * 8, cudaMemcpyDeviceToDevice, c->s));
    }
    // the multigrid kernels return at once on a finished solve: re-open it
    CK(cudaMemsetAsync(&c->ctrl->done, 0, sizeof(int), c->s));
  }
  auto launch = [&]() -> int {
    switch (kernel) {
      case 0: {
        // predictor on the live state, without rotating the flux ring
        void* saved[3][3];
        memcpy(saved, c->fu, sizeof saved);
        int st = c->mixed ? predict_t<float>(c, 3) : predict_t<double>(c, 3);
        memcpy(c->fu, saved, sizeof saved);
        return st;
      }
      case 1: return c->mixed ? rhs_t<float>(c) : rhs_t<double>(c);
      case 2: return c->mixed ? correct_t<float>(c) : correct_t<double>(c);
      case 5:
      case 6: {
        int pre, post;
        mg_smooth_cfg(c, &pre, &post);
        const float om = (float)mg_omega_of(c);
        if (kernel == 5) launch_mg_down(c->mg[0], c->mg[1], om, pre, true, c->ctrl, c->s);
        else launch_mg_up(c->mg[0], c->mg[1], om, post, p_scratch, c->ctrl, c->s);
        c->launches++;
        CKL();
        return O3D_OK;
      }
      case 9:
      case 10:
      case 11:
        launch_post_pass(kernel - 9, c->mg[0], c->mg[1], (float)mg_omega_of(c), p_scratch, c->ctrl, c->s);
        c->launches++;
        CKL();
        return O3D_OK;
      case 7:
      case 8:
        if (c->mixed) launch_level_kernel<float, float>(kernel - 5, c->pp, c->rhs32, c->mg[0], c->ctrl, c->s, c->pdf);
        else launch_level_kernel<double, double>(kernel - 5, c->pp, (const double*)c->rhs, c->mg[0], c->ctrl, c->s, false);
        c->launches++;
        CKL();
        return O3D_OK;
      default:
        if (c->mixed && c->rhs_f32)
          launch_level_kernel<float, float>(kernel - 3, c->pp, c->rhs32, c->mg[0], c->ctrl, c->s, c->pdf);
        else if (c->mixed)
          launch_level_kernel<float, double>(kernel - 3, c->pp, (const double*)c->rhs, c->mg[0], c->ctrl, c->s,
                                             c->pdf);
        else
          launch_level_kernel<double, double>(kernel - 3, c->pp, (const double*)c->rhs, c->mg[0], c->ctrl, c->s,
                                              false);
        c->launches++;
        CKL();
        return O3D_OK;
    }
  };
  int st = launch();  // warm
  if (st) return st;
  CK(cudaEventRecord(c->ev[2], c->s));
  for (int q = 0; q < reps; ++q)
    if ((st = launch())) return st;
  CK(cudaEventRecord(c->ev[3], c->s));
  CK(cudaEventSynchronize(c->ev[3]));
  float ms = 0.f;
  CK(cudaEventElapsedTime(&ms, c->ev[2], c->ev[3]));
  *ms_per_launch = ms / reps;
  if (kernel >= 3) CK(cudaMemsetAsync(&c->ctrl->done, 0xff, sizeof(int), c->s));
  CK(cudaStreamSynchronize(c->s));
  if (p_scratch) CK(cudaFree(p_scratch));
  return O3D_OK;
}

}  // extern "C"

int o3d_write_output(o3d_ctx* c, const char* dir, int num, double time) {
  if (!c || !dir) return O3D_ERR_BADARG;
  const char* names[8] = {"ux", "uy", "uz", "pp", "vort", "qcrit", nullptr, nullptr};
  int nf = 6;
  if (c->P.nscr == 1) names[nf++] = "phi";
  if (c->P.iles == 1) names[nf++] = "nu_t";
  double* snap = nullptr;
  int st = out_prepare(&c->out, c->g.n, nf, &snap);
  if (st) return st;
  const long long n = c->g.n;
  double* outs[5] = {snap, snap + n, snap + 2 * n, snap + 4 * n, snap + 5 * n};
  if (c->mixed) {
    const float* u[3] = {(const float*)c->u[0], (const float*)c->u[1], (const float*)c->u[2]};
    launch_out_snapshot<float>(u, outs, c->g, cast_coef<float>(c->cf), c->s);
  } else {
    const double* u[3] = {(const double*)c->u[0], (const double*)c->u[1], (const double*)c->u[2]};
    launch_out_snapshot<double>(u, outs, c->g, c->cf, c->s);
  }
  c->launches++;
  CKL();
  if (c->pdf) launch_join_pair(c->pp, snap + 3 * n, n, c->s);
  else CK(cudaMemcpyAsync(snap + 3 * n, c->pp, (size_t)n * 8, cudaMemcpyDeviceToDevice, c->s));
  int q = 6;
  for (void* f : {c->P.nscr == 1 ? c->phi : nullptr, c->P.iles == 1 ? c->nu_t : nullptr}) {
    if (!f) continue;
    if (c->mixed) {
      launch_convert<float, double>((const float*)f, snap + (size_t)q * n, n, c->s);
      c->launches++;
      CKL();
    } else {
      CK(cudaMemcpyAsync(snap + (size_t)q * n, f, (size_t)n * 8, cudaMemcpyDeviceToDevice, c->s));
    }
    ++q;
  }
  OutRequest r;
  r.dir = dir;
  r.num = num;
  r.time = time;
  r.nx = c->g.nx;
  r.ny = c->g.ny;
  r.nz = c->g.nz;
  r.dx = c->dx;
  r.dy = c->dy;
  r.dz = c->dz;
  r.x0 = c->P.x0;
  r.y0 = c->P.y0;
  r.z0 = c->P.z0;
  return out_submit(c->out, r, names, nf, c->s);
}

int o3d_output_wait(o3d_ctx* c) {
  if (!c) return O3D_ERR_BADARG;
  return out_wait(c->out);
}
