// o3d_kernels.h -- argument blocks and launchers shared by the kernel files
// and the host orchestration in o3d_api.cu.
#pragma once

#include "o3d_internal.cuh"

struct o3d_unet;

namespace o3d {

// the network of the learned guess (o3d_unet_host.cu)
int unet_enqueue_forward(o3d_unet* n, const float* d_in, float* d_out, cudaStream_t s, long long* nl);
int unet_sync(o3d_unet* n);
int unet_grid(const o3d_unet* n, int* nx, int* ny, int* nz, int* in_ch);

template <class T>
struct PredArgs {
  const T* u[3];
  T* up[3];
  T* fnew[3];
  const T* f2[3];  // previous flux (nullptr when its AB weight is zero)
  const T* f3[3];  // flux two steps back (nullptr when its AB weight is zero)
  T* nu_t;
  Grid g;
  Coef3<T> cf;
  T adu, bdu, cdu, onere, csd2;
  int les;
};

template <class T, class P>
struct CorrArgs {
  const P* p;
  const T* up[3];
  T* u[3];
  Grid g;
  Coef3<T> cf;
  T dt;
  double* part;  // 10 doubles per block: min[3], max[3], |max|[3], nan
};

template <class T>
struct ScalArgs {
  const T* phi;
  T* phi_out;
  const T* u[3];
  const T* src;
  const T* nu_t;
  T* fnew;
  const T* f2;
  const T* f3;
  Grid g;
  Coef3<T> cf;
  T adu, bdu, cdu, alpha0, sc;
  int les;
  double* part;  // 3 doubles per block
};

void set_error(const char* fmt, ...);

long long pt_blocks(const Grid& g);
// blocks of the z-marching (2.5D) kernels: divergence and correction
long long z_blocks(const Grid& g);
// blocks (statistics and weighted-sum records) of the divergence kernel that
// launch_div runs for field type T, and of the correction kernel of
// launch_correct
template <class T>
long long div_blocks(const Grid& g);
template <class T>
long long corr_blocks(const Grid& g);

template <class T>
void launch_der(const T* f, T* df, const Grid& g, const AxisCoef<T>& c, int axis, int order,
                int odd, cudaStream_t s);
// output snapshot: u, v, w in FP64, |curl u| and Q into out[0..4]
template <class T>
void launch_out_snapshot(const T* const u[3], double* const out[5], const Grid& g, const Coef3<T>& cf,
                         cudaStream_t s);
template <class T>
void launch_predict(const PredArgs<T>& a, cudaStream_t s);
// the FP32 2.5D kernels with two x-adjacent points per thread
// (k_stencil25v.cu), for grids with nx a multiple of 4
bool stencil_v_ok(const Grid& g);
void launch_predict_v(const PredArgs<float>& a, cudaStream_t s);
template <class O>
void launch_div_v(const float* fx, const float* fy, const float* fz, O* out, const Grid& g, const Coef3<float>& cf,
                  int odd, float dt, int divide, StatPart* part, cudaStream_t s, double* wpart, int wmask);
void launch_correct_v(const CorrArgs<float, double>& a, cudaStream_t s);
void launch_correct_v(const CorrArgs<float, float>& a, cudaStream_t s);
long long div_v_blocks(const Grid& g);
long long corr_v_blocks(const Grid& g);
void launch_transeq_v(const ScalArgs<float>& a, cudaStream_t s);
long long transeq_v_blocks(const Grid& g);
// planes per block of the two-point kernels for `per_sm` resident blocks
int v_chunk(const Grid& g, int per_sm);
template <class T>
void launch_nu_t(const T* ux, const T* uy, const T* uz, T* nu, const Grid& g, const Coef3<T>& cf,
                 T csd2, cudaStream_t s);
template <class T, class O>
void launch_div(const T* fx, const T* fy, const T* fz, O* out, const Grid& g, const Coef3<T>& cf,
                int odd, T dt, int divide, StatPart* part, cudaStream_t s, double* wpart = nullptr,
                int wmask = 0);
template <class T, class P>
void launch_correct(const CorrArgs<T, P>& a, cudaStream_t s);
template <class T>
void launch_stats(const T* ux, const T* uy, const T* uz, const Grid& g, const Coef3<T>& cf,
                  double xnu, double* part, cudaStream_t s);
template <class T>
void launch_transeq(const ScalArgs<T>& a, const double* sums, cudaStream_t s, long long* nl);
void launch_finalize(const double* part, long long nblk, int M, unsigned long long opmask,
                     double* out, cudaStream_t s);
void launch_finalize_stats(const StatPart* part, long long nblk, const Grid& g, double* out6,
                           cudaStream_t s);
template <class S, class D>
void launch_convert(const S* s_, D* d, long long n, cudaStream_t s);
// FP64 field <-> double-float pair buffer (PPair layout: hi plane, lo plane)
void launch_split_pair(const double* x, void* pair, long long n, cudaStream_t s);
void launch_join_pair(const void* pair, double* x, long long n, cudaStream_t s);

// ---- pressure solve (k_poisson.cu) ----------------------------------------

// 7-point operator of src/poisson.f90:95-98 on one grid level.
template <class T>
struct PoiCoef {
  T ox, oy, oz;   // 1/dx^2, 1/dy^2, 1/dz^2
  T A;            // -(2/dx^2 + 2/dy^2 + 2/dz^2)
  T invA;
};
template <class T>
inline PoiCoef<T> make_poi(double dx, double dy, double dz) {
  PoiCoef<T> c;
  double ox = 1.0 / (dx * dx), oy = 1.0 / (dy * dy), oz = 1.0 / (dz * dz);
  double A = -(2.0 * ox + 2.0 * oy + 2.0 * oz);
  c.ox = (T)ox; c.oy = (T)oy; c.oz = (T)oz; c.A = (T)A; c.invA = (T)(1.0 / A);
  return c;
}

// Largest coarsest level solved in one block's shared memory (16 KB per array).
template <class T>
constexpr int coarse_max() { return (int)(16384 / sizeof(T)); }

// One level of the multigrid hierarchy.
struct MGLevel {
  Grid g;
  double h[3];
  int coarsen[3];   // per axis towards the next level: 0 kept, 1 halved onto every other node, 2 non-nested
  void* e;          // correction (T)
  void* r;          // right-hand side (T)
  void* t;          // residual scratch (T); the smoothed e between the fused kernels
  int fused;        // pre/post-smoothing, residual and transfers by k_mg_down / k_mg_up
  int fuse_all;     // k_mg_down even where the 2.5D one-pass kernels would serve (o3d_params.mg_kernels = 2)
  int plain;        // the plain one-pass kernels only (o3d_params.mg_kernels = 1): the reference path of the tests
};

// fused FP32 level kernels (k_mgfused.cu)
int mg_fused_setup();
bool mg_fusable(const MGLevel& L, int pre, int post, bool any_size);
void launch_mg_down(const MGLevel& L, const MGLevel& C, float om, int pre, bool zero, const SolveCtrl* ctrl,
                    cudaStream_t s);
// p: the finest level's pressure as a double-float pair buffer (p += e), or nullptr
void launch_mg_up(const MGLevel& L, const MGLevel& C, float om, int post, double* p, SolveCtrl* ctrl,
                  cudaStream_t s);

// context state for checkpoint and restart (o3d_api.cu, used by o3d_io.cu)
int ctx_geometry(o3d_ctx* c, o3d_params* p, int* nx, int* ny, int* nz, double* dx, double* dy, double* dz);
// the SOR omega and the previous pressures kept for the extrapolated and
// learned guesses: *nprev of them (0..2); prev_host receives number `which`
// (1 = the newest)
int ctx_history_state(o3d_ctx* c, double* omega, int* nprev, double* prev_host, int which);
int ctx_restore_history(o3d_ctx* c, double omega, int nprev, const double* prev1, const double* prev2);
// whether the context holds its pressures as double-float pairs, and their
// raw buffers (n doubles' size: hi plane, lo plane): `which` 0 = the
// pressure, 1 and 2 = the previous ones; to_device copies host -> device
// (allocating a missing history buffer and marking it valid)
int ctx_pressure_pairs(const o3d_ctx* c);
int ctx_pressure_raw(o3d_ctx* c, int which, void* host, int to_device);

// output-cadence diagnostics (k_diag.cu)
template <class T>
void launch_vorticity(const T* const u[3], T* rx, T* ry, T* rz, T* q, const Grid& g, const Coef3<T>& cf,
                      cudaStream_t s);
template <class T>
void launch_vel_residuals(const T* const u[3], const T* const old[3], const Grid& g, double dt, void* scratch,
                          cudaStream_t s);
size_t vel_residual_scratch_bytes(const Grid& g);
size_t vel_residual_result_offset(const Grid& g);

// one red-black sweep (plus the seam-class passes of odd periodic axes);
// returns the kernels launched
int launch_sor_sweep_ctrl(double* p, const double* rhs, const Grid& g, const PoiCoef<double>& c,
                          SolveCtrl* ctrl, cudaStream_t s);
void launch_sor_control(SolveCtrl* ctrl, cudaStream_t s);
void launch_sor_fixed(double* p, const double* rhs, const Grid& g, const PoiCoef<double>& c,
                      double omega, SolveCtrl* ctrl, cudaStream_t s);

// Multigrid: T is the arithmetic of the cycles, R the type of the top rhs.
// One outer iteration = launch_mg_resid (FP64 residual into the finest
// level's r) + launch_mg_cycles (V-cycles, p += e, stop test).
template <class T, class R>
void launch_mg_outer(double* p, const R* rhs, MGLevel* lv, int nlev, int pre, int post,
                     int coarse_sweeps, T smooth_omega, int cycles, SolveCtrl* ctrl, cudaStream_t s,
                     long long* nl);
template <class T, class R>
void launch_mg_resid(double* p, const R* rhs, MGLevel* lv, SolveCtrl* ctrl, cudaStream_t s, long long* nl);
template <class T>
void launch_mg_cycles(double* p, MGLevel* lv, int nlev, int pre, int post, int coarse_sweeps, T smooth_omega,
                      int cycles, bool from_e, SolveCtrl* ctrl, cudaStream_t s, long long* nl);
// pair: the buffers hold double-float pairs (the mixed multigrid method)
void launch_extrapolate(double* p, double* pprev, long long n, cudaStream_t s, bool pair);
void launch_extrapolate2(double* p, const double* pprev, double* pprev2, long long n, cudaStream_t s, bool pair);

// learned warm start: the network works on multigrid level ll
template <class T>
void launch_learn_extrapolate(double* p, double* pprev, MGLevel* lv, cudaStream_t s, long long* nl, bool pair);
template <class T>
void launch_learn_features(MGLevel* lv, int ll, SolveCtrl* ctrl, float* feat, cudaStream_t s, long long* nl);
template <class T>
void launch_learn_apply(double* p, const float* y, MGLevel* lv, int ll, bool add_to_p, SolveCtrl* ctrl,
                        cudaStream_t s, long long* nl);
template <class T>
void launch_learn_target(const double* p, const double* pprev, MGLevel* lv, int ll, SolveCtrl* ctrl,
                         const float* ch1, float* tgt, cudaStream_t s, long long* nl);

// one finest-level kernel for timing: 0 smoother (one sweep), 1 FP64 residual
template <class T, class R>
void launch_level_kernel(int which, double* p, const R* rhs, const MGLevel& L, SolveCtrl* ctrl,
                         cudaStream_t s, bool pair);
// one pass of the post-smoothing of a large fused level as the step runs it
// on the finest level of the cycle that updates the pressure, for timing:
// 0 the prolongation-add into t (k_prolong_cell), 1 the red pass in place on
// t (k_smooth), 2 the black pass with the pair update p += e (k_smooth_upd)
void launch_post_pass(int which, const MGLevel& L, const MGLevel& C, float om, double* p, SolveCtrl* ctrl,
                      cudaStream_t s);
template <class R>
void launch_rhs_wmean(const R* rhs, const Grid& g, double* part, SolveCtrl* ctrl, cudaStream_t s,
                      long long* nl);
void launch_rhs_wmean_final(const double* part, long long nblk, const Grid& g, SolveCtrl* ctrl, cudaStream_t s,
                            long long* nl);
template <class R>
void launch_residual_inf(const double* p, const R* rhs, const Grid& g, const PoiCoef<double>& c, SolveCtrl* ctrl,
                         bool shift, cudaStream_t s, bool pair);
template <class R>
void launch_rhs_shift(R* rhs, long long n, SolveCtrl* ctrl, cudaStream_t s);

}  // namespace o3d
