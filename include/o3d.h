/*
 * o3d.h -- C ABI of libo3d.so, the GB300 (sm_103a) implementation of
 * osinco3d's per-step hot path: the 6th/4th-order stencils, the Smagorinsky
 * eddy viscosity, the AB1/AB2/AB3 predictor, the projection and the pressure
 * Poisson solve.
 *
 * Conventions
 *  - Fields are column-major (nx, ny, nz) with x fastest, exactly as the
 *    Fortran driver's real(8) arrays; a Fortran caller passes c_loc(ux) etc.
 *  - Every function returns an int status: O3D_OK (0), a positive warning or
 *    a negative error.  Nothing here calls exit() or abort().
 *  - A context owns its device memory and one CUDA stream; fields stay
 *    device-resident between calls.  A context is not thread-safe.
 *  - Host-pointer entry points copy in and out; *_dev entry points take
 *    device pointers and run on the context's stream.
 *
 * Each entry point names the reference routine it replaces (file:line in the
 * osinco3d source tree).
 */
#ifndef O3D_H
#define O3D_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define O3D_ABI_VERSION 1

#if defined(__GNUC__)
#define O3D_API __attribute__((visibility("default")))
#else
#define O3D_API
#endif

/* ---- status codes ------------------------------------------------------ */
enum {
  O3D_OK = 0,
  O3D_WARN_POISSON_MAXIT = 1,   /* solver stopped at kmax (src/poisson.f90:53) */
  O3D_WARN_STAGNATION = 2,      /* |dmax_old - dmax| < eps/1000 (src/poisson.f90:111-114) */
  O3D_ERR_BADARG = -1,          /* unsupported size/BC/option (src/initialization.f90:238-242) */
  O3D_ERR_CUDA = -2,            /* a CUDA call failed; see o3d_last_error() */
  O3D_ERR_NONFINITE = -3,       /* NaN or max(u) > 1000 after correction (src/integration.f90:309-325) */
  O3D_ERR_NOMEM = -4,           /* device allocation failed */
  O3D_ERR_NOT_BUILT = -5        /* feature compiled out or network weights missing */
};

/* boundary codes, src/initialization.f90:74-75 */
enum { O3D_BC_PERIODIC = 0, O3D_BC_FREE_SLIP = 1 };

/* arithmetic of the step */
enum {
  O3D_PREC_FP64 = 0,   /* every kernel in FP64 (the plain method) */
  O3D_PREC_MIXED = 1   /* FP32 stencils and V-cycles inside an FP64 defect-correction loop */
};

/* pressure solver */
enum {
  O3D_SOLVER_SOR = 0,  /* red-black SOR, same operator, stop test and dynamic omega as src/poisson.f90 */
  O3D_SOLVER_MG = 1    /* geometric multigrid V(pre,post) cycles, FP64 outer correction loop */
};

/* initial guess of each pressure solve */
enum {
  O3D_GUESS_PREVIOUS = 0, /* previous step's pressure (the reference: pp persists) */
  O3D_GUESS_ZERO = 1,
  O3D_GUESS_LEARNED = 2,  /* extrapolated pressure plus a 3D U-Net correction (below) */
  O3D_GUESS_EXTRAPOLATED = 3, /* 2 p(n) - p(n-1): linear extrapolation in time */
  O3D_GUESS_EXTRAPOLATED2 = 4 /* 3 p(n) - 3 p(n-1) + p(n-2): quadratic extrapolation in time
                                 (the first solves take the previous, then the linear guess) */
};

/* field identifiers for o3d_upload / o3d_download */
enum {
  O3D_FIELD_UX = 0, O3D_FIELD_UY = 1, O3D_FIELD_UZ = 2, O3D_FIELD_PP = 3,
  O3D_FIELD_UX_PRED = 4, O3D_FIELD_UY_PRED = 5, O3D_FIELD_UZ_PRED = 6,
  O3D_FIELD_PHI = 7, O3D_FIELD_SRC = 8, O3D_FIELD_NU_T = 9,
  O3D_FIELD_RHS = 10,     /* last Poisson right-hand side, div(u*)/dt */
  /* flux history: component c (0..2), age h (0 = newest, 1 = one step older) */
  O3D_FIELD_FU0 = 16,     /* + 2*c + h */
  O3D_FIELD_FPHI0 = 24    /* + h */
};

/* Mirrors the namelists of parameters.o3d (src/initialization.f90:117-125)
 * plus the options this implementation adds. */
typedef struct o3d_params {
  /* &Domain */
  int nx, ny, nz;
  double xlx, yly, zlz;   /* node-inclusive: dx = xlx/(nx-1), src/initialization.f90:182 */
  double x0, y0, z0;
  /* &BoundaryConditions: 0 periodic, 1 free-slip; on x also 2, open: inflow at
   * x(1) (u, v, w and phi held at their values there), outflow at x(nx), the
   * derivatives closed one-sidedly as the reference's dery1D
   * (src/derivation.f90:950-992) and dp/dx = 0 on both faces; it needs
   * free-slip y and z.  The reference declares code 2 but binds no scheme
   * for it (src/initialization.f90:228-242), so this closure is this
   * library's definition. */
  int nbcx1, nbcxn, nbcy1, nbcyn, nbcz1, nbczn, sim2d;
  /* &AdvanceTime */
  int itscheme;           /* 1 Euler, 2 AB2, 3 AB3 */
  double dt;
  /* &FlowParam */
  double re;
  /* &PoissonEq */
  double omega, eps;
  int kmax, idyn;
  /* &Scalar */
  int nscr;
  double sc;
  /* &LES */
  int iles;
  double cs;
  /* additions */
  int precision;          /* O3D_PREC_* */
  int solver;             /* O3D_SOLVER_* */
  int mg_levels;          /* 0 = as many as the grid allows */
  int mg_pre, mg_post;    /* smoothing sweeps; 0 -> V(2,2) in FP64, V(1,1) mixed */
  int guess;              /* O3D_GUESS_* */
  int diagnostics;        /* 1: per-step div/CFL/min-max reductions as the driver prints them */
  int mg_cycles;          /* V-cycles per FP64 residual; 0 -> 1 */
  double mg_omega;        /* relaxation of the red-black smoother; 0 -> 1 (Gauss-Seidel)
                             in FP64, 1.25 mixed */
  int mg_kernels;         /* mixed multigrid: 0 = fused level kernels on the levels large
                             enough to fill the GPU (at least 152 blocks), except that a
                             V-cycle from zero with one pre-sweep on a level of 2^22
                             points or more runs its pre-smoothing, residual and
                             restriction as one-pass 2.5D kernels, and the cycle that
                             updates the pressure its post-smoothing as one-pass
                             kernels with the update in the last black pass (so does
                             an unfused finest level); 1 = one plain kernel
                             per pass (no fused, 2.5D or staged forms); 2 = fused on
                             every level they can serve (same
                             results in all three; 1 and 2 are for comparison and tests) */
} o3d_params;

/* Fills *p with the defaults of the reference's namelists (periodic 64^3);
 * the namelists are read by parameters(), src/initialization.f90:114-126. */
O3D_API void o3d_default_params(o3d_params *p);

/* What one time step reports (the values the reference prints each step). */
typedef struct o3d_step_info {
  int poisson_status;       /* O3D_OK / O3D_WARN_* */
  int poisson_iters;        /* SOR sweeps or MG outer iterations */
  int poisson_cycles;       /* V-cycles (MG) */
  double poisson_dmax;      /* last max |p_gs - p| (SOR) or max |correction| (MG) */
  double poisson_res_inf;   /* max |rhs - A p| after the solve, FP64 */
  double omega;             /* SOR relaxation after the dynamic update */
  int diverged;             /* 1 if NaN or max(u) > 1000 */
  double divu_pred_stats[6];/* min, max, mean, imax, jmax, kmax of div(u*) */
  double divu_stats[6];     /* same for div(u) after the correction */
  double cfl[3];            /* src/utils.f90:202-204 */
  double umin[3], umax[3];  /* velocity extrema per component */
  double poisson_ms;        /* device time of the pressure solve */
  double step_ms;           /* device time of the whole step */
} o3d_step_info;

typedef struct o3d_ctx o3d_ctx;

/* Creates a context: validates the parameters like schemes()
 * (src/initialization.f90:226-304), allocates device fields, zeroes them
 * (src/initialization.f90:170-178) and sets dx, AB coefficients and the LES
 * width (src/initialization.f90:182-209). */
O3D_API int o3d_create(const o3d_params *p, o3d_ctx **out);
O3D_API int o3d_destroy(o3d_ctx *ctx);
O3D_API const char *o3d_last_error(void);
/* Number of kernel launches this context has issued. */
O3D_API long long o3d_launch_count(const o3d_ctx *ctx);
/* The context's CUDA stream (a cudaStream_t) for callers that enqueue work. */
O3D_API void *o3d_stream(o3d_ctx *ctx);

/* Field transfer, host buffers of nx*ny*nz doubles: the module arrays that
 * src/initialization.f90:158-160 allocates (ux, uy, uz, pp, ...) live on the
 * device instead, and the driver copies them only at output. */
O3D_API int o3d_upload(o3d_ctx *ctx, int field, const double *host);
O3D_API int o3d_download(o3d_ctx *ctx, int field, double *host);

/* der_type(df, f, d), src/initialization.f90:86-91: one derivative of f along
 * axis (0 x, 1 y, 2 z), order 1 (6th-order, src/derivation.f90:6-479) or 2
 * (4th-order, src/derivation.f90:497-932), parity 0 = even ("p" routines),
 * 1 = odd ("i" routines), using the context's boundary types and spacing.
 * FP64, host buffers. */
O3D_API int o3d_der(o3d_ctx *ctx, int axis, int order, int odd, const double *f, double *df);
O3D_API int o3d_der_dev(o3d_ctx *ctx, int axis, int order, int odd, const double *d_f, double *d_df);

/* divergence(divf, fx, fy, fz, ..., odd), src/differential_operators.f90:7-38. FP64, host. */
O3D_API int o3d_divergence(o3d_ctx *ctx, const double *fx, const double *fy,
                   const double *fz, int odd, double *divf);
/* calculate_nu_t from the context's velocity into O3D_FIELD_NU_T,
 * src/les_turbulence.f90:10-97. */
O3D_API int o3d_calculate_nu_t(o3d_ctx *ctx);

/* predict_velocity(...), src/integration.f90:14-197: context fields
 * ux,uy,uz and the flux history -> ux_pred.., new flux, history rotated. */
O3D_API int o3d_predict_velocity(o3d_ctx *ctx, int itime);
/* correct_pression(...), src/integration.f90:199-255: rhs = div(u*)/dt and
 * the pressure solve; omega is read and written back like the Fortran
 * intent(inout) argument. */
O3D_API int o3d_correct_pression(o3d_ctx *ctx, double *omega, o3d_step_info *info);
/* correct_velocity(...), src/integration.f90:257-330. Returns
 * O3D_ERR_NONFINITE where the reference stops. */
O3D_API int o3d_correct_velocity(o3d_ctx *ctx);
/* transeq(...), src/integration.f90:332-468 (passive scalar). */
O3D_API int o3d_transeq(o3d_ctx *ctx, int itime);

/* poi_type(pp, rhs, dx,dy,dz, nx,ny,nz, omega, eps, kmax, idyn),
 * src/initialization.f90:93-102: solve A pp = rhs with the context's
 * solver, host buffers, pp is the initial guess and the result. */
O3D_API int o3d_poisson_solve(o3d_ctx *ctx, double *pp, const double *rhs, double *omega,
                      double eps, int kmax, int idyn, int *iters, double *dmax);

/* One iteration of the time loop, src/osinco3d_main.f90:104-128, without I/O. */
O3D_API int o3d_step(o3d_ctx *ctx, int itime, o3d_step_info *info);
/* Same, with the driver's host arrays: ux,uy,uz,pp are copied in before the
 * step and out after it (the flux history stays on the device). */
O3D_API int o3d_step_host(o3d_ctx *ctx, int itime, double *ux, double *uy, double *uz,
                  double *pp, o3d_step_info *info);

/* statistics_calc(...), src/utils.f90:243-375: out[17] = t, E_k, eps, eps2,
 * dzeta, <u^2>, <v^2>, <w^2>, nine <(du_i/dx_j)^2>, FP64 reductions. */
O3D_API int o3d_statistics_calc(o3d_ctx *ctx, double t, double out[17]);

/* ---- output-cadence diagnostics ------------------------------------------
 * rotational(rotx, roty, rotz, ux, uy, uz, ...) and calculate_Q_criterion
 * (src/differential_operators.f90:40-108) of the current velocity into host
 * arrays of nx*ny*nz doubles; any pointer may be NULL. */
O3D_API int o3d_vorticity(o3d_ctx *ctx, double *rotx, double *roty, double *rotz, double *q_criterion);

/* write_all_data(...) + write_xdmf(...), src/visualization.f90:242-341, as
 * called every nfre steps by src/osinco3d_main.f90:147-150: writes
 * <dir>/ux_<num>.bin, uy, uz, pp, vort (|curl u|), qcrit, and phi (nscr = 1)
 * and nu_t (iles = 1) -- raw FP64 column-major nx*ny*nz arrays, no record
 * markers -- and <dir>/output_<num>.xdmf describing them, in the reference's
 * layouts.  Asynchronous: the call snapshots the fields on the device and
 * returns; the device->host copies run on a separate stream and a host
 * thread writes the files while later steps run.  The next call,
 * o3d_output_wait or o3d_destroy waits for it.  The driver keeps num
 * (write_xdmf's counter) and time. */
O3D_API int o3d_write_output(o3d_ctx *ctx, const char *dir, int num, double time);
/* Waits until the files of the last o3d_write_output are written; returns
 * O3D_ERR_BADARG (with o3d_last_error) if a file could not be written. */
O3D_API int o3d_output_wait(o3d_ctx *ctx);
/* old_values (src/utils.f90:209-218): keep the current velocity on the
 * device for o3d_velocity_residuals. */
O3D_API int o3d_save_old_velocity(o3d_ctx *ctx);
/* calculate_residuals (src/utils.f90:93-163) of the current velocity against
 * the one kept by o3d_save_old_velocity: out = res_u, res_v, res_w (rms of
 * |old - u|/(2 dt) over the interior points, normalised by nx*ny*nz),
 * linf_u, linf_v, linf_w (max), each scaled by t_ref/u_ref, then the
 * 1-based (i, j, k) of each max (the last in i-fastest order on ties). */
O3D_API int o3d_velocity_residuals(o3d_ctx *ctx, double t_ref, double u_ref, double out[15]);

/* ---- checkpoint and restart ----------------------------------------------
 * save_fields / read_fields (src/IOfunctions.f90:360-470): the flow-state
 * file of the reference, stream-unformatted: time (f8), nx ny nz (int32),
 * x, y, z (f8), then ux, uy, uz, pp, phi (f8, column-major); phi is written
 * as zeros without a scalar.  o3d_load_fields checks the grid and uploads
 * the fields; *time may be NULL. */
O3D_API int o3d_save_fields(o3d_ctx *ctx, const char *path, double time);
O3D_API int o3d_load_fields(o3d_ctx *ctx, const char *path, double *time);
/* What the flow-state file lacks for an exact restart: the Adams-Bashforth
 * flux history of the velocity and the scalar, the previous pressure of the
 * extrapolated and learned guesses and the dynamic SOR omega; in the mixed
 * multigrid method, which holds its pressures as double-float pairs of FP32
 * values, also the current pressure as that pair (the FP64 value in the
 * flow-state file may round it).  Load the history after the fields: with
 * both files a restarted run continues bit for bit.  No counterpart in the
 * reference (its restart resets the history). */
O3D_API int o3d_save_history(o3d_ctx *ctx, const char *path);
O3D_API int o3d_load_history(o3d_ctx *ctx, const char *path);

/* ---- learned Poisson warm start ------------------------------------------
 * A 3D U-Net (BF16 tensor-core convolutions, FP32 accumulation) corrects the
 * extrapolated pressure p_ex = 2 p(n) - p(n-1).  Its input, on the multigrid
 * level ll of o3d_guess_grid (the pressure grid coarsened 1 to 3 times, at
 * least 16 points per axis): the restricted FP64 residual of p_ex times
 * h_ll^2, divided by its rms S_r, and the restricted last increment
 * p(n) - p(n-1), divided by its rms.  Its output y predicts
 * restrict(p(n+1) - p_ex) / S_r, mean removed (the solver leaves the
 * constant of the singular operator free).  The correction prolong(S_r y)
 * starts the first V-cycle of the multigrid solve (the residual already
 * computed is reused), or is added to p_ex before SOR; the solver then
 * iterates to eps as usual, so the converged pressure does not depend on
 * the network.  No counterpart in the reference. */
typedef struct o3d_unet o3d_unet;
/* nx, ny, nz: the network grid (that of o3d_guess_grid); periodic[a] = 1
 * wraps axis a in the convolutions; base_channels (16) doubles per level. */
O3D_API int o3d_unet_create(int nx, int ny, int nz, const int periodic[3], int base_channels, int levels,
                            int in_channels, unsigned long long seed, o3d_unet **out);
O3D_API int o3d_unet_destroy(o3d_unet *net);
O3D_API long long o3d_unet_num_params(const o3d_unet *net);
/* FP32 master parameters (host buffers of o3d_unet_num_params floats) */
O3D_API int o3d_unet_get_params(o3d_unet *net, float *host);
O3D_API int o3d_unet_set_params(o3d_unet *net, const float *host);
/* d_in: in_channels x nvox FP32 device buffer (channel-major, x fastest);
 * d_out: nvox FP32; `wait` is a cudaStream_t ordered before and after. */
O3D_API int o3d_unet_forward_dev(o3d_unet *net, const float *d_in, float *d_out, void *wait);
/* MSE loss and parameter gradients of one sample (host_grad may be NULL) */
O3D_API int o3d_unet_gradients(o3d_unet *net, const float *d_in, const float *d_target, float *loss,
                               float *host_grad);
/* one Adam step (beta 0.9 / 0.999) on one sample */
O3D_API int o3d_unet_train_step(o3d_unet *net, const float *d_in, const float *d_target, float lr, float *loss);
/* the grid of the guess features for this context (dims[3]) */
O3D_API int o3d_guess_grid(o3d_ctx *ctx, int dims[3]);
/* use `net` for O3D_GUESS_LEARNED (NULL detaches); the caller keeps ownership */
O3D_API int o3d_attach_unet(o3d_ctx *ctx, o3d_unet *net);
/* Training data: with device buffers set (features 2 x n, target n on the
 * guess grid), every multigrid solve with the extrapolated or learned guess
 * that has a previous pressure writes the network input before and the
 * target, restrict(p(n+1) - p_ex) / S_r with its mean removed, after
 * (O3D_ERR_BADARG otherwise). */
O3D_API int o3d_set_sample_buffers(o3d_ctx *ctx, float *d_feat, float *d_tgt);
/* 1 when the last solve wrote a sample */
O3D_API int o3d_sample_ready(const o3d_ctx *ctx);

/* Device time of one launch of a hot kernel on the live state, averaged over
 * `reps` back-to-back launches timed with CUDA events on the context's stream.
 * kernel: 0 fused predictor, 1 divergence -> rhs, 2 velocity correction,
 * 3 multigrid smoother colour pass on the finest level, 4 FP64 residual of
 * the defect-correction loop, 5 fused pre-smoothing + residual + restriction
 * of the finest level (mixed method, from a zero correction), 6 fused
 * prolongation + post-smoothing + p += e of the finest level (mixed method;
 * the update goes to a scratch copy of p), 7 the finest level's first sweep
 * from a zero correction and 8 its residual, in the form a large level runs
 * them before the fused up kernel; 9, 10 and 11 the post-smoothing passes of
 * the finest level in the cycle that updates the pressure: the
 * prolongation-add, the red pass and the black pass with p += e (on a
 * scratch copy of p).  The launches only rewrite
 * scratch outputs (u*, the free flux slot, rhs, the multigrid levels'
 * corrections and residuals) or recompute the velocity identically from u*
 * and p.  No counterpart in the reference (measurement hook). */
O3D_API int o3d_time_kernel(o3d_ctx *ctx, int kernel, int reps, double *ms_per_launch);

/* Self-check of the binary64 <-> binary32 conversions the kernels perform on
 * the integer pipe (round to nearest even): converts n seeded pseudo-random
 * bit patterns (normal, subnormal, zero, tie and out-of-range cases) both
 * ways on the device, and splits each binary64 value into the double-float
 * pair hi = RN32(x), lo = RN32(x - hi) of the mixed method's residual, and
 * counts results that differ bit-wise from the FP64 instructions.  No
 * counterpart in the reference. */
O3D_API int o3d_check_conversions(long long n, unsigned long long seed, long long *mismatches);

/* divergence(divf, fx, fy, fz, ..., odd) with function_stats of the result
 * (src/differential_operators.f90:7-38, src/functions.f90:27-63) for callers
 * that cannot allocate device memory.  No counterpart in the reference: it
 * exists for hosts that give all device memory to their own allocator, time
 * loops that must avoid the device-wide synchronisation of cudaMalloc and
 * cudaFree, and code where allocation is forbidden.  It needs no context and
 * calls no allocating routine.  d_fx, d_fy, d_fz and d_div are the caller's
 * device buffers of nx*ny*nz doubles (d_div may be NULL); dx, dy, dz are the
 * node spacings, bc* the O3D_BC_* code of each axis, odd selects the "i"
 * closures; the work runs on `stream` (a cudaStream_t, NULL = default) and the
 * call returns after stats = min, max, mean, imax, jmax, kmax (1-based) are in
 * host memory.  Scratch: a fixed 768 KiB array in device memory, shared by
 * every call, of O3D_NOALLOC_MAX_RECORDS block records.  A grid needs
 * ceil(nx/32) * ceil(ny/8) * ceil(nz/28) of them (19456 for 512^3, 16128 for
 * 768 x 384 x 384); a grid needing more is rejected with O3D_ERR_BADARG before
 * any device work.  Calls that overlap on the GPU race on the array.  The
 * first call on each device looks up the array's device address.  Every call
 * synchronizes `stream` and copies the statistics into pageable host memory,
 * so it must not be called while `stream` is being captured into a graph. */
#define O3D_NOALLOC_MAX_RECORDS 24576
O3D_API int o3d_divergence_stats_noalloc(const double *d_fx, const double *d_fy, const double *d_fz,
                                         double *d_div, int nx, int ny, int nz, double dx, double dy,
                                         double dz, int bcx, int bcy, int bcz, int odd, void *stream,
                                         double stats[6]);

/* Red-black SOR sweep(s) alone on device buffers: for tests of the kernel
 * that replaces the lexicographic sweeps of src/poisson.f90:6-130. */
O3D_API int o3d_rbsor_sweeps_dev(o3d_ctx *ctx, double *d_pp, const double *d_rhs, double omega,
                         int nsweeps, double *dmax_last);

#ifdef __cplusplus
}
#endif
#endif
