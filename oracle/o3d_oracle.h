/*
 * o3d_oracle.h -- FP64 CPU restatement of osinco3d's per-step hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This is the checker the CUDA library is compared
 * against; only the tests, the smoke check and the CPU-baseline leg of the
 * benchmark may load it.  The product (libo3d.so) never links or calls it.
 *
 * Every routine follows the Fortran reference statement by statement and
 * cites the file:line it restates (paths relative to the osinco3d source
 * tree).  Arrays are column-major (nx, ny, nz) with x fastest, 0-based:
 * element (i, j, k) lives at i + nx*(j + ny*k).
 */
#ifndef O3D_ORACLE_H
#define O3D_ORACLE_H
#ifdef __cplusplus
extern "C" {
#endif

/* closure codes: how a derivative treats the two ends of an axis */
enum { ORC_PERIODIC = 0, ORC_EVEN = 1, ORC_ODD = 2, ORC_ZERO = 3, ORC_OPEN = 4 };

/* ---- derivation.f90 --------------------------------------------------- */
/* 6th-order first derivative along `axis` (0=x,1=y,2=z). */
void orc_der1(double *df, const double *f, int nx, int ny, int nz,
              int axis, int closure, double d);
/* 4th-order second derivative along `axis`. */
void orc_der2(double *df, const double *f, int nx, int ny, int nz,
              int axis, int closure, double d);

/* ---- model description (initialization.f90) --------------------------- */
typedef struct orc_model {
  int nx, ny, nz;
  double dx, dy, dz;
  int bcx, bcy, bcz;      /* 0 periodic, 1 free-slip (per axis, both ends), 2 open (x only) */
  int sim2d;
  int itscheme;
  double dt, re, sc;
  double adt[3], bdt[3], cdt[3];
  int iles;
  double cs, delta;
  int nscr;
} orc_model;

/* Fills the derived members (dx.., adt.., delta) from the grid and dt the
 * way variables() does, initialization.f90:182-209. */
void orc_model_init(orc_model *m, int nx, int ny, int nz, double xlx,
                    double yly, double zlz, int bcx, int bcy, int bcz,
                    int sim2d, int itscheme, double dt, double re, double sc,
                    int iles, double cs, int nscr);

/* ---- differential_operators.f90, les_turbulence.f90 -------------------- */
void orc_divergence(const orc_model *m, double *divf, const double *fx,
                    const double *fy, const double *fz, int odd);
void orc_nu_t(const orc_model *m, double *nu_t, const double *ux,
              const double *uy, const double *uz);

/* ---- integration.f90 ---------------------------------------------------- */
/* fu: 9 fields, fu[3*c + h] is component c (0 ux, 1 uy, 2 uz), history slot
 * h (0 newest).  nu_t is written when iles==1 and zeroed otherwise. */
void orc_predict_velocity(const orc_model *m, double *upred[3],
                          double *u[3], double *fu[9], double *nu_t,
                          int itime);
/* returns solver status (ORC_SOR_*), sweeps performed in *iters, the last
 * sweep's max|p_gs - p| in *dmax; *omega is updated in place (idyn). */
int orc_correct_pressure(const orc_model *m, double *pp,
                         double *const upred[3], double *omega, double eps,
                         int kmax, int idyn, int *iters, double *dmax);
int orc_poisson_sor(const orc_model *m, double *pp, const double *rhs,
                    double *omega, double eps, int kmax, int idyn,
                    int *iters, double *dmax);
/* returns 0, or 1 if a component holds a NaN or exceeds 1000 */
int orc_correct_velocity(const orc_model *m, double *u[3],
                         double *const upred[3], const double *pp);
void orc_transeq(const orc_model *m, double *phi, double *const u[3],
                 const double *src, double *fphi[3], const double *nu_t,
                 int itime);

enum { ORC_SOR_CONVERGED = 0, ORC_SOR_STAGNATED = 1, ORC_SOR_MAXIT = 2 };

/* ---- diagnostics (functions.f90, utils.f90) ----------------------------- */
/* out: min, max, mean, imax, jmax, kmax (1-based indices as in Fortran) */
void orc_function_stats(const double *f, int n1, int n2, int n3, double out[6]);
void orc_cfl(const orc_model *m, double *const u[3], double out[3]);
/* out[17] = t, E_k, eps, eps2, dzeta, <u^2>,<v^2>,<w^2>, 9 x <(du_i/dx_j)^2> */
void orc_statistics(const orc_model *m, double *const u[3], double t,
                    double out[17]);
void orc_rotational(const orc_model *m, double *const u[3], double *rot[3]);
void orc_q_criterion(const orc_model *m, double *q, double *const u[3]);
void orc_residuals(const orc_model *m, double *const u[3], double *const old[3], double dt,
                   double t_ref, double u_ref, double out[15]);

/* ---- initial_conditions.f90 -------------------------------------------- */
void orc_init_tgv(const orc_model *m, double x0, double y0, double z0,
                  double u0, double l0, double ratio, int nscr,
                  double *ux, double *uy, double *uz, double *pp,
                  double *phi);
void orc_init_mixing_layer(const orc_model *m, double x0, double y0,
                           double z0, double u0, double l0, double ratio,
                           int nscr, double *ux, double *uy, double *uz,
                           double *pp, double *phi);
/* initialize_coplanar_jet, src/initial_conditions.f90:244-327 (no noise) */
void orc_init_coplanar_jet(const orc_model *m, double y0, double u0, double l0,
                           double ratio, int nscr, double *ux, double *uy,
                           double *uz, double *pp, double *phi);

/* ---- one iteration of the time loop, osinco3d_main.f90:97-128 ---------- */
typedef struct orc_step_info {
  int sor_status, sor_iters;
  double sor_dmax, omega;
  int diverged;
  double divu_pred_stats[6], divu_stats[6];
  double cfl[3];
} orc_step_info;

typedef struct orc_state {
  double *u[3], *upred[3], *pp, *fu[9], *nu_t, *phi, *src, *fphi[3];
  double omega, eps;
  int kmax, idyn;
} orc_state;

void orc_step(const orc_model *m, orc_state *s, int itime, orc_step_info *info);

/* ---- red-black ordering (poisson_multigrid.f90:80-121) ------------------ */
/* One red-black SOR sweep on the same 7-point operator and boundary remap
 * as the lexicographic solvers; returns max|p_gs - p| over the sweep.
 * Used to check the GPU red-black kernel sweep by sweep. */
double orc_rbsor_sweep(const orc_model *m, double *pp, const double *rhs,
                       double omega);

/* The reference's SOR control loop (poisson.f90:52-123: stop on dmax < eps,
 * stagnation on |dmax_old - dmax| < eps/1000, dynamic omega with the
 * variant's factor, kmax) driving orc_rbsor_sweep instead of the
 * lexicographic sweep: the solve the GPU red-black SOR performs.  If
 * omega_trace is not NULL, omega_trace[iter-1] and dmax_trace[iter-1] hold
 * omega and dmax after the control step of each sweep. */
int orc_poisson_rbsor(const orc_model *m, double *pp, const double *rhs,
                      double *omega_io, double eps, int kmax, int idyn,
                      int *iters, double *dmax_out, double *omega_trace,
                      double *dmax_trace);

#ifdef __cplusplus
}
#endif
#endif
