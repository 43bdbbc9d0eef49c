/*
 * o3d_oracle.c -- FP64 CPU restatement of osinco3d's per-step hot path.
 *
 * TEST INFRASTRUCTURE ONLY: the checker for the CUDA library (see the header
 * of o3d_oracle.h).  Built with -ffp-contract=off so that every expression is
 * evaluated in the same order, with the same roundings, as gfortran evaluates
 * the Fortran statement it restates (no fused multiply-add, no reassociation).
 *
 * Citations are file:line in the osinco3d source tree (src/...).
 */
#include "o3d_oracle.h"

#include <float.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>

#define IDX(m, i, j, k) ((size_t)(i) + (size_t)(m)->nx * ((size_t)(j) + (size_t)(m)->ny * (size_t)(k)))

/* ------------------------------------------------------------------------ */
/* 1D line kernels.  A "line" is n values f[0], f[s], ..., f[(n-1)s].       */
/* Each one restates the explicit boundary rows of the Fortran routine.     */
/* ------------------------------------------------------------------------ */
#define F(q) f[(size_t)(q) * s]
#define D(q) df[(size_t)(q) * s]

/* derx_00 / dery_00 / derz_00, src/derivation.f90:34-56 */
static void d1_periodic(double *df, const double *f, int n, size_t s,
                        double a, double b, double c) {
  D(0) = a * (F(3) - F(n - 3)) - b * (F(2) - F(n - 2)) + c * (F(1) - F(n - 1));
  D(1) = a * (F(4) - F(n - 2)) - b * (F(3) - F(n - 1)) + c * (F(2) - F(0));
  D(2) = a * (F(5) - F(n - 1)) - b * (F(4) - F(0)) + c * (F(3) - F(1));
  for (int i = 3; i <= n - 4; ++i)
    D(i) = a * (F(i + 3) - F(i - 3)) - b * (F(i + 2) - F(i - 2)) + c * (F(i + 1) - F(i - 1));
  D(n - 3) = a * (F(0) - F(n - 6)) - b * (F(n - 1) - F(n - 5)) + c * (F(n - 2) - F(n - 4));
  D(n - 2) = a * (F(1) - F(n - 5)) - b * (F(0) - F(n - 4)) + c * (F(n - 1) - F(n - 3));
  D(n - 1) = a * (F(2) - F(n - 4)) - b * (F(1) - F(n - 3)) + c * (F(0) - F(n - 2));
}

/* derxp_11 / deryp_11 / derzp_11 (mirror closure), src/derivation.f90:87-105 */
static void d1_even(double *df, const double *f, int n, size_t s,
                    double a, double b, double c) {
  D(0) = 0.0;
  D(1) = a * (F(4) - F(2)) - b * (F(3) - F(1)) + c * (F(2) - F(0));
  D(2) = a * (F(5) - F(1)) - b * (F(4) - F(0)) + c * (F(3) - F(1));
  for (int i = 3; i <= n - 4; ++i)
    D(i) = a * (F(i + 3) - F(i - 3)) - b * (F(i + 2) - F(i - 2)) + c * (F(i + 1) - F(i - 1));
  D(n - 3) = a * (F(n - 2) - F(n - 6)) - b * (F(n - 1) - F(n - 5)) + c * (F(n - 2) - F(n - 4));
  D(n - 2) = a * (F(n - 3) - F(n - 5)) - b * (F(n - 2) - F(n - 4)) + c * (F(n - 1) - F(n - 3));
  D(n - 1) = 0.0;
}

/* derxi_11 / deryi_11 / derzi_11 (anti-mirror closure), src/derivation.f90:137-159 */
static void d1_odd(double *df, const double *f, int n, size_t s,
                   double a, double b, double c) {
  D(0) = a * (F(3) + F(3)) - b * (F(2) + F(2)) + c * (F(1) + F(1));
  D(1) = a * (F(4) + F(2)) - b * (F(3) + F(1)) + c * (F(2) - F(0));
  D(2) = a * (F(5) + F(1)) - b * (F(4) - F(0)) + c * (F(3) - F(1));
  for (int i = 3; i <= n - 4; ++i)
    D(i) = a * (F(i + 3) - F(i - 3)) - b * (F(i + 2) - F(i - 2)) + c * (F(i + 1) - F(i - 1));
  D(n - 3) = a * (-F(n - 2) - F(n - 6)) - b * (F(n - 1) - F(n - 5)) + c * (F(n - 2) - F(n - 4));
  D(n - 2) = a * (-F(n - 3) - F(n - 5)) - b * (-F(n - 2) - F(n - 4)) + c * (F(n - 1) - F(n - 3));
  D(n - 1) = a * (-F(n - 4) - F(n - 4)) - b * (-F(n - 3) - F(n - 3)) + c * (-F(n - 2) - F(n - 2));
}

/* derxx_00 / deryy_00 / derzz_00, src/derivation.f90:521-539 */
static void d2_periodic(double *df, const double *f, int n, size_t s,
                        double a, double b, double c) {
  D(0) = -a * (F(n - 2) + F(2)) + b * (F(n - 1) + F(1)) - c * F(0);
  D(1) = -a * (F(n - 1) + F(3)) + b * (F(0) + F(2)) - c * F(1);
  for (int i = 2; i <= n - 3; ++i)
    D(i) = -a * (F(i - 2) + F(i + 2)) + b * (F(i - 1) + F(i + 1)) - c * F(i);
  D(n - 2) = -a * (F(n - 4) + F(0)) + b * (F(n - 3) + F(n - 1)) - c * F(n - 2);
  D(n - 1) = -a * (F(n - 3) + F(1)) + b * (F(n - 2) + F(0)) - c * F(n - 1);
}

/* derxxp_11 / deryyp_11 / derzzp_11 (mirror), src/derivation.f90:618-636 */
static void d2_even(double *df, const double *f, int n, size_t s,
                    double a, double b, double c) {
  D(0) = -a * (F(2) + F(2)) + b * (F(1) + F(1)) - c * F(0);
  D(1) = -a * (F(1) + F(3)) + b * (F(0) + F(2)) - c * F(1);
  for (int i = 2; i <= n - 3; ++i)
    D(i) = -a * (F(i - 2) + F(i + 2)) + b * (F(i - 1) + F(i + 1)) - c * F(i);
  D(n - 2) = -a * (F(n - 4) + F(n - 2)) + b * (F(n - 3) + F(n - 1)) - c * F(n - 2);
  D(n - 1) = -a * (F(n - 3) + F(n - 3)) + b * (F(n - 2) + F(n - 2)) - c * F(n - 1);
}

/* derxxi_11 / deryyi_11 / derzzi_11 (anti-mirror), src/derivation.f90:570-588 */
static void d2_odd(double *df, const double *f, int n, size_t s,
                   double a, double b, double c) {
  D(0) = -a * (-F(2) + F(2)) + b * (-F(1) + F(1)) - c * F(0);
  D(1) = -a * (-F(1) + F(3)) + b * (F(0) + F(2)) - c * F(1);
  for (int i = 2; i <= n - 3; ++i)
    D(i) = -a * (F(i - 2) + F(i + 2)) + b * (F(i - 1) + F(i + 1)) - c * F(i);
  D(n - 2) = -a * (F(n - 4) - F(n - 2)) + b * (F(n - 3) + F(n - 1)) - c * F(n - 2);
  D(n - 1) = -a * (F(n - 3) - F(n - 3)) + b * (F(n - 2) - F(n - 2)) - c * F(n - 1);
}
/* Open x axis: no reference routine (src/initialization.f90:228-242 stops on
 * nbcx = 2).  First derivative: the one-sided closure of dery1D,
 * src/derivation.f90:975-989, with the 6th-order interior; second
 * derivative (this build's choice): 2nd-order one-sided at the end nodes,
 * 2nd-order central next to them, the 4th-order interior elsewhere.  d is
 * the node spacing. */
static void d1_open(double *df, const double *f, int n, size_t s,
                    double a, double b, double c, double d) {
  D(0) = (-F(2) + 4.0 * F(1) - 3.0 * F(0)) / (2.0 * d);
  D(1) = (F(2) - F(0)) / (2.0 * d);
  D(2) = (-F(4) + 8.0 * F(3) - 8.0 * F(1) + F(0)) / (12.0 * d);
  for (int i = 3; i <= n - 4; ++i)
    D(i) = a * (F(i + 3) - F(i - 3)) - b * (F(i + 2) - F(i - 2)) + c * (F(i + 1) - F(i - 1));
  D(n - 3) = (-F(n - 1) + 8.0 * F(n - 2) - 8.0 * F(n - 4) + F(n - 5)) / (12.0 * d);
  D(n - 2) = (F(n - 1) - F(n - 3)) / (2.0 * d);
  D(n - 1) = (3.0 * F(n - 1) - 4.0 * F(n - 2) + F(n - 3)) / (2.0 * d);
}

static void d2_open(double *df, const double *f, int n, size_t s,
                    double a, double b, double c, double d) {
  D(0) = (2.0 * F(0) - 5.0 * F(1) + 4.0 * F(2) - F(3)) / (d * d);
  D(1) = (F(0) - 2.0 * F(1) + F(2)) / (d * d);
  for (int i = 2; i <= n - 3; ++i)
    D(i) = -a * (F(i - 2) + F(i + 2)) + b * (F(i - 1) + F(i + 1)) - c * F(i);
  D(n - 2) = (F(n - 3) - 2.0 * F(n - 2) + F(n - 1)) / (d * d);
  D(n - 1) = (2.0 * F(n - 1) - 5.0 * F(n - 2) + 4.0 * F(n - 3) - F(n - 4)) / (d * d);
}
#undef F
#undef D

typedef void (*line_fn)(double *, const double *, int, size_t, double, double, double);
typedef void (*line_fn_d)(double *, const double *, int, size_t, double, double, double, double);

static void apply_lines(double *df, const double *f, int nx, int ny, int nz,
                        int axis, line_fn fn, double a, double b, double c) {
  size_t sx = 1, sy = (size_t)nx, sz = (size_t)nx * ny;
#ifdef _OPENMP
#pragma omp parallel for collapse(2) schedule(static)
#endif
  for (int q = 0; q < (axis == 2 ? ny : nz); ++q) {
    for (int p = 0; p < (axis == 0 ? ny : nx); ++p) {
      size_t base;
      int n;
      size_t s;
      if (axis == 0) { base = sy * p + sz * q; n = nx; s = sx; }
      else if (axis == 1) { base = sx * p + sz * q; n = ny; s = sy; }
      else { base = sx * p + sy * q; n = nz; s = sz; }
      fn(df + base, f + base, n, s, a, b, c);
    }
  }
}

static void apply_lines_d(double *df, const double *f, int nx, int ny, int nz,
                          int axis, line_fn_d fn, double a, double b, double c, double d) {
  size_t sx = 1, sy = (size_t)nx, sz = (size_t)nx * ny;
  for (int q = 0; q < (axis == 2 ? ny : nz); ++q)
    for (int p = 0; p < (axis == 0 ? ny : nx); ++p) {
      size_t base;
      int n;
      size_t s;
      if (axis == 0) { base = sy * p + sz * q; n = nx; s = sx; }
      else if (axis == 1) { base = sx * p + sz * q; n = ny; s = sy; }
      else { base = sx * p + sy * q; n = nz; s = sz; }
      fn(df + base, f + base, n, s, a, b, c, d);
    }
}

void orc_der1(double *df, const double *f, int nx, int ny, int nz, int axis,
              int closure, double d) {
  size_t n = (size_t)nx * ny * nz;
  if (closure == ORC_ZERO) { /* derz_2dsim: df = 0*f*dz, src/derivation.f90:492 */
    for (size_t q = 0; q < n; ++q) df[q] = 0.0 * f[q] * d;
    return;
  }
  /* coefficients, src/derivation.f90:26-30 */
  double sixtyd = 60.0 * d;
  double a = 1.0 / sixtyd, b = 9.0 / sixtyd, c = 45.0 / sixtyd;
  if (closure == ORC_OPEN) {
    apply_lines_d(df, f, nx, ny, nz, axis, d1_open, a, b, c, d);
    return;
  }
  line_fn fn = closure == ORC_PERIODIC ? d1_periodic : closure == ORC_EVEN ? d1_even : d1_odd;
  apply_lines(df, f, nx, ny, nz, axis, fn, a, b, c);
}

void orc_der2(double *df, const double *f, int nx, int ny, int nz, int axis,
              int closure, double d) {
  size_t n = (size_t)nx * ny * nz;
  if (closure == ORC_ZERO) { /* derzz_2dsim, src/derivation.f90:946 */
    for (size_t q = 0; q < n; ++q) df[q] = 0.0 * f[q] * d;
    return;
  }
  /* coefficients, src/derivation.f90:518-522 */
  double twelved2 = 12.0 * d * d;
  double a = 1.0 / twelved2, b = 16.0 / twelved2, c = 30.0 / twelved2;
  if (closure == ORC_OPEN) {
    apply_lines_d(df, f, nx, ny, nz, axis, d2_open, a, b, c, d);
    return;
  }
  line_fn fn = closure == ORC_PERIODIC ? d2_periodic : closure == ORC_EVEN ? d2_even : d2_odd;
  apply_lines(df, f, nx, ny, nz, axis, fn, a, b, c);
}

/* ------------------------------------------------------------------------ */
/* Procedure-pointer binding, src/initialization.f90:226-281.               */
/* parity 'p' -> even closure on a free-slip axis, 'i' -> odd closure.      */
/* ------------------------------------------------------------------------ */
static int closure_of(const orc_model *m, int axis, int odd) {
  if (axis == 2 && m->sim2d) return ORC_ZERO;
  int bc = axis == 0 ? m->bcx : axis == 1 ? m->bcy : m->bcz;
  if (bc == 0) return ORC_PERIODIC;
  if (bc == 2) return ORC_OPEN;
  return odd ? ORC_ODD : ORC_EVEN;
}
static double step_of(const orc_model *m, int axis) {
  return axis == 0 ? m->dx : axis == 1 ? m->dy : m->dz;
}
static void der1(const orc_model *m, double *df, const double *f, int axis, int odd) {
  orc_der1(df, f, m->nx, m->ny, m->nz, axis, closure_of(m, axis, odd), step_of(m, axis));
}
static void der2(const orc_model *m, double *df, const double *f, int axis, int odd) {
  orc_der2(df, f, m->nx, m->ny, m->nz, axis, closure_of(m, axis, odd), step_of(m, axis));
}
static size_t npts(const orc_model *m) { return (size_t)m->nx * m->ny * m->nz; }
static double *fld(const orc_model *m) { return (double *)malloc(npts(m) * sizeof(double)); }

void orc_model_init(orc_model *m, int nx, int ny, int nz, double xlx,
                    double yly, double zlz, int bcx, int bcy, int bcz,
                    int sim2d, int itscheme, double dt, double re, double sc,
                    int iles, double cs, int nscr) {
  memset(m, 0, sizeof(*m));
  m->nx = nx; m->ny = ny; m->nz = nz;
  m->bcx = bcx; m->bcy = bcy; m->bcz = bcz; m->sim2d = sim2d;
  m->itscheme = itscheme; m->re = re; m->sc = sc;
  m->iles = iles; m->cs = cs; m->nscr = nscr;
  /* src/initialization.f90:182-202 */
  m->dx = xlx / (double)(nx - 1);
  m->dy = yly / (double)(ny - 1);
  m->dz = zlz / (double)(nz - 1);
  m->delta = pow(m->dx * m->dy * m->dz, 1.0 / 3.0);
  m->dt = dt;
  m->adt[0] = dt; m->bdt[0] = 0.0; m->cdt[0] = 0.0;
  m->adt[1] = 3.0 * dt / 2.0; m->bdt[1] = -1.0 * dt / 2.0; m->cdt[1] = 0.0;
  m->adt[2] = 23.0 * dt / 12.0; m->bdt[2] = -16.0 * dt / 12.0; m->cdt[2] = 5.0 * dt / 12.0;
}

/* divergence, src/differential_operators.f90:25-35 */
void orc_divergence(const orc_model *m, double *divf, const double *fx,
                    const double *fy, const double *fz, int odd) {
  double *dfx = fld(m), *dfy = fld(m), *dfz = fld(m);
  der1(m, dfx, fx, 0, odd);
  der1(m, dfy, fy, 1, odd);
  der1(m, dfz, fz, 2, odd);
  size_t n = npts(m);
  for (size_t q = 0; q < n; ++q) divf[q] = dfx[q] + dfy[q] + dfz[q];
  free(dfx); free(dfy); free(dfz);
}

/* calculate_nu_t, src/les_turbulence.f90:54-88 */
void orc_nu_t(const orc_model *m, double *nu_t, const double *ux,
              const double *uy, const double *uz) {
  double *g[9];
  for (int q = 0; q < 9; ++q) g[q] = fld(m);
  der1(m, g[0], ux, 0, 1); der1(m, g[1], ux, 1, 0); der1(m, g[2], ux, 2, 0);
  der1(m, g[3], uy, 0, 0); der1(m, g[4], uy, 1, 1); der1(m, g[5], uy, 2, 0);
  der1(m, g[6], uz, 0, 0); der1(m, g[7], uz, 1, 0); der1(m, g[8], uz, 2, 1);
  double csd = m->cs * m->delta;
  double csd2 = csd * csd;
  size_t n = npts(m);
  for (size_t q = 0; q < n; ++q) {
    double s11 = g[0][q], s22 = g[4][q], s33 = g[8][q];
    double s12 = 0.5 * (g[1][q] + g[3][q]);
    double s13 = 0.5 * (g[2][q] + g[6][q]);
    double s23 = 0.5 * (g[5][q] + g[7][q]);
    double smag = sqrt(2.0 * (s11 * s11 + s22 * s22 + s33 * s33 +
                              2.0 * (s12 * s12 + s13 * s13 + s23 * s23)));
    nu_t[q] = csd2 * smag;
  }
  for (int q = 0; q < 9; ++q) free(g[q]);
}

/* AB coefficient choice, src/integration.f90:84-105 */
static void ab_coefs(const orc_model *m, int itime, double *a, double *b, double *c) {
  int s = (m->itscheme == 1 || itime == 1) ? 0 : (m->itscheme == 2 || itime == 2) ? 1 : 2;
  *a = m->adt[s]; *b = m->bdt[s]; *c = m->cdt[s];
}

/* predict_velocity, src/integration.f90:106-188 */
void orc_predict_velocity(const orc_model *m, double *upred[3], double *u[3],
                          double *fu[9], double *nu_t, int itime) {
  double adu, bdu, cdu;
  ab_coefs(m, itime, &adu, &bdu, &cdu);
  double onere = 1.0 / m->re;
  size_t n = npts(m);
  if (m->iles == 1) orc_nu_t(m, nu_t, u[0], u[1], u[2]);
  else for (size_t q = 0; q < n; ++q) nu_t[q] = 0.0;
  double *nu_eff = fld(m);
  for (size_t q = 0; q < n; ++q) nu_eff[q] = onere + nu_t[q];
  double *d1[3], *d2[3];
  for (int a = 0; a < 3; ++a) { d1[a] = fld(m); d2[a] = fld(m); }
  for (int c = 0; c < 3; ++c) {
    /* component c is odd along its own axis (derxi for ux, deryi for uy, ...) */
    for (int a = 0; a < 3; ++a) {
      der1(m, d1[a], u[c], a, a == c);
      der2(m, d2[a], u[c], a, a == c);
    }
    double *f1 = fu[3 * c + 0], *f2 = fu[3 * c + 1], *f3 = fu[3 * c + 2];
    const double *uc = u[c];
    double *up = upred[c];
    for (size_t q = 0; q < n; ++q) {
      f1[q] = nu_eff[q] * (d2[0][q] + d2[1][q] + d2[2][q]) -
              (u[0][q] * d1[0][q] + u[1][q] * d1[1][q] + u[2][q] * d1[2][q]);
      up[q] = uc[q] + adu * f1[q] + bdu * f2[q] + cdu * f3[q];
      if (m->bcx == 2 && q % (size_t)m->nx == 0) up[q] = uc[q]; /* open x: inflow held */
    }
  }
  /* history shift, src/integration.f90:176-188 */
  for (int c = 0; c < 3; ++c) {
    if (m->itscheme == 2) {
      memcpy(fu[3 * c + 1], fu[3 * c + 0], n * sizeof(double));
    } else if (m->itscheme == 3) {
      memcpy(fu[3 * c + 2], fu[3 * c + 1], n * sizeof(double));
      memcpy(fu[3 * c + 1], fu[3 * c + 0], n * sizeof(double));
    }
  }
  for (int a = 0; a < 3; ++a) { free(d1[a]); free(d2[a]); }
  free(nu_eff);
}

/* poisson_solver_0000 / _0011 / _111111, src/poisson.f90:41-123.
 * The three routines differ only in the neighbour remap of each axis and in
 * the dynamic-omega factor; the solver is chosen from the x and y boundary
 * types, src/initialization.f90:283-301 (z follows the chosen routine). */
int orc_poisson_sor(const orc_model *m, double *pp, const double *rhs,
                    double *omega_io, double eps, int kmax, int idyn,
                    int *iters, double *dmax_out) {
  const int nx = m->nx, ny = m->ny, nz = m->nz;
  int mirx, miry, mirz;
  double factor;
  if (m->bcx == 0 && m->bcy == 0) { mirx = 0; miry = 0; mirz = 0; factor = 1.05; }
  else if (m->bcx == 0 && m->bcy == 1) { mirx = 0; miry = 1; mirz = 0; factor = 1.01; }
  else { mirx = 1; miry = 1; mirz = 1; factor = 1.05; }
  double omega = *omega_io;
  double dx2 = m->dx * m->dx, dy2 = m->dy * m->dy, dz2 = m->dz * m->dz;
  double oneondx2 = 1.0 / dx2, oneondy2 = 1.0 / dy2, oneondz2 = 1.0 / dz2;
  double twoondx2 = 2.0 * oneondx2, twoondy2 = 2.0 * oneondy2, twoondz2 = 2.0 * oneondz2;
  double A = -(twoondx2 + twoondy2 + twoondz2);
  double dmax_old = 1609.0, dmax = 0.0;
  int status = ORC_SOR_MAXIT, iter;
  for (iter = 1; iter <= kmax; ++iter) {
    dmax = 0.0;
    for (int k = 0; k < nz; ++k) {
      int km1, kp1;
      if (k == 0) { km1 = mirz ? 1 : nz - 1; kp1 = 1; }
      else if (k == nz - 1) { km1 = nz - 2; kp1 = mirz ? nz - 2 : 0; }
      else { km1 = k - 1; kp1 = k + 1; }
      for (int j = 0; j < ny; ++j) {
        int jm1, jp1;
        if (j == 0) { jm1 = miry ? 1 : ny - 1; jp1 = 1; }
        else if (j == ny - 1) { jm1 = ny - 2; jp1 = miry ? ny - 2 : 0; }
        else { jm1 = j - 1; jp1 = j + 1; }
        for (int i = 0; i < nx; ++i) {
          int im1, ip1;
          if (i == 0) { im1 = mirx ? 1 : nx - 1; ip1 = 1; }
          else if (i == nx - 1) { im1 = nx - 2; ip1 = mirx ? nx - 2 : 0; }
          else { im1 = i - 1; ip1 = i + 1; }
          size_t c = IDX(m, i, j, k);
          double pn = (-oneondx2 * (pp[IDX(m, im1, j, k)] + pp[IDX(m, ip1, j, k)]) -
                       oneondy2 * (pp[IDX(m, i, jm1, k)] + pp[IDX(m, i, jp1, k)]) -
                       oneondz2 * (pp[IDX(m, i, j, km1)] + pp[IDX(m, i, j, kp1)]) +
                       rhs[c]) / A;
          double d = fabs(pn - pp[c]);
          dmax = d > dmax ? d : dmax; /* Fortran max(d, dmax) */
          pp[c] = (1.0 - omega) * pp[c] + omega * pn;
        }
      }
    }
    if (dmax < eps) { status = ORC_SOR_CONVERGED; break; }
    if (fabs(dmax_old - dmax) < eps / 1000.0) { status = ORC_SOR_STAGNATED; break; }
    if (iter > 1 && idyn == 1) {
      if (dmax > dmax_old) omega = omega * (2.0 - factor);
      else if (dmax < 0.1 * dmax_old) omega = fmin(omega * factor, 2.0);
    }
    dmax_old = dmax;
  }
  *iters = iter > kmax ? kmax : iter;
  *dmax_out = dmax;
  *omega_io = omega;
  return status;
}

/* correct_pression, src/integration.f90:234-247 (SOR branch) */
int orc_correct_pressure(const orc_model *m, double *pp, double *const upred[3],
                         double *omega, double eps, int kmax, int idyn,
                         int *iters, double *dmax) {
  size_t n = npts(m);
  double *div = fld(m), *rhs = fld(m);
  orc_divergence(m, div, upred[0], upred[1], upred[2], 1);
  for (size_t q = 0; q < n; ++q) rhs[q] = div[q] / m->dt;
  if (m->bcx == 2) {
    /* open x axis (this library's definition): the net flux through the
     * inflow and outflow faces makes the all-Neumann problem incompatible;
     * the trapezoid-weighted mean of the rhs (weight 1/2 at the end nodes of
     * every axis) is removed before the solve */
    double sw = 0.0, swr = 0.0;
    for (int k = 0; k < m->nz; ++k)
      for (int j = 0; j < m->ny; ++j)
        for (int i = 0; i < m->nx; ++i) {
          double w = (i == 0 || i == m->nx - 1) ? 0.5 : 1.0;
          if (j == 0 || j == m->ny - 1) w *= 0.5;
          if (k == 0 || k == m->nz - 1) w *= 0.5;
          sw += w;
          swr += w * rhs[IDX(m, i, j, k)];
        }
    double mean = swr / sw;
    for (size_t q = 0; q < n; ++q) rhs[q] = rhs[q] - mean;
  }
  int st = orc_poisson_sor(m, pp, rhs, omega, eps, kmax, idyn, iters, dmax);
  free(div); free(rhs);
  return st;
}

static int bad_component(const double *f, size_t n) {
  /* contains_nan + maxval > 1000, src/integration.f90:309-325 */
  double mx = -INFINITY;
  for (size_t q = 0; q < n; ++q) {
    if (isnan(f[q])) return 1;
    if (f[q] > mx) mx = f[q];
  }
  return mx > 1000.0;
}

/* correct_velocity, src/integration.f90:297-325 */
int orc_correct_velocity(const orc_model *m, double *u[3], double *const upred[3],
                         const double *pp) {
  size_t n = npts(m);
  double *g = fld(m);
  int bad = 0;
  for (int a = 0; a < 3; ++a) {
    der1(m, g, pp, a, 0);
    for (size_t q = 0; q < n; ++q) u[a][q] = upred[a][q] - m->dt * g[q];
    if (m->bcx == 2) /* open x: the inflow nodes keep their prescribed value */
      for (size_t q = 0; q < n; q += (size_t)m->nx) u[a][q] = upred[a][q];
  }
  for (int a = 0; a < 3 && !bad; ++a) bad = bad_component(u[a], n);
  free(g);
  return bad;
}

/* transeq, src/integration.f90:388-459 */
void orc_transeq(const orc_model *m, double *phi, double *const u[3],
                 const double *src, double *fphi[3], const double *nu_t, int itime) {
  double adu, bdu, cdu;
  ab_coefs(m, itime, &adu, &bdu, &cdu);
  size_t n = npts(m);
  double *d1[3], *d2[3];
  for (int a = 0; a < 3; ++a) {
    d1[a] = fld(m); d2[a] = fld(m);
    der1(m, d1[a], phi, a, 0);
  }
  for (int a = 0; a < 3; ++a) der2(m, d2[a], phi, a, 0);
  double base = 1.0 / (m->re * m->sc);
  for (size_t q = 0; q < n; ++q) {
    double alpha = m->iles == 1 ? base + nu_t[q] / m->sc : base;
    fphi[0][q] = alpha * (d2[0][q] + d2[1][q] + d2[2][q]) -
                 (u[0][q] * d1[0][q] + u[1][q] * d1[1][q] + u[2][q] * d1[2][q]) + src[q];
    if (!(m->bcx == 2 && q % (size_t)m->nx == 0)) /* open x: inflow held */
      phi[q] = phi[q] + adu * fphi[0][q] + bdu * fphi[1][q] + cdu * fphi[2][q];
  }
  /* conservative clipping, src/integration.f90:432-450 */
  double sum_old = 0.0;
  for (size_t q = 0; q < n; ++q) sum_old += phi[q];
  double old_avg = sum_old / (double)n;
  double sum_new = 0.0;
  for (size_t q = 0; q < n; ++q) {
    phi[q] = fmax(0.0, fmin(1.0, phi[q]));
    sum_new += phi[q];
  }
  double excess = old_avg - sum_new / (double)n;
  /* open x: the held inflow nodes take no part of the excess */
  const size_t held = m->bcx == 2 ? (size_t)m->nx : 0;
  double wsum = 0.0;
  for (size_t q = 0; q < n; ++q) wsum += (held && q % held == 0) ? 0.0 : fmin(phi[q], 1.0 - phi[q]);
  /* All points clipped to a bound leaves no weight to spread the excess
   * over (the Fortran divides by zero there); the redistribution is skipped. */
  if (wsum != 0.0) {
    for (size_t q = 0; q < n; ++q) {
      if (held && q % held == 0) continue;
      double w = fmin(phi[q], 1.0 - phi[q]) / wsum;
      phi[q] = fmax(0.0, fmin(1.0, phi[q] + excess * w));
    }
  }
  if (m->itscheme == 2) {
    memcpy(fphi[1], fphi[0], n * sizeof(double));
  } else if (m->itscheme == 3) {
    memcpy(fphi[2], fphi[1], n * sizeof(double));
    memcpy(fphi[1], fphi[0], n * sizeof(double));
  }
  for (int a = 0; a < 3; ++a) { free(d1[a]); free(d2[a]); }
}

/* function_stats, src/functions.f90:27-63 */
void orc_function_stats(const double *f, int n1, int n2, int n3, double out[6]) {
  double sum = 0.0, fmn = 1.79769313486231571e308, fmx = -1.79769313486231571e308;
  int im = 1, jm = 1, km = 1;
  size_t q = 0;
  for (int k = 0; k < n3; ++k)
    for (int j = 0; j < n2; ++j)
      for (int i = 0; i < n1; ++i, ++q) {
        sum = sum + f[q];
        if (f[q] < fmn) fmn = f[q];
        if (f[q] > fmx) { fmx = f[q]; im = i + 1; jm = j + 1; km = k + 1; }
      }
  out[0] = fmn; out[1] = fmx; out[2] = sum / (double)((size_t)n1 * n2 * n3);
  out[3] = im; out[4] = jm; out[5] = km;
}

/* compute_cfl, src/utils.f90:202-204 */
void orc_cfl(const orc_model *m, double *const u[3], double out[3]) {
  size_t n = npts(m);
  double h[3] = {m->dx, m->dy, m->dz};
  for (int a = 0; a < 3; ++a) {
    double mx = 0.0;
    for (size_t q = 0; q < n; ++q) mx = fmax(mx, fabs(u[a][q]));
    out[a] = mx * m->dt / h[a];
  }
}

/* average_3d_array, src/functions.f90:123-155 (sums with i outermost) */
static double average_sq(const orc_model *m, const double *f) {
  double sum = 0.0;
  for (int i = 0; i < m->nx; ++i)
    for (int j = 0; j < m->ny; ++j)
      for (int k = 0; k < m->nz; ++k) {
        double v = f[IDX(m, i, j, k)];
        sum = sum + v * v;
      }
  return sum / (double)npts(m);
}

/* statistics_calc, src/utils.f90:277-367 */
void orc_statistics(const orc_model *m, double *const u[3], double t, double out[17]) {
  size_t n = npts(m);
  double *g[9];
  for (int q = 0; q < 9; ++q) g[q] = fld(m);
  out[0] = t;
  out[5] = average_sq(m, u[0]);
  out[6] = average_sq(m, u[1]);
  out[7] = average_sq(m, u[2]);
  der1(m, g[0], u[0], 0, 1); der1(m, g[1], u[0], 1, 0); der1(m, g[2], u[0], 2, 0);
  der1(m, g[3], u[1], 0, 0); der1(m, g[4], u[1], 1, 1); der1(m, g[5], u[1], 2, 0);
  der1(m, g[6], u[2], 0, 0); der1(m, g[7], u[2], 1, 0); der1(m, g[8], u[2], 2, 1);
  for (int q = 0; q < 9; ++q) out[8 + q] = average_sq(m, g[q]);
  double xnu = 1.0 / m->re;
  double ek = 0.0, eps = 0.0, dz = 0.0;
  for (size_t q = 0; q < n; ++q) {
    double ux = u[0][q], uy = u[1][q], uz = u[2][q];
    ek = ek + 0.5 * (ux * ux + uy * uy + uz * uz);
    double a = 2.0 * g[0][q], b = 2.0 * g[4][q], c = 2.0 * g[8][q];
    double s12 = g[1][q] + g[3][q], s13 = g[2][q] + g[6][q], s23 = g[5][q] + g[7][q];
    eps = eps + 0.5 * xnu * (a * a + b * b + c * c + 2.0 * (s12 * s12) +
                             2.0 * (s13 * s13) + 2.0 * (s23 * s23));
    double w1 = g[7][q] - g[5][q], w2 = g[2][q] - g[6][q], w3 = g[3][q] - g[1][q];
    dz = dz + 0.5 * (w1 * w1 + w2 * w2 + w3 * w3);
  }
  out[1] = ek / (double)n;
  out[2] = eps / (double)n;
  out[4] = dz / (double)n;
  der2(m, g[0], u[0], 0, 1); der2(m, g[1], u[0], 1, 0); der2(m, g[2], u[0], 2, 0);
  der2(m, g[3], u[1], 0, 0); der2(m, g[4], u[1], 1, 1); der2(m, g[5], u[1], 2, 0);
  der2(m, g[6], u[2], 0, 0); der2(m, g[7], u[2], 1, 0); der2(m, g[8], u[2], 2, 1);
  double eps2 = 0.0;
  for (size_t q = 0; q < n; ++q) {
    double t1 = (-xnu) * (u[0][q] * (g[0][q] + g[1][q] + g[2][q]) +
                          u[1][q] * (g[3][q] + g[4][q] + g[5][q]) +
                          u[2][q] * (g[6][q] + g[7][q] + g[8][q]));
    eps2 = eps2 + t1;
  }
  out[3] = eps2 / (double)n;
  for (int q = 0; q < 9; ++q) free(g[q]);
}

/* grid coordinates, src/initialization.f90:211-219 */
static double coord(double o, double h, int i) { return o + (double)i * h; }

/* initialize_taylor_green_vortex, src/initial_conditions.f90:139-167 */
void orc_init_tgv(const orc_model *m, double x0, double y0, double z0,
                  double u0, double l0, double ratio, int nscr, double *ux,
                  double *uy, double *uz, double *pp, double *phi) {
  for (int k = 0; k < m->nz; ++k) {
    double z = coord(z0, m->dz, k);
    double twoz = 2.0 * z;
    for (int j = 0; j < m->ny; ++j) {
      double y = coord(y0, m->dy, j);
      double twoy = 2.0 * y;
      for (int i = 0; i < m->nx; ++i) {
        double x = coord(x0, m->dx, i);
        double twox = 2.0 * x;
        size_t c = IDX(m, i, j, k);
        ux[c] = ratio * u0 / l0 * sin(x) * cos(y) * cos(z);
        uy[c] = -ratio * u0 / l0 * cos(x) * sin(y) * cos(z);
        uz[c] = 0.0;
        pp[c] = 0.0625 * (cos(twox) + cos(twoy)) * (cos(twoz) + 2.0);
      }
    }
  }
  if (nscr == 1) {
    double xn = coord(x0, m->dx, m->nx - 1), yn = coord(y0, m->dy, m->ny - 1),
           zn = coord(z0, m->dz, m->nz - 1);
    double R = 0.25 * (xn - x0);
    double cx = 0.5 * (x0 + xn), cy = 0.5 * (y0 + yn), cz = 0.5 * (z0 + zn);
    for (int k = 0; k < m->nz; ++k)
      for (int j = 0; j < m->ny; ++j)
        for (int i = 0; i < m->nx; ++i) {
          double x = coord(x0, m->dx, i), y = coord(y0, m->dy, j), z = coord(z0, m->dz, k);
          double dist = sqrt((x - cx) * (x - cx) + (y - cy) * (y - cy) + (z - cz) * (z - cz));
          /* the reference divides by the LES filter width `delta` here */
          phi[IDX(m, i, j, k)] = 0.5 * (1.0 - tanh((dist - R) / m->delta));
        }
  }
}

/* initialize_mixing_layer, src/initial_conditions.f90:364-389 */
void orc_init_mixing_layer(const orc_model *m, double x0, double y0, double z0,
                           double u0, double l0, double ratio, int nscr,
                           double *ux, double *uy, double *uz, double *pp,
                           double *phi) {
  (void)x0; (void)z0;
  double u1, u2;
  if (ratio < 1e-12 && ratio > -1e-12) { u2 = u0; u1 = 0.0; }
  else { u2 = u0 / (1.0 - ratio); u1 = u2 * ratio; }
  double theta_o = 1.0 / (13.0 * l0);
  double t1 = 0.5 * (u2 + u1), t2 = 0.5 * (u1 - u2);
  for (int k = 0; k < m->nz; ++k)
    for (int j = 0; j < m->ny; ++j) {
      double y = coord(y0, m->dy, j);
      double t3 = y * log(2.0) / (2.0 * theta_o);
      for (int i = 0; i < m->nx; ++i) {
        size_t c = IDX(m, i, j, k);
        ux[c] = t1 - t2 * tanh(t3);
        uy[c] = 0.0;
        uz[c] = 0.0;
        if (nscr == 1) phi[c] = 0.5 - 0.5 * tanh(t3);
        pp[c] = 1.0;
      }
    }
}

/* initialize_coplanar_jet, src/initial_conditions.f90:244-327: an inner jet
 * of velocity u1 = u0/ratio within |y| < (h1 + h2)/2, an outer co-flow u0
 * beyond, zero velocity outside the outer layer; tanh shear layers of
 * momentum thickness h1/10 and h2/25; p = 0 */
void orc_init_coplanar_jet(const orc_model *m, double y0, double u0, double l0,
                           double ratio, int nscr, double *ux, double *uy,
                           double *uz, double *pp, double *phi) {
  double u2 = u0, u1 = u2 / ratio, u3 = 0.0 * u2;
  double d1 = l0, d2 = 2.0 * d1, h1 = 0.5 * d1, h2 = 0.5 * d2;
  double theta_1 = h1 / 10.0, theta_2 = h2 / 25.0, hm = 0.5 * (h1 + h2);
  for (int k = 0; k < m->nz; ++k)
    for (int j = 0; j < m->ny; ++j) {
      double y = coord(y0, m->dy, j), ay = fabs(y);
      for (int i = 0; i < m->nx; ++i) {
        size_t c = IDX(m, i, j, k);
        if (ay < hm) {
          ux[c] = 0.5 * (u1 + u2) + 0.5 * (u2 - u1) * tanh((ay - h1) / (2.0 * theta_1));
          if (nscr == 1) phi[c] = 0.5 * (0.0 + 1.0) + 0.5 * (1.0 - 0.0) * tanh((ay - h1) / (2.0 * theta_1));
        } else {
          ux[c] = 0.5 * (u2 + u3) + 0.5 * (u3 - u2) * tanh((ay - h2) / (2.0 * theta_2));
          if (nscr == 1) phi[c] = 0.5 * (1.0 + 0.0) + 0.5 * (0.0 - 1.0) * tanh((ay - h2) / (2.0 * theta_2));
        }
        uy[c] = 0.0;
        uz[c] = 0.0;
        pp[c] = 0.0;
      }
    }
}

/* rotational(rotx, roty, rotz, ux, uy, uz, ...), src/differential_operators.f90:
 * 40-77: the curl with the even ("p") closures of the bound derivatives */
void orc_rotational(const orc_model *m, double *const u[3], double *rot[3]) {
  double *a = fld(m), *b = fld(m);
  size_t n = npts(m);
  der1(m, a, u[2], 1, 0); der1(m, b, u[1], 2, 0);          /* deryp(uz), derzp(uy) */
  for (size_t q = 0; q < n; ++q) rot[0][q] = a[q] - b[q];
  der1(m, a, u[0], 2, 0); der1(m, b, u[2], 0, 0);          /* derzp(ux), derxp(uz) */
  for (size_t q = 0; q < n; ++q) rot[1][q] = a[q] - b[q];
  der1(m, a, u[1], 0, 0); der1(m, b, u[0], 1, 0);          /* derxp(uy), deryp(ux) */
  for (size_t q = 0; q < n; ++q) rot[2][q] = a[q] - b[q];
  free(a); free(b);
}

/* calculate_Q_criterion, src/differential_operators.f90:79-108 */
void orc_q_criterion(const orc_model *m, double *q, double *const u[3]) {
  size_t n = npts(m);
  double *g[9];
  for (int k = 0; k < 9; ++k) g[k] = fld(m);
  der1(m, g[0], u[0], 0, 1); der1(m, g[1], u[1], 1, 1); der1(m, g[2], u[2], 2, 1); /* derxi, deryi, derzi */
  der1(m, g[3], u[0], 1, 0); der1(m, g[4], u[0], 2, 0); der1(m, g[5], u[1], 0, 0); /* duxdy, duxdz, duydx */
  der1(m, g[6], u[1], 2, 0); der1(m, g[7], u[2], 0, 0); der1(m, g[8], u[2], 1, 0); /* duydz, duzdx, duzdy */
  for (size_t c = 0; c < n; ++c) {
    q[c] = -0.5 * (pow(g[0][c], 2.0) + pow(g[1][c], 2.0) + pow(g[2][c], 2.0)) -
           g[3][c] * g[5][c] - g[4][c] * g[7][c] - g[6][c] * g[8][c];
  }
  for (int k = 0; k < 9; ++k) free(g[k]);
}

/* calculate_residuals, src/utils.f90:93-163: over the interior points
 * (2..n-1 in Fortran indexing) of each component, the rms and the max of
 * |old - u| / (2 dt), scaled by t_ref / u_ref, the rms normalised by all
 * nx ny nz points; the max's location is the last one in loop order
 * (i fastest), 1-based.  out = res_u, res_v, res_w, linf_u, linf_v, linf_w,
 * then (i, j, k) of each max. */
void orc_residuals(const orc_model *m, double *const u[3], double *const old[3], double dt,
                   double t_ref, double u_ref, double out[15]) {
  int nx = m->nx, ny = m->ny, nz = m->nz;
  for (int a = 0; a < 3; ++a) {
    double res = 0.0, linf = 0.0;
    int ia = 0, ja = 0, ka = 0;
    for (int k = 1; k < nz - 1; ++k)
      for (int j = 1; j < ny - 1; ++j)
        for (int i = 1; i < nx - 1; ++i) {
          size_t c = IDX(m, i, j, k);
          double v = fabs(old[a][c] - u[a][c]) / (2.0 * dt);
          res += pow(v, 2.0);
          if (v > linf) linf = v;
        }
    for (int k = 1; k < nz - 1; ++k)
      for (int j = 1; j < ny - 1; ++j)
        for (int i = 1; i < nx - 1; ++i) {
          size_t c = IDX(m, i, j, k);
          double v = fabs(old[a][c] - u[a][c]) / (2.0 * dt);
          if (fabs(linf - v) <= DBL_MIN) { ia = i + 1; ja = j + 1; ka = k + 1; }
        }
    out[a] = (t_ref / u_ref) * sqrt((1.0 / (double)((long long)nx * ny * nz)) * res);
    out[3 + a] = (t_ref / u_ref) * linf;
    out[6 + 3 * a] = ia; out[7 + 3 * a] = ja; out[8 + 3 * a] = ka;
  }
}

/* one pass of the time loop body, src/osinco3d_main.f90:104-128, no I/O */
void orc_step(const orc_model *m, orc_state *s, int itime, orc_step_info *info) {
  memset(info, 0, sizeof(*info));
  orc_predict_velocity(m, s->upred, s->u, s->fu, s->nu_t, itime);
  info->sor_status = orc_correct_pressure(m, s->pp, s->upred, &s->omega, s->eps,
                                          s->kmax, s->idyn, &info->sor_iters,
                                          &info->sor_dmax);
  info->omega = s->omega;
  info->diverged = orc_correct_velocity(m, s->u, s->upred, s->pp);
  if (m->nscr == 1) orc_transeq(m, s->phi, s->u, s->src, s->fphi, s->nu_t, itime);
  double *div = fld(m);
  orc_divergence(m, div, s->upred[0], s->upred[1], s->upred[2], 1);
  orc_function_stats(div, m->nx, m->ny, m->nz, info->divu_pred_stats);
  orc_divergence(m, div, s->u[0], s->u[1], s->u[2], 1);
  orc_function_stats(div, m->nx, m->ny, m->nz, info->divu_stats);
  orc_cfl(m, s->u, info->cfl);
  free(div);
}

/* Red-black SOR sweep: red points (i+j+k even, 0-based) first, then black,
 * each with the neighbour remap of the lexicographic solver. */
double orc_rbsor_sweep(const orc_model *m, double *pp, const double *rhs, double omega) {
  const int nx = m->nx, ny = m->ny, nz = m->nz;
  int mirx, miry, mirz;
  if (m->bcx == 0 && m->bcy == 0) { mirx = 0; miry = 0; mirz = 0; }
  else if (m->bcx == 0 && m->bcy == 1) { mirx = 0; miry = 1; mirz = 0; }
  else { mirx = 1; miry = 1; mirz = 1; }
  double dx2 = m->dx * m->dx, dy2 = m->dy * m->dy, dz2 = m->dz * m->dz;
  double ox = 1.0 / dx2, oy = 1.0 / dy2, oz = 1.0 / dz2;
  double A = -(2.0 * ox + 2.0 * oy + 2.0 * oz);
  double dmax = 0.0;
  for (int color = 0; color < 2; ++color)
    for (int k = 0; k < nz; ++k) {
      int km1 = k == 0 ? (mirz ? 1 : nz - 1) : k - 1;
      int kp1 = k == nz - 1 ? (mirz ? nz - 2 : 0) : k + 1;
      for (int j = 0; j < ny; ++j) {
        int jm1 = j == 0 ? (miry ? 1 : ny - 1) : j - 1;
        int jp1 = j == ny - 1 ? (miry ? ny - 2 : 0) : j + 1;
        for (int i = (j + k + color) & 1; i < nx; i += 2) {
          int im1 = i == 0 ? (mirx ? 1 : nx - 1) : i - 1;
          int ip1 = i == nx - 1 ? (mirx ? nx - 2 : 0) : i + 1;
          size_t c = IDX(m, i, j, k);
          double pn = (-ox * (pp[IDX(m, im1, j, k)] + pp[IDX(m, ip1, j, k)]) -
                       oy * (pp[IDX(m, i, jm1, k)] + pp[IDX(m, i, jp1, k)]) -
                       oz * (pp[IDX(m, i, j, km1)] + pp[IDX(m, i, j, kp1)]) + rhs[c]) / A;
          double d = fabs(pn - pp[c]);
          dmax = d > dmax ? d : dmax;
          pp[c] = (1.0 - omega) * pp[c] + omega * pn;
        }
      }
    }
  return dmax;
}

/* poisson.f90:52-123's control loop (same tests, same order, same factors
 * as orc_poisson_sor above) around one red-black sweep per iteration */
int orc_poisson_rbsor(const orc_model *m, double *pp, const double *rhs,
                      double *omega_io, double eps, int kmax, int idyn,
                      int *iters, double *dmax_out, double *omega_trace,
                      double *dmax_trace) {
  double factor;
  if (m->bcx == 0 && m->bcy == 0) factor = 1.05;       /* poisson.f90:35 */
  else if (m->bcx == 0 && m->bcy == 1) factor = 1.01;  /* poisson.f90:162 */
  else factor = 1.05;                                  /* poisson.f90:288 */
  double omega = *omega_io;
  double dmax_old = 1609.0, dmax = 0.0;
  int status = ORC_SOR_MAXIT, iter;
  for (iter = 1; iter <= kmax; ++iter) {
    dmax = orc_rbsor_sweep(m, pp, rhs, omega);
    int stop = 0;
    if (dmax < eps) { status = ORC_SOR_CONVERGED; stop = 1; }
    else if (fabs(dmax_old - dmax) < eps / 1000.0) { status = ORC_SOR_STAGNATED; stop = 1; }
    else {
      if (iter > 1 && idyn == 1) {
        if (dmax > dmax_old) omega = omega * (2.0 - factor);
        else if (dmax < 0.1 * dmax_old) omega = fmin(omega * factor, 2.0);
      }
      dmax_old = dmax;
    }
    if (omega_trace) omega_trace[iter - 1] = omega;
    if (dmax_trace) dmax_trace[iter - 1] = dmax;
    if (stop) break;
  }
  *iters = iter > kmax ? kmax : iter;
  *dmax_out = dmax;
  *omega_io = omega;
  return status;
}
