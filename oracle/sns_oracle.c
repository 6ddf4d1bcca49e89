/*
 * TEST INFRASTRUCTURE ONLY -- CPU oracle for the SMR-RK3 step (see
 * sns_oracle.h). Restated from the reference's published algorithm; every
 * floating-point expression is kept in the reference's evaluation order (the
 * citation above each one gives file:line), because the GPU path is checked
 * against this code for identical bits.
 */
#include <float.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif
#include "rfft.h"
#include "sns_oracle.h"

#define ORACLE_PI 3.1415926535897932 /* include/common.h:7 */
#define T_XM (+0.5)                  /* include/temperature.h:22 */
#define T_XP (-0.5)                  /* include/temperature.h:23 */

struct oracle_case {
  int nx, ny; /* itot, jtot */
  double lx, ly, dy, Ra, Pr;
  double *xf, *xc, *dxf, *dxc;
  int with_temperature, with_thermal_forcing;
  double rk_a[3], rk_b[3], rk_g[3];
  double dt, time;
  int step, implicitx, implicity;
  double costs[2][2];
  /* state, reference layouts */
  double *ux, *uy, *p, *psi, *temp, *tforce;
  double *sux_a, *sux_b, *sux_g, *suy_a, *suy_b, *suy_g, *st_a, *st_b, *st_g;
  oracle_rfft_plan fft;
};

/* ---------------------------------------------------------------- layouts */
/* include/arrays/fluid.h and temperature.h: x fastest, halo rows j=0,jtot+1 */
static inline long iu(const oracle_case *c, int i, int j) { return (long)j * (c->nx + 1) + (i - 1); }
static inline long ic(const oracle_case *c, int i, int j) { return (long)j * (c->nx + 2) + i; }
static inline long isx(const oracle_case *c, int i, int j) { return (long)(j - 1) * (c->nx - 1) + (i - 2); }
static inline long isc(const oracle_case *c, int i, int j) { return (long)(j - 1) * c->nx + (i - 1); }
/* include/arrays/param.h */
#define DXF(i) (c->dxf[(i)-1])
#define DXC(i) (c->dxc[(i)-1])
#define XF(i) (c->xf[(i)-1])
#define XC(i) (c->xc[(i)])

static int g_threads = 1;
void oracle_set_threads(int nthreads) { g_threads = nthreads > 0 ? nthreads : 1; }

/* ------------------------------------------------------------ grid set-up */
static void build_grid(oracle_case *c, double stretch_in) {
  const int nx = c->nx, ny = c->ny;
  c->xf = calloc(nx + 1, sizeof(double));
  c->xc = calloc(nx + 2, sizeof(double));
  c->dxf = calloc(nx, sizeof(double));
  c->dxc = calloc(nx + 1, sizeof(double));
  /* src/param/init.c:142-166: uniform when stretch >= itot/2 (integer
   * division, stretch truncated to int), else clipped Chebyshev */
  int stretch = (int)stretch_in;
  if (stretch < 0) stretch = 0;
  if (stretch >= nx / 2) {
    const double dx = c->lx / nx;
    for (int i = 1; i <= nx + 1; i++) XF(i) = 1. * (i - 1) * dx;
  } else {
    for (int i = 1; i <= nx + 1; i++)
      XF(i) = cos(ORACLE_PI * (1. * (i - 1) + stretch) / (nx + 2. * stretch));
    const double lo = XF(1), hi = XF(nx + 1);
    for (int i = 1; i <= nx + 1; i++) XF(i) = c->lx * (XF(i) - lo) / (hi - lo);
  }
  XF(1) = 0.;
  XF(nx + 1) = c->lx;
  for (int i = 1; i <= nx; i++) DXF(i) = XF(i + 1) - XF(i);       /* :170-172 */
  XC(0) = XF(1);                                                  /* :175-179 */
  for (int i = 1; i <= nx; i++) XC(i) = 0.5 * (XF(i) + XF(i + 1));
  XC(nx + 1) = XF(nx + 1);
  for (int i = 1; i <= nx + 1; i++) DXC(i) = XC(i) - XC(i - 1);   /* :182-185 */
  c->dy = c->ly / ny;                                             /* :187 */
  (void)ny;
}

static void set_rk(oracle_case *c) {
  /* src/param/init.c:197-213 */
  c->rk_a[0] = 32. / 60.; c->rk_b[0] = 0. / 60.;
  c->rk_a[1] = 25. / 60.; c->rk_b[1] = -17. / 60.;
  c->rk_a[2] = 45. / 60.; c->rk_b[2] = -25. / 60.;
  for (int k = 0; k < 3; k++) c->rk_g[k] = c->rk_a[k] + c->rk_b[k];
}

/* ------------------------------------------------------------- boundaries */
/* src/fluid/boundary_conditions.c:6-21 */
static void bc_ux(oracle_case *c) {
  const int nx = c->nx, ny = c->ny;
  for (int i = 2; i <= nx; i++) {
    c->ux[iu(c, i, 0)] = c->ux[iu(c, i, ny)];
    c->ux[iu(c, i, ny + 1)] = c->ux[iu(c, i, 1)];
  }
  for (int j = 0; j <= ny + 1; j++) {
    c->ux[iu(c, 1, j)] = 0.;
    c->ux[iu(c, nx + 1, j)] = 0.;
  }
}

/* src/fluid/boundary_conditions.c:23-38 */
static void bc_uy(oracle_case *c) {
  const int nx = c->nx, ny = c->ny;
  for (int i = 1; i <= nx; i++) {
    c->uy[ic(c, i, 0)] = c->uy[ic(c, i, ny)];
    c->uy[ic(c, i, ny + 1)] = c->uy[ic(c, i, 1)];
  }
  for (int j = 0; j <= ny + 1; j++) {
    c->uy[ic(c, 0, j)] = 0.;
    c->uy[ic(c, nx + 1, j)] = 0.;
  }
}

/* src/fluid/boundary_conditions.c:40-55 (also applied to psi, compute_potential.c:159) */
static void bc_p(oracle_case *c, double *f) {
  const int nx = c->nx, ny = c->ny;
  for (int i = 1; i <= nx; i++) {
    f[ic(c, i, 0)] = f[ic(c, i, ny)];
    f[ic(c, i, ny + 1)] = f[ic(c, i, 1)];
  }
  for (int j = 0; j <= ny + 1; j++) {
    f[ic(c, 0, j)] = f[ic(c, 1, j)];
    f[ic(c, nx + 1, j)] = f[ic(c, nx, j)];
  }
}

/* src/temperature/boundary_conditions.c:6-21: walls only on j in [1, jtot] */
static void bc_temp(oracle_case *c) {
  const int nx = c->nx, ny = c->ny;
  for (int i = 1; i <= nx; i++) {
    c->temp[ic(c, i, 0)] = c->temp[ic(c, i, ny)];
    c->temp[ic(c, i, ny + 1)] = c->temp[ic(c, i, 1)];
  }
  for (int j = 1; j <= ny; j++) {
    c->temp[ic(c, 0, j)] = T_XM;
    c->temp[ic(c, nx + 1, j)] = T_XP;
  }
}

/* ------------------------------------------------------ tridiagonal solves */
/* src/linalg.c:9-30 (Thomas with the |pivot| < DBL_EPSILON guard) */
static void thomas(int n, double *l, double *d, double *u, double *q) {
  u[0] = u[0] / d[0];
  q[0] = q[0] / d[0];
  for (int i = 1; i <= n - 1; i++) {
    double v = d[i] - l[i] * u[i - 1];
    if (fabs(v) < DBL_EPSILON) {
      u[i] = 0.;
      q[i] = 0.;
    } else {
      v = 1. / v;
      u[i] = v * u[i];
      q[i] = v * (q[i] - l[i] * q[i - 1]);
    }
  }
  for (int i = n - 2; i >= 0; i--) q[i] -= u[i] * q[i + 1];
}

/* src/linalg.c:32-50: same recurrence on a complex right-hand side; real
 * matrix times complex value acts on both parts separately */
static void thomas_cplx(int n, double *l, double *d, double *u, double *qr, double *qi) {
  u[0] = u[0] / d[0];
  qr[0] = qr[0] / d[0];
  qi[0] = qi[0] / d[0];
  for (int i = 1; i <= n - 1; i++) {
    double v = d[i] - l[i] * u[i - 1];
    if (fabs(v) < DBL_EPSILON) {
      u[i] = 0.;
      qr[i] = 0.;
      qi[i] = 0.;
    } else {
      v = 1. / v;
      u[i] = v * u[i];
      qr[i] = v * (qr[i] - l[i] * qr[i - 1]);
      qi[i] = v * (qi[i] - l[i] * qi[i - 1]);
    }
  }
  for (int i = n - 2; i >= 0; i--) {
    qr[i] -= u[i] * qr[i + 1];
    qi[i] -= u[i] * qi[i + 1];
  }
}

/* src/linalg.c:52-108: periodic system as two Thomas solves of size n-1 and
 * a rank-one closure for the last unknown */
static void thomas_periodic(int n, const double *l, const double *d, const double *u, double *q) {
  double *l0 = malloc(sizeof(double) * (n - 1)), *d0 = malloc(sizeof(double) * (n - 1));
  double *u0 = malloc(sizeof(double) * (n - 1)), *q0 = malloc(sizeof(double) * (n - 1));
  double *l1 = malloc(sizeof(double) * (n - 1)), *d1 = malloc(sizeof(double) * (n - 1));
  double *u1 = malloc(sizeof(double) * (n - 1)), *q1 = malloc(sizeof(double) * (n - 1));
  for (int i = 0; i < n - 1; i++) {
    l0[i] = l1[i] = l[i];
    d0[i] = d1[i] = d[i];
    u0[i] = u1[i] = u[i];
    q0[i] = q[i];
    q1[i] = i == 0 ? -l[i] : i == n - 2 ? -u[i] : 0.;
  }
  thomas(n - 1, l0, d0, u0, q0);
  thomas(n - 1, l1, d1, u1, q1);
  q[n - 1] = (q[n - 1] - u[n - 1] * q0[0] - l[n - 1] * q0[n - 2])
           / (d[n - 1] + u[n - 1] * q1[0] + l[n - 1] * q1[n - 2]);
  for (int i = 0; i <= n - 2; i++) q[i] = q0[i] + q[n - 1] * q1[i];
  free(l0); free(d0); free(u0); free(q0);
  free(l1); free(d1); free(u1); free(q1);
}

/* implicit y: one periodic solve per x-column of a jtot-row increment field
 * stored x fastest with row stride `width`; columns [i_lo, i_hi) in storage
 * coordinates. Equivalent to the reference's transpose, solve per column and
 * transpose back (src/fluid/update_velocity.c:281-333). */
static void solve_y_columns(oracle_case *c, double *q, int width, int i_lo, int i_hi, double pf) {
  const int ny = c->ny;
  const double dy = c->dy;
#pragma omp parallel for num_threads(g_threads) schedule(static)
  for (int i = i_lo; i < i_hi; i++) {
    double *l = malloc(sizeof(double) * ny), *d = malloc(sizeof(double) * ny);
    double *u = malloc(sizeof(double) * ny), *r = malloc(sizeof(double) * ny);
    for (int j = 0; j < ny; j++) {
      const double cm = 1. / dy / dy, cp = 1. / dy / dy; /* update_velocity.c:306-308 */
      const double c0 = -cm - cp;
      l[j] = -pf * cm;
      u[j] = -pf * cp;
      d[j] = 1. - pf * c0;
      r[j] = q[(long)j * width + i];
    }
    thomas_periodic(ny, l, d, u, r);
    for (int j = 0; j < ny; j++) q[(long)j * width + i] = r[j];
    free(l); free(d); free(u); free(r);
  }
}

/* ----------------------------------------------------------- temperature */
/* src/temperature/force.c:6-32 */
static void temp_force(oracle_case *c) {
  const int nx = c->nx, ny = c->ny;
  for (int j = 1; j <= ny; j++)
    for (int i = 2; i <= nx; i++) {
      const long k = isx(c, i, j);
      if (c->with_thermal_forcing) {
        const double tm = c->temp[ic(c, i - 1, j)], tp = c->temp[ic(c, i, j)];
        c->tforce[k] = 0.5 * tm + 0.5 * tp;
      } else {
        c->tforce[k] = 0.;
      }
    }
}

/* src/temperature/update.c:11-87 */
static void temp_rhs(oracle_case *c) {
  const int nx = c->nx, ny = c->ny, impx = c->implicitx, impy = c->implicity;
  const double dy = c->dy, Ra = c->Ra, Pr = c->Pr;
  const double *T = c->temp, *ux = c->ux, *uy = c->uy;
  memcpy(c->st_b, c->st_a, sizeof(double) * nx * ny);
#pragma omp parallel for num_threads(g_threads) schedule(static)
  for (int j = 1; j <= ny; j++)
    for (int i = 1; i <= nx; i++) {
      const double gxm = (-T[ic(c, i - 1, j)] + T[ic(c, i, j)]) / DXC(i);
      const double gxp = (-T[ic(c, i, j)] + T[ic(c, i + 1, j)]) / DXC(i + 1);
      const double gym = (-T[ic(c, i, j - 1)] + T[ic(c, i, j)]) / dy;
      const double gyp = (-T[ic(c, i, j)] + T[ic(c, i, j + 1)]) / dy;
      const double cxm = DXC(i) / (2. * DXF(i)), cxp = DXC(i + 1) / (2. * DXF(i));
      const double axm = ux[iu(c, i, j)], axp = ux[iu(c, i + 1, j)];
      const double adv1 = -cxm * axm * gxm - cxp * axp * gxp;
      const double aym = uy[ic(c, i, j)], ayp = uy[ic(c, i, j + 1)];
      const double adv2 = -0.5 * aym * gym - 0.5 * ayp * gyp;
      const double kappa = 1. / sqrt(Pr) / sqrt(Ra);
      const double dif1 = kappa * (gxp - gxm) / DXF(i);
      const double dif2 = kappa * (gyp - gym) / dy;
      c->st_a[isc(c, i, j)] = +(adv1 + adv2) + (1. - 1. * impx) * dif1 + (1. - 1. * impy) * dif2;
      c->st_g[isc(c, i, j)] = +(+1. * impx) * dif1 + (+1. * impy) * dif2;
    }
}

/* src/temperature/update.c:89-231 */
static void temp_advance(oracle_case *c, int rk) {
  const int nx = c->nx, ny = c->ny;
  const double a = c->rk_a[rk], b = c->rk_b[rk], g = c->rk_g[rk], dt = c->dt;
  double *q = malloc(sizeof(double) * nx * ny); /* qx, x fastest, rows j=1..jtot */
  for (int j = 1; j <= ny; j++)
    for (int i = 1; i <= nx; i++) {
      const long k = isc(c, i, j);
      q[k] = +a * dt * c->st_a[k] + b * dt * c->st_b[k] + g * dt * c->st_g[k];
    }
  if (c->implicitx) {
#pragma omp parallel for num_threads(g_threads) schedule(static)
    for (int j = 1; j <= ny; j++) {
      double *l = malloc(sizeof(double) * nx), *d = malloc(sizeof(double) * nx);
      double *u = malloc(sizeof(double) * nx), *r = malloc(sizeof(double) * nx);
      for (int i = 1; i <= nx; i++) {
        const double pf = (g * dt) / (2. * sqrt(c->Pr) * sqrt(c->Ra));
        const double cm = 1. / DXF(i) / DXC(i), cp = 1. / DXF(i) / DXC(i + 1);
        const double c0 = -cm - cp;
        l[i - 1] = -pf * cm;
        u[i - 1] = -pf * cp;
        d[i - 1] = 1. - pf * c0;
        r[i - 1] = q[isc(c, i, j)];
      }
      thomas(nx, l, d, u, r);
      for (int i = 1; i <= nx; i++) q[isc(c, i, j)] = r[i - 1];
      free(l); free(d); free(u); free(r);
    }
  }
  if (c->implicity) {
    const double pf = (g * dt) / (2. * sqrt(c->Pr) * sqrt(c->Ra));
    solve_y_columns(c, q, nx, 0, nx, pf);
  }
  for (int j = 1; j <= ny; j++)
    for (int i = 1; i <= nx; i++) c->temp[ic(c, i, j)] += q[isc(c, i, j)];
  free(q);
  bc_temp(c);
}

/* --------------------------------------------------------------- velocity */
/* src/fluid/update_velocity.c:11-104 */
static void ux_rhs(oracle_case *c) {
  const int nx = c->nx, ny = c->ny, impx = c->implicitx, impy = c->implicity;
  const double dy = c->dy, Ra = c->Ra, Pr = c->Pr;
  const double *ux = c->ux, *uy = c->uy, *p = c->p;
  memcpy(c->sux_b, c->sux_a, sizeof(double) * (nx - 1) * ny);
#pragma omp parallel for num_threads(g_threads) schedule(static)
  for (int j = 1; j <= ny; j++)
    for (int i = 2; i <= nx; i++) {
      const double gxm = (-ux[iu(c, i - 1, j)] + ux[iu(c, i, j)]) / DXF(i - 1);
      const double gxp = (-ux[iu(c, i, j)] + ux[iu(c, i + 1, j)]) / DXF(i);
      const double gym = (-ux[iu(c, i, j - 1)] + ux[iu(c, i, j)]) / dy;
      const double gyp = (-ux[iu(c, i, j)] + ux[iu(c, i, j + 1)]) / dy;
      const double cxm = DXF(i - 1) / (2. * DXC(i)), cxp = DXF(i) / (2. * DXC(i));
      const double vxm = 0.5 * ux[iu(c, i - 1, j)] + 0.5 * ux[iu(c, i, j)];
      const double vxp = 0.5 * ux[iu(c, i, j)] + 0.5 * ux[iu(c, i + 1, j)];
      const double adv1 = -cxm * vxm * gxm - cxp * vxp * gxp;
      const double vym = cxm * uy[ic(c, i - 1, j)] + cxp * uy[ic(c, i, j)];
      const double vyp = cxm * uy[ic(c, i - 1, j + 1)] + cxp * uy[ic(c, i, j + 1)];
      const double adv2 = -0.5 * vym * gym - 0.5 * vyp * gyp;
      const double nu = sqrt(Pr) / sqrt(Ra);
      const double dif1 = nu * (gxp - gxm) / DXC(i);
      const double dif2 = nu * (gyp - gym) / dy;
      const double pre = -(p[ic(c, i, j)] - p[ic(c, i - 1, j)]) / DXC(i);
      const double buoy = c->tforce[isx(c, i, j)];
      const long k = isx(c, i, j);
      c->sux_a[k] = +(adv1 + adv2) + (1. - 1. * impx) * dif1 + (1. - 1. * impy) * dif2 + buoy;
      c->sux_g[k] = +(+1. * impx) * dif1 + (+1. * impy) * dif2 + pre;
    }
}

/* src/fluid/update_velocity.c:106-192 */
static void uy_rhs(oracle_case *c) {
  const int nx = c->nx, ny = c->ny, impx = c->implicitx, impy = c->implicity;
  const double dy = c->dy, Ra = c->Ra, Pr = c->Pr;
  const double *ux = c->ux, *uy = c->uy, *p = c->p;
  memcpy(c->suy_b, c->suy_a, sizeof(double) * nx * ny);
#pragma omp parallel for num_threads(g_threads) schedule(static)
  for (int j = 1; j <= ny; j++)
    for (int i = 1; i <= nx; i++) {
      const double gxm = (-uy[ic(c, i - 1, j)] + uy[ic(c, i, j)]) / DXC(i);
      const double gxp = (-uy[ic(c, i, j)] + uy[ic(c, i + 1, j)]) / DXC(i + 1);
      const double gym = (-uy[ic(c, i, j - 1)] + uy[ic(c, i, j)]) / dy;
      const double gyp = (-uy[ic(c, i, j)] + uy[ic(c, i, j + 1)]) / dy;
      const double cxm = DXC(i) / (2. * DXF(i)), cxp = DXC(i + 1) / (2. * DXF(i));
      const double vxm = 0.5 * ux[iu(c, i, j - 1)] + 0.5 * ux[iu(c, i, j)];
      const double vxp = 0.5 * ux[iu(c, i + 1, j - 1)] + 0.5 * ux[iu(c, i + 1, j)];
      const double adv1 = -cxm * vxm * gxm - cxp * vxp * gxp;
      const double vym = 0.5 * uy[ic(c, i, j - 1)] + 0.5 * uy[ic(c, i, j)];
      const double vyp = 0.5 * uy[ic(c, i, j)] + 0.5 * uy[ic(c, i, j + 1)];
      const double adv2 = -0.5 * vym * gym - 0.5 * vyp * gyp;
      const double nu = sqrt(Pr) / sqrt(Ra);
      const double dif1 = nu * (gxp - gxm) / DXF(i);
      const double dif2 = nu * (gyp - gym) / dy;
      const double pre = -(p[ic(c, i, j)] - p[ic(c, i, j - 1)]) / dy;
      const long k = isc(c, i, j);
      c->suy_a[k] = +(adv1 + adv2) + (1. - 1. * impx) * dif1 + (1. - 1. * impy) * dif2;
      c->suy_g[k] = +(+1. * impx) * dif1 + (+1. * impy) * dif2 + pre;
    }
}

/* src/fluid/update_velocity.c:194-344 */
static void ux_advance(oracle_case *c, int rk) {
  const int nx = c->nx, ny = c->ny, w = nx + 1;
  const double a = c->rk_a[rk], b = c->rk_b[rk], g = c->rk_g[rk], dt = c->dt;
  double *q = malloc(sizeof(double) * (size_t)w * ny); /* x fastest, i=1..itot+1 at [i-1] */
  for (int j = 1; j <= ny; j++)
    for (int i = 1; i <= nx + 1; i++)
      q[(long)(j - 1) * w + (i - 1)] =
          i == 1 ? 0. : i == nx + 1 ? 0.
                  : +a * dt * c->sux_a[isx(c, i, j)] + b * dt * c->sux_b[isx(c, i, j)] + g * dt * c->sux_g[isx(c, i, j)];
  if (c->implicitx) {
#pragma omp parallel for num_threads(g_threads) schedule(static)
    for (int j = 1; j <= ny; j++) {
      double *l = malloc(sizeof(double) * w), *d = malloc(sizeof(double) * w);
      double *u = malloc(sizeof(double) * w), *r = malloc(sizeof(double) * w);
      for (int i = 1; i <= nx + 1; i++) {
        if (i == 1 || i == nx + 1) { /* :249-253 */
          l[i - 1] = 0.;
          u[i - 1] = 0.;
          d[i - 1] = 1.;
        } else {
          const double pf = (g * dt * sqrt(c->Pr)) / (2. * sqrt(c->Ra));
          const double cm = 1. / DXC(i) / DXF(i - 1), cp = 1. / DXC(i) / DXF(i);
          const double c0 = -cm - cp;
          l[i - 1] = -pf * cm;
          u[i - 1] = -pf * cp;
          d[i - 1] = 1. - pf * c0;
        }
        r[i - 1] = q[(long)(j - 1) * w + (i - 1)];
      }
      thomas(w, l, d, u, r);
      for (int i = 1; i <= nx + 1; i++) q[(long)(j - 1) * w + (i - 1)] = r[i - 1];
      free(l); free(d); free(u); free(r);
    }
  }
  if (c->implicity) {
    const double pf = (g * dt * sqrt(c->Pr)) / (2. * sqrt(c->Ra));
    solve_y_columns(c, q, w, 0, w, pf);
  }
  for (int j = 1; j <= ny; j++)
    for (int i = 2; i <= nx; i++) c->ux[iu(c, i, j)] += q[(long)(j - 1) * w + (i - 1)];
  free(q);
  bc_ux(c);
}

/* src/fluid/update_velocity.c:346-488 */
static void uy_advance(oracle_case *c, int rk) {
  const int nx = c->nx, ny = c->ny;
  const double a = c->rk_a[rk], b = c->rk_b[rk], g = c->rk_g[rk], dt = c->dt;
  double *q = malloc(sizeof(double) * (size_t)nx * ny);
  for (int j = 1; j <= ny; j++)
    for (int i = 1; i <= nx; i++) {
      const long k = isc(c, i, j);
      q[k] = +a * dt * c->suy_a[k] + b * dt * c->suy_b[k] + g * dt * c->suy_g[k];
    }
  if (c->implicitx) {
#pragma omp parallel for num_threads(g_threads) schedule(static)
    for (int j = 1; j <= ny; j++) {
      double *l = malloc(sizeof(double) * nx), *d = malloc(sizeof(double) * nx);
      double *u = malloc(sizeof(double) * nx), *r = malloc(sizeof(double) * nx);
      for (int i = 1; i <= nx; i++) {
        const double pf = (g * dt * sqrt(c->Pr)) / (2. * sqrt(c->Ra));
        const double cm = 1. / DXF(i) / DXC(i), cp = 1. / DXF(i) / DXC(i + 1);
        const double c0 = -cm - cp;
        l[i - 1] = -pf * cm;
        u[i - 1] = -pf * cp;
        d[i - 1] = 1. - pf * c0;
        r[i - 1] = q[isc(c, i, j)];
      }
      thomas(nx, l, d, u, r);
      for (int i = 1; i <= nx; i++) q[isc(c, i, j)] = r[i - 1];
      free(l); free(d); free(u); free(r);
    }
  }
  if (c->implicity) {
    const double pf = (g * dt * sqrt(c->Pr)) / (2. * sqrt(c->Ra));
    solve_y_columns(c, q, nx, 0, nx, pf);
  }
  for (int j = 1; j <= ny; j++)
    for (int i = 1; i <= nx; i++) c->uy[ic(c, i, j)] += q[isc(c, i, j)];
  free(q);
  bc_uy(c);
}

/* ---------------------------------------------------------------- Poisson */
/* src/fluid/compute_potential.c:15-168 */
static void potential(oracle_case *c, int rk) {
  const int nx = c->nx, ny = c->ny, nh = ny / 2 + 1;
  const double g = c->rk_g[rk], dt = c->dt, dy = c->dy;
  /* spectrum, mode-major: re/im of mode J at x index i at spec[2*(J*nx + i-1)] */
  double *spec = malloc(sizeof(double) * 2 * (size_t)nh * nx);
#pragma omp parallel num_threads(g_threads)
  {
    double *col = malloc(sizeof(double) * ny), *work = malloc(sizeof(double) * ny);
#pragma omp for schedule(static)
    for (int i = 1; i <= nx; i++) {
      for (int j = 1; j <= ny; j++) { /* :74-86 */
        const double uxm = c->ux[iu(c, i, j)], uxp = c->ux[iu(c, i + 1, j)];
        const double uym = c->uy[ic(c, i, j)], uyp = c->uy[ic(c, i, j + 1)];
        col[j - 1] = 1. / (g * dt) * (+(uxp - uxm) / DXF(i) + (uyp - uym) / dy);
      }
      oracle_rfft_forward(&c->fft, col, 1, spec + 2L * (i - 1), nx, work); /* :88-92 */
    }
    free(col);
    free(work);
  }
#pragma omp parallel num_threads(g_threads)
  {
    double *l = malloc(sizeof(double) * nx), *d = malloc(sizeof(double) * nx);
    double *u = malloc(sizeof(double) * nx);
    double *qr = malloc(sizeof(double) * nx), *qi = malloc(sizeof(double) * nx);
#pragma omp for schedule(static)
    for (int J = 0; J < nh; J++) { /* :109-136 */
      const double eig = -4. / pow(dy, 2.) * pow(sin(ORACLE_PI * (J) / (1. * ny)), 2.);
      for (int i = 1; i <= nx; i++) {
        l[i - 1] = 1. / DXC(i) / DXF(i);
        u[i - 1] = 1. / DXC(i + 1) / DXF(i);
      }
      for (int i = 1; i <= nx; i++) d[i - 1] = -l[i - 1] - u[i - 1] + eig;
      d[0] += l[0];
      d[nx - 1] += u[nx - 1];
      for (int i = 0; i < nx; i++) {
        qr[i] = spec[2 * ((long)J * nx + i)];
        qi[i] = spec[2 * ((long)J * nx + i) + 1];
      }
      thomas_cplx(nx, l, d, u, qr, qi);
      for (int i = 0; i < nx; i++) {
        spec[2 * ((long)J * nx + i)] = qr[i];
        spec[2 * ((long)J * nx + i) + 1] = qi[i];
      }
    }
    free(l); free(d); free(u); free(qr); free(qi);
  }
#pragma omp parallel num_threads(g_threads)
  {
    double *col = malloc(sizeof(double) * ny), *work = malloc(sizeof(double) * ny);
#pragma omp for schedule(static)
    for (int i = 1; i <= nx; i++) {
      oracle_rfft_backward(&c->fft, spec + 2L * (i - 1), nx, col, 1, work); /* :147-151 */
      for (int j = 1; j <= ny; j++) c->psi[ic(c, i, j)] = col[j - 1] / (1. * ny); /* :153-157 */
    }
    free(col);
    free(work);
  }
  free(spec);
  bc_p(c, c->psi);
}

/* src/fluid/correct_velocity.c:6-42 */
static void correct(oracle_case *c, int rk) {
  const int nx = c->nx, ny = c->ny;
  const double g = c->rk_g[rk], dt = c->dt, dy = c->dy;
  for (int j = 1; j <= ny; j++)
    for (int i = 2; i <= nx; i++) {
      const double dxi = 1. / DXC(i);
      const double pp = c->psi[ic(c, i, j)], pm = c->psi[ic(c, i - 1, j)];
      c->ux[iu(c, i, j)] -= g * dt * (pp - pm) * dxi;
    }
  bc_ux(c);
  for (int j = 1; j <= ny; j++)
    for (int i = 1; i <= nx; i++) {
      const double pp = c->psi[ic(c, i, j)], pm = c->psi[ic(c, i, j - 1)];
      c->uy[ic(c, i, j)] -= g * dt * (pp - pm) / dy;
    }
  bc_uy(c);
}

/* src/fluid/update_pressure.c:7-60 */
static void pressure(oracle_case *c, int rk) {
  const int nx = c->nx, ny = c->ny;
  const double Re = sqrt(c->Ra) / sqrt(c->Pr);
  const double g = c->rk_g[rk], dt = c->dt, dy = c->dy;
  const double *psi = c->psi;
  for (int j = 1; j <= ny; j++)
    for (int i = 1; i <= nx; i++) c->p[ic(c, i, j)] += psi[ic(c, i, j)];
  if (c->implicitx) {
    for (int j = 1; j <= ny; j++)
      for (int i = 1; i <= nx; i++) {
        const double gm = (-psi[ic(c, i - 1, j)] + psi[ic(c, i, j)]) / DXC(i);
        const double gp = (-psi[ic(c, i, j)] + psi[ic(c, i + 1, j)]) / DXC(i + 1);
        c->p[ic(c, i, j)] += -(g * dt) / (2. * Re) * (+(gp - gm) / DXF(i));
      }
  }
  if (c->implicity) {
    for (int j = 1; j <= ny; j++)
      for (int i = 1; i <= nx; i++) {
        const double gm = (-psi[ic(c, i, j - 1)] + psi[ic(c, i, j)]) / dy;
        const double gp = (-psi[ic(c, i, j)] + psi[ic(c, i, j + 1)]) / dy;
        c->p[ic(c, i, j)] += -(g * dt) / (2. * Re) * (+(gp - gm) / dy);
      }
  }
  bc_p(c, c->p);
}

/* ------------------------------------------------------------ public API */
oracle_case *oracle_create(int itot, int jtot, double ly, double stretch, double Ra, double Pr,
                           int with_temperature, int with_thermal_forcing) {
  if (itot < 2 || jtot < 2 || (jtot & (jtot - 1)) != 0) return NULL;
  oracle_case *c = calloc(1, sizeof(oracle_case));
  c->nx = itot;
  c->ny = jtot;
  c->lx = 1.; /* include/param.h:13 */
  c->ly = ly;
  c->Ra = Ra;
  c->Pr = Pr;
  c->with_temperature = with_temperature;
  c->with_thermal_forcing = with_thermal_forcing;
  build_grid(c, stretch);
  set_rk(c);
  if (oracle_rfft_plan_init(&c->fft, jtot) != 0) {
    oracle_destroy(c);
    return NULL;
  }
  const size_t nu = (size_t)(itot + 1) * (jtot + 2), nc = (size_t)(itot + 2) * (jtot + 2);
  const size_t sx = (size_t)(itot - 1) * jtot, sc = (size_t)itot * jtot;
  c->ux = calloc(nu, sizeof(double));
  c->uy = calloc(nc, sizeof(double));
  c->p = calloc(nc, sizeof(double));
  c->psi = calloc(nc, sizeof(double));
  c->temp = calloc(nc, sizeof(double));
  c->tforce = calloc(sx, sizeof(double));
  c->sux_a = calloc(sx, sizeof(double));
  c->sux_b = calloc(sx, sizeof(double));
  c->sux_g = calloc(sx, sizeof(double));
  c->suy_a = calloc(sc, sizeof(double));
  c->suy_b = calloc(sc, sizeof(double));
  c->suy_g = calloc(sc, sizeof(double));
  c->st_a = calloc(sc, sizeof(double));
  c->st_b = calloc(sc, sizeof(double));
  c->st_g = calloc(sc, sizeof(double));
  bc_ux(c);
  bc_uy(c);
  bc_p(c, c->p);
  /* src/temperature/init.c:30-41 after srand(0) (src/parallel/init.c:25) */
  srand(0);
  for (int j = 1; j <= jtot; j++)
    for (int i = 1; i <= itot; i++) {
      const double x = XC(i);
      const double r = -0.5 + 1. * rand() / RAND_MAX;
      c->temp[ic(c, i, j)] = (T_XP - T_XM) * x + T_XM + 0.1 * r;
    }
  bc_temp(c);
  c->costs[0][0] = 1.;
  c->costs[0][1] = 2.;
  c->costs[1][0] = 2.;
  c->costs[1][1] = 3.;
  return c;
}

void oracle_destroy(oracle_case *c) {
  if (!c) return;
  free(c->xf); free(c->xc); free(c->dxf); free(c->dxc);
  free(c->ux); free(c->uy); free(c->p); free(c->psi); free(c->temp); free(c->tforce);
  free(c->sux_a); free(c->sux_b); free(c->sux_g);
  free(c->suy_a); free(c->suy_b); free(c->suy_g);
  free(c->st_a); free(c->st_b); free(c->st_g);
  oracle_rfft_plan_free(&c->fft);
  free(c);
}

void oracle_set_costs(oracle_case *c, const double w[4]) {
  c->costs[0][0] = w[0];
  c->costs[0][1] = w[1];
  c->costs[1][0] = w[2];
  c->costs[1][1] = w[3];
}

void oracle_set_dt(oracle_case *c, double dt, int implicitx, int implicity) {
  c->dt = dt;
  c->implicitx = implicitx;
  c->implicity = implicity;
}

void oracle_get_dt(const oracle_case *c, double *dt, int *implicitx, int *implicity, double *time, int *step) {
  *dt = c->dt;
  *implicitx = c->implicitx;
  *implicity = c->implicity;
  *time = c->time;
  *step = c->step;
}

void oracle_set_time(oracle_case *c, double time, int step) {
  c->time = time;
  c->step = step;
}

/* src/param/decide_dt.c:11-101 */
int oracle_decide_dt(oracle_case *c) {
  const int nx = c->nx, ny = c->ny;
  const double safe_adv = 0.7, safe_dif = 0.9;
  const double diffusivity = fmax(sqrt(c->Pr) / sqrt(c->Ra), 1. / sqrt(c->Pr) / sqrt(c->Ra));
  const double small = 1.e-8;
  double dt_adv = 5.e-2;
  for (int j = 1; j <= ny; j++)
    for (int i = 2; i <= nx; i++) {
      const double vel = fmax(fabs(c->ux[iu(c, i, j)]), small);
      dt_adv = fmin(dt_adv, DXC(i) / vel);
    }
  for (int j = 1; j <= ny; j++)
    for (int i = 1; i <= nx; i++) {
      const double vel = fmax(fabs(c->uy[ic(c, i, j)]), small);
      dt_adv = fmin(dt_adv, c->dy / vel);
    }
  dt_adv *= safe_adv;
  double dx = c->lx;
  for (int i = 2; i <= nx; i++) dx = fmin(dx, DXC(i));
  double dt_dif_x = 0.25 / diffusivity * pow(dx, 2.);
  double dt_dif_y = 0.25 / diffusivity * pow(c->dy, 2.);
  dt_dif_x *= safe_dif;
  dt_dif_y *= safe_dif;
  double dt = 1.e-2, best = DBL_MAX;
  int bx = -1, by = -1;
  for (int y = 0; y < 2; y++)
    for (int x = 0; x < 2; x++) {
      const double cand = x ? (y ? dt_adv : fmin(dt_adv, dt_dif_y))
                            : (y ? fmin(dt_adv, dt_dif_x) : fmin(dt_adv, fmin(dt_dif_x, dt_dif_y)));
      const double wt = c->costs[y][x] * (1. / cand);
      if (wt < best) {
        dt = cand;
        best = wt;
        bx = x;
        by = y;
      }
    }
  c->implicitx = bx;
  c->implicity = by;
  c->dt = dt;
  return 0;
}

int oracle_update_boundaries(oracle_case *c) {
  bc_ux(c);
  bc_uy(c);
  bc_p(c, c->p);
  if (c->with_temperature) bc_temp(c);
  return 0;
}

int oracle_temperature_force_and_update(oracle_case *c, int rkstep) {
  bc_temp(c);
  temp_force(c);
  temp_rhs(c);
  temp_advance(c, rkstep);
  return 0;
}

int oracle_fluid_update_velocity(oracle_case *c, int rkstep) {
  ux_rhs(c);
  uy_rhs(c);
  ux_advance(c, rkstep);
  uy_advance(c, rkstep);
  return 0;
}

int oracle_fluid_compute_potential(oracle_case *c, int rkstep) { potential(c, rkstep); return 0; }
int oracle_fluid_correct_velocity(oracle_case *c, int rkstep) { correct(c, rkstep); return 0; }
int oracle_fluid_update_pressure(oracle_case *c, int rkstep) { pressure(c, rkstep); return 0; }

/* src/main.c:80-99 */
int oracle_substage(oracle_case *c, int rk) {
  bc_ux(c);
  bc_uy(c);
  bc_p(c, c->p);
  if (c->with_temperature) {
    bc_temp(c);
    temp_force(c);
    temp_rhs(c);
    temp_advance(c, rk);
  }
  ux_rhs(c);
  uy_rhs(c);
  ux_advance(c, rk);
  uy_advance(c, rk);
  potential(c, rk);
  correct(c, rk);
  pressure(c, rk);
  return 0;
}

int oracle_run(oracle_case *c, int nsteps, int decide) {
  for (int s = 0; s < nsteps; s++) {
    if (decide) oracle_decide_dt(c);
    for (int rk = 0; rk < 3; rk++) oracle_substage(c, rk);
    c->step += 1;
    c->time += c->dt;
  }
  return 0;
}

void oracle_get_state(const oracle_case *c, double *ux, double *uy, double *p, double *psi, double *temp) {
  const size_t nu = (size_t)(c->nx + 1) * (c->ny + 2), nc = (size_t)(c->nx + 2) * (c->ny + 2);
  if (ux) memcpy(ux, c->ux, sizeof(double) * nu);
  if (uy) memcpy(uy, c->uy, sizeof(double) * nc);
  if (p) memcpy(p, c->p, sizeof(double) * nc);
  if (psi) memcpy(psi, c->psi, sizeof(double) * nc);
  if (temp) memcpy(temp, c->temp, sizeof(double) * nc);
}

void oracle_set_state(oracle_case *c, const double *ux, const double *uy, const double *p, const double *temp) {
  const size_t nu = (size_t)(c->nx + 1) * (c->ny + 2), nc = (size_t)(c->nx + 2) * (c->ny + 2);
  if (ux) memcpy(c->ux, ux, sizeof(double) * nu);
  if (uy) memcpy(c->uy, uy, sizeof(double) * nc);
  if (p) memcpy(c->p, p, sizeof(double) * nc);
  if (temp) memcpy(c->temp, temp, sizeof(double) * nc);
}

void oracle_get_sources(const oracle_case *c, double *srcuxa, double *srcuya, double *srctempa) {
  if (srcuxa) memcpy(srcuxa, c->sux_a, sizeof(double) * (c->nx - 1) * c->ny);
  if (srcuya) memcpy(srcuya, c->suy_a, sizeof(double) * c->nx * c->ny);
  if (srctempa) memcpy(srctempa, c->st_a, sizeof(double) * c->nx * c->ny);
}

void oracle_set_sources(oracle_case *c, const double *srcuxa, const double *srcuya, const double *srctempa) {
  if (srcuxa) memcpy(c->sux_a, srcuxa, sizeof(double) * (c->nx - 1) * c->ny);
  if (srcuya) memcpy(c->suy_a, srcuya, sizeof(double) * c->nx * c->ny);
  if (srctempa) memcpy(c->st_a, srctempa, sizeof(double) * c->nx * c->ny);
}

void oracle_get_grid(const oracle_case *c, double *xf, double *xc, double *dxf, double *dxc, double *dy) {
  memcpy(xf, c->xf, sizeof(double) * (c->nx + 1));
  memcpy(xc, c->xc, sizeof(double) * (c->nx + 2));
  memcpy(dxf, c->dxf, sizeof(double) * c->nx);
  memcpy(dxc, c->dxc, sizeof(double) * (c->nx + 1));
  *dy = c->dy;
}

/* -------------------------------------------------------------- diagnostics */
/* src/analyses.c:8-33 */
static double kdiss_x(const oracle_case *c, int i, int j) {
  const double *ux = c->ux, dy = c->dy;
  double s = 0.;
  if (i != 1) {
    const double du = ux[iu(c, i, j)] - ux[iu(c, i - 1, j)];
    const double g = du / DXF(i - 1);
    s += 0.5 / DXC(i) * du * g;
  }
  if (i != c->nx + 1) {
    const double du = ux[iu(c, i + 1, j)] - ux[iu(c, i, j)];
    const double g = du / DXF(i);
    s += 0.5 / DXC(i) * du * g;
  }
  {
    const double du = ux[iu(c, i, j)] - ux[iu(c, i, j - 1)];
    const double g = du / dy;
    s += 0.5 / dy * du * g;
  }
  {
    const double du = ux[iu(c, i, j + 1)] - ux[iu(c, i, j)];
    const double g = du / dy;
    s += 0.5 / dy * du * g;
  }
  return sqrt(c->Pr) / sqrt(c->Ra) * s;
}

/* src/analyses.c:35-72 (also the thermal version :74-110 with 1/sqrt(Pr)) */
static double cdiss(const oracle_case *c, const double *f, int i, int j, double pref) {
  const double dy = c->dy;
  double s = 0.;
  {
    const double w = i == 1 ? 1. : 0.5;
    const double d = f[ic(c, i, j)] - f[ic(c, i - 1, j)];
    const double g = d / DXC(i);
    s += w / DXF(i) * d * g;
  }
  {
    const double w = i == c->nx ? 1. : 0.5;
    const double d = f[ic(c, i + 1, j)] - f[ic(c, i, j)];
    const double g = d / DXC(i + 1);
    s += w / DXF(i) * d * g;
  }
  {
    const double d = f[ic(c, i, j)] - f[ic(c, i, j - 1)];
    const double g = d / dy;
    s += 0.5 / dy * d * g;
  }
  {
    const double d = f[ic(c, i, j + 1)] - f[ic(c, i, j)];
    const double g = d / dy;
    s += 0.5 / dy * d * g;
  }
  return pref * s;
}

void oracle_diagnostics(const oracle_case *c, double out[11]) {
  const int nx = c->nx, ny = c->ny;
  const double dy = c->dy, Ra = c->Ra, Pr = c->Pr, lx = c->lx, ly = c->ly;
  const double *ux = c->ux, *uy = c->uy, *T = c->temp;
  double divmax = 0., divsum = 0.; /* src/logging.c:36-80 */
  for (int j = 1; j <= ny; j++)
    for (int i = 1; i <= nx; i++) {
      const double div = (ux[iu(c, i + 1, j)] - ux[iu(c, i, j)]) / DXF(i) + (uy[ic(c, i, j + 1)] - uy[ic(c, i, j)]) / dy;
      divmax = fmax(divmax, fabs(div));
      divsum += div;
    }
  double mx = 0., my = 0.; /* :82-122 */
  for (int j = 1; j <= ny; j++)
    for (int i = 1; i <= nx + 1; i++) mx += ux[iu(c, i, j)] * (DXC(i) * dy);
  for (int j = 1; j <= ny; j++)
    for (int i = 1; i <= nx; i++) my += uy[ic(c, i, j)] * (DXF(i) * dy);
  double e0 = 0., e1 = 0., e2 = 0.; /* :124-173 */
  for (int j = 1; j <= ny; j++)
    for (int i = 1; i <= nx + 1; i++) e0 += 0.5 * pow(ux[iu(c, i, j)], 2.) * (DXC(i) * dy);
  for (int j = 1; j <= ny; j++)
    for (int i = 1; i <= nx; i++) e1 += 0.5 * pow(uy[ic(c, i, j)], 2.) * (DXF(i) * dy);
  for (int j = 1; j <= ny; j++)
    for (int i = 1; i <= nx; i++) e2 += 0.5 * pow(T[ic(c, i, j)], 2.) * (DXF(i) * dy);
  double nu_wall = 0.; /* :191-203 */
  for (int j = 1; j <= ny; j++) {
    const double g0 = (T[ic(c, 1, j)] - T[ic(c, 0, j)]) / DXC(1);
    const double g1 = (T[ic(c, nx + 1, j)] - T[ic(c, nx, j)]) / DXC(nx + 1);
    nu_wall -= 0.5 * (g0 + g1) * dy;
  }
  nu_wall /= ly;
  double nu_inje = 0.; /* :204-219 */
  for (int j = 1; j <= ny; j++)
    for (int i = 1; i <= nx + 1; i++) {
      const double integrand = ux[iu(c, i, j)] * 0.5 * (T[ic(c, i - 1, j)] + T[ic(c, i, j)]);
      const double cellsize = DXC(i) * dy;
      nu_inje += sqrt(Pr) * sqrt(Ra) * integrand * cellsize;
    }
  nu_inje /= lx * ly;
  nu_inje += 1.;
  double nu_ek = 0.; /* :220-243 */
  for (int j = 1; j <= ny; j++)
    for (int i = 1; i <= nx + 1; i++) {
      const double cellsize = DXC(i) * dy;
      nu_ek += sqrt(Pr) * sqrt(Ra) * kdiss_x(c, i, j) * cellsize;
    }
  for (int j = 1; j <= ny; j++)
    for (int i = 1; i <= nx; i++) {
      const double cellsize = DXF(i) * dy;
      nu_ek += sqrt(Pr) * sqrt(Ra) * cdiss(c, uy, i, j, sqrt(Pr) / sqrt(Ra)) * cellsize;
    }
  nu_ek /= lx * ly;
  nu_ek += 1.;
  double nu_eh = 0.; /* :244-258 */
  for (int j = 1; j <= ny; j++)
    for (int i = 1; i <= nx; i++) {
      const double cellsize = DXF(i) * dy;
      nu_eh += sqrt(Pr) * sqrt(Ra) * cdiss(c, T, i, j, 1. / sqrt(Pr) / sqrt(Ra)) * cellsize;
    }
  nu_eh /= lx * ly;
  out[0] = divmax; out[1] = divsum; out[2] = mx; out[3] = my;
  out[4] = e0; out[5] = e1; out[6] = e2;
  out[7] = nu_wall; out[8] = nu_inje; out[9] = nu_ek; out[10] = nu_eh;
}
