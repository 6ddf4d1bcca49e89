/*
 * TEST INFRASTRUCTURE ONLY -- drives the reference's own compiled sources
 * (everything under src/ except main.c and parallel/transpose.c) from Python
 * through ctypes, so that tests/golden/make_golden.py can record what the
 * reference itself computes.
 *
 * The per-substage call sequence is the one of the reference's static
 * integrate() (src/main.c:79-101) and the per-step bookkeeping is that of its
 * main loop (src/main.c:28-35), with two documented deviations:
 *   - param_estimate_cost (src/param/estimate_cost.c:44-74) is not run; the
 *     caller supplies expimp_wtimes so that param_decide_dt is deterministic;
 *   - the loop runs a given number of steps instead of stopping on timemax or
 *     wall time, and writes no logs or snapshots unless asked.
 * Configuration goes through the same environment variables that
 * param_init reads (src/param/init.c:87-122).
 */
#define _GNU_SOURCE
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <unistd.h>
#include "mpi.h"
#include "param.h"
#include "parallel.h"
#include "fluid.h"
#include "temperature.h"
#include "logging.h"
#include "save.h"
#include "statistics.h"

static param_t *g_param;
static parallel_t *g_parallel;
static fluid_t *g_fluid;
static temperature_t *g_temperature;

static void set_double(const char *name, double v) {
  char buf[64];
  snprintf(buf, sizeof buf, "%.17g", v);
  setenv(name, buf, 1);
}

static void set_int(const char *name, int v) {
  char buf[32];
  snprintf(buf, sizeof buf, "%d", v);
  setenv(name, buf, 1);
}

/* restart_dir: NULL for the reference's own initial condition (u = p = 0,
 * T = linear + rand() noise after srand(0)); otherwise a directory holding
 * step/time/ux/uy/p/temp .npy files in the reference's save layout. */
int ref_open(int itot, int jtot, double ly, double stretch, double Ra, double Pr,
             int with_temperature, int with_thermal_forcing, const char *restart_dir) {
  if (g_param) return 1;
  unsetenv("dirname_restart");
  if (restart_dir) setenv("dirname_restart", restart_dir, 1);
  set_int("itot", itot);
  set_int("jtot", jtot);
  set_double("ly", ly);
  set_double("stretch", stretch);
  set_double("Ra", Ra);
  set_double("Pr", Pr);
  setenv("with_temperature", with_temperature ? "true" : "false", 1);
  setenv("with_thermal_forcing", with_thermal_forcing ? "true" : "false", 1);
  set_double("timemax", 1e30);
  set_double("wtimemax", 1e30);
  int saved = dup(1);
  fflush(stdout);
  FILE *devnull = fopen("/dev/null", "w");
  if (devnull) dup2(fileno(devnull), 1);
  MPI_Init(NULL, NULL);
  g_param = param_init();
  g_parallel = parallel_init();
  g_fluid = fluid_init(g_param, g_parallel);
  g_temperature = temperature_init(g_param, g_parallel);
  fflush(stdout);
  dup2(saved, 1);
  close(saved);
  if (devnull) fclose(devnull);
  return 0;
}

void ref_close(void) {
  if (!g_param) return;
  temperature_finalise(g_temperature);
  fluid_finalise(g_fluid);
  parallel_finalise(g_parallel);
  param_finalise(g_param);
  g_param = NULL;
  g_parallel = NULL;
  g_fluid = NULL;
  g_temperature = NULL;
}

void ref_set_costs(const double w[4]) {
  g_param->expimp_wtimes[0][0] = w[0];
  g_param->expimp_wtimes[0][1] = w[1];
  g_param->expimp_wtimes[1][0] = w[2];
  g_param->expimp_wtimes[1][1] = w[3];
}

void ref_set_dt(double dt, int implicitx, int implicity) {
  g_param->dt = dt;
  g_param->implicitx = implicitx;
  g_param->implicity = implicity;
}

void ref_get_dt(double *dt, int *implicitx, int *implicity, double *time, int *step) {
  *dt = g_param->dt;
  *implicitx = g_param->implicitx;
  *implicity = g_param->implicity;
  *time = g_param->time;
  *step = g_param->step;
}

int ref_decide_dt(void) { return param_decide_dt(g_param, g_parallel, g_fluid); }

/* one Runge-Kutta substage in the order of src/main.c:80-99 */
int ref_substage(int rkstep) {
  fluid_update_boundaries_ux(g_param, g_parallel, g_fluid->ux);
  fluid_update_boundaries_uy(g_param, g_parallel, g_fluid->uy);
  fluid_update_boundaries_p(g_param, g_parallel, g_fluid->p);
  if (g_param->with_temperature) {
    temperature_update_boundaries_temp(g_param, g_parallel, g_temperature->temp);
    temperature_compute_force(g_param, g_parallel, g_temperature);
    temperature_update_temp(g_param, g_parallel, rkstep, g_fluid, g_temperature);
  }
  fluid_update_velocity(g_param, g_parallel, rkstep, g_fluid, g_temperature);
  fluid_compute_potential(g_param, g_parallel, rkstep, g_fluid);
  fluid_correct_velocity(g_param, g_parallel, rkstep, g_fluid);
  fluid_update_pressure(g_param, g_parallel, rkstep, g_fluid);
  return 0;
}

/* nsteps time steps; decide != 0 calls param_decide_dt first each step
 * (src/main.c:30), otherwise the dt/scheme last set is kept */
int ref_run(int nsteps, int decide) {
  for (int s = 0; s < nsteps; s++) {
    if (decide) param_decide_dt(g_param, g_parallel, g_fluid);
    for (int rk = 0; rk < RKSTEPMAX; rk++) ref_substage(rk);
    g_param->step += 1;
    g_param->time += g_param->dt;
  }
  return 0;
}

/* whole arrays, halos included, in the reference's layout */
static size_t n_ux(void) { return (size_t)(g_param->itot + 1) * (g_param->jtot + 2); }
static size_t n_p(void) { return (size_t)(g_param->itot + 2) * (g_param->jtot + 2); }
static size_t n_srcx(void) { return (size_t)(g_param->itot - 1) * g_param->jtot; }
static size_t n_srcc(void) { return (size_t)g_param->itot * g_param->jtot; }

void ref_get_state(double *ux, double *uy, double *p, double *psi, double *temp) {
  memcpy(ux, g_fluid->ux, sizeof(double) * n_ux());
  memcpy(uy, g_fluid->uy, sizeof(double) * n_p());
  memcpy(p, g_fluid->p, sizeof(double) * n_p());
  memcpy(psi, g_fluid->psi, sizeof(double) * n_p());
  memcpy(temp, g_temperature->temp, sizeof(double) * n_p());
}

void ref_set_state(const double *ux, const double *uy, const double *p, const double *temp) {
  memcpy(g_fluid->ux, ux, sizeof(double) * n_ux());
  memcpy(g_fluid->uy, uy, sizeof(double) * n_p());
  memcpy(g_fluid->p, p, sizeof(double) * n_p());
  memcpy(g_temperature->temp, temp, sizeof(double) * n_p());
}

/* explicit Runge-Kutta sources of the last substage (srcuxa, srcuya, srctempa) */
void ref_get_sources(double *srcuxa, double *srcuya, double *srctempa) {
  memcpy(srcuxa, g_fluid->srcuxa, sizeof(double) * n_srcx());
  memcpy(srcuya, g_fluid->srcuya, sizeof(double) * n_srcc());
  memcpy(srctempa, g_temperature->srctempa, sizeof(double) * n_srcc());
}

void ref_get_grid(double *xf, double *xc, double *dxf, double *dxc, double *dy) {
  const int itot = g_param->itot;
  memcpy(xf, g_param->xf, sizeof(double) * (itot + 1));
  memcpy(xc, g_param->xc, sizeof(double) * (itot + 2));
  memcpy(dxf, g_param->dxf, sizeof(double) * itot);
  memcpy(dxc, g_param->dxc, sizeof(double) * (itot + 1));
  *dy = g_param->dy;
}

/* the reference's own diagnostics (src/logging.c:274-281) written as text
 * under <dir>/output/log; the caller parses them */
int ref_logging(const char *dir) {
  char cwd[4096];
  if (!getcwd(cwd, sizeof cwd)) return 1;
  if (chdir(dir) != 0) return 2;
  logging(g_param, g_parallel, g_fluid, g_temperature);
  int rc = chdir(cwd);
  return rc == 0 ? 0 : 3;
}

/* the reference's snapshot writer (src/save.c:52-68) under <dir>/output/save */
/* nsteps steps with statistics_collect after each (src/main.c:46-50), then
 * statistics_output (it writes output/stat/step%010d under dir) */
int ref_stats_run(int nsteps, const char *dir) {
  statistics_t *st = statistics_init(g_param, g_parallel);
  for (int s = 0; s < nsteps; s++) {
    ref_run(1, 1);
    statistics_collect(g_param, g_parallel, g_fluid, g_temperature, st);
  }
  char cwd[4096];
  int rc = 0;
  if (!getcwd(cwd, sizeof cwd)) rc = 1;
  if (!rc && chdir(dir) != 0) rc = 2;
  if (!rc) {
    statistics_output(g_param, g_parallel, st);
    if (chdir(cwd) != 0) rc = 3;
  }
  statistics_finalise(st);
  return rc;
}

int ref_save(const char *dir) {
  char cwd[4096];
  if (!getcwd(cwd, sizeof cwd)) return 1;
  if (chdir(dir) != 0) return 2;
  save(g_param, g_parallel, g_fluid, g_temperature);
  int rc = chdir(cwd);
  return rc == 0 ? 0 : 3;
}
