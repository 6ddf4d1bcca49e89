/*
 * TEST INFRASTRUCTURE ONLY -- the CPU oracle for the SMR-RK3 time step.
 *
 * A plain-C restatement of the reference's FP64 algorithm (NaokiHori/
 * SimpleNavierStokesSolver, src/fluid/*.c, src/temperature/*.c, src/linalg.c,
 * src/param/{init,decide_dt}.c, src/logging.c, src/analyses.c), single rank.
 * Every floating-point expression keeps the reference's operation order, so
 * on the same machine it reproduces the reference bit for bit; that claim is
 * checked against the reference itself (compiled from its own sources with
 * the stand-ins in shim/) by tests/test_oracle_pinning.py and the fixtures in
 * tests/golden/.
 *
 * Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use
 * this library, always as the checker or the timed CPU baseline; the product
 * never links it.
 *
 * Arrays use the reference's layouts (include/arrays/{fluid,temperature,
 * param}.h): x fastest, one halo row at j=0 and j=jtot+1,
 *   ux  : (itot+1) x (jtot+2), i in [1, itot+1]
 *   uy, p, psi, temp : (itot+2) x (jtot+2), i in [0, itot+1]
 *   srcux* : (itot-1) x jtot ; srcuy*, srctemp* : itot x jtot
 */
#ifndef SNS_ORACLE_H
#define SNS_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

typedef struct oracle_case oracle_case;

/* builds the grid (src/param/init.c:124-195), the RK coefficients (:197-213)
 * and the initial state (src/fluid/init.c:31-83, src/temperature/init.c:
 * 19-46 with srand(0) as src/parallel/init.c:25 does for rank 0).
 * Returns NULL on invalid sizes (itot < 2, jtot not a power of two >= 2). */
oracle_case *oracle_create(int itot, int jtot, double ly, double stretch, double Ra, double Pr,
                           int with_temperature, int with_thermal_forcing);
void oracle_destroy(oracle_case *c);

/* OpenMP threads for the line/cell loops (results do not depend on it) */
void oracle_set_threads(int nthreads);

void oracle_set_costs(oracle_case *c, const double w[4]); /* expimp_wtimes[y][x] = w[2y+x] */
void oracle_set_dt(oracle_case *c, double dt, int implicitx, int implicity);
void oracle_get_dt(const oracle_case *c, double *dt, int *implicitx, int *implicity, double *time, int *step);
void oracle_set_time(oracle_case *c, double time, int step);

int oracle_decide_dt(oracle_case *c);          /* src/param/decide_dt.c:11-101 */
int oracle_substage(oracle_case *c, int rkstep); /* src/main.c:80-99, one substage */
int oracle_run(oracle_case *c, int nsteps, int decide); /* src/main.c:28-35 without I/O */

/* the individual hot-path operations, for per-function parity tests */
int oracle_update_boundaries(oracle_case *c);  /* ux, uy, p, temp halos and walls */
int oracle_temperature_force_and_update(oracle_case *c, int rkstep);
int oracle_fluid_update_velocity(oracle_case *c, int rkstep);
int oracle_fluid_compute_potential(oracle_case *c, int rkstep);
int oracle_fluid_correct_velocity(oracle_case *c, int rkstep);
int oracle_fluid_update_pressure(oracle_case *c, int rkstep);

void oracle_get_state(const oracle_case *c, double *ux, double *uy, double *p, double *psi, double *temp);
void oracle_set_state(oracle_case *c, const double *ux, const double *uy, const double *p, const double *temp);
void oracle_get_sources(const oracle_case *c, double *srcuxa, double *srcuya, double *srctempa);
void oracle_set_sources(oracle_case *c, const double *srcuxa, const double *srcuya, const double *srctempa);
void oracle_get_grid(const oracle_case *c, double *xf, double *xc, double *dxf, double *dxc, double *dy);

/* the reference's log quantities (src/logging.c:36-272), in its summation
 * order: out[0..1] divergence max, sum; [2..3] x/y momentum;
 * [4..6] kinetic x, kinetic y, thermal energy; [7..10] Nu wall, injection,
 * kinetic dissipation, thermal dissipation */
void oracle_diagnostics(const oracle_case *c, double out[11]);

#ifdef __cplusplus
}
#endif
#endif
