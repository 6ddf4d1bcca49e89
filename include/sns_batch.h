/*
 * sns_batch.h -- C ABI of the batched precision form of libsns_gpu.so.
 *
 * Many independent Rayleigh-Benard cases of uneven grid size and Ra/Pr
 * advance together: every kernel launch of a time step covers all resident
 * cases (work lists of (case, tile) units), and the step is replayed as one
 * CUDA graph. Stencils, RK3 updates and halo traffic run in FP32; the Poisson
 * solve (real DFT along y, tridiagonal along x), the divergence, the pressure
 * and the scalar potential stay FP64. Results therefore differ from the
 * reference by round-off growth, not bit for bit (the plain path of
 * sns_gpu.h is the bit-exact drop-in).
 *
 * Scheme: the reference's SMR-RK3 step (src/main.c:79-101) with explicit
 * diffusion in both directions; dt per case from the reference's advective
 * limit (src/param/decide_dt.c:35-50) and the explicit diffusive limits, or a
 * fixed dt. No reference counterpart exists for the batching itself: the
 * reference runs one case per MPI job.
 *
 * Memory: one device arena of the size given at creation; a case is admitted
 * only if its footprint (sns_batch_case_bytes) fits, so admission control
 * by HBM footprint is a call away. Fields stay device-resident until read.
 *
 * Limits: jtot a power of two in [8, 8192]; itot a multiple of 32 in
 * [64, 4096]; lx = 1.
 */
#ifndef SNS_BATCH_H
#define SNS_BATCH_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct sns_batch sns_batch;

typedef struct sns_case_desc {
  int itot, jtot;            /* cells in x (wall-bounded) and y (periodic) */
  double ly;                 /* domain height in y; lx is 1 */
  double stretch;            /* >= itot/2: uniform x grid, else clipped Chebyshev (src/param/init.c:148-166) */
  double Ra, Pr;
  int with_temperature, with_thermal_forcing;
  long long steps;           /* steps after which the case is complete (0: never) */
  unsigned long long seed;   /* 0: the reference's own initial noise (srand(0); rand()),
                                else SplitMix64(seed) uniform noise in [-0.05, 0.05] */
  double fixed_dt;           /* > 0: use this dt every step instead of the CFL decision */
  int compensated;           /* 1: stencil terms, coefficients and increments as float-float
                                pairs (about 48 bits, on the FP32 pipes) and the divergence
                                from both words in FP64; 0: FP32 terms */
} sns_case_desc;

/* Launch shapes of the step's kernels. The defaults (64, 8, 4, 0) are set at
 * creation; sns_batch_autotune measures alternatives on the resident cases. */
typedef struct sns_batch_tuning {
  int tile_x;          /* stencil / correction block width: 32, 64 or 128 columns */
  int tile_rows;       /* rows each stencil / correction thread marches: 1 .. 64 */
  int modes_per_block; /* tridiagonal mode lines (warps) per block: 2, 4 or 8 */
  int fcols_shift;     /* DFT columns per block: the per-case default times 2^shift, -3 .. 3 */
} sns_batch_tuning;

/* a batch with a device arena of hbm_bytes and room for max_cases cases */
extern sns_batch *sns_batch_create(size_t hbm_bytes, int max_cases);
extern int sns_batch_destroy(sns_batch *batch);
/* arena bytes one case of this description occupies */
extern size_t sns_batch_case_bytes(const sns_case_desc *desc);
/* free arena bytes (largest contiguous block) */
extern size_t sns_batch_free_bytes(const sns_batch *batch);
/* admits a case; temp_init: optional initial temperature in the reference's
 * (jtot+2) x (itot+2) layout (interior used). Fails with SNS_ERR_OOM when it
 * does not fit, SNS_ERR_UNSUPPORTED for sizes outside the limits. */
extern int sns_batch_add(sns_batch *batch, const sns_case_desc *desc, const double *temp_init, int *slot);
/* releases a case's slot and arena memory (waits for queued work first) */
extern int sns_batch_remove(sns_batch *batch, int slot);
/* every resident, unfinished case advances nsteps time steps; enqueued on the
 * batch's stream, returns without waiting */
extern int sns_batch_step(sns_batch *batch, int nsteps);
extern int sns_batch_synchronize(sns_batch *batch);
extern void *sns_batch_stream(const sns_batch *batch);
/* state of one case in the reference's layouts, as FP64 (halos and walls
 * filled by the reference's rules); any pointer may be NULL. Waits. */
extern int sns_batch_state(sns_batch *batch, int slot, double *ux, double *uy, double *p, double *psi,
                           double *temp);
/* time, dt of the next step, completed steps, done flag (steps reached).
 * Returns SNS_ERR_NONFINITE (outputs filled) once the case has written a NaN
 * or infinity to its velocity or pressure (a diverged case; the flag is
 * sticky). Waits. */
extern int sns_batch_case_status(sns_batch *batch, int slot, double *time, double *dt, long long *step, int *done);
/* Bounded wait of the tridiagonal launch (its bulk copies complete on an
 * mbarrier), no counterpart in the reference: it gives up after `polls`
 * polls (0: the default, about a second), sets this batch's error word, and
 * the next sns_batch_synchronize returns SNS_ERR_STATE. stale != 0 makes the
 * next step issue no copy so that every wait runs out: a test of the error
 * path that faults nothing. */
extern int sns_batch_set_wait_limit(sns_batch *batch, unsigned polls, int stale);
/* One persistent cooperative launch per RK substage (on != 0) instead of
 * five per-phase launches; no counterpart in the reference. The launch's
 * blocks are all resident, walk each phase's work list (stencil tiles,
 * column groups, mode lines, correction tiles) and meet at a grid barrier
 * between phases (a bounded wait: a barrier that gives up makes the next
 * sns_batch_synchronize return SNS_ERR_STATE). The arithmetic per work item
 * is the per-phase kernels' (the same device functions; the compiler may
 * pair multiply-adds differently, so FP32 results agree to their rounding);
 * the step graph holds 4 launches instead of 16. Default off: measured against the
 * per-phase launches on the 64-case ensemble (bench key
 * ensemble_64.persistent_substage). */
extern int sns_batch_set_persistent(sns_batch *batch, int on);
/* number of resident cases; their slots written to slots[0..max) */
extern int sns_batch_cases(const sns_batch *batch, int *slots, int max);
/* cells summed over resident unfinished cases (the host knows every case's
 * step count: each sns_batch_step step advances every unfinished case once) */
extern long long sns_batch_active_cells(const sns_batch *batch);
/* the initial temperature a case of this description starts from, in the
 * reference's (jtot+2) x (itot+2) layout (for checking against other solvers) */
extern int sns_batch_initial_temperature(const sns_case_desc *desc, double *temp);
/* sns_diagnostics (include/sns_gpu.h) for one case of the batch: FP64
 * compensated reductions over its FP32 fields. Waits. */
extern int sns_batch_diagnostics(sns_batch *batch, int slot, double out[11]);
/* errors of these calls are reported by sns_last_error() (include/sns_gpu.h) */

/* Continuous batching in real time. Request r (description reqs[r], which
 * must set steps > 0) arrives arrival_s[r] seconds after the call starts
 * (non-decreasing). Arrived requests wait in FIFO order and are admitted
 * into a batch with an hbm_bytes arena as soon as their footprint fits; all
 * admitted cases advance together, chunk_steps steps per launch round, and
 * each finished case is retired at the next round boundary, which returns
 * its memory for the waiting requests. For each request: admit_s[r] and
 * done_s[r] (seconds since the start; done_s - arrival_s is its
 * time-to-completion). on_done, if not NULL, is called for each finished
 * request before its retirement, with the batch and slot so that the caller
 * can read its state. Returns SNS_OK or an error; a request larger than the
 * whole arena is an SNS_ERR_OOM error. *busy_s receives the wall time from
 * the first admission to the last completion. */
typedef void (*sns_done_fn)(int request, sns_batch *batch, int slot, void *user);
extern int sns_serve(const sns_case_desc *reqs, const double *arrival_s, int n, size_t hbm_bytes, int max_cases,
                     int chunk_steps, double *admit_s, double *done_s, double *busy_s, sns_done_fn on_done,
                     void *user);

/* A case's state in the reference's save layout (src/save.c:13-68): the
 * files sns_checkpoint (sns_gpu.h) writes for the plain path, with velocity
 * and temperature widened from their compensated FP32 pairs. An FP32 case's
 * pairs fit FP64 exactly, so a restart continues bit for bit; a compensated
 * case's pairs may hold more bits, and its restart resumes from them
 * rounded to FP64 (a relative 2^-53 per value). Blocks. */
extern int sns_batch_checkpoint(sns_batch *batch, int slot, const char *dirname);
/* Admits a case from a directory in that layout (written by the reference's
 * save(), sns_checkpoint or sns_batch_checkpoint): step, time, ux, uy, p and
 * temp; the explicit sources start at zero as in a restarted reference run,
 * the first dt follows from the restored velocity. desc->steps is the step
 * index at which the case completes (it counts from the restored step). */
extern int sns_batch_add_restart(sns_batch *batch, const sns_case_desc *desc, const char *dirname, int *slot);

/* current launch shapes */
extern int sns_batch_get_tuning(const sns_batch *batch, sns_batch_tuning *tuning);
/* fixed launch shapes (SNS_ERR_ARG outside the ranges above); results do not
 * depend on them: every shape computes the same arithmetic per point */
extern int sns_batch_set_tuning(sns_batch *batch, const sns_batch_tuning *tuning);
/* Autotuner: a coordinate search over tile_rows {4, 8, 16}, tile_x {32, 64,
 * 128}, fcols_shift {-1, 0, 1} and modes_per_block {2, 4, 8}, each candidate
 * timed with CUDA events over `steps` graph replays of the resident cases.
 * The cases' device state is copied aside (arena up to its high-water mark
 * and the case table: SNS_ERR_OOM if that much memory is not free) and put
 * back after every candidate, so tuning leaves every case where it was. The
 * fastest shapes are kept; chosen and ms_per_step (optional) report them. */
extern int sns_batch_autotune(sns_batch *batch, int steps, sns_batch_tuning *chosen, double *ms_per_step);

#ifdef __cplusplus
}
#endif
#endif /* SNS_BATCH_H */
