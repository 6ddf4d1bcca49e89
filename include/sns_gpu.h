/*
 * sns_gpu.h -- C ABI of libsns_gpu.so, the GB300 (sm_103a) implementation of
 * the SMR-RK3 time step of NaokiHori/SimpleNavierStokesSolver.
 *
 * The structures below have the reference's exact member order and types, so
 * the reference's own driver, logging, save and statistics code
 * (src/main.c, src/logging.c, src/save.c, src/statistics/) compiles against
 * them unchanged. The hot-path entry points keep the reference's names and
 * signatures; each comment names the reference interface it replaces.
 *
 * Ownership and residency. fluid_init / temperature_init allocate the host
 * arrays of the structure (reference layouts, include/arrays/ headers) and a device
 * mirror that holds the authoritative state from then on. The hot-path calls
 * only enqueue GPU work on the solver's CUDA stream; the host arrays are
 * refreshed by sns_sync_to_host (call it before logging/saving/statistics)
 * and pushed to the device by sns_sync_to_device (after writing into them,
 * e.g. when loading a restart).
 *
 * Errors. Every int-returning call returns SNS_OK (0) on success and a
 * nonzero SNS_ERR_* code otherwise (the reference returns 0 unconditionally
 * and aborts on allocation failure, src/common.c:8-15); sns_last_error()
 * returns a message. Constructors return NULL on failure.
 *
 * Scope: one MPI rank (parallel->mpisize == 1), one GPU, jtot a power of two,
 * itot >= 2. All arithmetic is IEEE binary64 without contraction, in the
 * reference's operation order: results equal the reference's bit for bit on
 * the same host (same libm for the host-side grid set-up).
 */
#ifndef SNS_GPU_H
#define SNS_GPU_H

#include <stdbool.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ------------------------------------------------------------------ types */
/* include/structure.h:4-7 */
typedef struct param_t_ param_t;
typedef struct parallel_t_ parallel_t;
typedef struct fluid_t_ fluid_t;
typedef struct temperature_t_ temperature_t;

/* include/param.h:10-13 */
#define RKSTEPMAX 3
#define LX 1.

/* include/param.h:15-25 */
typedef struct rkcoef_t_ {
  double alpha;
  double beta;
  double gamma;
} rkcoef_t;

typedef struct schedule_t_ {
  double rate;
  double after;
  double next;
} schedule_t;

/* include/param.h:28-54 (member order and types kept for ABI compatibility) */
struct param_t_ {
  bool load_flow_field;
  char *dirname_restart;
  bool with_temperature;
  bool with_thermal_forcing;
  int itot, jtot;
  double lx, ly;
  double stretch;
  double *xf, *xc;
  double *dxf, *dxc;
  double *yf, *yc;
  double dy;
  double Ra, Pr;
  rkcoef_t rkcoefs[3];
  double time, dt;
  int step, implicitx, implicity;
  double expimp_wtimes[2][2];
  double timemax, wtimemax;
  schedule_t log, save, stat;
};

/* include/parallel.h:10-13 */
struct parallel_t_ {
  int mpisize, mpirank;
  int ymrank, yprank;
};

/* include/fluid.h:8-13 */
struct fluid_t_ {
  double *ux, *uy;
  double *p, *psi;
  double *srcuxa, *srcuxb, *srcuxg;
  double *srcuya, *srcuyb, *srcuyg;
};

/* include/temperature.h:8-12 */
struct temperature_t_ {
  double *temp;
  double *tempforcex;
  double *srctempa, *srctempb, *srctempg;
};

/* include/temperature.h:22-23 */
#define TEMP_XM +0.5
#define TEMP_XP -0.5

/* ------------------------------------------------------------ status codes */
#define SNS_OK 0
#define SNS_ERR_ARG 1         /* NULL or inconsistent argument */
#define SNS_ERR_UNSUPPORTED 2 /* mpisize != 1, jtot not a power of two, ... */
#define SNS_ERR_CUDA 3        /* CUDA launch or runtime error */
#define SNS_ERR_OOM 4         /* device or host allocation failed */
#define SNS_ERR_STATE 5       /* call out of order (e.g. object already finalised) */
/* the state holds NaN or infinity (a diverged run): reported by param_decide_dt
 * (after deciding dt as the reference would) and by sns_run, which stops
 * stepping; the batched form reports it per case */
#define SNS_ERR_NONFINITE 6

/* ----------------------------------------------- reference hot-path entries */
/* include/fluid.h:15 (src/fluid/init.c:85-92): allocates the structure, its
 * host arrays and the device mirror; u = p = 0 with the reference's
 * boundary values. Restart loading (param->load_flow_field) is not done here:
 * write the loaded fields into the host arrays and call sns_sync_to_device. */
extern fluid_t *fluid_init(const param_t *param, const parallel_t *parallel);
/* include/fluid.h:16 (src/fluid/finalise.c) */
extern int fluid_finalise(fluid_t *fluid);

/* include/fluid.h:19-21 (src/fluid/boundary_conditions.c:6-55). Apply the
 * reference's single-rank halo and wall rules in place to the host array
 * passed (O(itot + jtot) host work). The device copy never stores halo or
 * wall values (they are implied by index logic in every kernel), so these
 * calls do not touch the device state. */
extern int fluid_update_boundaries_ux(const param_t *param, const parallel_t *parallel, double *ux);
extern int fluid_update_boundaries_uy(const param_t *param, const parallel_t *parallel, double *uy);
extern int fluid_update_boundaries_p(const param_t *param, const parallel_t *parallel, double *p);

/* include/fluid.h:23 (src/fluid/update_velocity.c:490-498): momentum sources
 * and RK3 / Crank-Nicolson prediction of ux, uy */
extern int fluid_update_velocity(const param_t *param, const parallel_t *parallel, const int rkstep,
                                 fluid_t *fluid, const temperature_t *temperature);
/* include/fluid.h:24 (src/fluid/compute_potential.c:15-168): Poisson solve for
 * the scalar potential psi (real DFT along y, tridiagonal along x) */
extern int fluid_compute_potential(const param_t *param, const parallel_t *parallel, const int rkstep,
                                   fluid_t *fluid);
/* include/fluid.h:25 (src/fluid/correct_velocity.c:6-42). Its launch waits
 * for the next fluid_update_pressure of the same substage (one kernel for
 * both); any other call of this solver launches it first, so every call sees
 * the corrected velocity. */
extern int fluid_correct_velocity(const param_t *param, const parallel_t *parallel, const int rkstep,
                                  fluid_t *fluid);
/* include/fluid.h:26 (src/fluid/update_pressure.c:7-60) */
extern int fluid_update_pressure(const param_t *param, const parallel_t *parallel, const int rkstep,
                                 fluid_t *fluid);

/* include/temperature.h:14 (src/temperature/init.c:48-55): linear profile plus
 * the reference's rand() noise (call srand(0) first, as parallel_init does for
 * rank 0, src/parallel/init.c:25, to reproduce the reference's initial field) */
extern temperature_t *temperature_init(const param_t *param, const parallel_t *parallel);
/* include/temperature.h:15 */
extern int temperature_finalise(temperature_t *temperature);
/* include/temperature.h:17 (src/temperature/force.c:6-32): buoyancy from the
 * current temperature, consumed by the next fluid_update_velocity */
extern int temperature_compute_force(const param_t *param, const parallel_t *parallel,
                                     temperature_t *temperature);
/* include/temperature.h:18 (src/temperature/update.c:233-238). With the
 * explicit scheme its launch waits for the next fluid_compute_potential of
 * the same substage, which runs it inside the fused Poisson launch; any other
 * call of this solver launches it first, so every call sees the updated
 * temperature. */
extern int temperature_update_temp(const param_t *param, const parallel_t *parallel, const int rkstep,
                                   const fluid_t *fluid, temperature_t *temperature);
/* include/temperature.h:20 (src/temperature/boundary_conditions.c:6-21), same
 * convention as fluid_update_boundaries_* */
extern int temperature_update_boundaries_temp(const param_t *param, const parallel_t *parallel,
                                              double *temp);

/* include/param.h:59 (src/param/decide_dt.c:11-101): advective limit from a
 * device reduction over ux, uy; diffusive limits and the EXP/IMP choice from
 * param->expimp_wtimes on the host. Blocks until the reduction is done. */
extern int param_decide_dt(param_t *param, const parallel_t *parallel, const fluid_t *fluid);

/* ------------------------------------------------------------ sns helpers */
/* param_t built from arguments instead of environment variables; grid and RK
 * coefficients as src/param/init.c:124-213 (uniform grid when
 * stretch >= itot/2, clipped Chebyshev otherwise). expimp_wtimes defaults to
 * {{1,2},{2,3}} (explicit preferred when dt limits tie). */
extern param_t *sns_param_create(int itot, int jtot, double ly, double stretch, double Ra, double Pr,
                                 int with_temperature, int with_thermal_forcing);
extern int sns_param_destroy(param_t *param);
/* single-rank parallel_t {1, 0, 0, 0}; also calls srand(0) like
 * src/parallel/init.c:25 does on rank 0 */
extern parallel_t *sns_parallel_create(void);
extern int sns_parallel_destroy(parallel_t *parallel);

/* device -> host arrays (reference layouts, halos filled by the reference's
 * rules); either pointer may be NULL. Blocks until the copies are done. */
extern int sns_sync_to_host(const param_t *param, fluid_t *fluid, temperature_t *temperature);
/* host arrays -> device (interior values are taken; halos are implied) */
extern int sns_sync_to_device(const param_t *param, fluid_t *fluid, temperature_t *temperature);
/* the same two copies restricted to ux, uy, p and temp, the whole input and
 * output of a time step taken with sns_integrate / sns_run (psi is written
 * before it is read, the first substage multiplies the previous sources by
 * zero and the buoyancy is recomputed from temp): psi, srcuxa, srcuya,
 * srctempa and tempforcex stay as they are on the side being written. Not
 * for use between the reference-named calls of one step. */
extern int sns_sync_state_to_host(const param_t *param, fluid_t *fluid, temperature_t *temperature);
extern int sns_sync_state_to_device(const param_t *param, fluid_t *fluid, temperature_t *temperature);
/* waits for all GPU work queued for this fluid's solver */
extern int sns_synchronize(const fluid_t *fluid);
/* the CUDA stream (cudaStream_t) the solver enqueues on */
extern void *sns_stream(const fluid_t *fluid);

/* one full time step's three RK substages (src/main.c:79-101) with the dt and
 * scheme currently in param, using fused kernels; with_temperature honoured */
extern int sns_integrate(const param_t *param, const parallel_t *parallel, fluid_t *fluid,
                         temperature_t *temperature);
/* nsteps of { param_decide_dt; sns_integrate; step += 1; time += dt }
 * (src/main.c:28-35 without logging/saving/statistics) */
extern int sns_run(param_t *param, const parallel_t *parallel, fluid_t *fluid, temperature_t *temperature,
                   int nsteps);

/* the reference's log quantities (src/logging.c:36-272) computed on the
 * device in FP64 with compensated summation, without a host copy of the
 * fields: out[0..1] divergence max and sum, [2..3] x and y momentum,
 * [4..6] kinetic energy of ux and uy and thermal energy, [7..10] Nusselt
 * number from the wall heat flux, the energy injection, the kinetic and the
 * thermal dissipation. Blocks until done. */
extern int sns_diagnostics(const param_t *param, const fluid_t *fluid, const temperature_t *temperature,
                           double out[11]);

/* sns_diagnostics without any allocation; no counterpart in the reference.
 * For callers that cannot allocate: a monitoring thread sampling a run in
 * flight (cudaMalloc / cudaFree may synchronise the device and stall the
 * solver) and a process whose HBM is committed to a batch arena. The block
 * partials live in a fixed file-scope device array (4096 blocks, 672 KiB) and
 * are summed on the device with the same compensated sums in the same order,
 * so out[] equals sns_diagnostics's bit for bit. A grid needing more than
 * 4096 partials, ceil((itot+1)/64) * ceil(jtot/16) > 4096 (1024 x 2048
 * fits, 1024 x 4096 does not), returns SNS_ERR_UNSUPPORTED with a message. Every call
 * looks the scratch up (cudaGetSymbolAddress, with the case's device current;
 * cheap once the module is loaded, and never stale after a device reset); the
 * first call on a device may load the module, so make it before any stream
 * capture. sns_allocations() does not move across a call. Nothing in the scratch needs
 * to start at zero. There is one scratch per device: calls that overlap on
 * one device (several threads, several cases) race on it; serialise them.
 * Blocks until done. */
extern int sns_diagnostics_static(const param_t *param, const fluid_t *fluid, const temperature_t *temperature,
                                  double out[11]);

/* param_estimate_cost (include/param.h, src/param/estimate_cost.c:44-74)
 * with a deterministic cost model instead of wall-clock emulation: fills
 * expimp_wtimes[implicity][implicitx] with the predicted seconds of one RK
 * substage for this grid on the current device (its SM count and clock), so
 * param_decide_dt picks the same treatment in every run. */
extern int param_estimate_cost(param_t *param, const parallel_t *parallel);
/* the same model for a given device description, host only:
 * out[2*implicity + implicitx] in seconds per substage */
extern int sns_cost_model(int itot, int jtot, int sm_count, double clock_ghz, int with_temperature, double out[4]);
/* the reference's wall-clock estimate (emulate(), src/param/estimate_cost.c:
 * 11-42) measured with CUDA events on this device: out[2*implicity +
 * implicitx] in seconds per substage over `reps` substages. Like the
 * reference it creates fresh fields through fluid_init/temperature_init,
 * which draw from rand(). param's dt and treatment are restored. */
extern int sns_measure_cost(param_t *param, const parallel_t *parallel, int reps, double out[4]);

/* statistics_t (include/statistics.h:8-13): the number of samples and host
 * arrays in the reference's layouts (include/arrays/statistics.h: ux1/ux2
 * (jtot+2) x (itot+1), uy1/uy2/temp1/temp2 (jtot+2) x (itot+2)). The running
 * sums live on the device; the host arrays are filled by statistics_output
 * and sns_statistics_output_to. */
typedef struct statistics_t_ {
  int num;
  double *ux1, *ux2;
  double *uy1, *uy2;
  double *temp1, *temp2;
} statistics_t;

/* include/statistics.h:15-19 (src/statistics/{init,finalise,collect,output}.c):
 * collect adds u and u^2 of the current device state on the solver's stream
 * (asynchronous); output writes NPY files to output/stat/step%010d relative to
 * the working directory, as the reference does, byte for byte. */
extern statistics_t *statistics_init(const param_t *param, const parallel_t *parallel);
extern int statistics_finalise(statistics_t *statistics);
extern int statistics_collect(param_t *param, const parallel_t *parallel, const fluid_t *fluid,
                              const temperature_t *temperature, statistics_t *statistics);
extern int statistics_output(const param_t *param, const parallel_t *parallel, const statistics_t *statistics);
/* statistics_output into a given directory (created if needed) */
extern int sns_statistics_output_to(const param_t *param, const statistics_t *statistics, const char *dirname);

/* Checkpoint of the device state in the reference's save layout
 * (src/save.c:13-68, src/fileio.c:226-345, src/simple_npyio.c:1222):
 * dirname/{step,itot,jtot,time,lx,ly,Ra,Pr,xf,xc,yf,yc,ux,uy,p[,temp]}.npy,
 * byte for byte the files the reference's save() writes for the same state
 * (it writes into output/save/step%010d). dirname is created if needed.
 * Asynchronous: ux, uy, p and T are copied on the device in stream order,
 * the copy to pinned host memory runs on a separate stream and a host thread
 * writes the files; the call returns after enqueuing the device copy, so
 * the solver may keep stepping. One checkpoint per solver is in flight; a
 * second call waits for the first. */
extern int sns_checkpoint(const param_t *param, const fluid_t *fluid, const temperature_t *temperature,
                          const char *dirname);
/* waits for the last checkpoint of this solver; its status and message */
extern int sns_checkpoint_wait(const fluid_t *fluid);
/* Restart from a directory written by the reference's save() or by
 * sns_checkpoint (src/param/init.c:245-247, src/fluid/init.c:53-81,
 * src/temperature/init.c:51): step and time into param, rows 1..jtot of ux,
 * uy, p and temp into the host arrays, the boundary rules, zeroed explicit
 * sources, then sns_sync_to_device. Shapes and dtypes are checked
 * (SNS_ERR_ARG with the file's name otherwise). */
extern int sns_restart(param_t *param, fluid_t *fluid, temperature_t *temperature, const char *dirname);
/* Host-only NPY helpers with the reference's file format (no device needed):
 * dtype is the reference's descriptor text, "'float64'" or "'int32'"; the
 * reader also accepts numpy's '<f8' / '<i4' and checks ndim and shape. */
extern int sns_npy_write(const char *path, const char *dtype, int ndim, const size_t *shape, const void *data,
                         size_t nbytes);
extern int sns_npy_read(const char *path, const char *dtype, int ndim, const size_t *shape, void *data,
                        size_t nbytes);

/* The Poisson solve (and, with the explicit scheme, the temperature update of
 * the fused step) runs as one cooperative launch by default: the serial
 * tridiagonal sweeps on a few SMs, the DFTs and the temperature update on
 * the others, pipelined column by column; identical results to the
 * three-kernel form. on = 0 selects the three-kernel form for this solver
 * (for comparisons); sizes the device cannot hold cooperatively fall back
 * by themselves. */
extern int sns_set_fused(const fluid_t *fluid, int on);

/* Arithmetic form of the plain path; no counterpart in the reference.
 * SNS_FORM_EXACT (default): every operation of the reference in its order,
 * without contraction, the Poisson lines by the reference's Thomas
 * recurrence (src/fluid/compute_potential.c:109-136, src/linalg.c:32-50):
 * results identical to the reference's bit for bit. On GB300 the
 * recurrence's serial chain of dependent FP64 operations sets the step's
 * critical path.
 * SNS_FORM_PARALLEL: the Poisson lines by the partition method with
 * warp-shuffle parallel cyclic reduction (one warp per Fourier mode, one lane
 * per segment of itot/32 rows), the Crank-Nicolson lines (src/linalg.c:9-108)
 * by the same method (32 segments per row or column, the periodic y lines
 * with a cyclic interface system; the serial sweep where a line is not a
 * multiple of 32 rows of at least 64), the DFTs by a radix-8 Stockham FFT,
 * and every other kernel compiled with fused multiply-adds. Results differ
 * from the reference's by rounding, held to 1e-12 relative L2 per field
 * after the stated step counts. Needs itot in [64, 14048] and a grid on
 * which the mean mode's last Thomas pivot vanishes (uniform grids with a
 * power-of-two itot), otherwise SNS_ERR_UNSUPPORTED and the form is
 * unchanged. The first switch to it computes the Poisson factors (host,
 * O(itot * jtot)) and allocates them on the device; the Crank-Nicolson
 * factors are recomputed on the host every implicit substage (they depend
 * on dt). */
#define SNS_FORM_EXACT 0
#define SNS_FORM_PARALLEL 1
extern int sns_set_form(const fluid_t *fluid, int form);
/* the current form, or -1 for a foreign structure */
extern int sns_get_form(const fluid_t *fluid);

/* Bounded device waits, no counterpart in the reference. The fused Poisson
 * launch (SNS_FORM_EXACT) polls completion flags written by other blocks
 * of the same launch, and the partition-method launch (SNS_FORM_PARALLEL) waits for its
 * bulk copies; every such wait gives up after `polls` polls (0: the default,
 * about a second), sets an error word, and the next synchronising call of
 * this solver returns SNS_ERR_STATE (the fused form is then switched off for
 * this solver, see sns_set_fused). stale != 0 makes the next launch wait for
 * a flag that nothing sets (fused form) or issue no copy (parallel form), so
 * that its wait runs out: a test of the error path that faults nothing. */
extern int sns_set_wait_limit(const fluid_t *fluid, unsigned polls, int stale);

/* per-kernel device time: with profiling enabled every kernel launched for
 * this solver is bracketed by CUDA events on its stream. sns_profile(f, 1)
 * resets the totals and starts, sns_profile(f, 0) stops. sns_profile_read
 * fills ms[k] (summed milliseconds) and count[k] (launches) for the first n
 * kernel kinds and returns the number of kinds; sns_profile_kind_name names
 * kind k. */
extern int sns_profile(const fluid_t *fluid, int enable);
extern int sns_profile_read(const fluid_t *fluid, double *ms, long long *count, int n);
extern const char *sns_profile_kind_name(int kind);

/* FP64 issue rate of the current device in Gop/s, no counterpart in the
 * reference: out[0] additions, out[1] multiplications, each from eight
 * independent chains per thread on every SM, timed by CUDA events. The plain
 * FP64 kernels are bound by FP64 issue on GB300; this is the denominator of
 * their FP64 roofline. Takes a few milliseconds. */
extern int sns_fp64_issue_rate(double out[2]);

/* message of the last error on this thread ("" if none) */
extern const char *sns_last_error(void);
/* number of kernel launches issued by this process so far */
extern long long sns_kernel_launches(void);
/* number of device and pinned host allocations (cudaMalloc, cudaHostAlloc)
 * the library has made in this process so far; no counterpart in the
 * reference. Steady-state stepping and sns_diagnostics_static make none. */
extern long long sns_allocations(void);
/* struct layout as compiled into the library, for binding checks: writes up to
 * n values -- sizeof(param_t), offsetof(param_t, itot / dy / rkcoefs / time /
 * dt / step / expimp_wtimes / timemax / log / stat), sizeof(parallel_t),
 * sizeof(fluid_t), offsetof(fluid_t, srcuyg), sizeof(temperature_t),
 * sizeof(sns_case_desc), offsetof(sns_case_desc, fixed_dt / compensated)
 * (include/sns_batch.h) -- and returns how many it wrote (18) */
extern int sns_abi_layout(size_t *out, int n);

#ifdef __cplusplus
}
#endif
#endif /* SNS_GPU_H */
