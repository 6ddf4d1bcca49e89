/*
 * A plain C99 host program on the C ABI of libsns_gpu.so, written the way
 * the reference's own driver is (src/main.c:19-35 and the static integrate()
 * of src/main.c:79-101): structures from the constructors, then per step
 * param_decide_dt and, per RK substage, the boundary calls, the temperature
 * force and update, and the four fluid calls. It runs the 32 x 64,
 * Ra = 1e8, Pr = 1 Rayleigh-Benard case for 25 steps with the fixed cost
 * table (1, 2, 2, 3) and writes the final ux, uy, p and temp arrays (the
 * reference's layouts, halos included) as raw doubles to argv[1].
 */
#include <stdio.h>
#include <stdlib.h>

#include "sns_gpu.h"

static int check(int rc, const char *what) {
  if (rc != SNS_OK) {
    fprintf(stderr, "%s failed (%d): %s\n", what, rc, sns_last_error());
    exit(1);
  }
  return rc;
}

int main(int argc, char **argv) {
  const int itot = 32, jtot = 64, steps = 25;
  param_t *param;
  parallel_t *parallel;
  fluid_t *fluid;
  temperature_t *temperature;
  FILE *fp;
  int step, rk;
  if (argc < 2) {
    fprintf(stderr, "usage: %s OUTPUT\n", argv[0]);
    return 2;
  }
  param = sns_param_create(itot, jtot, 2.0, 1.e9, 1.e8, 1.0, 1, 1);
  if (!param) return 1;
  param->expimp_wtimes[0][0] = 1.;
  param->expimp_wtimes[0][1] = 2.;
  param->expimp_wtimes[1][0] = 2.;
  param->expimp_wtimes[1][1] = 3.;
  parallel = sns_parallel_create();
  fluid = fluid_init(param, parallel);
  temperature = temperature_init(param, parallel);
  if (!fluid || !temperature) {
    fprintf(stderr, "init failed: %s\n", sns_last_error());
    return 1;
  }
  for (step = 0; step < steps; step++) {
    check(param_decide_dt(param, parallel, fluid), "param_decide_dt");
    for (rk = 0; rk < RKSTEPMAX; rk++) {
      check(fluid_update_boundaries_ux(param, parallel, fluid->ux), "fluid_update_boundaries_ux");
      check(fluid_update_boundaries_uy(param, parallel, fluid->uy), "fluid_update_boundaries_uy");
      check(fluid_update_boundaries_p(param, parallel, fluid->p), "fluid_update_boundaries_p");
      check(temperature_update_boundaries_temp(param, parallel, temperature->temp),
            "temperature_update_boundaries_temp");
      check(temperature_compute_force(param, parallel, temperature), "temperature_compute_force");
      check(temperature_update_temp(param, parallel, rk, fluid, temperature), "temperature_update_temp");
      check(fluid_update_velocity(param, parallel, rk, fluid, temperature), "fluid_update_velocity");
      check(fluid_compute_potential(param, parallel, rk, fluid), "fluid_compute_potential");
      check(fluid_correct_velocity(param, parallel, rk, fluid), "fluid_correct_velocity");
      check(fluid_update_pressure(param, parallel, rk, fluid), "fluid_update_pressure");
    }
    param->step += 1;
    param->time += param->dt;
  }
  check(sns_sync_to_host(param, fluid, temperature), "sns_sync_to_host");
  fp = fopen(argv[1], "wb");
  if (!fp) return 1;
  fwrite(fluid->ux, sizeof(double), (size_t)(itot + 1) * (jtot + 2), fp);
  fwrite(fluid->uy, sizeof(double), (size_t)(itot + 2) * (jtot + 2), fp);
  fwrite(fluid->p, sizeof(double), (size_t)(itot + 2) * (jtot + 2), fp);
  fwrite(temperature->temp, sizeof(double), (size_t)(itot + 2) * (jtot + 2), fp);
  fwrite(&param->time, sizeof(double), 1, fp);
  fwrite(&param->dt, sizeof(double), 1, fp);
  fclose(fp);
  printf("step %d time %.17g dt %.17g\n", param->step, param->time, param->dt);
  temperature_finalise(temperature);
  fluid_finalise(fluid);
  sns_parallel_destroy(parallel);
  sns_param_destroy(param);
  return 0;
}
