/*
 * TEST INFRASTRUCTURE ONLY -- CPU oracle. See rfft.h for the contract.
 *
 * Stands in for FFTW3's r2c/c2r transforms that the reference plans in
 * src/fluid/compute_potential.c:54-67 and executes at :90 (forward) and :149
 * (backward). Algorithm: published radix-2/4 decimation-in-time Cooley-Tukey
 * on the packed half-length complex sequence plus the real-FFT split step.
 */
#include <stdlib.h>
#include <math.h>
#include "rfft.h"

#define ORACLE_PI 3.14159265358979323846

void oracle_twiddle(int n, int t, double *re, double *im) {
  /* theta = 2 pi t / n = (pi/2) (q + r/n) with 4t = q n + r, 0 <= r < n */
  const long t4 = 4L * (long)t;
  const long q = t4 / n;
  const long r = t4 - q * (long)n;
  double c, s;
  if (2 * r <= n) {
    const double a = (ORACLE_PI * (double)r) / (2.0 * (double)n);
    c = cos(a);
    s = sin(a);
  } else {
    const double a = (ORACLE_PI * (double)(n - r)) / (2.0 * (double)n);
    c = sin(a);
    s = cos(a);
  }
  double cq, sq;
  switch (q & 3) {
    case 0: cq = c; sq = s; break;
    case 1: cq = -s; sq = c; break;
    case 2: cq = -c; sq = -s; break;
    default: cq = s; sq = -c; break;
  }
  *re = cq;
  *im = -sq;
}

int oracle_rfft_plan_init(oracle_rfft_plan *plan, int n) {
  if (n < 2 || (n & (n - 1)) != 0) return 1;
  plan->n = n;
  plan->m = n / 2;
  int p = 0;
  while ((1 << p) < plan->m) p++;
  plan->nstages = 0;
  if (p & 1) plan->radix[plan->nstages++] = 2;
  for (int s = 0; s < p / 2; s++) plan->radix[plan->nstages++] = 4;
  plan->tw = (double *)malloc(sizeof(double) * 2 * (size_t)n);
  plan->pos = (int *)malloc(sizeof(int) * (size_t)plan->m);
  if (!plan->tw || !plan->pos) return 2;
  for (int t = 0; t < n; t++) oracle_twiddle(n, t, &plan->tw[2 * t], &plan->tw[2 * t + 1]);
  for (int idx = 0; idx < plan->m; idx++) {
    int rest = idx, span = plan->m, slot = 0;
    for (int s = plan->nstages - 1; s >= 0; s--) {
      const int rdx = plan->radix[s];
      const int dig = rest % rdx;
      rest /= rdx;
      span /= rdx;
      slot += dig * span;
    }
    plan->pos[idx] = slot;
  }
  return 0;
}

void oracle_rfft_plan_free(oracle_rfft_plan *plan) {
  free(plan->tw);
  free(plan->pos);
  plan->tw = NULL;
  plan->pos = NULL;
}

/* one in-place decimation-in-time stage: sub-transforms of length L are
 * combined R at a time into transforms of length R*L. dir = -1 forward,
 * +1 backward (conjugate twiddles, +i in the radix-4 kernel). */
static void dit_stage(double *a, int M, int N, int R, int L, const double *tw, int dir) {
  const int span = R * L;
  const int tstep = N / span;
  const int nbfly = M / R;
  for (int b = 0; b < nbfly; b++) {
    const int k = b % L;
    const int base = (b / L) * span + k;
    double vr[4], vi[4];
    for (int r = 0; r < R; r++) {
      vr[r] = a[2 * (base + r * L)];
      vi[r] = a[2 * (base + r * L) + 1];
    }
    if (L > 1) {
      for (int r = 1; r < R; r++) {
        const int t = r * k * tstep;
        const double wr = tw[2 * t], wi = tw[2 * t + 1];
        const double xr = vr[r], xi = vi[r];
        if (dir < 0) {
          vr[r] = xr * wr - xi * wi;
          vi[r] = xr * wi + xi * wr;
        } else {
          vr[r] = xr * wr + xi * wi;
          vi[r] = xi * wr - xr * wi;
        }
      }
    }
    if (R == 2) {
      a[2 * base] = vr[0] + vr[1];
      a[2 * base + 1] = vi[0] + vi[1];
      a[2 * (base + L)] = vr[0] - vr[1];
      a[2 * (base + L) + 1] = vi[0] - vi[1];
    } else {
      const double t0r = vr[0] + vr[2], t0i = vi[0] + vi[2];
      const double t1r = vr[0] - vr[2], t1i = vi[0] - vi[2];
      const double t2r = vr[1] + vr[3], t2i = vi[1] + vi[3];
      const double t3r = vr[1] - vr[3], t3i = vi[1] - vi[3];
      /* forward: s = -i * t3 ; backward: s = +i * t3 (exact sign swaps) */
      const double sr = dir < 0 ? t3i : -t3i;
      const double si = dir < 0 ? -t3r : t3r;
      a[2 * base] = t0r + t2r;
      a[2 * base + 1] = t0i + t2i;
      a[2 * (base + L)] = t1r + sr;
      a[2 * (base + L) + 1] = t1i + si;
      a[2 * (base + 2 * L)] = t0r - t2r;
      a[2 * (base + 2 * L) + 1] = t0i - t2i;
      a[2 * (base + 3 * L)] = t1r - sr;
      a[2 * (base + 3 * L) + 1] = t1i - si;
    }
  }
}

static void run_stages(const oracle_rfft_plan *plan, double *a, int dir) {
  int L = 1;
  for (int s = 0; s < plan->nstages; s++) {
    dit_stage(a, plan->m, plan->n, plan->radix[s], L, plan->tw, dir);
    L *= plan->radix[s];
  }
}

void oracle_rfft_forward(const oracle_rfft_plan *plan, const double *x, long xs,
                         double *X, long Xs, double *work) {
  const int M = plan->m;
  for (int m = 0; m < M; m++) {
    const int p = plan->pos[m];
    work[2 * p] = x[(long)(2 * m) * xs];
    work[2 * p + 1] = x[(long)(2 * m + 1) * xs];
  }
  run_stages(plan, work, -1);
  const double z0r = work[0], z0i = work[1];
  X[0] = z0r + z0i;
  X[1] = 0.0;
  X[2 * (long)M * Xs] = z0r - z0i;
  X[2 * (long)M * Xs + 1] = 0.0;
  for (int k = 1; 2 * k <= M; k++) {
    const double ar = work[2 * k], ai = work[2 * k + 1];
    const double br = work[2 * (M - k)], bi = work[2 * (M - k) + 1];
    const double sre = ar + br, dim = ai - bi, dre = ar - br, sim = ai + bi;
    const double er = 0.5 * sre, ei = 0.5 * dim;
    const double orr = 0.5 * sim, oi = -(0.5 * dre);
    const double wr = plan->tw[2 * k], wi = plan->tw[2 * k + 1];
    const double wor = wr * orr - wi * oi;
    const double woi = wr * oi + wi * orr;
    X[2 * (long)k * Xs] = er + wor;
    X[2 * (long)k * Xs + 1] = ei + woi;
    if (2 * k != M) {
      X[2 * (long)(M - k) * Xs] = er - wor;
      X[2 * (long)(M - k) * Xs + 1] = woi - ei;
    }
  }
}

void oracle_rfft_backward(const oracle_rfft_plan *plan, const double *X, long Xs,
                          double *x, long xs, double *work) {
  const int M = plan->m;
  const double x0r = X[0], xmr = X[2 * (long)M * Xs];
  const int p0 = plan->pos[0];
  work[2 * p0] = x0r + xmr;
  work[2 * p0 + 1] = x0r - xmr;
  for (int k = 1; 2 * k <= M; k++) {
    const double ar = X[2 * (long)k * Xs], ai = X[2 * (long)k * Xs + 1];
    const double br = X[2 * (long)(M - k) * Xs], bi = X[2 * (long)(M - k) * Xs + 1];
    const double er = ar + br, ei = ai - bi, dr = ar - br, di = ai + bi;
    const double wr = plan->tw[2 * k], wi = plan->tw[2 * k + 1];
    const double orr = dr * wr + di * wi;
    const double oi = di * wr - dr * wi;
    const int pk = plan->pos[k];
    work[2 * pk] = er - oi;
    work[2 * pk + 1] = ei + orr;
    if (2 * k != M) {
      const int pm = plan->pos[M - k];
      work[2 * pm] = er + oi;
      work[2 * pm + 1] = orr - ei;
    }
  }
  run_stages(plan, work, +1);
  for (int m = 0; m < M; m++) {
    x[(long)(2 * m) * xs] = work[2 * m];
    x[(long)(2 * m + 1) * xs] = work[2 * m + 1];
  }
}
