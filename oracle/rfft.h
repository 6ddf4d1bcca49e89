/*
 * TEST INFRASTRUCTURE ONLY -- part of the CPU oracle. Nothing in the product
 * (the CUDA library and its host-side wrapper) links or calls this file; the
 * tests, smoke() and the CPU-baseline leg of bench.py use it as the checker.
 *
 * The real-to-complex / complex-to-real DFT used along the periodic (y)
 * direction of the Poisson solve.
 *
 * The reference calls FFTW3 (not vendored, unpinned; `apt-get install
 * libfftw3-dev` in Dockerfile:1-3) through
 *   fftw_plan_guru_dft_r2c / fftw_plan_guru_dft_c2r / fftw_execute
 * (src/fluid/compute_potential.c:54-67,90,149). FFTW is absent here, so the
 * transform is restated from the published algorithm (radix-2/4 Cooley-Tukey
 * decimation in time on the half-length complex sequence z[m] = x[2m]+i x[2m+1],
 * followed by the standard real-FFT split step) with FFTW's conventions:
 *   forward  X[k] = sum_n x[n] exp(-2 pi i k n / N), k = 0..N/2 (N/2+1 bins),
 *   backward x[n] = sum_{k=0}^{N-1} X[k] exp(+2 pi i k n / N), unnormalised,
 *            imaginary parts of X[0] and X[N/2] ignored.
 * The exact operation order written here is the contract shared with the
 * GPU kernels: the device FFT performs the same floating-point operations in
 * the same order on the same twiddle table, so both produce identical bits.
 *
 * Supported lengths: N = 2^p, p >= 1.
 */
#ifndef SNS_ORACLE_RFFT_H
#define SNS_ORACLE_RFFT_H

#ifdef __cplusplus
extern "C" {
#endif

typedef struct {
  int n;          /* real length N */
  int m;          /* complex length M = N/2 */
  int nstages;    /* number of butterfly stages on the length-M sequence */
  int radix[32];  /* radix of each stage, first applied first (2 or 4) */
  double *tw;     /* tw[2t], tw[2t+1] = cos(2 pi t/N), -sin(2 pi t/N), t in [0, N) */
  int *pos;       /* pos[m]: slot of input element m before the in-place stages */
} oracle_rfft_plan;

/* returns 0 on success, nonzero when n is not a power of two >= 2 */
int oracle_rfft_plan_init(oracle_rfft_plan *plan, int n);
void oracle_rfft_plan_free(oracle_rfft_plan *plan);

/* x: n reals read with stride xs; X: n/2+1 complex written (interleaved re,im)
 * with complex stride Xs; work: 2*(n/2) doubles */
void oracle_rfft_forward(const oracle_rfft_plan *plan, const double *x, long xs,
                         double *X, long Xs, double *work);
/* X: n/2+1 complex read with complex stride Xs; x: n reals written with stride xs */
void oracle_rfft_backward(const oracle_rfft_plan *plan, const double *X, long Xs,
                          double *x, long xs, double *work);

/* the shared twiddle rule: exact at multiples of pi/2, libm cos/sin only on
 * arguments in [0, pi/4] */
void oracle_twiddle(int n, int t, double *re, double *im);

#ifdef __cplusplus
}
#endif
#endif
