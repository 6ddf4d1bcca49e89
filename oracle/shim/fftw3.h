/*
 * TEST INFRASTRUCTURE ONLY -- FFTW3-API stand-in for compiling the reference's
 * own sources into the CPU oracle (oracle/_ref). FFTW3 is not in this image
 * and is not vendored by the reference (Dockerfile:1-3 installs it with apt,
 * unpinned). Only the calls the reference makes are declared, with FFTW's
 * public signatures (src/fluid/compute_potential.c:54-67,90,149,165-166):
 * rank-1 guru r2c/c2r plans with one howmany dimension. The transform itself
 * is oracle/rfft.c (FFTW's conventions: unnormalised, n/2+1 bins).
 */
#ifndef ORACLE_SHIM_FFTW3_H
#define ORACLE_SHIM_FFTW3_H

#include <stddef.h>

/* as in FFTW: C99 complex when <complex.h> was included first */
#if defined(_Complex_I) && defined(complex) && defined(I)
typedef double _Complex fftw_complex;
#else
typedef double fftw_complex[2];
#endif

typedef struct oracle_fftw_plan_s *fftw_plan;
typedef struct { int n, is, os; } fftw_iodim;

#define FFTW_ESTIMATE (1U << 6)

fftw_plan fftw_plan_guru_dft_r2c(int rank, const fftw_iodim *dims, int howmany_rank,
                                 const fftw_iodim *howmany_dims, double *in, fftw_complex *out,
                                 unsigned flags);
fftw_plan fftw_plan_guru_dft_c2r(int rank, const fftw_iodim *dims, int howmany_rank,
                                 const fftw_iodim *howmany_dims, fftw_complex *in, double *out,
                                 unsigned flags);
void fftw_execute(const fftw_plan plan);
void fftw_destroy_plan(fftw_plan plan);

#endif
