/*
 * TEST INFRASTRUCTURE ONLY -- FFTW3-API stand-in (see fftw3.h), backed by the
 * oracle's real FFT (oracle/rfft.c).
 */
#include <stdio.h>
#include <stdlib.h>
#include "fftw3.h"
#include "../rfft.h"

struct oracle_fftw_plan_s {
  int forward;
  int howmany;
  int in_elem_stride, out_elem_stride; /* strides along the transform, in elements */
  int in_batch_stride, out_batch_stride;
  void *in, *out;
  oracle_rfft_plan rfft;
  double *work;
};

static fftw_plan make_plan(int forward, int rank, const fftw_iodim *dims, int howmany_rank,
                           const fftw_iodim *hdims, void *in, void *out) {
  if (rank != 1 || howmany_rank != 1) {
    fprintf(stderr, "fftw stand-in: only rank-1 transforms with one howmany dim\n");
    abort();
  }
  fftw_plan p = (fftw_plan)calloc(1, sizeof(*p));
  p->forward = forward;
  p->howmany = hdims[0].n;
  p->in_elem_stride = dims[0].is;
  p->out_elem_stride = dims[0].os;
  p->in_batch_stride = hdims[0].is;
  p->out_batch_stride = hdims[0].os;
  p->in = in;
  p->out = out;
  if (oracle_rfft_plan_init(&p->rfft, dims[0].n) != 0) {
    fprintf(stderr, "fftw stand-in: unsupported length %d (power of two required)\n", dims[0].n);
    abort();
  }
  p->work = (double *)malloc(sizeof(double) * (size_t)dims[0].n);
  return p;
}

fftw_plan fftw_plan_guru_dft_r2c(int rank, const fftw_iodim *dims, int howmany_rank,
                                 const fftw_iodim *howmany_dims, double *in, fftw_complex *out,
                                 unsigned flags) {
  (void)flags;
  return make_plan(1, rank, dims, howmany_rank, howmany_dims, in, out);
}

fftw_plan fftw_plan_guru_dft_c2r(int rank, const fftw_iodim *dims, int howmany_rank,
                                 const fftw_iodim *howmany_dims, fftw_complex *in, double *out,
                                 unsigned flags) {
  (void)flags;
  return make_plan(0, rank, dims, howmany_rank, howmany_dims, in, out);
}

void fftw_execute(const fftw_plan p) {
  for (int b = 0; b < p->howmany; b++) {
    if (p->forward) {
      const double *x = (const double *)p->in + (long)b * p->in_batch_stride;
      double *X = (double *)p->out + 2L * b * p->out_batch_stride;
      oracle_rfft_forward(&p->rfft, x, p->in_elem_stride, X, p->out_elem_stride, p->work);
    } else {
      const double *X = (const double *)p->in + 2L * b * p->in_batch_stride;
      double *x = (double *)p->out + (long)b * p->out_batch_stride;
      oracle_rfft_backward(&p->rfft, X, p->in_elem_stride, x, p->out_elem_stride, p->work);
    }
  }
}

void fftw_destroy_plan(fftw_plan p) {
  if (!p) return;
  oracle_rfft_plan_free(&p->rfft);
  free(p->work);
  free(p);
}
