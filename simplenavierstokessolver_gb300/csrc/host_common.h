// Host-side numerics shared by the plain path (sns_api.cpp) and the batched
// FP32-stencil engine (batch_api.cpp). Compiled without floating-point
// contraction: these values feed kernels that must reproduce the reference's
// rounding.
#pragma once

#include <cfloat>
#include <cmath>
#include <cstdint>
#include <vector>

namespace sns {

constexpr double kPiRef = 3.1415926535897932;  // include/common.h:7 of the reference

// src/param/init.c:124-195: face/centre coordinates and spacings (0-based
// arrays: xf[i-1] = XF(i), xc[i] = XC(i), dxf[i-1] = DXF(i), dxc[i-1] = DXC(i))
inline void make_grid(int itot, int jtot, double lx, double ly, double stretch_in, double *xf, double *xc,
                      double *dxf, double *dxc, double *yf, double *yc, double *dy) {
  int stretch = (int)stretch_in;
  if (stretch < 0) stretch = 0;
  if (stretch >= itot / 2) {
    const double dx = lx / itot;
    for (int i = 1; i <= itot + 1; i++) xf[i - 1] = 1. * (i - 1) * dx;
  } else {
    for (int i = 1; i <= itot + 1; i++) xf[i - 1] = cos(kPiRef * (1. * (i - 1) + stretch) / (itot + 2. * stretch));
    const double mn = xf[0], mx = xf[itot];
    for (int i = 1; i <= itot + 1; i++) xf[i - 1] = lx * (xf[i - 1] - mn) / (mx - mn);
  }
  xf[0] = 0.;
  xf[itot] = lx;
  for (int i = 1; i <= itot; i++) dxf[i - 1] = xf[i] - xf[i - 1];
  xc[0] = xf[0];
  for (int i = 1; i <= itot; i++) xc[i] = 0.5 * (xf[i - 1] + xf[i]);
  xc[itot + 1] = xf[itot];
  for (int i = 1; i <= itot + 1; i++) dxc[i - 1] = xc[i] - xc[i - 1];
  *dy = ly / jtot;
  if (yf)
    for (int j = 1; j <= jtot + 1; j++) yf[j - 1] = 1. * (j - 1) * (*dy);
  if (yc)
    for (int j = 1; j <= jtot; j++) yc[j - 1] = 0.5 * (2 * j - 1) * (*dy);
}

// Thomas forward elimination of a constant matrix (src/linalg.c:11-24), the
// RHS-independent part: normalised upper diagonal and 1/pivot, with 1/pivot
// = +0 marking the |pivot| < DBL_EPSILON rows that the reference zeroes.
inline void factorize(int n, const double *l, const double *d, const double *u, double *inv, double *up) {
  up[0] = u[0] / d[0];
  inv[0] = 0.0;
  for (int i = 1; i <= n - 1; i++) {
    double v = d[i] - l[i] * up[i - 1];
    if (std::fabs(v) < DBL_EPSILON) {
      up[i] = 0.;
      inv[i] = 0.;
    } else {
      v = 1. / v;
      up[i] = v * u[i];
      inv[i] = v;
    }
  }
}

// exp(-2 pi i t/n) with the CPU FFT's rule: exact at multiples of pi/2, libm
// cos/sin evaluated only on [0, pi/4]
inline void twiddle(int n, int t, double *re, double *im) {
  const long t4 = 4L * t;
  const long q = t4 / n;
  const long r = t4 - q * (long)n;
  double c, s;
  if (2 * r <= n) {
    const double a = (3.14159265358979323846 * (double)r) / (2.0 * (double)n);
    c = std::cos(a);
    s = std::sin(a);
  } else {
    const double a = (3.14159265358979323846 * (double)(n - r)) / (2.0 * (double)n);
    c = std::sin(a);
    s = std::cos(a);
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

inline std::vector<double> twiddle_table(int n) {
  std::vector<double> tw(2 * (size_t)n);
  for (int t = 0; t < n; t++) twiddle(n, t, &tw[2 * t], &tw[2 * t + 1]);
  return tw;
}

// Fourier eigenvalue of mode J of the periodic second difference
// (src/fluid/compute_potential.c:112-115)
inline double poisson_eigenvalue(double dy, int jtot, int J) {
  return -4. / pow(dy, 2.) * pow(sin(kPiRef * (J) / (1. * jtot)), 2.);
}

// stage layout of the length-jtot/2 complex FFT: radix 2 first when
// log2(jtot/2) is odd, then radix 4
inline void fft_layout(int jtot, int *nst, int *first2) {
  int p = 0;
  while ((1 << p) < jtot / 2) p++;
  *first2 = p & 1;
  *nst = (p & 1) + p / 2;
}

}  // namespace sns
