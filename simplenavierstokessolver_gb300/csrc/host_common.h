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

// ------------------------------------------------ partition method (PCR)
// A tridiagonal line of n rows is split into kPartSeg segments of m = n /
// kPartSeg rows, one per lane of a warp. Row e = k m + m - 1, the last of
// segment k, is its interface unknown; the m - 1 rows before it are the
// segment's interior. With the interface values known, an interior is the
// solution y of its own block (zero boundary values) plus multiples of two
// spikes: x_i = y_i + v_i x_{e(k-1)} + w_i x_{e(k)}. Substituting into the
// interface rows gives a tridiagonal system of kPartSeg unknowns, solved by
// parallel cyclic reduction in kPartLevels levels of warp shuffles.
// Everything here is independent of the right-hand side and computed once.
constexpr int kPartSeg = 32;
constexpr int kPartLevels = 5;  // log2(kPartSeg)

// doubles per line of the factor block written by partition_factors
inline size_t partition_stride(int n) { return 4 * (size_t)n + 2 * kPartLevels * kPartSeg + kPartSeg; }

// Factors of one line of n rows with sub-diagonal a_i, diagonal d_i and
// super-diagonal c_i. periodic: row 0 couples to row n-1 through a_0 and row
// n-1 to row 0 through c_{n-1}, so the interface system is cyclic (lane k
// couples to lanes k -+ 2^lev modulo kPartSeg at every level; after the last
// level both couplings fold into the diagonal); otherwise a_0 and c_{n-1} are
// ignored and the couplings past either end are zero. pin_last: the singular
// mean mode of the Poisson lines, whose last unknown the reference's Thomas
// solve sets to zero (its last pivot vanishes, src/linalg.c:36-38). Output
// (doubles): inv[n] up[n] v[n] w[n] (interior Thomas factors and spikes by
// row) alpha[kPartLevels][kPartSeg] beta[kPartLevels][kPartSeg] rD[kPartSeg].
// interleave: the four row arrays hold row k m + r at index r kPartSeg + k,
// so that the 32 lanes, each walking its own segment, touch 32 consecutive
// words at every step.
inline void partition_factors_tri(int n, const double *a_in, const double *d, const double *c_in, bool periodic,
                                  bool pin_last, bool interleave, double *out) {
  const int m = n / kPartSeg;
  std::vector<double> a(a_in, a_in + n), c(c_in, c_in + n);
  if (!periodic) {
    a[0] = 0.0;
    c[n - 1] = 0.0;
  }
  std::vector<double> inv(n, 0.0), up(n, 0.0), v(n, 0.0), w(n, 0.0);
  double *alpha = out + 4 * (size_t)n, *beta = alpha + kPartLevels * kPartSeg, *rD = beta + kPartLevels * kPartSeg;
  std::vector<double> L(kPartSeg), D(kPartSeg), U(kPartSeg);
  for (int k = 0; k < kPartSeg; k++) {
    const int s = k * m, e = s + m - 1;
    // interior block rows s..e-1
    inv[s] = 1.0 / d[s];
    up[s] = c[s] * inv[s];
    for (int i = s + 1; i < e; i++) {
      inv[i] = 1.0 / (d[i] - a[i] * up[i - 1]);
      up[i] = c[i] * inv[i];
    }
    auto solve = [&](std::vector<double> &r) {  // r over rows s..e-1 (index i - s)
      r[0] *= inv[s];
      for (int i = s + 1; i < e; i++) r[i - s] = inv[i] * (r[i - s] - a[i] * r[i - s - 1]);
      for (int i = e - 2; i >= s; i--) r[i - s] -= up[i] * r[i - s + 1];
    };
    std::vector<double> rv(m - 1, 0.0), rw(m - 1, 0.0);
    rv[0] = -a[s];
    rw[m - 2] = -c[e - 1];
    solve(rv);
    solve(rw);
    for (int i = s; i < e; i++) {
      v[i] = rv[i - s];
      w[i] = rw[i - s];
    }
  }
  for (int k = 0; k < kPartSeg; k++) {
    const int s = k * m, e = s + m - 1;
    const double ae = a[e], ce = c[e];
    L[k] = ae * v[e - 1];
    D[k] = ae * w[e - 1] + d[e];
    U[k] = 0.0;
    if (periodic || k < kPartSeg - 1) {
      const int s1 = (s + m) % n;  // the next segment's first interior row
      D[k] += ce * v[s1];
      U[k] = ce * w[s1];
    }
  }
  if (pin_last) {
    L[kPartSeg - 1] = 0.0;
    D[kPartSeg - 1] = 1.0;
    U[kPartSeg - 1] = 0.0;
  }
  for (int lev = 0; lev < kPartLevels; lev++) {
    const int dd = 1 << lev;
    std::vector<double> L2(kPartSeg), D2(kPartSeg), U2(kPartSeg);
    for (int k = 0; k < kPartSeg; k++) {
      const bool has_m = periodic || k - dd >= 0, has_p = periodic || k + dd < kPartSeg;
      const int km = (k - dd + kPartSeg) % kPartSeg, kp = (k + dd) % kPartSeg;
      const double al = has_m ? -L[k] / D[km] : 0.0;
      const double be = has_p ? -U[k] / D[kp] : 0.0;
      alpha[lev * kPartSeg + k] = al;
      beta[lev * kPartSeg + k] = be;
      L2[k] = has_m ? al * L[km] : 0.0;
      U2[k] = has_p ? be * U[kp] : 0.0;
      D2[k] = D[k] + (has_m ? al * U[km] : 0.0) + (has_p ? be * L[kp] : 0.0);
    }
    L = L2;
    D = D2;
    U = U2;
  }
  // cyclic: the last level leaves L and U on the unknown itself
  for (int k = 0; k < kPartSeg; k++) rD[k] = periodic ? 1.0 / (D[k] + L[k] + U[k]) : 1.0 / D[k];
  for (int i = 0; i < n; i++) {
    const size_t o = interleave ? (size_t)(i % m) * kPartSeg + i / m : (size_t)i;
    out[o] = inv[i];
    out[n + o] = up[i];
    out[2 * (size_t)n + o] = v[i];
    out[3 * (size_t)n + o] = w[i];
  }
}

// The Poisson lines: diagonal d_i = -l_raw_i - u_raw_i + eig with the
// Neumann closure (src/fluid/compute_potential.c:116-127: the first and last
// diagonal entries absorb l_raw_0 and u_raw_{n-1}), a_0 = c_{n-1} = 0.
inline void partition_factors(int n, const double *a, const double *c, const double *l_raw, const double *u_raw,
                              double eig, bool pin_last, bool interleave, double *out) {
  std::vector<double> d(n);
  for (int i = 0; i < n; i++) d[i] = -l_raw[i] - u_raw[i] + eig;
  d[0] += l_raw[0];
  d[n - 1] += u_raw[n - 1];
  partition_factors_tri(n, a, d.data(), c, false, pin_last, interleave, out);
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
