// CPU check of the partition-method factors (csrc/host_common.h,
// partition_factors_tri): solves random tridiagonal lines with the
// operations the GPU kernels apply to those factors (k_par_cn in
// csrc/plain_parallel.cu: interior elimination and substitution per
// segment, interface right-hand sides, PCR over the 32 interface unknowns
// with cyclic lane indices, spikes) and compares the result with a dense
// Gaussian elimination of the same system. Prints one line per case:
// n periodic constant max_relative_error. With the argument "nowrap" the
// solve drops the periodic lines' wrap-around couplings (the dense system
// keeps them): the check's own sensitivity to a wrong coupling.
#include <cmath>
#include <cstdio>
#include <random>
#include <string>
#include <vector>

#include "host_common.h"

using namespace sns;

// dense solve with partial pivoting; A row-major n x n, b overwritten by x
static void dense_solve(int n, std::vector<double> A, std::vector<double> &b) {
  for (int k = 0; k < n; k++) {
    int p = k;
    for (int i = k + 1; i < n; i++)
      if (std::fabs(A[(size_t)i * n + k]) > std::fabs(A[(size_t)p * n + k])) p = i;
    if (p != k) {
      for (int j = 0; j < n; j++) std::swap(A[(size_t)k * n + j], A[(size_t)p * n + j]);
      std::swap(b[k], b[p]);
    }
    for (int i = k + 1; i < n; i++) {
      const double f = A[(size_t)i * n + k] / A[(size_t)k * n + k];
      for (int j = k; j < n; j++) A[(size_t)i * n + j] -= f * A[(size_t)k * n + j];
      b[i] -= f * b[k];
    }
  }
  for (int i = n - 1; i >= 0; i--) {
    double s = b[i];
    for (int j = i + 1; j < n; j++) s -= A[(size_t)i * n + j] * b[j];
    b[i] = s / A[(size_t)i * n + i];
  }
}

static bool g_nowrap = false;

// the kernels' operations on factors in natural row order (row k m + r of
// segment k at index k m + r)
static std::vector<double> partition_solve(int n, const std::vector<double> &a, const std::vector<double> &c,
                                           bool periodic, const std::vector<double> &fac, std::vector<double> q) {
  const int m = n / kPartSeg;
  const double *inv = fac.data(), *up = inv + n, *vv = inv + 2 * n, *ww = inv + 3 * n;
  const double *alpha = inv + 4 * (size_t)n, *beta = alpha + kPartLevels * kPartSeg, *rD = beta + kPartLevels * kPartSeg;
  std::vector<double> first(kPartSeg), last(kPartSeg), R(kPartSeg), xe(kPartSeg);
  for (int k = 0; k < kPartSeg; k++) {
    const int s = k * m;
    double y = q[s] * inv[s];
    q[s] = y;
    for (int r = 1; r < m - 1; r++) {
      const double g = a[s + r] * inv[s + r];
      y = std::fma(-g, y, inv[s + r] * q[s + r]);
      q[s + r] = y;
    }
    last[k] = y;
    for (int r = m - 3; r >= 0; r--) {
      y = std::fma(-up[s + r], y, q[s + r]);
      q[s + r] = y;
    }
    first[k] = y;
  }
  for (int k = 0; k < kPartSeg; k++) {
    const int e = k * m + m - 1;
    const bool wrap = periodic && !g_nowrap;
    const double ae = a[e], ce = (wrap || k < kPartSeg - 1) ? c[e] : 0.0;
    R[k] = std::fma(-ce, first[(k + 1) % kPartSeg], std::fma(-ae, last[k], q[e]));
  }
  for (int lev = 0; lev < kPartLevels; lev++) {
    const int d = 1 << lev;
    std::vector<double> Rn(kPartSeg);
    for (int k = 0; k < kPartSeg; k++) {
      const double rm = R[(k - d + kPartSeg) % kPartSeg], rp = R[(k + d) % kPartSeg];
      Rn[k] = std::fma(beta[lev * kPartSeg + k], rp, std::fma(alpha[lev * kPartSeg + k], rm, R[k]));
    }
    R = Rn;
  }
  for (int k = 0; k < kPartSeg; k++) xe[k] = R[k] * rD[k];
  for (int k = 0; k < kPartSeg; k++) {
    const int s = k * m;
    const double xl = (k == 0 && g_nowrap) ? 0.0 : xe[(k - 1 + kPartSeg) % kPartSeg];
    q[s + m - 1] = xe[k];
    for (int r = 0; r < m - 1; r++) q[s + r] = std::fma(ww[s + r], xe[k], std::fma(vv[s + r], xl, q[s + r]));
  }
  return q;
}

static double run_case(int n, bool periodic, bool constant, std::mt19937_64 &rng) {
  std::uniform_real_distribution<double> U(-1.0, 1.0);
  std::vector<double> a(n), d(n), c(n), q(n);
  const double s = 0.5 + 4.0 * std::fabs(U(rng));  // Crank-Nicolson-like: d = 1 + 2 s, a = c = -s
  for (int i = 0; i < n; i++) {
    a[i] = constant ? -s : -s * (1.0 + 0.3 * U(rng));
    c[i] = constant ? -s : -s * (1.0 + 0.3 * U(rng));
    d[i] = 1.0 + std::fabs(a[i]) + std::fabs(c[i]) + (constant ? 0.0 : 0.1 * std::fabs(U(rng)));
    q[i] = U(rng);
  }
  if (!periodic) {
    a[0] = 0.0;
    c[n - 1] = 0.0;
  }
  std::vector<double> fac(partition_stride(n));
  partition_factors_tri(n, a.data(), d.data(), c.data(), periodic, false, false, fac.data());
  const std::vector<double> x = partition_solve(n, a, c, periodic, fac, q);
  std::vector<double> A((size_t)n * n, 0.0), b = q;
  for (int i = 0; i < n; i++) {
    A[(size_t)i * n + i] = d[i];
    if (i > 0) A[(size_t)i * n + i - 1] = a[i];
    if (i < n - 1) A[(size_t)i * n + i + 1] = c[i];
  }
  if (periodic) {
    A[(size_t)0 * n + n - 1] += a[0];
    A[(size_t)(n - 1) * n + 0] += c[n - 1];
  }
  dense_solve(n, A, b);
  double num = 0.0, den = 0.0;
  for (int i = 0; i < n; i++) {
    num = std::fmax(num, std::fabs(x[i] - b[i]));
    den = std::fmax(den, std::fabs(b[i]));
  }
  return num / den;
}

int main(int argc, char **argv) {
  g_nowrap = argc > 1 && std::string(argv[1]) == "nowrap";
  std::mt19937_64 rng(20261203);
  const int sizes[] = {64, 96, 128, 256, 512};
  for (int n : sizes)
    for (int periodic = 0; periodic < 2; periodic++)
      for (int constant = 0; constant < 2; constant++)
        std::printf("%d %d %d %.3e\n", n, periodic, constant, run_case(n, periodic != 0, constant != 0, rng));
  return 0;
}
