// Deterministic cost of one RK substage per diffusive treatment, the GPU
// counterpart of param_estimate_cost (src/param/estimate_cost.c:44-74),
// which times every EXP/IMP combination by wall clock and so makes the
// choice of param_decide_dt (src/param/decide_dt.c:76-100) vary from run to
// run. Here each kernel's time is predicted from the grid and the device's
// SM count and clock with constants measured on GB300:
//  * FP64-throughput kernels (stencils, FFTs): FP64 instructions per cell at
//    one warp instruction per kFp64CyclesPerWarpInst cycles per SM, at
//    kStencilEfficiency of that rate;
//  * serial line recurrences (Thomas sweeps): cycles per element of one line
//    times the line length, or the FP64 throughput bound when the lines
//    outnumber the SM sub-partitions;
//  * memory-bound kernels: bytes over kHbmBytesPerSecond;
//  * kLaunchSeconds per launch.
// The same grid and device always give the same costs, hence the same
// scheme for the same dt.
#include <algorithm>
#include <cmath>

#include "sns_internal.h"

namespace sns {

namespace {
constexpr double kFp64CyclesPerWarpInst = 19.9;  // per SM: 1.61 lane-ops/clk/SM measured
constexpr double kStencilEfficiency = 0.8;
constexpr double kHbmBytesPerSecond = 6.0e12;
constexpr double kLaunchSeconds = 2.5e-6;
// cycles per element of one serial sweep (forward + backward), measured
constexpr double kCyclesPoissonLine = 530.0;
constexpr double kCyclesSolveX = 540.0;
constexpr double kCyclesSolveY = 700.0;  // periodic: second pass over the line
constexpr double kOpsPerLineElement = 6.0;

// FP64 instructions per real sample of the length-ny real FFT of the Poisson
// kernels (radix-2 first stage when log2(ny/2) is odd, radix-4 stages with
// twiddles after the first, the real split step)
double fft_ops_per_sample(int ny) {
  const int m = ny / 2;
  int p = 0;
  while ((1 << (p + 1)) <= m) p++;
  double ops = 0.0;
  int L = 1;
  auto stage = [&](int r) {
    const int nb = m / r;
    ops += (double)nb * ((r == 2 ? 4 : 16) + (L > 1 ? (r - 1) * 6 : 0));
    L *= r;
  };
  if (p % 2) stage(2);
  for (int s = 0; s < p / 2; s++) stage(4);
  ops += (double)(m / 2) * 18 + 2;
  return ops / ny;
}
}  // namespace

void cost_model(int nx, int ny, int sms, double clock_hz, bool with_t, double out[2][2]) {
  const double cells = (double)nx * ny;
  const double warp_inst_rate = (double)sms * clock_hz / kFp64CyclesPerWarpInst;  // FP64 warp instructions / s
  auto fp64 = [&](double ops_per_cell) {
    return ops_per_cell * cells / 32.0 / (warp_inst_rate * kStencilEfficiency) + kLaunchSeconds;
  };
  auto lines = [&](int nlines, int length, double cycles_per_element) {
    const double latency = length * cycles_per_element / clock_hz;
    const double warps = std::ceil(nlines / 32.0);
    const double throughput = warps * length * kOpsPerLineElement / warp_inst_rate;
    return std::max(latency, throughput) + kLaunchSeconds;
  };
  auto memory = [&](double bytes_per_cell) { return bytes_per_cell * cells / kHbmBytesPerSecond + kLaunchSeconds; };
  const int nh = ny / 2 + 1;
  double base = fp64(81.0)                                   // velocity
                + fp64(fft_ops_per_sample(ny) + 6.0)         // divergence + forward FFT
                + lines(2 * nh, nx, kCyclesPoissonLine)      // Poisson tridiagonal
                + fp64(fft_ops_per_sample(ny) + 1.0)         // inverse FFT
                + fp64(9.0);                                 // correction + pressure
  if (with_t) base += fp64(27.0);                            // temperature
  const int fields = with_t ? 3 : 2;
  for (int iy = 0; iy < 2; iy++)
    for (int ix = 0; ix < 2; ix++) {
      double t = base;
      if (ix) t += fields * (lines(ny, nx, kCyclesSolveX) + memory(24.0));
      if (iy) t += fields * (lines(nx, ny, kCyclesSolveY) + memory(24.0));
      out[iy][ix] = t;
    }
}

}  // namespace sns
