// Device diagnostics (diagnostics.cu): arguments and launch helpers.
#pragma once

#include <cmath>
#include <cstddef>

#include <cuda_runtime.h>

namespace sns {

constexpr int kDiagSums = 10;  // compensated sums per block
constexpr int kDiagRows = 16;  // rows per thread

// dense fields (x fastest, no halos), metrics as DXF(i) = dxf[i-1], DXC(i) = dxc[i-1]
template <typename F>
struct DiagArgs {
  int nx, ny;
  double dy, ly;
  double sqrt_pr_ra;  // sqrt(Pr)*sqrt(Ra)
  double nu;          // sqrt(Pr)/sqrt(Ra)
  double kappa;       // 1./sqrt(Pr)/sqrt(Ra)
  const double *dxf, *dxc;
  const F *ux, *uy, *t;
  // low words of compensated FP32 storage (value = hi + lo), or nullptr
  const float *uxl = nullptr, *uyl = nullptr, *tl = nullptr;
};

template <typename F>
cudaError_t launch_diag(const DiagArgs<F> &a, double *partials, int *nblocks, cudaStream_t st);
size_t diag_partials_words(int nx, int ny);
// out: divergence max, sum; x, y momentum; kinetic x, y and thermal energy;
// Nu from wall flux, injection, kinetic dissipation, thermal dissipation
void diag_finish(const double *partials, int nblocks, double ly, double out[11]);

// allocation-free form: block partials in a fixed file-scope device array of
// kDiagStaticBlocks blocks (672 KiB), the final sum on the device; grids with
// more blocks (diag_blocks) are rejected. Blocks until done.
constexpr int kDiagStaticBlocks = 4096;
int diag_blocks(int nx, int ny);
cudaError_t diag_static(const DiagArgs<double> &a, cudaStream_t st, double out[11]);

}  // namespace sns
