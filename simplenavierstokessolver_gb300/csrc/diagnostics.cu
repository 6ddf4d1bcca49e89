// Device diagnostics of a Rayleigh-Benard state: the quantities the
// reference writes to its logs (src/logging.c:36-272 with the dissipation
// stencils of src/analyses.c:8-121): maximum and sum of the divergence,
// x/y momentum, kinetic (x, y) and thermal energy, and the Nusselt number
// from the wall heat flux, the energy injection, the kinetic and the thermal
// dissipation. All arithmetic is FP64; every sum is accumulated with
// Neumaier's compensated summation per thread, merged per block with the
// compensation carried along, and finished on the host in the same way, so
// the result agrees with the reference's sequential sums to their own
// round-off. Fields may be FP64 (plain path) or FP32 (batched form); FP32
// values are widened exactly.
#include <cstdint>
#include <mutex>

#include "diag_internal.h"

namespace sns {
namespace {

struct Neu {
  double s, c;
  __device__ __forceinline__ void add(double v) {
    const double t = s + v;
    c += fabs(s) >= fabs(v) ? (s - t) + v : (v - t) + s;
    s = t;
  }
};

template <typename F>
__global__ void __launch_bounds__(64) k_diag(DiagArgs<F> a, double *partials) {
  const int nx = a.nx, ny = a.ny;
  const int x = blockIdx.x * blockDim.x + threadIdx.x;  // ux point i = x+1 in [1, nx+1]
  const int y0 = blockIdx.y * kDiagRows, y1 = min(y0 + kDiagRows, ny);
  Neu acc[kDiagSums];
#pragma unroll
  for (int k = 0; k < kDiagSums; ++k) acc[k] = {0.0, 0.0};
  double divmax = 0.0;
  if (x <= nx) {
    const double dy = a.dy, q = a.sqrt_pr_ra, nu = a.nu, kap = a.kappa;
    const bool cell = x < nx;  // cell centre i = x+1 <= nx
    auto LD = [](const F *hi, const float *lo, size_t k) -> double {
      return lo ? (double)hi[k] + (double)lo[k] : (double)hi[k];
    };
    auto UX = [&](int xi, int y) -> double {  // ux at i = xi+1; walls i = 1 and nx+1 are zero
      return (xi <= 0 || xi >= nx) ? 0.0 : LD(a.ux, a.uxl, (size_t)y * nx + xi);
    };
    auto UY = [&](int xi, int y) -> double {  // uy at i = xi+1, zero at i = 0 and nx+1
      return (xi < 0 || xi >= nx) ? 0.0 : LD(a.uy, a.uyl, (size_t)y * nx + xi);
    };
    auto TT = [&](int xi, int y) -> double {
      return xi < 0 ? 0.5 : xi >= nx ? -0.5 : LD(a.t, a.tl, (size_t)y * nx + xi);
    };
    const double dxc = a.dxc[x];                 // DXC(i), i = x+1 <= nx+1
    const double dxf = cell ? a.dxf[x] : 1.0;    // DXF(i)
    const double dxf_m = x >= 1 ? a.dxf[x - 1] : 1.0;
    const double dxc_p = cell ? a.dxc[x + 1] : 1.0;
    for (int y = y0; y < y1; ++y) {
      const int ym = y == 0 ? ny - 1 : y - 1, yp = y + 1 == ny ? 0 : y + 1;
      // ---- ux point i (src/logging.c:95-100, 139-144, 208-214, 224-230)
      const double u = UX(x, y);
      const double cs_u = dxc * dy;
      acc[0].add(u * cs_u);
      acc[2].add(0.5 * (u * u) * cs_u);
      acc[5].add(q * (u * 0.5 * (TT(x - 1, y) + TT(x, y))) * cs_u);
      {  // src/analyses.c:8-33
        double s = 0.0;
        if (x != 0) {
          const double du = u - UX(x - 1, y);
          s += 0.5 / dxc * du * (du / dxf_m);
        }
        if (x != nx) {
          const double du = UX(x + 1, y) - u;
          s += 0.5 / dxc * du * (du / dxf);
        }
        const double dm = u - UX(x, ym), dp = UX(x, yp) - u;
        s += 0.5 / dy * dm * (dm / dy);
        s += 0.5 / dy * dp * (dp / dy);
        acc[6].add(q * (nu * s) * cs_u);
      }
      if (!cell) continue;
      // ---- cell centre i
      const double v = UY(x, y), tc = TT(x, y);
      const double cs_c = dxf * dy;
      const double div = (UX(x + 1, y) - u) / dxf + (UY(x, yp) - v) / dy;  // src/logging.c:51-57
      divmax = fmax(divmax, fabs(div));
      acc[7].add(div);
      acc[1].add(v * cs_c);
      acc[3].add(0.5 * (v * v) * cs_c);
      acc[4].add(0.5 * (tc * tc) * cs_c);
      {  // src/analyses.c:35-72 (uy) and :74-110 (temperature)
        const double wl = x == 0 ? 1. : 0.5, wr = x == nx - 1 ? 1. : 0.5;
        double s = 0.0, r = 0.0;
        double d = v - UY(x - 1, y);
        s += wl / dxf * d * (d / dxc);
        d = UY(x + 1, y) - v;
        s += wr / dxf * d * (d / dxc_p);
        d = v - UY(x, ym);
        s += 0.5 / dy * d * (d / dy);
        d = UY(x, yp) - v;
        s += 0.5 / dy * d * (d / dy);
        acc[6].add(q * (nu * s) * cs_c);
        d = tc - TT(x - 1, y);
        r += wl / dxf * d * (d / dxc);
        d = TT(x + 1, y) - tc;
        r += wr / dxf * d * (d / dxc_p);
        d = tc - TT(x, ym);
        r += 0.5 / dy * d * (d / dy);
        d = TT(x, yp) - tc;
        r += 0.5 / dy * d * (d / dy);
        acc[8].add(q * (kap * r) * cs_c);
      }
      if (x == 0) {  // wall heat flux (src/logging.c:195-199)
        const double g0 = (TT(0, y) - TT(-1, y)) / a.dxc[0];
        const double g1 = (TT(nx, y) - TT(nx - 1, y)) / a.dxc[nx];
        acc[9].add(-(0.5 * (g0 + g1) * dy));
      }
    }
  }
  // block merge: sums and compensations separately, then the block's result
  __shared__ double sh[64];
  double *out = partials + ((size_t)blockIdx.y * gridDim.x + blockIdx.x) * (2 * kDiagSums + 1);
  for (int k = 0; k < kDiagSums; ++k) {
    for (int part = 0; part < 2; ++part) {
      sh[threadIdx.x] = part == 0 ? acc[k].s : acc[k].c;
      __syncthreads();
      if (threadIdx.x == 0) {
        Neu m{0.0, 0.0};
        for (int t = 0; t < (int)blockDim.x; ++t) m.add(sh[t]);
        out[2 * k + part] = m.s + m.c;
      }
      __syncthreads();
    }
  }
  sh[threadIdx.x] = divmax;
  __syncthreads();
  if (threadIdx.x == 0) {
    double m = 0.0;
    for (int t = 0; t < (int)blockDim.x; ++t) m = fmax(m, sh[t]);
    out[2 * kDiagSums] = m;
  }
}

}  // namespace

template <typename F>
cudaError_t launch_diag(const DiagArgs<F> &a, double *partials, int *nblocks, cudaStream_t st) {
  const dim3 grid((a.nx + 1 + 63) / 64, (a.ny + kDiagRows - 1) / kDiagRows);
  *nblocks = grid.x * grid.y;
  k_diag<F><<<grid, 64, 0, st>>>(a, partials);
  return cudaGetLastError();
}

template cudaError_t launch_diag<double>(const DiagArgs<double> &, double *, int *, cudaStream_t);
template cudaError_t launch_diag<float>(const DiagArgs<float> &, double *, int *, cudaStream_t);

size_t diag_partials_words(int nx, int ny) {
  return (size_t)((nx + 1 + 63) / 64) * ((ny + kDiagRows - 1) / kDiagRows) * (2 * kDiagSums + 1);
}

// host finish: compensated sum of the block partials into the 11 log values
void diag_finish(const double *partials, int nblocks, double ly, double out[11]) {
  double s[kDiagSums] = {}, c[kDiagSums] = {};
  double divmax = 0.0;
  for (int b = 0; b < nblocks; ++b) {
    const double *p = partials + (size_t)b * (2 * kDiagSums + 1);
    for (int k = 0; k < kDiagSums; ++k) {
      for (int part = 0; part < 2; ++part) {
        const double v = p[2 * k + part];
        const double t = s[k] + v;
        c[k] += std::fabs(s[k]) >= std::fabs(v) ? (s[k] - t) + v : (v - t) + s[k];
        s[k] = t;
      }
    }
    divmax = std::fmax(divmax, p[2 * kDiagSums]);
  }
  double r[kDiagSums];
  for (int k = 0; k < kDiagSums; ++k) r[k] = s[k] + c[k];
  const double lx = 1.0;
  out[0] = divmax;
  out[1] = r[7];
  out[2] = r[0];
  out[3] = r[1];
  out[4] = r[2];
  out[5] = r[3];
  out[6] = r[4];
  out[7] = r[9] / ly;
  out[8] = r[5] / (lx * ly) + 1.;
  out[9] = r[6] / (lx * ly) + 1.;
  out[10] = r[8] / (lx * ly);
}

// ---------------------------------------------------------------------------
// Allocation-free variant (sns_diagnostics_static in sns_api.cpp).
//
// Some callers cannot allocate: a monitoring thread that samples a run while
// its kernels are in flight (cudaMalloc and cudaFree may synchronise the
// device and stall the solver's stream, and the first call of the allocating
// entry point makes a cudaMalloc), and a process whose device memory is
// committed to a batch arena sized to the whole HBM (an allocation there
// fails with out-of-memory). For them the block partials live in one
// file-scope device array of fixed size, the final compensated sum runs on
// the device, and the 11 results are copied straight into the caller's array:
// no device or host memory is allocated.
//
// Scratch layout: kDiagStaticBlocks block partials of 2*kDiagSums+1 words,
// then the 11 results. Nothing in it needs to start at zero: k_diag writes
// every partial word of every block it launches and k_diag_finish reads only
// those, then writes all 11 results. There is one scratch per device, so two
// calls that overlap on one device (other host threads, other cases) race on
// it and may return each other's or mixed results: serialise them.
namespace {

constexpr size_t kDiagStaticWords = (size_t)kDiagStaticBlocks * (2 * kDiagSums + 1);
static __device__ __align__(256) double g_diag_scratch[kDiagStaticWords + 16];

// the same compensated sums in the same order as diag_finish, one thread per
// sum, so the results equal those of sns_diagnostics bit for bit
__global__ void __launch_bounds__(32) k_diag_finish(const double *partials, int nblocks, double ly, double *out) {
  __shared__ double r[kDiagSums + 1];
  const int k = threadIdx.x;
  if (k < kDiagSums) {
    Neu m{0.0, 0.0};
    for (int b = 0; b < nblocks; ++b) {
      const double *p = partials + (size_t)b * (2 * kDiagSums + 1);
      m.add(p[2 * k]);
      m.add(p[2 * k + 1]);
    }
    r[k] = m.s + m.c;
  } else if (k == kDiagSums) {
    double divmax = 0.0;
    for (int b = 0; b < nblocks; ++b) divmax = fmax(divmax, partials[(size_t)b * (2 * kDiagSums + 1) + 2 * kDiagSums]);
    r[kDiagSums] = divmax;
  }
  __syncthreads();
  if (k == 0) {
    const double lx = 1.0;
    out[0] = r[kDiagSums];
    out[1] = r[7];
    out[2] = r[0];
    out[3] = r[1];
    out[4] = r[2];
    out[5] = r[3];
    out[6] = r[4];
    out[7] = r[9] / ly;
    out[8] = r[5] / (lx * ly) + 1.;
    out[9] = r[6] / (lx * ly) + 1.;
    out[10] = r[8] / (lx * ly);
  }
}

// The scratch's device address, looked up on every call with the caller's
// device current: an address kept from an earlier call could belong to a
// context that no longer exists (after cudaDeviceReset the module is loaded
// again, possibly elsewhere). The lookup is cheap once the module is loaded;
// the first call on a device may load it, so make that call before any
// stream capture.
cudaError_t scratch_for_current_device(double **ptr) {
  void *p = nullptr;
  const cudaError_t e = cudaGetSymbolAddress(&p, g_diag_scratch);
  if (e != cudaSuccess) return e;
  *ptr = static_cast<double *>(p);
  return cudaSuccess;
}

}  // namespace

int diag_blocks(int nx, int ny) { return ((nx + 1 + 63) / 64) * ((ny + kDiagRows - 1) / kDiagRows); }

cudaError_t diag_static(const DiagArgs<double> &a, cudaStream_t st, double out[11]) {
  if (diag_blocks(a.nx, a.ny) > kDiagStaticBlocks) return cudaErrorInvalidValue;
  double *scratch = nullptr;
  cudaError_t e = scratch_for_current_device(&scratch);
  if (e != cudaSuccess) return e;
  int nb = 0;
  if ((e = launch_diag(a, scratch, &nb, st)) != cudaSuccess) return e;
  double *res = scratch + kDiagStaticWords;
  k_diag_finish<<<1, 32, 0, st>>>(scratch, nb, a.ly, res);
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  if ((e = cudaMemcpyAsync(out, res, 11 * sizeof(double), cudaMemcpyDeviceToHost, st)) != cudaSuccess) return e;
  return cudaStreamSynchronize(st);
}

}  // namespace sns
