// Parallel form of the plain FP64 step's line solves and DFTs on GB300.
//
// The reference solves each Fourier mode's x-line with a serial Thomas
// recurrence (src/fluid/compute_potential.c:109-136, src/linalg.c:32-50).
// Reproduced bit for bit, that recurrence is a chain of 3 + 2 dependent FP64
// operations per x, which on GB300 (~70 cycles per dependent FP64 operation)
// bounds the plain step no matter how many lines run side by side. This
// form solves the same lines by the partition method with warp-shuffle
// parallel cyclic reduction (PCR): a warp per part (real, imaginary) of a
// mode line, one lane per segment of nx/32 rows, a 32-unknown interface
// system reduced in 5 shuffle levels. All RHS-independent factors (interior
// Thomas factors, spikes, PCR coefficients) are computed once on the host.
// Its results differ from the Thomas recurrence by rounding only, so the
// form is held to the path's tolerance (1e-12 relative L2 per field after
// the stated step counts) rather than to bit identity, and this unit is
// compiled with floating-point contraction.
//
// Layout: the spectrum is mode-major, spec[J * nx + p], with the rows of a
// mode line in the interleaved order p = (x % m) * 32 + x / m (m = nx / 32):
// lane k walks segment k, and at every step the 32 lanes touch 32
// consecutive elements, in global and in shared memory alike. The forward
// and inverse DFTs write and read that order: a radix-8 Stockham FFT in
// registers for 16 <= jtot <= 8192 (fft_stockham.cuh), the Thomas form's
// radix-2/4 FFT otherwise.
//
// The Crank-Nicolson lines (src/linalg.c:9-108) are solved by the same
// partition method: one warp per row along x (k_par_cn), one thread per
// segment of a column along y (k_par_cn_cols).
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>

#include "fft_dev.cuh"
#include "fft_stockham.cuh"
#include "host_common.h"
#include "sns_gpu.h"
#include "sns_internal.h"

namespace sns {
namespace {

constexpr int kParWarpsMax = 8;  // warps per block of the PCR kernel (two per mode line)
constexpr size_t kParSmemMax = 220 * 1024;

struct ParArgs {
  DevGrid g;
  StageScalars s;
  const double *ux, *uy;
  double2 *spec;  // [nh][nx], interleaved rows
  double *psi;
  int cols;       // adjacent x columns per block of the DFT kernels
  int m;          // rows per segment, nx / 32
};

// line position of column x (rows of a mode line interleaved by segment)
__device__ __forceinline__ int par_p(int x, int m) { return (x % m) * kPartSeg + x / m; }

// src/fluid/compute_potential.c:69-92: (div u*)/(gamma dt) and its real DFT
// along y, for the adjacent columns x0 .. x0+cols-1 (coalesced reads of the
// velocity); each column's spectrum goes to its line position
__global__ void __launch_bounds__(256) k_par_fwd(const ParArgs a) {
  extern __shared__ double2 z[];
  const int nx = a.g.nx, ny = a.g.ny, M = ny / 2, C = a.cols;
  const int x0 = blockIdx.x * C;
  double *zd = reinterpret_cast<double *>(z);
  const double rdy = a.g.rdy, rgdt = a.s.rgdt;
  for (int e = threadIdx.x; e < C * ny; e += blockDim.x) {
    const int c = e % C, y = e / C, x = x0 + c;
    double d = 0.0;
    if (x < nx) {
      const size_t r = (size_t)y * nx + x;
      const double uxm = a.ux[r];
      const double uxp = x == nx - 1 ? 0.0 : a.ux[r + 1];
      const double uym = a.uy[r];
      const double uyp = a.uy[(size_t)(y + 1 == ny ? 0 : y + 1) * nx + x];
      d = rgdt * ((uxp - uxm) * a.g.rdxf[x] + (uyp - uym) * rdy);
    }
    zd[2 * (c * M + fft::fft_slot(y >> 1, M, a.g.fft_nst, a.g.fft_first2)) + (y & 1)] = d;
  }
  __syncthreads();
  const double2 *tw = reinterpret_cast<const double2 *>(a.g.tw);
  fft::fft_stages<true>(z, C, M, ny, a.g.fft_nst, a.g.fft_first2, tw);
  const int half = M / 2 + 1;
  for (int e = threadIdx.x; e < C * half; e += blockDim.x) {
    const int c = e % C, k = e / C, x = x0 + c;
    if (x < nx) fft::rfft_post(z + c * M, a.spec + par_p(x, a.m), M, k, tw, (size_t)nx);
  }
}

// src/fluid/compute_potential.c:146-157: inverse real DFT and 1/jtot
__global__ void __launch_bounds__(256) k_par_bwd(const ParArgs a) {
  extern __shared__ double2 z[];
  const int nx = a.g.nx, ny = a.g.ny, M = ny / 2, C = a.cols;
  const int x0 = blockIdx.x * C;
  const double2 *tw = reinterpret_cast<const double2 *>(a.g.tw);
  const int half = M / 2 + 1;
  for (int e = threadIdx.x; e < C * half; e += blockDim.x) {
    const int c = e % C, k = e / C, x = x0 + c;
    double2 *zc = z + c * M;
    if (x >= nx) {
      zc[fft::fft_slot(k, M, a.g.fft_nst, a.g.fft_first2)] = make_double2(0.0, 0.0);
      if (k > 0) zc[fft::fft_slot(M - k, M, a.g.fft_nst, a.g.fft_first2)] = make_double2(0.0, 0.0);
      continue;
    }
    fft::rfft_pre(a.spec + par_p(x, a.m), zc, M, k, tw, a.g.fft_nst, a.g.fft_first2, (size_t)nx);
  }
  __syncthreads();
  fft::fft_stages<false>(z, C, M, ny, a.g.fft_nst, a.g.fft_first2, tw);
  const double *zd = reinterpret_cast<const double *>(z);
  for (int e = threadIdx.x; e < C * ny; e += blockDim.x) {
    const int c = e % C, y = e / C, x = x0 + c;
    if (x >= nx) continue;
    a.psi[(size_t)y * nx + x] = zd[2 * (c * M + (y >> 1)) + (y & 1)] * a.s.rny;
  }
}

// ---- the same two transforms by the radix-8 Stockham FFT (fft_stockham.cuh),
// for 16 <= jtot <= 8192. The solve is linear, so this pair moves two
// constant factors to the inverse's final scale: the forward transforms
// div u* without the factor 1/(gamma dt) and leaves the real FFT's split
// step unhalved (2 X), and the inverse multiplies by 1/(gamma dt) / (2 jtot)
// (an exact power-of-two scaling of 1/(gamma dt)). Both kernels run C
// columns per block on C jtot / 16 threads, 8 complex values per thread.

// src/fluid/compute_potential.c:69-92: div u* along two rows per complex
// element (z[m] = d[2m] + i d[2m+1]), its FFT, and 2 X[k] of the real
// transform at the columns' line positions
__global__ void __launch_bounds__(512) k_par_fwd8(const ParArgs a) {
  extern __shared__ double2 z[];
  const int nx = a.g.nx, ny = a.g.ny, M = ny / 2, C = a.cols;
  const int x0 = blockIdx.x * C;
  const double rdy = a.g.rdy;
  const double2 *tw = reinterpret_cast<const double2 *>(a.g.tw);
  for (int e = threadIdx.x; e < C * M; e += blockDim.x) {
    const int c = e % C, mm = e / C, x = x0 + c;
    double2 d = make_double2(0.0, 0.0);
    if (x < nx) {
      const size_t r0 = (size_t)(2 * mm) * nx + x, r1 = r0 + nx;
      const size_t r2 = (size_t)(2 * mm + 2 == ny ? 0 : 2 * mm + 2) * nx + x;
      const bool right = x == nx - 1;
      const double rdx = a.g.rdxf[x];
      const double u0m = a.ux[r0], u0p = right ? 0.0 : a.ux[r0 + 1];
      const double u1m = a.ux[r1], u1p = right ? 0.0 : a.ux[r1 + 1];
      const double v0 = a.uy[r0], v1 = a.uy[r1], v2 = a.uy[r2];
      d.x = (u0p - u0m) * rdx + (v1 - v0) * rdy;
      d.y = (u1p - u1m) * rdx + (v2 - v1) * rdy;
    }
    z[c * M + fft8::swz(mm)] = d;
  }
  __syncthreads();
  fft8::transform<true, 1>(z, C, M, tw);
  // split step for the bin pair (k, M-k): 2 X[k] = (Z[k] + conj Z[M-k]) +
  // w^k (Z[k] - conj Z[M-k]) / i, w = exp(-2 pi i / jtot)
  const int half = M / 2 + 1;
  for (int e = threadIdx.x; e < C * half; e += blockDim.x) {
    const int c = e % C, k = e / C, x = x0 + c;
    if (x >= nx) continue;
    const double2 *zc = z + c * M;
    double2 *out = a.spec + par_p(x, a.m);
    const size_t os = (size_t)nx;
    if (k == 0) {
      const double2 z0 = zc[0];
      const double s = z0.x + z0.y, t = z0.x - z0.y;
      out[0] = make_double2(s + s, 0.0);
      out[(size_t)M * os] = make_double2(t + t, 0.0);
    } else {
      const double2 A = zc[fft8::swz(k)], B = zc[fft8::swz(M - k)];
      const double sre = A.x + B.x, dim = A.y - B.y, dre = A.x - B.x, sim = A.y + B.y;
      const double2 w = tw[k];
      const double wor = w.x * sim + w.y * dre;
      const double woi = w.y * sim - w.x * dre;
      out[(size_t)k * os] = make_double2(sre + wor, dim + woi);
      if (2 * k != M) out[(size_t)(M - k) * os] = make_double2(sre - wor, woi - dim);
    }
  }
}

// src/fluid/compute_potential.c:146-157: the inverse (2 Z[k] from the bin
// pair, FFT, psi rows 2m and 2m+1 from element m) and the final scale
__global__ void __launch_bounds__(512) k_par_bwd8(const ParArgs a) {
  extern __shared__ double2 z[];
  const int nx = a.g.nx, ny = a.g.ny, M = ny / 2, C = a.cols;
  const int x0 = blockIdx.x * C;
  const double2 *tw = reinterpret_cast<const double2 *>(a.g.tw);
  const int half = M / 2 + 1;
  for (int e = threadIdx.x; e < C * half; e += blockDim.x) {
    const int c = e % C, k = e / C, x = x0 + c;
    double2 *zc = z + c * M;
    if (x >= nx) {
      zc[fft8::swz(k)] = make_double2(0.0, 0.0);
      if (k > 0) zc[fft8::swz(M - k)] = make_double2(0.0, 0.0);
      continue;
    }
    const double2 *in = a.spec + par_p(x, a.m);
    const size_t is = (size_t)nx;
    if (k == 0) {
      // imaginary parts of X[0] and X[M] ignored (FFTW's c2r convention)
      const double x0r = in[0].x, xmr = in[(size_t)M * is].x;
      zc[0] = make_double2(x0r + xmr, x0r - xmr);
    } else {
      const double2 A = in[(size_t)k * is], B = in[(size_t)(M - k) * is];
      const double er = A.x + B.x, ei = A.y - B.y, dr = A.x - B.x, di = A.y + B.y;
      const double2 w = tw[k];
      const double orr = dr * w.x + di * w.y;
      const double oi = di * w.x - dr * w.y;
      zc[fft8::swz(k)] = make_double2(er - oi, ei + orr);
      if (2 * k != M) zc[fft8::swz(M - k)] = make_double2(er + oi, orr - ei);
    }
  }
  __syncthreads();
  fft8::transform<false, 1>(z, C, M, tw);
  const double scale = a.s.rgdt * (0.5 * a.s.rny);
  for (int e = threadIdx.x; e < C * M; e += blockDim.x) {
    const int c = e % C, mm = e / C, x = x0 + c;
    if (x >= nx) continue;
    const double2 v = z[c * M + fft8::swz(mm)];
    const size_t r0 = (size_t)(2 * mm) * nx + x;
    a.psi[r0] = v.x * scale;
    a.psi[r0 + nx] = v.y * scale;
  }
}

struct ParTriArgs {
  double2 *spec;       // [nh][nx], interleaved rows
  const double *fac;   // [nh][stride]: inv g up v w (interleaved rows, g = a inv), alpha, beta, rD
  const double *lo;    // [nx] sub-diagonal a_i, interleaved rows (a_0 = 0)
  const double *hi;    // [nx] super-diagonal c_i, interleaved rows (c_{nx-1} = 0)
  size_t stride;       // doubles per mode in fac
  int nx, nh, m;
  unsigned *err;       // set to 1 when a copy wait gave up (the line is then left unsolved)
  unsigned spin_limit; // polls of a copy wait before it gives up
  int stale;           // test of the bounded wait: issue no copy, so the wait runs out
};

// polls of the wait that lets a warp's copies land after its first wait gave
// up, so that no copy into the warp's shared memory outlives the warp
constexpr unsigned kParDrainSpins = 1u << 22;

__device__ __forceinline__ bool mbar_try(unsigned bar, unsigned parity) {
  unsigned ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(bar), "r"(parity)
      : "memory");
  return ok != 0;
}

__device__ __forceinline__ unsigned smem_u32(const void *p) { return (unsigned)__cvta_generic_to_shared(p); }

// rows per chunk of the segment sweeps: the next chunk's factors are loaded
// while the current chunk is eliminated, off the dependent chain
constexpr int kParChunk = 8;

// src/fluid/compute_potential.c:109-136 by the partition method: two warps
// per mode line, one for its real and one for its imaginary part (both see
// the same real matrix and never mix, so each part takes the operations it
// took when one warp carried both). The first warp's lane 0 moves the line
// (16 nx bytes) into shared memory with a bulk asynchronous copy (completion
// on an mbarrier both warps wait on, bounded), STAGED: also the mode's factor
// block; otherwise the factors are read from global memory, coalesced by the
// interleaved row order, a chunk ahead. Each warp solves its part in shared
// memory and writes it back.
template <bool STAGED>
__global__ void __launch_bounds__(32 * kParWarpsMax) k_par_tri(const ParTriArgs a) {
  extern __shared__ __align__(128) unsigned char sm[];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int li = w >> 1, comp = w & 1;  // line of the block, part (0 real, 1 imaginary)
  const int J = blockIdx.x * (blockDim.x >> 6) + li;
  if (J >= a.nh) return;  // both warps of the line
  const int n = a.nx, m = a.m;
  const size_t per_line = 16 * (size_t)n + (STAGED ? 8 * a.stride : 0);
  double2 *line = reinterpret_cast<double2 *>(sm + 128 + (size_t)li * per_line);
  double *lc = reinterpret_cast<double *>(line) + comp;  // this part of element i at lc[2 i]
  double *fs = reinterpret_cast<double *>(line + n);
  double2 *gline = a.spec + (size_t)J * n;
  const double *gfac = a.fac + (size_t)J * a.stride;
  const unsigned bar = smem_u32(reinterpret_cast<unsigned long long *>(sm) + li);
  const unsigned line_bytes = 16u * (unsigned)n, fac_bytes = STAGED ? 8u * (unsigned)a.stride : 0u;
  if (comp == 0 && lane == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bar) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(line_bytes + fac_bytes)
                 : "memory");
    if (!a.stale) {
      asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                       smem_u32(line)),
                   "l"(__cvta_generic_to_global(gline)), "r"(line_bytes), "r"(bar)
                   : "memory");
      if (STAGED)
        asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                         smem_u32(fs)),
                     "l"(__cvta_generic_to_global(gfac)), "r"(fac_bytes), "r"(bar)
                     : "memory");
    }
  }
  // the line's two warps: the mbarrier is initialised before either waits on it
  asm volatile("bar.sync %0, 64;" ::"r"(1 + li) : "memory");
  const double *f = STAGED ? fs : gfac;
  auto ld = [&](const double *p) -> double {
    if constexpr (STAGED) {
      return *p;
    } else {
      return __ldg(p);
    }
  };
  const double *inv = f, *gg = f + n, *up = f + 2 * n, *vv = f + 3 * n, *ww = f + 4 * n;
  const double *alpha = f + 5 * n, *beta = alpha + kPartLevels * kPartSeg, *rD = beta + kPartLevels * kPartSeg;
  // global form: the first chunk's factors while the copy lands
  double ci[kParChunk], cg[kParChunk];
  const double inv0 = STAGED ? 0.0 : ld(inv + lane);
  if constexpr (!STAGED) {
#pragma unroll
    for (int k = 0; k < kParChunk; ++k) {
      const int r = 1 + k, i = r * kPartSeg + lane;
      ci[k] = r < m - 1 ? ld(inv + i) : 0.0;
      cg[k] = r < m - 1 ? ld(gg + i) : 0.0;
    }
  }
  bool done = false;
  for (unsigned k = 0; k < a.spin_limit && !done; ++k) done = mbar_try(bar, 0u);
  if (!done) {
    if (lane == 0) atomicOr(a.err, 1u);
    // leave the line unsolved, but only once the copies issued into this
    // line's shared memory have landed (bounded as well)
    if (!a.stale)
      for (unsigned k = 0; k < kParDrainSpins && !mbar_try(bar, 0u); ++k) {
      }
    return;
  }
  if constexpr (STAGED) {
#pragma unroll
    for (int k = 0; k < kParChunk; ++k) {
      const int r = 1 + k, i = r * kPartSeg + lane;
      ci[k] = r < m - 1 ? ld(inv + i) : 0.0;
      cg[k] = r < m - 1 ? ld(gg + i) : 0.0;
    }
  }
  // 1) the segment's interior rows r = 0 .. m-2 (line index r*32 + lane)
  //    with zero boundary values: forward elimination and back substitution.
  //    y_r = inv_r q_r - g_r y_{r-1} with g_r = a_r inv_r: one FMA per row on
  //    the dependent chain, the product inv_r q_r off it
  double y = lc[2 * lane];
  {
    const double i0 = STAGED ? ld(inv + lane) : inv0;
    y *= i0;
  }
  lc[2 * lane] = y;
#pragma unroll 1
  for (int b = 1; b < m - 1; b += kParChunk) {
    double ni[kParChunk], ng[kParChunk];
#pragma unroll
    for (int k = 0; k < kParChunk; ++k) {
      const int r = b + kParChunk + k, i = r * kPartSeg + lane;
      ni[k] = r < m - 1 ? ld(inv + i) : 0.0;
      ng[k] = r < m - 1 ? ld(gg + i) : 0.0;
    }
#pragma unroll
    for (int k = 0; k < kParChunk; ++k) {
      const int r = b + k, i = r * kPartSeg + lane;
      if (r < m - 1) {
        const double q = fma(-cg[k], y, ci[k] * lc[2 * i]);
        lc[2 * i] = q;
        y = q;
      }
    }
#pragma unroll
    for (int k = 0; k < kParChunk; ++k) {
      ci[k] = ni[k];
      cg[k] = ng[k];
    }
  }
  const double ylast = y;  // row m-2
  double cu[kParChunk];
#pragma unroll
  for (int k = 0; k < kParChunk; ++k) {
    const int r = m - 3 - k;
    cu[k] = r >= 0 ? ld(up + r * kPartSeg + lane) : 0.0;
  }
#pragma unroll 1
  for (int b = m - 3; b >= 0; b -= kParChunk) {
    double nu[kParChunk];
#pragma unroll
    for (int k = 0; k < kParChunk; ++k) {
      const int r = b - kParChunk - k;
      nu[k] = r >= 0 ? ld(up + r * kPartSeg + lane) : 0.0;
    }
#pragma unroll
    for (int k = 0; k < kParChunk; ++k) {
      const int r = b - k, i = r * kPartSeg + lane;
      if (r >= 0) {
        const double q = fma(-cu[k], y, lc[2 * i]);
        lc[2 * i] = q;
        y = q;
      }
    }
#pragma unroll
    for (int k = 0; k < kParChunk; ++k) cu[k] = nu[k];
  }
  // y: the first interior value (row 0). 2) right-hand side of the interface
  // row e: r_e - a_e y_{e-1} - c_e y'_0 (y'_0 of the next segment)
  const int ie = (m - 1) * kPartSeg + lane;
  const double yn = __shfl_down_sync(0xffffffffu, y, 1);
  const double re = lc[2 * ie];
  const double ae = __ldg(a.lo + ie), ce = lane < kPartSeg - 1 ? __ldg(a.hi + ie) : 0.0;
  double R = re - ae * ylast - ce * (lane < kPartSeg - 1 ? yn : 0.0);
  if (J == 0 && lane == kPartSeg - 1) R = 0.0;  // the mean mode: last unknown pinned to 0
  // 3) parallel cyclic reduction of the 32 interface equations
#pragma unroll
  for (int lev = 0; lev < kPartLevels; ++lev) {
    const int d = 1 << lev;
    const double mv = __shfl_up_sync(0xffffffffu, R, d);
    const double pv = __shfl_down_sync(0xffffffffu, R, d);
    const double al = ld(alpha + lev * kPartSeg + lane), be = ld(beta + lev * kPartSeg + lane);
    const double lm = lane >= d ? mv : 0.0;
    const double lp = lane + d < kPartSeg ? pv : 0.0;
    R = fma(be, lp, fma(al, lm, R));
  }
  const double xe = R * ld(rD + lane);
  lc[2 * ie] = xe;
  // 4) interiors from the spikes: x_i = y_i + v_i x_{e(k-1)} + w_i x_{e(k)}
  const double xl = __shfl_up_sync(0xffffffffu, xe, 1);
  const double lx = lane > 0 ? xl : 0.0;
#pragma unroll 1
  for (int b = 0; b < m - 1; b += kParChunk) {
    double cv[kParChunk], cw[kParChunk];
#pragma unroll
    for (int k = 0; k < kParChunk; ++k) {
      const int r = b + k, i = r * kPartSeg + lane;
      cv[k] = r < m - 1 ? ld(vv + i) : 0.0;
      cw[k] = r < m - 1 ? ld(ww + i) : 0.0;
    }
#pragma unroll
    for (int k = 0; k < kParChunk; ++k) {
      const int r = b + k, i = r * kPartSeg + lane;
      if (r < m - 1) lc[2 * i] = fma(cw[k], xe, fma(cv[k], lx, lc[2 * i]));
    }
  }
  __syncwarp();
  double *gc = reinterpret_cast<double *>(gline) + comp;
  for (int i = lane; i < n; i += 32) gc[2 * i] = lc[2 * i];
}

// ------------------------------------------------------------------------
// Crank-Nicolson lines by the partition method: src/linalg.c:9-30 along x
// (rows of a field, wall-bounded: src/temperature/update.c:141-157,
// src/fluid/update_velocity.c:249-280 and :500-520) and src/linalg.c:52-108
// along y (columns, periodic: src/temperature/update.c:189-207,
// src/fluid/update_velocity.c:404-430). A line of n rows is cut into 32
// segments of m = n / 32 rows; a periodic line's interface system is
// cyclic (its PCR levels couple modulo 32). All RHS-independent factors are
// computed on the host per substage (they depend on dt). Both kernels do
// the same operations on every element, in the same order.

constexpr int kCnWarpsMax = 8;
constexpr int kCnLoad = 8;  // elements in flight per thread while gathering a row

// factor block of a field's lines: inv g up v w (rows interleaved: row r of
// segment k at r * 32 + k), alpha beta (PCR levels), rD, then the interface
// rows' sub- and super-diagonals
struct CnFac {
  const double *inv, *gg, *up, *vv, *ww, *alpha, *beta, *rD, *ae, *ce;
  __device__ __forceinline__ CnFac(const double *f, int n)
      : inv(f), gg(f + n), up(f + 2 * n), vv(f + 3 * n), ww(f + 4 * n), alpha(f + 5 * (size_t)n),
        beta(alpha + kPartLevels * kPartSeg), rD(beta + kPartLevels * kPartSeg), ae(rD + kPartSeg),
        ce(ae + kPartSeg) {}
};

__device__ __forceinline__ ParCnField cn_field(const ParCnArgs &a) {
  // a select, not an index into the parameter array (which would copy the
  // array to the stack)
  return blockIdx.y == 0 ? a.f[0] : blockIdx.y == 1 ? a.f[1] : a.f[2];
}

__device__ __forceinline__ int cn_pos(int e, int m, int s) {
  const int k = e / m;
  return k * s + (e - k * m);
}

// Rows along x (wall-bounded): one warp per row, one lane per segment; the
// row is gathered into shared memory with each segment at a stride s = m | 1
// (odd, so that the 32 lanes' accesses at one row fall on distinct bank
// pairs), solved there and written back, coalesced both ways.
__global__ void __launch_bounds__(32 * kCnWarpsMax) k_par_cn(const ParCnArgs a) {
  extern __shared__ __align__(16) double cn_sm[];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, wpb = blockDim.x >> 5;
  const ParCnField F = cn_field(a);
  const int n = a.n, m = a.m, s = a.s;
  const int line = F.first + blockIdx.x * wpb + w;
  if (line >= a.lines) return;  // the whole warp
  double *sl = cn_sm + (size_t)w * ((size_t)kPartSeg * s + 8);
  const double *src = F.q + (size_t)line * a.ls;
  for (int e0 = lane; e0 < n; e0 += 32 * kCnLoad) {
    double v[kCnLoad];
#pragma unroll
    for (int k = 0; k < kCnLoad; ++k) {
      const int e = e0 + 32 * k;
      v[k] = e < n ? src[e] : 0.0;
    }
#pragma unroll
    for (int k = 0; k < kCnLoad; ++k) {
      const int e = e0 + 32 * k;
      if (e < n) sl[cn_pos(e, m, s)] = v[k];
    }
  }
  __syncwarp();
  const CnFac f(F.fac, n);
  double *seg = sl + lane * s;
  // 1) interior rows r = 0 .. m-2 with zero interface values:
  //    y_r = inv_r q_r - g_r y_{r-1}, then y_r -= up_r y_{r+1}
  double y = seg[0] * __ldg(f.inv + lane);
  seg[0] = y;
  double ci[kParChunk], cg[kParChunk];
#pragma unroll
  for (int k = 0; k < kParChunk; ++k) {
    const int r = 1 + k, i = r * kPartSeg + lane;
    ci[k] = r < m - 1 ? __ldg(f.inv + i) : 0.0;
    cg[k] = r < m - 1 ? __ldg(f.gg + i) : 0.0;
  }
#pragma unroll 1
  for (int b = 1; b < m - 1; b += kParChunk) {
    double ni[kParChunk], ng[kParChunk];
#pragma unroll
    for (int k = 0; k < kParChunk; ++k) {
      const int r = b + kParChunk + k, i = r * kPartSeg + lane;
      ni[k] = r < m - 1 ? __ldg(f.inv + i) : 0.0;
      ng[k] = r < m - 1 ? __ldg(f.gg + i) : 0.0;
    }
#pragma unroll
    for (int k = 0; k < kParChunk; ++k) {
      const int r = b + k;
      if (r < m - 1) {
        y = fma(-cg[k], y, ci[k] * seg[r]);
        seg[r] = y;
      }
    }
#pragma unroll
    for (int k = 0; k < kParChunk; ++k) {
      ci[k] = ni[k];
      cg[k] = ng[k];
    }
  }
  const double ylast = y;  // row m-2
  double cu[kParChunk];
#pragma unroll
  for (int k = 0; k < kParChunk; ++k) {
    const int r = m - 3 - k;
    cu[k] = r >= 0 ? __ldg(f.up + r * kPartSeg + lane) : 0.0;
  }
#pragma unroll 1
  for (int b = m - 3; b >= 0; b -= kParChunk) {
    double nu[kParChunk];
#pragma unroll
    for (int k = 0; k < kParChunk; ++k) {
      const int r = b - kParChunk - k;
      nu[k] = r >= 0 ? __ldg(f.up + r * kPartSeg + lane) : 0.0;
    }
#pragma unroll
    for (int k = 0; k < kParChunk; ++k) {
      const int r = b - k;
      if (r >= 0) {
        y = fma(-cu[k], y, seg[r]);
        seg[r] = y;
      }
    }
#pragma unroll
    for (int k = 0; k < kParChunk; ++k) cu[k] = nu[k];
  }
  // 2) interface row e of segment k: q_e - a_e y_{e-1} - c_e y'_0 (the next
  //    segment's first interior value; c_e = 0 for the last segment)
  const double ynext = __shfl_sync(0xffffffffu, y, (lane + 1) & 31);
  double R = fma(-__ldg(f.ce + lane), ynext, fma(-__ldg(f.ae + lane), ylast, seg[m - 1]));
  // 3) PCR of the 32 interface equations; the host zeroes the couplings
  //    past the ends of the line
#pragma unroll
  for (int lev = 0; lev < kPartLevels; ++lev) {
    const int d = 1 << lev;
    const double rm = __shfl_sync(0xffffffffu, R, (lane - d) & 31);
    const double rp = __shfl_sync(0xffffffffu, R, (lane + d) & 31);
    R = fma(__ldg(f.beta + lev * kPartSeg + lane), rp, fma(__ldg(f.alpha + lev * kPartSeg + lane), rm, R));
  }
  const double xe = R * __ldg(f.rD + lane);
  seg[m - 1] = xe;
  // 4) interiors: x_r = y_r + v_r x_{e(k-1)} + w_r x_{e(k)} (v = 0 in the
  //    first segment)
  const double xl = __shfl_sync(0xffffffffu, xe, (lane - 1) & 31);
#pragma unroll 1
  for (int b = 0; b < m - 1; b += kParChunk) {
    double cv[kParChunk], cw[kParChunk];
#pragma unroll
    for (int k = 0; k < kParChunk; ++k) {
      const int r = b + k, i = r * kPartSeg + lane;
      cv[k] = r < m - 1 ? __ldg(f.vv + i) : 0.0;
      cw[k] = r < m - 1 ? __ldg(f.ww + i) : 0.0;
    }
#pragma unroll
    for (int k = 0; k < kParChunk; ++k) {
      const int r = b + k;
      if (r < m - 1) seg[r] = fma(cw[k], xe, fma(cv[k], xl, seg[r]));
    }
  }
  __syncwarp();
  double *dstq = F.q + (size_t)line * a.ls;
  for (int e = lane; e < n; e += 32) dstq[e] = sl[cn_pos(e, m, s)];
}

// Columns along y (periodic): a block takes kCnCols adjacent columns and
// all 32 segments of each, thread t column t % kCnCols and segment
// t / kCnCols, and walks its segment in place in global memory; a warp's
// access covers 8 rows of kCnCols columns (whole 32-byte sectors). The
// first interior values, the interface right-hand sides and the interface
// solutions pass between the threads of a column through shared memory;
// warp c solves column c's cyclic interface system with lane = segment.
// Same operations on every element as k_par_cn.
constexpr int kCnCols = 4;

__global__ void __launch_bounds__(32 * kCnCols) k_par_cn_cols(const ParCnArgs a) {
  __shared__ double ex[3][kCnCols][kPartSeg];
  const ParCnField F = cn_field(a);
  const int n = a.n, m = a.m;
  const int c = threadIdx.x % kCnCols, k = threadIdx.x / kCnCols;
  const int col = F.first + blockIdx.x * kCnCols + c;
  const bool live = col < a.lines;
  const size_t es = (size_t)a.es;
  double *q = F.q + (live ? col : 0);
  const CnFac f(F.fac, n);
  const size_t e0 = (size_t)k * m;  // first row of the segment
  double y = 0.0, ylast = 0.0;
  if (live) {
    // 1) interior rows r = 0 .. m-2: forward elimination, back substitution
    y = q[e0 * es] * __ldg(f.inv + k);
    q[e0 * es] = y;
#pragma unroll 4
    for (int r = 1; r < m - 1; ++r) {
      const size_t o = (e0 + r) * es;
      y = fma(-__ldg(f.gg + r * kPartSeg + k), y, __ldg(f.inv + r * kPartSeg + k) * q[o]);
      q[o] = y;
    }
    ylast = y;
#pragma unroll 4
    for (int r = m - 3; r >= 0; --r) {
      const size_t o = (e0 + r) * es;
      y = fma(-__ldg(f.up + r * kPartSeg + k), y, q[o]);
      q[o] = y;
    }
  }
  ex[0][c][k] = y;  // the segment's first interior value
  __syncthreads();
  // 2) interface row e of segment k (the next segment cyclically)
  double R = 0.0;
  if (live) {
    const double ynext = ex[0][c][(k + 1) & 31];
    R = fma(-__ldg(f.ce + k), ynext, fma(-__ldg(f.ae + k), ylast, q[(e0 + m - 1) * es]));
  }
  ex[1][c][k] = R;
  __syncthreads();
  // 3) PCR: warp w takes column w, lane = segment
  {
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    double Rw = ex[1][w][lane];
#pragma unroll
    for (int lev = 0; lev < kPartLevels; ++lev) {
      const int d = 1 << lev;
      const double rm = __shfl_sync(0xffffffffu, Rw, (lane - d) & 31);
      const double rp = __shfl_sync(0xffffffffu, Rw, (lane + d) & 31);
      Rw = fma(__ldg(f.beta + lev * kPartSeg + lane), rp, fma(__ldg(f.alpha + lev * kPartSeg + lane), rm, Rw));
    }
    ex[2][w][lane] = Rw * __ldg(f.rD + lane);
  }
  __syncthreads();
  if (!live) return;
  // 4) interiors from the spikes
  const double xe = ex[2][c][k], xl = ex[2][c][(k - 1) & 31];
  q[(e0 + m - 1) * es] = xe;
#pragma unroll 4
  for (int r = 0; r < m - 1; ++r) {
    const size_t o = (e0 + r) * es;
    q[o] = fma(__ldg(f.ww + r * kPartSeg + k), xe, fma(__ldg(f.vv + r * kPartSeg + k), xl, q[o]));
  }
}

// adjacent columns per block of the DFT kernels, where the shared memory
// allows it. Measured at 512 x 1024 (parallel-form step, CUDA events): 1, 2,
// 4 and 8 columns 0.513, 0.511, 0.538 and 0.724 ms per step: whole sectors
// of the velocity rows (4 and more) cost more in blocks per SM than they save
constexpr int kParCols = 2;
int par_cols(const DevGrid &g) {
  int c = kParCols;
  while (c > 1 && (size_t)c * g.ny * sizeof(double) > 128 * 1024) c /= 2;
  return c;
}

int par_threads(const DevGrid &g, int cols) {
  const int b = cols * (g.ny / 2) / 4;
  return b <= 64 ? 64 : b >= 256 ? 256 : (b + 31) / 32 * 32;
}

// mode lines per block: enough blocks to spread over the SMs twice, and at
// least two blocks per SM where the lines' shared memory allows it
int par_lines(int nx, size_t per_line, int nh) {
  const size_t room = 2 * per_line + 256 <= kParSmemMax ? kParSmemMax / 2 - 128 : kParSmemMax - 128;
  const int by_smem = (int)std::min<size_t>(kParWarpsMax / 2, room / per_line);
  const int spread = (nh + 2 * 152 - 1) / (2 * 152);
  return std::max(0, std::min(by_smem, std::max(1, spread)));
}

// the factor block goes to shared memory along with the line when both fit
// twice per SM (lines up to itot 1024: the copy engine brings them in one
// go); longer lines read their factors from global memory a chunk ahead
bool par_staged(int nx, size_t stride) { return 2 * (16 * (size_t)nx + 8 * stride) + 256 <= kParSmemMax; }

}  // namespace

bool parallel_tri_supported(int nx, int ny) {
  return nx >= 2 * kPartSeg && nx % kPartSeg == 0 && ny >= 4 && 16 * (size_t)nx + 128 <= kParSmemMax;
}

namespace {
// the radix-8 Stockham pair: 16 <= jtot <= 8192 (at most 512 threads a block)
bool par_fft8(const DevGrid &g) { return g.ny >= 16 && g.ny <= 8192; }

void par_dft_attributes() {
  static bool attr = false;
  if (!attr) {
    cudaFuncSetAttribute(k_par_fwd, cudaFuncAttributeMaxDynamicSharedMemorySize, 160 * 1024);
    cudaFuncSetAttribute(k_par_bwd, cudaFuncAttributeMaxDynamicSharedMemorySize, 160 * 1024);
    cudaFuncSetAttribute(k_par_fwd8, cudaFuncAttributeMaxDynamicSharedMemorySize, 160 * 1024);
    cudaFuncSetAttribute(k_par_bwd8, cudaFuncAttributeMaxDynamicSharedMemorySize, 160 * 1024);
    attr = true;
  }
}

// columns per block of the radix-8 pair: C jtot / 16 threads, C jtot 8 bytes
int par_cols8(const DevGrid &g) {
  int c = kParCols;
  while (c > 1 && ((size_t)c * g.ny * sizeof(double) > 128 * 1024 || c * g.ny / 16 > 512)) c /= 2;
  return c;
}
}  // namespace

cudaError_t launch_par_fwd(const DevGrid &g, const StageScalars &s, const double *ux, const double *uy,
                           double2 *spec, cudaStream_t st) {
  par_dft_attributes();
  if (par_fft8(g)) {
    const int C = par_cols8(g);
    const ParArgs a{g, s, ux, uy, spec, nullptr, C, g.nx / kPartSeg};
    k_par_fwd8<<<(g.nx + C - 1) / C, C * g.ny / 16, (size_t)C * g.ny * sizeof(double), st>>>(a);
  } else {
    const int C = par_cols(g);
    const ParArgs a{g, s, ux, uy, spec, nullptr, C, g.nx / kPartSeg};
    k_par_fwd<<<(g.nx + C - 1) / C, par_threads(g, C), (size_t)C * g.ny * sizeof(double), st>>>(a);
  }
  count_launches(1);
  return cudaGetLastError();
}

cudaError_t launch_par_tri(const DevGrid &g, double2 *spec, const ParFactors &pf, cudaStream_t st) {
  static bool attr = false;
  if (!attr) {
    cudaFuncSetAttribute(k_par_tri<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kParSmemMax);
    cudaFuncSetAttribute(k_par_tri<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kParSmemMax);
    attr = true;
  }
  const bool staged = par_staged(g.nx, pf.stride);
  const size_t per_line = 16 * (size_t)g.nx + (staged ? 8 * pf.stride : 0);
  // mode lines per block, two warps each
  const int lpb = par_lines(g.nx, per_line, g.nh);
  if (lpb < 1) return cudaErrorInvalidValue;
  const ParTriArgs a{spec,  pf.fac, pf.lo, pf.hi, pf.stride, g.nx, g.nh, g.nx / kPartSeg, pf.err, pf.spin_limit,
                     pf.stale};
  const size_t smem = 128 + (size_t)lpb * per_line;
  if (staged) {
    k_par_tri<true><<<(g.nh + lpb - 1) / lpb, 64 * lpb, smem, st>>>(a);
  } else {
    k_par_tri<false><<<(g.nh + lpb - 1) / lpb, 64 * lpb, smem, st>>>(a);
  }
  count_launches(1);
  return cudaGetLastError();
}

size_t par_cn_stride(int n) { return 5 * (size_t)n + 2 * kPartLevels * kPartSeg + 3 * kPartSeg; }

namespace {
// doubles of shared memory per warp (one line)
size_t cn_warp_doubles(int n) { return (size_t)kPartSeg * ((n / kPartSeg) | 1) + 8; }
}  // namespace

bool parallel_cn_supported(int n) {
  return n >= 2 * kPartSeg && n % kPartSeg == 0 && cn_warp_doubles(n) * sizeof(double) <= kParSmemMax;
}

cudaError_t launch_par_cn(bool columns, ParCnArgs a, cudaStream_t st) {
  static bool attr = false;
  if (!attr) {
    cudaFuncSetAttribute(k_par_cn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kParSmemMax);
    attr = true;
  }
  if (!parallel_cn_supported(a.n) || a.nf < 1 || a.nf > 3) return cudaErrorInvalidValue;
  a.m = a.n / kPartSeg;
  a.s = a.m | 1;
  if (columns) {
    const dim3 grid((a.lines + kCnCols - 1) / kCnCols, a.nf);
    k_par_cn_cols<<<grid, 32 * kCnCols, 0, st>>>(a);
  } else {
    const size_t per = cn_warp_doubles(a.n) * sizeof(double);
    // warps (rows) per block: two blocks per SM where the rows fit
    int wpb = (int)std::min<size_t>(kCnWarpsMax, (kParSmemMax / 2) / per);
    if (wpb < 1) wpb = 1;
    const dim3 grid((a.lines + wpb - 1) / wpb, a.nf);
    k_par_cn<<<grid, 32 * wpb, wpb * per, st>>>(a);
  }
  count_launches(1);
  return cudaGetLastError();
}

cudaError_t launch_par_bwd(const DevGrid &g, const StageScalars &s, const double2 *spec, double *psi,
                           cudaStream_t st) {
  par_dft_attributes();
  if (par_fft8(g)) {
    const int C = par_cols8(g);
    const ParArgs a{g, s, nullptr, nullptr, const_cast<double2 *>(spec), psi, C, g.nx / kPartSeg};
    k_par_bwd8<<<(g.nx + C - 1) / C, C * g.ny / 16, (size_t)C * g.ny * sizeof(double), st>>>(a);
  } else {
    const int C = par_cols(g);
    const ParArgs a{g, s, nullptr, nullptr, const_cast<double2 *>(spec), psi, C, g.nx / kPartSeg};
    k_par_bwd<<<(g.nx + C - 1) / C, par_threads(g, C), (size_t)C * g.ny * sizeof(double), st>>>(a);
  }
  count_launches(1);
  return cudaGetLastError();
}

}  // namespace sns
