// Internal structures of the batched FP32-stencil / FP64-Poisson engine.
//
// Per-case device layout: FP32 fields ux, uy, T (two buffers each) and the RK
// sources, FP64 p and psi, all dense ny x nx, x fastest, no halos (walls and
// the periodic wrap are index logic, as in the plain path). The FP64
// spectrum is mode-major here: mode J of column x at spec[J*nx + x], so a
// warp solving one mode line reads contiguous segments.
#pragma once

#include <cstddef>
#include <cstdint>

#include <cuda_runtime.h>

namespace sns {

constexpr int kSeg = 32;      // partition-method segments per line (one per lane)
constexpr int kPcrLevels = 5; // log2(kSeg)

struct BCase {
  // ---- static
  int nx, ny, nh;
  int fft_nst, fft_first2, fcols;  // FFT stage layout, columns per FFT block
  int with_t, with_force;
  int seg;                         // rows per segment = nx / kSeg
  double dy, rdy;
  float rdy_f, kappa_f, nu_f;
  int x2;                          // compensated increments (sns_case_desc::compensated)
  double kappa, nu;
  double dt_dif;                   // explicit diffusive limit min(dt_dif_x, dt_dif_y)
  double fixed_dt;
  long long target_steps;
  const float *rdxf_f, *rdxc_f;    // [nx], [nx+1]
  const float *rdxf_l;             // [nx] low words of 1/DXF(i) (compensated cases: rdxf_f + rdxf_l)
  float rdy_l;                     // low word of 1/dy
  const float *ccm_f, *ccp_f;      // DXC(i)/(2 DXF(i)), DXC(i+1)/(2 DXF(i))
  const float *cfm_f, *cfp_f;      // DXF(i-1)/(2 DXC(i)), DXF(i)/(2 DXC(i))
  const double *rdxf, *rdxc, *dxi; // FP64 metrics
  const double *ccm, *ccp, *cfm, *cfp;  // the advective coefficients above in FP64 (compensated cases)
  const double *dxf, *dxc;         // DXF(i), DXC(i) (diagnostics)
  const double *tw;                // [2*ny]
  const double *lo, *hi;           // Poisson sub/super diagonals a_i, c_i (mode independent) [nx]
  const double *pfac;              // per mode: inv[nx] up[nx] v[nx] w[nx] alpha[5*32] beta[5*32] rD[32]
  size_t pstride;                  // doubles per mode in pfac
  // ---- fields
  float *ux[2], *uy[2], *t[2];
  // low words of the compensated storage: value = hi (ux/uy/t above) + lo,
  // double-buffered like the high words
  float *uxl[2], *uyl[2], *tl[2];
  float *aux, *auy, *at;
  float *auxl, *auyl, *atl;        // low words of the previous right-hand sides (compensated cases)
  double *p, *psi;
  double2 *spec;
  // ---- dynamic (device-owned)
  int par;                         // buffer holding the current ux, uy, T
  int done;
  long long step;
  double time, dt;
  double adt[3], bdt[3], gdt[3], rgdt[3];
  unsigned int umax[2];            // float bits of max |ux|/DXC and max |uy|/dy (next dt)
  int nonfinite;                   // sticky: a NaN or infinity was written to ux, uy or p
};

struct BTile {
  int c, x0, y0;
};
struct BCols {
  int c, x0;
};
struct BModes {
  int c, j0;
};

constexpr int kBTileX = 64;   // default stencil/correction block width (tunable: 32, 64, 128)
constexpr int kBTileXMax = 128;
constexpr int kBTileY = 8;    // default rows per stencil/correction thread (tunable: 4, 8, 16)
constexpr int kBCorrY = 4;
constexpr int kBModesPerBlock = 4;     // default tridiagonal warps per block (tunable: 2, 4, 8)
constexpr int kBModesPerBlockMax = 8;

cudaError_t batch_kernels_init();
// tiles[ntiles - ntiles_x2 ..] belong to compensated cases
cudaError_t launch_batch_stencil(const BCase *cases, const BTile *tiles, int ntiles, int ntiles_x2, int rk,
                                 int tile_x, int rows, cudaStream_t st);
cudaError_t launch_batch_fwd(const BCase *cases, const BCols *cols, int ncols, int rk, size_t smem, int threads,
                             cudaStream_t st);
// shared memory of the tridiagonal launch for lines up to nmax long
size_t batch_tri_smem(int nmax, int modes_per_block);
// err: the batch's error word, set when a bulk-copy wait gave up after
// `spin` polls; stale: issue no copy, so that every wait runs out (a test of
// the error path)
cudaError_t launch_batch_tri(const BCase *cases, const BModes *modes, int nmodes, int modes_per_block, int nmax,
                             unsigned *err, unsigned spin, int stale, cudaStream_t st);
cudaError_t launch_batch_bwd(const BCase *cases, const BCols *cols, int ncols, size_t smem, int threads,
                             cudaStream_t st);
// the five phases of substage rk in one persistent cooperative launch of
// `blocks` blocks of 256 threads (batch_substage_blocks: every block resident)
size_t batch_substage_smem(size_t fft_smem, int nmax, int mpb);
int batch_substage_blocks(size_t smem);
cudaError_t launch_batch_substage(BCase *cases, const BTile *tiles, int ntiles, int ntiles_x2, const BCols *cols,
                                  int ncols, const BModes *modes, int nmodes, int rk, int tile_x, int rows, int mpb,
                                  int nmax, size_t smem, unsigned *err, unsigned spin, unsigned *bar, int blocks,
                                  cudaStream_t st);
cudaError_t launch_batch_corr(const BCase *cases, const BTile *tiles, int ntiles, int rk, int tile_x, int rows,
                              cudaStream_t st);
cudaError_t launch_batch_dt(BCase *cases, int ncases, const double *rk_a, const double *rk_b, cudaStream_t st);

void count_launches(long long n);
// counts the device and pinned host allocations the library makes (process-wide)
void count_allocation();
#ifndef SNS_COUNTED_ALLOC
#define SNS_COUNTED_ALLOC
template <typename T>
inline cudaError_t counted_malloc(T **p, size_t bytes) {
  const cudaError_t e = cudaMalloc(reinterpret_cast<void **>(p), bytes);
  if (e == cudaSuccess) count_allocation();
  return e;
}
template <typename T>
inline cudaError_t counted_malloc_host(T **p, size_t bytes, unsigned flags = cudaHostAllocDefault) {
  const cudaError_t e = cudaHostAlloc(reinterpret_cast<void **>(p), bytes, flags);
  if (e == cudaSuccess) count_allocation();
  return e;
}
#endif
// sets the message returned by sns_last_error() on this thread
void record_error(const char *msg);

}  // namespace sns
