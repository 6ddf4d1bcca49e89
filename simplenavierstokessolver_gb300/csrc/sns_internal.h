// Internal declarations shared by the host-side C ABI (sns_api.cpp) and the
// CUDA kernels. Not part of the public interface.
//
// Device layout ("dense"): every field is ny rows by nx columns, x fastest,
// element (i, j) of the reference (1-based, include/arrays/*.h) at
// [(j-1)*nx + (i-1)]. No halo rows or columns are stored:
//   * y is periodic, so row j=0 is row ny and row ny+1 is row 1 (index wrap);
//   * wall values are implied by index logic: ux(1) = ux(nx+1) = 0 (ux(1) is
//     stored, always zero), uy(0) = uy(nx+1) = 0, p and psi Neumann
//     (p(0) = p(1), p(nx+1) = p(nx)), T(0) = +0.5, T(nx+1) = -0.5.
// The Poisson spectrum is stored x-major: mode J of column i at
// [(i-1)*jpitch + J] as double2, so line solves along x for fixed J read
// consecutive J across a warp.
#pragma once

#include <cstddef>
#include <cstdint>

#include <cuda_runtime.h>

namespace sns {

constexpr double kTempXm = +0.5;  // include/temperature.h:22
constexpr double kTempXp = -0.5;  // include/temperature.h:23

// Grid metrics on the device, all indexed by x = i-1.
struct DevGrid {
  int nx, ny, nh, jpitch;  // nh = ny/2 + 1 Fourier modes; jpitch >= nh
  bool rcp;                // every metric divisor is a power of two
  bool p2;                 // rcp, and every reciprocal spacing, advective and Poisson coefficient is 2^e, |e| <= 64
  double dy, rdy;
  const double *dxf;    // [nx]    DXF(i)
  const double *dxc;    // [nx+1]  DXC(i), i = 1..nx+1
  const double *rdxf;   // [nx]    1/DXF(i) (exact when rcp)
  const double *rdxc;   // [nx+1]  1/DXC(i) (exact when rcp)
  const double *dxi;    // [nx+1]  1./DXC(i) as src/fluid/correct_velocity.c:13
  const double *c_cm;   // [nx]    DXC(i)/(2.*DXF(i))     (T and uy advection)
  const double *c_cp;   // [nx]    DXC(i+1)/(2.*DXF(i))
  const double *c_fm;   // [nx]    DXF(i-1)/(2.*DXC(i))   (ux advection, i >= 2)
  const double *c_fp;   // [nx]    DXF(i)/(2.*DXC(i))
  // Poisson: Thomas factors of the per-mode x-systems (src/fluid/compute_potential.c:109-136)
  const double *pl;     // [nx]            lower diagonal 1./DXC(i)/DXF(i)
  const double *pd0;    // [nh]            first pivot per mode
  const double *pinv;   // [nx * jpitch]   1./pivot; 0 where |pivot| < DBL_EPSILON (row forced to 0)
  const double *pup;    // [nx * jpitch]   normalised upper diagonal
  const double *tw;     // [2*ny]          twiddles exp(-2 pi i t/ny), t < ny
  int fft_nst;          // stages of the length-ny/2 complex FFT
  int fft_first2;       // first stage radix 2 (else all radix 4)
};

// Factors of one constant-matrix Thomas system shared by all lines, uploaded
// per substage for the Crank-Nicolson solves (src/linalg.c:9-30).
struct LineFactors {
  int n;
  const double *l;      // [n] lower diagonal
  const double *inv;    // [n] 1./pivot, 0 where |pivot| < DBL_EPSILON (row forced to 0);
                        //     row 0 unused (first row divides by d0)
  const double *up;     // [n] normalised upper diagonal
  double d0;            // first pivot
};

// Periodic y system (src/linalg.c:52-108): Thomas factors of the (n-1)
// sub-system, the RHS-independent second solution q1 and the closure.
struct PeriodicFactors {
  LineFactors sub;     // size n-1, first_div mode
  const double *q1;    // [n-1]
  double l_last, u_last, den;  // l[n-1], u[n-1], d[n-1] + u[n-1]*q1[0] + l[n-1]*q1[n-2]
};

// RK substage scalars, computed on the host exactly as the reference does.
struct StageScalars {
  double adt, bdt, gdt;  // alpha*dt, beta*dt, gamma*dt
  bool has_b;            // beta != 0 (beta*dt*srcb contributes)
  double kappa;          // 1./sqrt(Pr)/sqrt(Ra)   (temperature diffusion)
  double nu;             // sqrt(Pr)/sqrt(Ra)      (momentum diffusion)
  double rgdt;           // 1./(gamma*dt)          (Poisson right-hand side)
  double rny;            // 1/jtot when jtot is a power of two
  double pcorr;          // -(gamma*dt)/(2.*Re)    (pressure correction, implicit)
};

struct Fields {
  double *ux, *uy;             // current velocity (dense)
  double *ux_alt, *uy_alt;     // prediction targets (swapped after update)
  double *p, *psi;
  double *aux, *auy;           // explicit RK sources srcuxa / srcuya (dense, in place)
  double *qx, *qy;             // increments for the implicit paths
  double2 *spec;               // Poisson spectrum [nx * jpitch]
  unsigned long long *colmax;  // [nx] max |ux| per column (bit patterns)
  unsigned long long *uymax;   // [1]
};

struct TempFields {
  double *t[3];   // rotation of temperature buffers
  double *at;     // srctempa (dense)
  double *qt;     // increment for the implicit paths
};

// ------------------------------------------------------------ launch types
// up to three independent fields (temperature, ux, uy) in one launch: their
// serial sweeps run side by side
struct SolveXSet {
  LineFactors f[3];
  int mode[3];
  double *q[3];
  int n;
};
struct SolveYSet {
  PeriodicFactors f[3];
  int first_col[3];
  double *q[3];
  int n;
};
// strided field copies in one launch (host arrays are pinned and read or
// written in place through their device alias): row y of field k moves
// width entries from src + y*sstride to dst + y*dstride
struct XferField {
  const double *src;
  double *dst;
  int sstride, dstride, width;
};
constexpr int kXferMax = 8;
struct XferList {
  XferField f[kXferMax];
  int n, rows;
};
// Whole reference-layout host arrays moved in one linear pass (pinned host
// memory read or written in place through its device alias, 16-byte pairs of
// elements, full cache lines on the link): `host` holds (ny+2) rows of W
// entries, `dev` the dense ny x nx field. To the host every entry is written:
// the interior from the device, halo rows and wall columns by the reference's
// boundary rules of the field's kind (src/fluid/boundary_conditions.c:6-55,
// src/temperature/boundary_conditions.c:6-21; the temperature's four corners,
// which those rules leave alone, are not written). To the device only the
// interior is read.
enum LinKind { LIN_UX = 0, LIN_UY = 1, LIN_P = 2, LIN_T = 3 };
struct LinField {
  double *host;
  double *dev;
  int W;     // nx+1 (ux) or nx+2
  int kind;  // LinKind
};
struct LinList {
  LinField f[kXferMax];
  int n, nx, ny;
};

// fused Poisson solve (+ explicit temperature update): device flag words,
// sized by fused_layout, zeroed once; epoch advances by one per launch
struct FusedState {
  unsigned *fwd_done = nullptr;          // [groups]
  unsigned long long *bwd_cnt = nullptr; // [spans]
  unsigned *err = nullptr;               // [1]
  unsigned epoch = 0;
  unsigned spin_limit = 0;               // polls of a wait before it gives up; 0: the default (~1 s)
  int stale = 0;                         // test of the bounded waits: the next launch waits for a flag nobody sets
};

// ------------------------------------------------- launches of plain_fp64.cu
inline namespace exact {
#include "plain_launch.inc"
}
namespace contract {
#include "plain_launch.inc"
}

// Partition-method (PCR) form of the Poisson solve (plain_parallel.cu):
// per-mode factor blocks and the interleaved sub/super diagonals
struct ParFactors {
  const double *fac = nullptr;           // [nh][stride]
  const double *lo = nullptr, *hi = nullptr;  // [nx], rows interleaved
  size_t stride = 0;
  unsigned *err = nullptr;               // [1] set when a copy wait gave up
  unsigned spin_limit = 1u << 22;        // polls of that wait
  int stale = 0;                         // test of the bounded wait: the next launch issues no copy
};
bool parallel_tri_supported(int nx, int ny);
cudaError_t launch_par_fwd(const DevGrid &g, const StageScalars &s, const double *ux, const double *uy,
                           double2 *spec, cudaStream_t st);
cudaError_t launch_par_tri(const DevGrid &g, double2 *spec, const ParFactors &pf, cudaStream_t st);
cudaError_t launch_par_bwd(const DevGrid &g, const StageScalars &s, const double2 *spec, double *psi,
                           cudaStream_t st);

// Partition-method form of the Crank-Nicolson solves (plain_parallel.cu):
// per field the right-hand sides (solved in place), the line factor block
// (par_cn_stride doubles, shared by all lines of the field) and the first
// line solved; one launch covers up to three fields of one direction
struct ParCnField {
  double *q = nullptr;
  const double *fac = nullptr;
  int first = 0;
};
struct ParCnArgs {
  ParCnField f[3];
  int nf = 0;
  int n = 0, m = 0, s = 0;  // rows per line, per segment, shared-memory stride of a segment
  int lines = 0;            // lines per field (a field's lines are first .. lines-1)
  long long es = 0, ls = 0; // strides of a line's elements and of consecutive lines in q
};
size_t par_cn_stride(int n);
bool parallel_cn_supported(int n);
// columns: periodic lines along y; otherwise wall-bounded rows along x
cudaError_t launch_par_cn(bool columns, ParCnArgs a, cudaStream_t st);

// kernel kinds for the optional per-launch event timing (sns_profile_*)
enum KernelKind {
  K_TEMP = 0, K_VEL, K_POI_FWD, K_POI_TRI, K_POI_BWD, K_CORR_PRES, K_CORR, K_PRES, K_UMAX, K_SOLVE_X, K_SOLVE_Y,
  K_ADD_INC, K_POI_FUSED, K_POI_PCR, K_NUM_KINDS
};

// counts kernel launches (process-wide)
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
// message returned by sns_last_error on this thread
void record_error(const char *msg);
// predicted seconds per RK substage, out[implicity][implicitx] (cost_model.cpp)
void cost_model(int nx, int ny, int sms, double clock_hz, bool with_t, double out[2][2]);

}  // namespace sns
