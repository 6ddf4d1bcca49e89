// Batched FP32-stencil / FP64-Poisson form of the SMR-RK3 step (sm_103a).
//
// One launch per phase covers every resident case: blocks read a work item
// (case, tile | column group | mode group) and the case's table entry.
// Stencils and RK3 updates are FP32 with fused multiply-adds; velocity and
// temperature are stored as compensated FP32 pairs (hi + lo, about 48
// significant bits) so that the per-substage rounding of the stored state
// does not accumulate, while every stencil reads the hi words only; the pressure gradient, the divergence, the FFTs, the
// tridiagonal solves, psi and p are FP64 (multiply-adds allowed: this form is
// compared with the FP64 reference by error norms, not bits). The equations
// are the reference's (src/temperature/update.c:11-87, src/fluid/
// update_velocity.c:11-192, src/fluid/compute_potential.c:69-157,
// src/fluid/correct_velocity.c:6-42, src/fluid/update_pressure.c:7-60) with
// explicit diffusion in both directions.
//
// The per-mode tridiagonal systems use a partition method instead of the
// serial Thomas sweep: a warp owns one line, lane k a segment of nx/32 rows;
// each lane eliminates its segment's interior with precomputed factors, the
// 32 interface unknowns form a tridiagonal system solved by parallel cyclic
// reduction across lanes (precomputed multipliers), and the interiors are
// recovered from the precomputed spike vectors. The critical path is
// nx/32 + 5 steps instead of nx.
#include <algorithm>
#include <cstdint>

#include "batch_internal.h"
#include "fft_dev.cuh"
#include "fft_stockham.cuh"

namespace sns {
namespace {

__device__ __forceinline__ int wup(int y, int ny) { return y + 1 == ny ? 0 : y + 1; }

// (hi + lo) + q in compensated FP32: the rounding error of hi + q (Knuth's
// TwoSum) joins the low word, then the pair is renormalised (Fast2Sum).
// Additions only, so no contraction can change the result.
__device__ __forceinline__ void acc2(float hi, float lo, float q, float &ho, float &lw) {
  const float s = hi + q;
  const float bp = s - hi;
  const float e = (hi - (s - bp)) + (q - bp);
  const float l = lo + e;
  const float h2 = s + l;
  lw = l - (h2 - s);
  ho = h2;
}
__device__ __forceinline__ int wdn(int y, int ny) { return y == 0 ? ny - 1 : y - 1; }

// ------------------------------------------------------------------ stencils
// A compensated value (hi + lo). Differences of neighbours use both words, so
// gradients and Laplacians are accurate to FP32 rounding of the difference
// itself rather than of the values; products and interpolations use hi.
struct F2 {
  float h, l;
};
__device__ __forceinline__ F2 ld2(const float *__restrict__ h, const float *__restrict__ l, size_t i) {
  return F2{h[i], l[i]};
}
__device__ __forceinline__ float dif(F2 a, F2 b) { return (a.h - b.h) + (a.l - b.l); }

// ------------------------------------------- float-float (compensated) terms
// Values as unevaluated sums h + l of two FP32 words (about 48 significant
// bits), built from error-free transformations: Knuth's TwoSum, Dekker's
// Fast2Sum (|a| >= |b| or a = 0) and the exact product error of one fused
// multiply-add. Cases with sns_case_desc::compensated compute every stencil
// term, coefficient and increment this way on the FP32 pipes, so the per-step
// rounding of the increments drops from FP32's 2^-24 to about 2^-44.
__device__ __forceinline__ F2 two_sum(float a, float b) {
  const float s = a + b;
  const float bp = s - a;
  return F2{s, (a - (s - bp)) + (b - bp)};
}
__device__ __forceinline__ F2 fast_two_sum(float a, float b) {
  const float s = a + b;
  return F2{s, b - (s - a)};
}
// the final renormalisation is a TwoSum too: under cancellation the low
// parts can outweigh the high sum, where Fast2Sum would not be exact
__device__ __forceinline__ F2 operator+(F2 x, F2 y) {
  const F2 s = two_sum(x.h, y.h);
  return two_sum(s.h, s.l + (x.l + y.l));
}
__device__ __forceinline__ F2 operator-(F2 x) { return F2{-x.h, -x.l}; }
__device__ __forceinline__ F2 operator-(F2 x, F2 y) { return x + (-y); }
__device__ __forceinline__ F2 operator*(F2 x, F2 y) {
  const float p = x.h * y.h;
  float e = fmaf(x.h, y.h, -p);
  e = fmaf(x.h, y.l, e);
  e = fmaf(x.l, y.h, e);
  return fast_two_sum(p, e);
}
__device__ __forceinline__ F2 halve(F2 x) { return F2{0.5f * x.h, 0.5f * x.l}; }
__device__ __forceinline__ F2 ff(double d) {
  const float h = (float)d;
  return F2{h, (float)(d - (double)h)};
}

// The stencil of k_b_stencil below for a compensated case: the same terms in
// the same order on float-float values; the previous right-hand sides are
// stored as pairs too (at/atl, aux/auxl, auy/auyl).
__device__ void stencil_x2(const BCase &C, int x, int y0, int y1, int rk) {
  const int nx = C.nx, ny = C.ny;
  const int pin = C.par ^ (rk & 1), pout = pin ^ 1;
  const float *__restrict__ ux = C.ux[pin];
  const float *__restrict__ uy = C.uy[pin];
  const float *__restrict__ T = C.t[pin];
  const float *__restrict__ uxl = C.uxl[pin];
  const float *__restrict__ uyl = C.uyl[pin];
  const float *__restrict__ Tl = C.tl[pin];
  float *__restrict__ uxo = C.ux[pout];
  float *__restrict__ uyo = C.uy[pout];
  float *__restrict__ To = C.t[pout];
  float *__restrict__ uxlo = C.uxl[pout];
  float *__restrict__ uylo = C.uyl[pout];
  float *__restrict__ Tlo = C.tl[pout];
  float *__restrict__ aux = C.aux;
  float *__restrict__ auy = C.auy;
  float *__restrict__ at = C.at;
  float *__restrict__ auxl = C.auxl;
  float *__restrict__ auyl = C.auyl;
  float *__restrict__ atl = C.atl;
  const double *__restrict__ p = C.p;
  const F2 adt = ff(C.adt[rk]), bdt = ff(C.bdt[rk]), gdt = ff(C.gdt[rk]);
  const bool hasb = rk > 0;
  const bool with_t = C.with_t != 0, force = C.with_t && C.with_force;
  const bool left = x == 0, right = x == nx - 1, has_ux = x >= 1;
  const F2 rdy = ff(C.rdy), kappa = ff(C.kappa), nu = ff(C.nu);
  const F2 rxc_m = ff(C.rdxc[x]), rxc_p = ff(C.rdxc[x + 1]), rxf = ff(C.rdxf[x]);
  const F2 rxf_m = has_ux ? ff(C.rdxf[x - 1]) : F2{0.f, 0.f};
  const F2 ccm = ff(C.ccm[x]), ccp = ff(C.ccp[x]), cfm = ff(C.cfm[x]), cfp = ff(C.cfp[x]);
  const double rdxc_d = C.rdxc[x], rdy_d = C.rdy;
  const F2 Z{0.f, 0.f};

  const int ym = wdn(y0, ny);
  const size_t r0 = (size_t)y0 * nx + x, rm = (size_t)ym * nx + x;
  F2 u0 = ld2(ux, uxl, r0), u1 = right ? Z : ld2(ux, uxl, r0 + 1);
  F2 um0 = ld2(ux, uxl, rm), um1 = right ? Z : ld2(ux, uxl, rm + 1);
  F2 v0 = ld2(uy, uyl, r0), vl = left ? Z : ld2(uy, uyl, r0 - 1);
  const F2 vm = ld2(uy, uyl, rm);
  F2 tc = ld2(T, Tl, r0);
  const F2 tm = ld2(T, Tl, rm);
  double pm = p[rm];
  F2 gym_u = (u0 - um0) * rdy;
  F2 pym_u = has_ux ? halve(cfm * vl + cfp * v0) * gym_u : Z;
  F2 gym_v = (v0 - vm) * rdy;
  F2 pym_v = halve(halve(vm + v0)) * gym_v;
  F2 gym_t = (tc - tm) * rdy;
  F2 pym_t = halve(v0) * gym_t;

  for (int y = y0; y < y1; ++y) {
    const int yp = wup(y, ny);
    const size_t r = (size_t)y * nx + x, rp = (size_t)yp * nx + x;
    const F2 u0n = ld2(ux, uxl, rp);
    const F2 u1n = right ? Z : ld2(ux, uxl, rp + 1);
    const F2 v0n = ld2(uy, uyl, rp);
    const F2 vln = left ? Z : ld2(uy, uyl, rp - 1);
    const F2 vr = right ? Z : ld2(uy, uyl, r + 1);
    const F2 tn = ld2(T, Tl, rp);
    const F2 tlv = left ? F2{0.5f, 0.f} : ld2(T, Tl, r - 1);  // T(0, j) = +0.5 (include/temperature.h)
    const double pc = p[r];
    if (with_t) {  // src/temperature/update.c:32-85
      const F2 trv = right ? F2{-0.5f, 0.f} : ld2(T, Tl, r + 1);
      const F2 gxm = (tc - tlv) * rxc_m, gxp = (trv - tc) * rxc_p, gyp = (tn - tc) * rdy;
      const F2 pyp = halve(v0n) * gyp;
      const F2 adv1 = -(ccm * u0 * gxm) - (ccp * u1 * gxp);
      const F2 adv2 = -pym_t - pyp;
      const F2 dfs = kappa * ((gxp - gxm) * rxf + (gyp - gym_t) * rdy);
      const F2 A = adv1 + adv2 + dfs;
      const F2 q = hasb ? adt * A + bdt * ld2(at, atl, r) : adt * A;
      at[r] = A.h;
      atl[r] = A.l;
      const F2 tn2 = tc + q;
      To[r] = tn2.h;
      Tlo[r] = tn2.l;
      gym_t = gyp;
      pym_t = pyp;
    } else {
      To[r] = tc.h;
      Tlo[r] = tc.l;
    }
    if (has_ux) {  // src/fluid/update_velocity.c:136-203
      const F2 ul = ld2(ux, uxl, r - 1);
      const F2 gxm = (u0 - ul) * rxf_m, gxp = (u1 - u0) * rxf, gyp = (u0n - u0) * rdy;
      const F2 vxm = halve(ul + u0), vxp = halve(u0 + u1);
      const F2 adv1 = -(cfm * vxm * gxm) - (cfp * vxp * gxp);
      const F2 pyp = halve(cfm * vln + cfp * v0n) * gyp;
      const F2 adv2 = -pym_u - pyp;
      const F2 dfs = nu * ((gxp - gxm) * rxc_m + (gyp - gym_u) * rdy);
      const F2 pre = ff(-((pc - p[r - 1]) * rdxc_d));
      F2 A = adv1 + adv2 + dfs;
      if (force) A = A + halve(tlv + tc);
      const F2 q = (hasb ? adt * A + bdt * ld2(aux, auxl, r) : adt * A) + gdt * pre;
      aux[r] = A.h;
      auxl[r] = A.l;
      const F2 un = u0 + q;
      uxo[r] = un.h;
      uxlo[r] = un.l;
      gym_u = gyp;
      pym_u = pyp;
    }
    {  // src/fluid/update_velocity.c:230-291
      const F2 gxm = (v0 - vl) * rxc_m, gxp = (vr - v0) * rxc_p, gyp = (v0n - v0) * rdy;
      const F2 wxm = halve(um0 + u0), wxp = halve(um1 + u1);
      const F2 adv1 = -(ccm * wxm * gxm) - (ccp * wxp * gxp);
      const F2 pyp = halve(halve(v0 + v0n)) * gyp;
      const F2 adv2 = -pym_v - pyp;
      const F2 dfs = nu * ((gxp - gxm) * rxf + (gyp - gym_v) * rdy);
      const F2 pre = ff(-((pc - pm) * rdy_d));
      const F2 A = adv1 + adv2 + dfs;
      const F2 q = (hasb ? adt * A + bdt * ld2(auy, auyl, r) : adt * A) + gdt * pre;
      auy[r] = A.h;
      auyl[r] = A.l;
      const F2 vn = v0 + q;
      uyo[r] = vn.h;
      uylo[r] = vn.l;
      gym_v = gyp;
      pym_v = pyp;
    }
    um0 = u0;
    um1 = u1;
    u0 = u0n;
    u1 = u1n;
    vl = vln;
    v0 = v0n;
    pm = pc;
    tc = tn;
  }
}

// the tiles of compensated cases (listed after the FP32 ones): a launch of
// its own, so that the FP32 stencil keeps its register budget
__global__ void __launch_bounds__(kBTileXMax) k_b_stencil_x2(const BCase *__restrict__ cases,
                                                            const BTile *__restrict__ tiles, int rk, int rows) {
  const BTile tile = tiles[blockIdx.x];
  const BCase &C = cases[tile.c];
  if (C.done) return;
  const int x = tile.x0 + threadIdx.x;
  if (x >= C.nx) return;
  stencil_x2(C, x, tile.y0, min(tile.y0 + rows, C.ny), rk);
}

// the FP32 stencil of column x, rows y0 .. y1-1 (one thread)
__device__ __forceinline__ void stencil_fp32(const BCase &C, int x, int y0, int y1, int rk) {
  const int nx = C.nx, ny = C.ny;
  const int pin = C.par ^ (rk & 1), pout = pin ^ 1;
  const float *__restrict__ ux = C.ux[pin];
  const float *__restrict__ uy = C.uy[pin];
  const float *__restrict__ T = C.t[pin];
  const float *__restrict__ uxl = C.uxl[pin];
  const float *__restrict__ uyl = C.uyl[pin];
  const float *__restrict__ Tl = C.tl[pin];
  float *__restrict__ uxo = C.ux[pout];
  float *__restrict__ uyo = C.uy[pout];
  float *__restrict__ To = C.t[pout];
  float *__restrict__ uxlo = C.uxl[pout];
  float *__restrict__ uylo = C.uyl[pout];
  float *__restrict__ Tlo = C.tl[pout];
  float *__restrict__ aux = C.aux;
  float *__restrict__ auy = C.auy;
  float *__restrict__ at = C.at;
  const double *__restrict__ p = C.p;
  const float adt = (float)C.adt[rk], bdt = (float)C.bdt[rk], gdt = (float)C.gdt[rk];
  const bool hasb = rk > 0;
  const bool with_t = C.with_t != 0, force = C.with_t && C.with_force;
  const bool left = x == 0, right = x == nx - 1, has_ux = x >= 1;
  const float rdy = C.rdy_f, kappa = C.kappa_f, nu = C.nu_f;
  const float rxc_m = C.rdxc_f[x], rxc_p = C.rdxc_f[x + 1], rxf = C.rdxf_f[x];
  const float rxf_m = has_ux ? C.rdxf_f[x - 1] : 0.f;
  const float ccm = C.ccm_f[x], ccp = C.ccp_f[x], cfm = C.cfm_f[x], cfp = C.cfp_f[x];
  const double rdxc_d = C.rdxc[x], rdy_d = C.rdy;
  const F2 Z{0.f, 0.f};

  const int ym = wdn(y0, ny);
  const size_t r0 = (size_t)y0 * nx + x, rm = (size_t)ym * nx + x;
  F2 u0 = ld2(ux, uxl, r0), u1 = right ? Z : ld2(ux, uxl, r0 + 1);
  F2 um0 = ld2(ux, uxl, rm), um1 = right ? Z : ld2(ux, uxl, rm + 1);
  F2 v0 = ld2(uy, uyl, r0), vl = left ? Z : ld2(uy, uyl, r0 - 1);
  const F2 vm = ld2(uy, uyl, rm);
  F2 tc = ld2(T, Tl, r0);
  const F2 tm = ld2(T, Tl, rm);
  double pm = p[rm];
  float gym_u = dif(u0, um0) * rdy;
  float pym_u = has_ux ? (0.5f * (cfm * vl.h + cfp * v0.h)) * gym_u : 0.f;
  float gym_v = dif(v0, vm) * rdy;
  float pym_v = (0.5f * (0.5f * (vm.h + v0.h))) * gym_v;
  float gym_t = dif(tc, tm) * rdy;
  float pym_t = (0.5f * v0.h) * gym_t;

  for (int y = y0; y < y1; ++y) {
    const int yp = wup(y, ny);
    const size_t r = (size_t)y * nx + x, rp = (size_t)yp * nx + x;
    const F2 u0n = ld2(ux, uxl, rp);
    const F2 u1n = right ? Z : ld2(ux, uxl, rp + 1);
    const F2 v0n = ld2(uy, uyl, rp);
    const F2 vln = left ? Z : ld2(uy, uyl, rp - 1);
    const F2 vr = right ? Z : ld2(uy, uyl, r + 1);
    const F2 tn = ld2(T, Tl, rp);
    const F2 tlv = left ? F2{0.5f, 0.f} : ld2(T, Tl, r - 1);  // T(0, j) = +0.5 (include/temperature.h)
    const double pc = p[r];
    if (with_t) {  // src/temperature/update.c:32-85
      const F2 trv = right ? F2{-0.5f, 0.f} : ld2(T, Tl, r + 1);
      const float gxm = dif(tc, tlv) * rxc_m, gxp = dif(trv, tc) * rxc_p, gyp = dif(tn, tc) * rdy;
      const float pyp = (0.5f * v0n.h) * gyp;
      const float adv1 = -(ccm * u0.h * gxm) - (ccp * u1.h * gxp);
      const float adv2 = -pym_t - pyp;
      const float dfs = kappa * ((gxp - gxm) * rxf + (gyp - gym_t) * rdy);
      const float A = adv1 + adv2 + dfs;
      const float q = hasb ? fmaf(adt, A, bdt * at[r]) : adt * A;
      at[r] = A;
      acc2(tc.h, tc.l, q, To[r], Tlo[r]);
      gym_t = gyp;
      pym_t = pyp;
    } else {
      To[r] = tc.h;  // uncoupled temperature is carried along unchanged
      Tlo[r] = tc.l;
    }
    if (has_ux) {  // src/fluid/update_velocity.c:136-203
      const F2 ul = ld2(ux, uxl, r - 1);
      const float gxm = dif(u0, ul) * rxf_m, gxp = dif(u1, u0) * rxf, gyp = dif(u0n, u0) * rdy;
      const float vxm = 0.5f * (ul.h + u0.h), vxp = 0.5f * (u0.h + u1.h);
      const float adv1 = -(cfm * vxm * gxm) - (cfp * vxp * gxp);
      const float pyp = (0.5f * (cfm * vln.h + cfp * v0n.h)) * gyp;
      const float adv2 = -pym_u - pyp;
      const float dfs = nu * ((gxp - gxm) * rxc_m + (gyp - gym_u) * rdy);
      const float pre = -(float)((pc - p[r - 1]) * rdxc_d);
      float A = adv1 + adv2 + dfs;
      if (force) A += 0.5f * ((tlv.h + tc.h) + (tlv.l + tc.l));
      float q = hasb ? fmaf(adt, A, bdt * aux[r]) : adt * A;
      q = fmaf(gdt, pre, q);
      aux[r] = A;
      acc2(u0.h, u0.l, q, uxo[r], uxlo[r]);
      gym_u = gyp;
      pym_u = pyp;
    }
    {  // src/fluid/update_velocity.c:230-291
      const float gxm = dif(v0, vl) * rxc_m, gxp = dif(vr, v0) * rxc_p, gyp = dif(v0n, v0) * rdy;
      const float wxm = 0.5f * (um0.h + u0.h), wxp = 0.5f * (um1.h + u1.h);
      const float adv1 = -(ccm * wxm * gxm) - (ccp * wxp * gxp);
      const float pyp = (0.5f * (0.5f * (v0.h + v0n.h))) * gyp;
      const float adv2 = -pym_v - pyp;
      const float dfs = nu * ((gxp - gxm) * rxf + (gyp - gym_v) * rdy);
      const float pre = -(float)((pc - pm) * rdy_d);
      const float A = adv1 + adv2 + dfs;
      float q = hasb ? fmaf(adt, A, bdt * auy[r]) : adt * A;
      q = fmaf(gdt, pre, q);
      auy[r] = A;
      acc2(v0.h, v0.l, q, uyo[r], uylo[r]);
      gym_v = gyp;
      pym_v = pyp;
    }
    um0 = u0;
    um1 = u1;
    u0 = u0n;
    u1 = u1n;
    vl = vln;
    v0 = v0n;
    pm = pc;
    tc = tn;
  }
}

__global__ void __launch_bounds__(kBTileXMax) k_b_stencil(const BCase *__restrict__ cases,
                                                         const BTile *__restrict__ tiles, int rk, int rows) {
  const BTile tile = tiles[blockIdx.x];
  const BCase &C = cases[tile.c];
  if (C.done) return;
  const int x = tile.x0 + threadIdx.x;
  if (x >= C.nx) return;
  stencil_fp32(C, x, tile.y0, min(tile.y0 + rows, C.ny), rk);
}

// ------------------------------------------------------------------- Poisson
// The column DFTs run the radix-8 Stockham FFT (fft_stockham.cuh, 8 values
// per thread) where the block's threads cover the column group that way, the
// radix-2/4 stages otherwise (the block size is set by the largest case of
// the batch)
__device__ __forceinline__ bool stockham8(int M, int nc) { return M >= 8 && nc * M <= 8 * (int)blockDim.x; }

// FP64 divergence of the FP32 predicted velocity (src/fluid/compute_potential.c:74-86)
// and the forward real DFT along y of `fcols` columns.
// the block's column group x0 .. x0+fcols-1 (every thread of the block)
__device__ __forceinline__ void fwd_cols(const BCase &C, int x0, int rk, double2 *zs) {
  const int nx = C.nx, ny = C.ny, M = ny / 2, nc = C.fcols;
  const int pu = C.par ^ (rk & 1) ^ 1;
  const float *__restrict__ ux = C.ux[pu];
  const float *__restrict__ uy = C.uy[pu];
  const float *__restrict__ uxl = C.uxl[pu];
  const float *__restrict__ uyl = C.uyl[pu];
  const double rgdt = C.rgdt[rk], rdy = C.rdy;
  const F2 rg2 = ff(rgdt);
  double *zd = reinterpret_cast<double *>(zs);
  const bool s8 = stockham8(M, nc);
  for (int e = threadIdx.x; e < nc * ny; e += blockDim.x) {
    const int c = e % nc, y = e / nc, x = x0 + c;
    double d = 0.0;
    if (x < nx) {
      const size_t r = (size_t)y * nx + x;
      const size_t ry = (size_t)wup(y, ny) * nx + x;
      if (C.x2) {  // float-float on the FP32 pipes, one conversion pair at the end
        const F2 u0{ux[r], uxl[r]};
        const F2 dux = x == nx - 1 ? -u0 : F2{ux[r + 1], uxl[r + 1]} - u0;
        const F2 duy = F2{uy[ry], uyl[ry]} - F2{uy[r], uyl[r]};
        const F2 v = (dux * F2{C.rdxf_f[x], C.rdxf_l[x]} + duy * F2{C.rdy_f, C.rdy_l}) * rg2;
        d = (double)v.h + (double)v.l;
      } else {
        const float dux = x == nx - 1 ? -(ux[r] + uxl[r]) : (ux[r + 1] - ux[r]) + (uxl[r + 1] - uxl[r]);
        const float duy = (uy[ry] - uy[r]) + (uyl[ry] - uyl[r]);
        d = rgdt * ((double)dux * C.rdxf[x] + (double)duy * rdy);
      }
    }
    const int m = y >> 1;
    zd[2 * (c * M + (s8 ? fft8::swz(m) : fft::fft_slot(m, M, C.fft_nst, C.fft_first2))) + (y & 1)] = d;
  }
  __syncthreads();
  const double2 *tw = reinterpret_cast<const double2 *>(C.tw);
  if (s8) {
    fft8::transform<true, 1>(zs, nc, M, tw);
  } else {
    fft::fft_stages<true>(zs, nc, M, ny, C.fft_nst, C.fft_first2, tw);
  }
  const int half = M / 2 + 1;
  for (int e = threadIdx.x; e < nc * half; e += blockDim.x) {
    const int c = e % nc, k = e / nc, x = x0 + c;
    if (x >= nx) continue;
    if (s8) {
      fft8::rfft_post(zs + c * M, C.spec + x, M, k, tw, (size_t)nx);
    } else {
      fft::rfft_post(zs + c * M, C.spec + x, M, k, tw, (size_t)nx);
    }
  }
}

__global__ void __launch_bounds__(256) k_b_fwd(const BCase *__restrict__ cases, const BCols *__restrict__ cols,
                                               int rk) {
  extern __shared__ double2 zs[];
  const BCols it = cols[blockIdx.x];
  const BCase &C = cases[it.c];
  if (C.done) return;
  fwd_cols(C, it.x0, rk, zs);
}

// inverse DFT and 1/jtot (src/fluid/compute_potential.c:146-157)
__device__ __forceinline__ void bwd_cols(const BCase &C, int x0, double2 *zs) {
  const int nx = C.nx, ny = C.ny, M = ny / 2, nc = C.fcols;
  const double2 *tw = reinterpret_cast<const double2 *>(C.tw);
  const bool s8 = stockham8(M, nc);
  const int half = M / 2 + 1;
  for (int e = threadIdx.x; e < nc * half; e += blockDim.x) {
    const int c = e % nc, k = e / nc, x = x0 + c;
    double2 *zc = zs + c * M;
    if (x >= nx) {
      zc[s8 ? fft8::swz(k) : fft::fft_slot(k, M, C.fft_nst, C.fft_first2)] = make_double2(0.0, 0.0);
      if (k > 0) zc[s8 ? fft8::swz(M - k) : fft::fft_slot(M - k, M, C.fft_nst, C.fft_first2)] = make_double2(0.0, 0.0);
      continue;
    }
    if (s8) {
      fft8::rfft_pre(C.spec + x, zc, M, k, tw, (size_t)nx);
    } else {
      fft::rfft_pre(C.spec + x, zc, M, k, tw, C.fft_nst, C.fft_first2, (size_t)nx);
    }
  }
  __syncthreads();
  if (s8) {
    fft8::transform<false, 1>(zs, nc, M, tw);
  } else {
    fft::fft_stages<false>(zs, nc, M, ny, C.fft_nst, C.fft_first2, tw);
  }
  const double *zd = reinterpret_cast<const double *>(zs);
  const double rny = 1.0 / ny;
  for (int e = threadIdx.x; e < nc * ny; e += blockDim.x) {
    const int c = e % nc, y = e / nc, x = x0 + c;
    const int m = y >> 1;
    if (x < nx) C.psi[(size_t)y * nx + x] = zd[2 * (c * M + (s8 ? fft8::swz(m) : m)) + (y & 1)] * rny;
  }
}

__global__ void __launch_bounds__(256) k_b_bwd(const BCase *__restrict__ cases, const BCols *__restrict__ cols) {
  extern __shared__ double2 zs[];
  const BCols it = cols[blockIdx.x];
  const BCase &C = cases[it.c];
  if (C.done) return;
  bwd_cols(C, it.x0, zs);
}

// Partition-method solve of the mode lines J = j0 .. j0+w-1 (one warp each).
// Per-mode factor block (doubles): inv[nx] up[nx] v[nx] w[nx] alpha[5][32]
// beta[5][32] rD[32]; rows are indexed by x. Each warp first moves its mode
// line (16 nx bytes) and factor block into shared memory with two bulk
// asynchronous copies (the TMA engine, completion on an mbarrier), solves
// there, and writes the line back with coalesced stores: the per-lane
// segment sweeps then read shared memory instead of scattered global lines.
// polls of the wait that lets a warp's copies land after its first wait gave
// up, so that no copy into the warp's shared memory outlives the warp
constexpr unsigned kTriDrainSpins = 1u << 22;

__device__ __forceinline__ unsigned smem_addr(const void *p) { return (unsigned)__cvta_generic_to_shared(p); }

__device__ __forceinline__ bool mbar_wait(unsigned bar, unsigned parity, unsigned spins) {
  for (unsigned k = 0; k < spins; ++k) {
    unsigned ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(bar), "r"(parity)
        : "memory");
    if (ok) return true;
  }
  return false;
}

// mode line J of case C by warp w of the block (its shared memory slot w)
__device__ __forceinline__ void tri_line(const BCase &C, int J, int w, unsigned char *tri_sm, int nmax, unsigned *err,
                                         unsigned spin, int stale) {
  const int lane = threadIdx.x & 31;
  const int n = C.nx, m = C.seg;
  const int s = lane * m, e = s + m - 1;
  double2 *gline = C.spec + (size_t)J * n;
  const size_t per_warp = 48 * (size_t)nmax + 8 * (2 * kPcrLevels * kSeg + kSeg);
  double2 *line = reinterpret_cast<double2 *>(tri_sm + 128 + (size_t)w * per_warp);
  double *f = reinterpret_cast<double *>(line + nmax);
  unsigned long long *bar = reinterpret_cast<unsigned long long *>(tri_sm) + w;
  const unsigned line_bytes = 16u * (unsigned)n, fac_bytes = 8u * (unsigned)C.pstride;
  __syncwarp();
  if (lane == 0) {
    // the slot's earlier generic reads and writes (a previous line, another
    // phase of a persistent launch) before the bulk copies write it
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    const unsigned b = smem_addr(bar);
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(b) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(b), "r"(line_bytes + fac_bytes)
                 : "memory");
  }
  if (lane == 0 && !stale) {
    const unsigned b = smem_addr(bar);
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     smem_addr(line)),
                 "l"(__cvta_generic_to_global(gline)), "r"(line_bytes), "r"(b)
                 : "memory");
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     smem_addr(f)),
                 "l"(__cvta_generic_to_global(C.pfac + (size_t)J * C.pstride)), "r"(fac_bytes), "r"(b)
                 : "memory");
  }
  __syncwarp();
  if (!mbar_wait(smem_addr(bar), 0, spin)) {
    if (lane == 0) atomicOr(err, 1u);
    // this line is left unsolved and the host reports the error, once the
    // copies issued into this warp's shared memory have landed
    if (!stale) mbar_wait(smem_addr(bar), 0, kTriDrainSpins);
    return;
  }
  const double *inv = f, *up = f + n, *vv = f + 2 * n, *ww = f + 3 * n;
  const double *alpha = f + 4 * n, *beta = alpha + kPcrLevels * kSeg, *rD = beta + kPcrLevels * kSeg;
  const double *lo = C.lo, *hi = C.hi;
  // 1) interior rows s..e-1 with zero boundary values: forward and back substitution
  double2 y = line[s];
  y.x *= inv[s];
  y.y *= inv[s];
  line[s] = y;
  for (int i = s + 1; i < e; ++i) {
    double2 r = line[i];
    const double a = lo[i], iv = inv[i];
    r.x = iv * fma(-a, y.x, r.x);
    r.y = iv * fma(-a, y.y, r.y);
    line[i] = r;
    y = r;
  }
  for (int i = e - 2; i >= s; --i) {
    double2 r = line[i];
    const double u = up[i];
    r.x = fma(-u, y.x, r.x);
    r.y = fma(-u, y.y, r.y);
    line[i] = r;
    y = r;
  }
  // y now holds the first interior value y_s; the last interior value y_{e-1}
  const double2 ylast = line[e - 1];
  // 2) reduced right-hand side of interface row e:
  //    R = r_e - a_e y_{e-1} - c_e y'_{s'} (y'_{s'} from the next lane)
  const double ynx = __shfl_down_sync(0xffffffffu, y.x, 1);
  const double yny = __shfl_down_sync(0xffffffffu, y.y, 1);
  const double2 re = line[e];
  const double ae = lo[e], ce = lane < kSeg - 1 ? hi[e] : 0.0;
  double Rx = re.x - ae * ylast.x - ce * (lane < kSeg - 1 ? ynx : 0.0);
  double Ry = re.y - ae * ylast.y - ce * (lane < kSeg - 1 ? yny : 0.0);
  if (J == 0 && lane == kSeg - 1) {  // singular mean mode: pin the last unknown to 0
    Rx = 0.0;
    Ry = 0.0;
  }
  // 3) parallel cyclic reduction over the 32 interface equations
#pragma unroll
  for (int lev = 0; lev < kPcrLevels; ++lev) {
    const int d = 1 << lev;
    const double mx = __shfl_up_sync(0xffffffffu, Rx, d), my = __shfl_up_sync(0xffffffffu, Ry, d);
    const double px = __shfl_down_sync(0xffffffffu, Rx, d), py = __shfl_down_sync(0xffffffffu, Ry, d);
    const double al = alpha[lev * kSeg + lane], be = beta[lev * kSeg + lane];
    const double lmx = lane >= d ? mx : 0.0, lmy = lane >= d ? my : 0.0;
    const double lpx = lane + d < kSeg ? px : 0.0, lpy = lane + d < kSeg ? py : 0.0;
    Rx = fma(be, lpx, fma(al, lmx, Rx));
    Ry = fma(be, lpy, fma(al, lmy, Ry));
  }
  const double xe_x = Rx * rD[lane], xe_y = Ry * rD[lane];
  line[e] = make_double2(xe_x, xe_y);
  // 4) interiors from the spikes: x_i = y_i + v_i x_{e(k-1)} + w_i x_{e(k)}
  const double xl_x = __shfl_up_sync(0xffffffffu, xe_x, 1), xl_y = __shfl_up_sync(0xffffffffu, xe_y, 1);
  const double lx_ = lane > 0 ? xl_x : 0.0, ly_ = lane > 0 ? xl_y : 0.0;
  for (int i = s; i < e; ++i) {
    double2 r = line[i];
    r.x = fma(ww[i], xe_x, fma(vv[i], lx_, r.x));
    r.y = fma(ww[i], xe_y, fma(vv[i], ly_, r.y));
    line[i] = r;
  }
  __syncwarp();
  for (int i = lane; i < n; i += 32) gline[i] = line[i];
  __syncwarp();  // the slot may take the next line
}

__global__ void __launch_bounds__(32 * kBModesPerBlockMax) k_b_tri(const BCase *__restrict__ cases,
                                                               const BModes *__restrict__ items, int nmax,
                                                               unsigned *err, unsigned spin, int stale) {
  extern __shared__ __align__(128) unsigned char tri_sm[];
  const BModes it = items[blockIdx.x];
  const BCase &C = cases[it.c];
  if (C.done) return;
  const int w = threadIdx.x >> 5;
  const int J = it.j0 + w;
  if (J >= C.nh) return;  // the whole warp
  tri_line(C, J, w, tri_sm, nmax, err, spin, stale);
}

// ---------------------------------------------------- correction and pressure
// correction and pressure of column tl.x0 + tx (tx < tile width); every lane
// of the warp calls it for the same tile (warp reductions at the end)
__device__ __forceinline__ void corr_col(BCase &C, const BTile tl, int tx, int rk, int rows) {
  const int nx = C.nx, ny = C.ny;
  const int x = tl.x0 + tx;
  const bool live = x < nx;
  float mx = 0.f, my = 0.f;
  bool nf = false;  // a NaN or infinity among the values written
  if (live) {
    const int y0 = tl.y0, y1 = min(y0 + rows, ny);
    const int pu = C.par ^ (rk & 1) ^ 1;
    float *__restrict__ ux = C.ux[pu];
    float *__restrict__ uy = C.uy[pu];
    float *__restrict__ uxl = C.uxl[pu];
    float *__restrict__ uyl = C.uyl[pu];
    const double *__restrict__ psi = C.psi;
    double *__restrict__ p = C.p;
    const double gdt = C.gdt[rk];
    const float rxc = C.rdxc_f[x], rdyf = C.rdy_f;
    // gamma dt / DXC and gamma dt / dy once per column: one FP64 product per
    // increment instead of two (the same value on grids whose spacings are
    // powers of two, where the division is an exact scaling)
    const double gx = gdt * C.dxi[x], gy = gdt * C.rdy;
    double sm = psi[(size_t)wdn(y0, ny) * nx + x];
    for (int y = y0; y < y1; ++y) {
      const size_t r = (size_t)y * nx + x;
      const double sc = psi[r];
      if (x >= 1) {  // src/fluid/correct_velocity.c:19-25
        float u, ul;
        const double du = -((sc - psi[r - 1]) * gx);
        if (C.x2) {
          const F2 w = F2{ux[r], uxl[r]} + ff(du);
          u = w.h;
          ul = w.l;
        } else {
          acc2(ux[r], uxl[r], (float)du, u, ul);
        }
        ux[r] = u;
        uxl[r] = ul;
        mx = fmaxf(mx, fabsf(u) * rxc);
        nf |= (__float_as_uint(u) & 0x7f800000u) == 0x7f800000u;
      }
      float v, vlo;
      const double dv = -((sc - sm) * gy);  // :31-37
      if (C.x2) {
        const F2 w = F2{uy[r], uyl[r]} + ff(dv);
        v = w.h;
        vlo = w.l;
      } else {
        acc2(uy[r], uyl[r], (float)dv, v, vlo);
      }
      uy[r] = v;
      uyl[r] = vlo;
      my = fmaxf(my, fabsf(v) * rdyf);
      const double pv = p[r] + sc;  // src/fluid/update_pressure.c:26-31
      p[r] = pv;
      nf |= ((__float_as_uint(v) & 0x7f800000u) == 0x7f800000u) |
            ((__double2hiint(pv) & 0x7ff00000) == 0x7ff00000);
      sm = sc;
    }
  }
  // a NaN or infinity written: the case is flagged (sticky) for the host
  if (__any_sync(0xffffffffu, nf) && (threadIdx.x & 31) == 0) atomicOr(&C.nonfinite, 1);
  if (rk == 2) {  // max |u|/dx for the next step's dt (src/param/decide_dt.c:35-50)
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
      mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, off));
      my = fmaxf(my, __shfl_xor_sync(0xffffffffu, my, off));
    }
    if ((threadIdx.x & 31) == 0) {
      atomicMax(&C.umax[0], __float_as_uint(mx));
      atomicMax(&C.umax[1], __float_as_uint(my));
    }
  }
}

__global__ void __launch_bounds__(kBTileXMax) k_b_corr(BCase *__restrict__ cases, const BTile *__restrict__ tiles,
                                                      int rk, int rows) {
  const BTile tl = tiles[blockIdx.x];
  BCase &C = cases[tl.c];
  if (C.done) return;
  corr_col(C, tl, threadIdx.x, rk, rows);
}

// ---------------------------------------------- one persistent launch per substage
// The five phases of a substage (stencils, forward DFT, tridiagonal, inverse
// DFT, correction) in one cooperative launch: every block of the grid is
// resident, walks each phase's work list with a grid stride, and the grid
// meets at a barrier between phases. The arithmetic per work item is that of
// the per-phase kernels above (the same device functions; with contraction
// on, the compiler may pair multiply-adds differently in this kernel, so FP32
// results agree to their rounding, not bit for bit). The barrier is a counter and a generation word in global
// memory; its wait is bounded: a block that gives up sets *err and goes on,
// so a launch always ends (the host then reports SNS_ERR_STATE).
constexpr unsigned kGridWaitSpins = 1u << 24;
// warps of a block that take mode lines in the tridiagonal phase: shared
// memory for four line slots leaves room for two blocks per SM
constexpr int kSubTriWarps = 4;

__device__ void grid_barrier(unsigned *count, unsigned *gen, unsigned *err) {
  __syncthreads();
  if (threadIdx.x == 0) {
    const unsigned g = *reinterpret_cast<volatile unsigned *>(gen);
    __threadfence();
    if (atomicAdd(count, 1u) == gridDim.x - 1) {
      atomicExch(count, 0u);
      __threadfence();
      atomicAdd(gen, 1u);
    } else {
      unsigned k = 0;
      while (*reinterpret_cast<volatile unsigned *>(gen) == g && ++k < kGridWaitSpins) {
      }
      if (k >= kGridWaitSpins) atomicOr(err, 2u);
    }
    __threadfence();
  }
  __syncthreads();
}

struct SubstageArgs {
  BCase *cases;
  const BTile *tiles;
  const BCols *cols;
  const BModes *modes;
  int ntiles, ntiles_x2, ncols, nmodes;
  int rk, tile_x, rows, mpb, nmax;
  unsigned *err;
  unsigned spin;
  unsigned *bar;  // [2]: arrival count, generation
};

__global__ void __launch_bounds__(256, 2) k_b_substage(const SubstageArgs a) {
  extern __shared__ __align__(128) unsigned char sm[];
  const int tid = threadIdx.x, nthr = blockDim.x;
  // 1) stencils: nthr / tile_x tiles per block at a time (FP32 tiles first,
  //    then compensated ones)
  {
    const int per = nthr / a.tile_x;
    for (int t0 = blockIdx.x * per; t0 < a.ntiles; t0 += gridDim.x * per) {
      const int t = t0 + tid / a.tile_x;
      if (t < a.ntiles) {
        const BTile tile = a.tiles[t];
        const BCase &C = a.cases[tile.c];
        const int x = tile.x0 + tid % a.tile_x;
        if (!C.done && x < C.nx) {
          const int y1 = min(tile.y0 + a.rows, C.ny);
          if (t >= a.ntiles - a.ntiles_x2) {
            stencil_x2(C, x, tile.y0, y1, a.rk);
          } else {
            stencil_fp32(C, x, tile.y0, y1, a.rk);
          }
        }
      }
    }
  }
  grid_barrier(a.bar, a.bar + 1, a.err);
  // 2) forward DFTs: one column group per block at a time
  double2 *zs = reinterpret_cast<double2 *>(sm);
  for (int i = blockIdx.x; i < a.ncols; i += gridDim.x) {
    const BCols it = a.cols[i];
    const BCase &C = a.cases[it.c];
    if (!C.done) fwd_cols(C, it.x0, a.rk, zs);
    __syncthreads();
  }
  grid_barrier(a.bar, a.bar + 1, a.err);
  // 3) tridiagonal: warps of the block take mode lines (mpb per work item)
  {
    const int w = tid >> 5;
    const int ipb = max(1, kSubTriWarps / a.mpb);
    for (int b0 = blockIdx.x * ipb; b0 < a.nmodes; b0 += gridDim.x * ipb) {
      const int item = b0 + w / a.mpb;
      if (w < ipb * a.mpb && item < a.nmodes) {
        const BModes it = a.modes[item];
        const BCase &C = a.cases[it.c];
        const int J = it.j0 + w % a.mpb;
        if (!C.done && J < C.nh) tri_line(C, J, w, sm, a.nmax, a.err, a.spin, 0);
      }
    }
  }
  grid_barrier(a.bar, a.bar + 1, a.err);
  // 4) inverse DFTs
  for (int i = blockIdx.x; i < a.ncols; i += gridDim.x) {
    const BCols it = a.cols[i];
    const BCase &C = a.cases[it.c];
    if (!C.done) bwd_cols(C, it.x0, zs);
    __syncthreads();
  }
  grid_barrier(a.bar, a.bar + 1, a.err);
  // 5) correction and pressure: whole warps per tile (tile_x is a multiple of 32)
  {
    const int per = nthr / a.tile_x;
    for (int t0 = blockIdx.x * per; t0 < a.ntiles; t0 += gridDim.x * per) {
      const int t = t0 + tid / a.tile_x;
      if (t < a.ntiles) {
        const BTile tile = a.tiles[t];
        BCase &C = a.cases[tile.c];
        if (!C.done) corr_col(C, tile, tid % a.tile_x, a.rk, a.rows);
      }
    }
  }
}

// end of a step for every case: step/time bookkeeping, buffer swap, done flag,
// dt of the next step (src/param/decide_dt.c:11-101, explicit scheme) and the
// RK scalars derived from it
struct RkCoefs {
  double a[3], b[3];
};

__global__ void k_b_dt(BCase *cases, int ncases, RkCoefs rk) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= ncases) return;
  BCase &C = cases[c];
  if (C.done) return;
  C.time += C.dt;
  C.step += 1;
  C.par ^= 1;
  if (C.target_steps > 0 && C.step >= C.target_steps) C.done = 1;
  const float ux_m = __uint_as_float(C.umax[0]), uy_m = __uint_as_float(C.umax[1]);
  C.umax[0] = 0u;
  C.umax[1] = 0u;
  double dt_adv = 5.e-2;
  if (ux_m > 0.f) dt_adv = fmin(dt_adv, 1.0 / (double)ux_m);
  if (uy_m > 0.f) dt_adv = fmin(dt_adv, 1.0 / (double)uy_m);
  dt_adv *= 0.7;
  double dt = fmin(dt_adv, C.dt_dif);
  if (C.fixed_dt > 0.0) dt = C.fixed_dt;
  C.dt = dt;
  for (int k = 0; k < 3; ++k) {
    C.adt[k] = rk.a[k] * dt;
    C.bdt[k] = rk.b[k] * dt;
    C.gdt[k] = (rk.a[k] + rk.b[k]) * dt;
    C.rgdt[k] = 1. / C.gdt[k];
  }
}

}  // namespace

// kernel attributes, set once outside any stream capture
cudaError_t batch_kernels_init() {
  cudaFuncSetAttribute(k_b_fwd, cudaFuncAttributeMaxDynamicSharedMemorySize, 160 * 1024);
  cudaFuncSetAttribute(k_b_bwd, cudaFuncAttributeMaxDynamicSharedMemorySize, 160 * 1024);
  cudaFuncSetAttribute(k_b_tri, cudaFuncAttributeMaxDynamicSharedMemorySize, 210 * 1024);
  return cudaGetLastError();
}

// the launch helpers below only enqueue: the graph replays are counted by sns_batch_step
cudaError_t launch_batch_stencil(const BCase *cases, const BTile *tiles, int ntiles, int ntiles_x2, int rk,
                                 int tile_x, int rows, cudaStream_t st) {
  const int nf = ntiles - ntiles_x2;
  if (nf > 0) {
    k_b_stencil<<<nf, tile_x, 0, st>>>(cases, tiles, rk, rows);
  }
  if (ntiles_x2 > 0) {
    k_b_stencil_x2<<<ntiles_x2, tile_x, 0, st>>>(cases, tiles + nf, rk, rows);
  }
  return cudaGetLastError();
}

cudaError_t launch_batch_fwd(const BCase *cases, const BCols *cols, int ncols, int rk, size_t smem, int threads,
                             cudaStream_t st) {
  if (ncols == 0) return cudaSuccess;
  k_b_fwd<<<ncols, threads, smem, st>>>(cases, cols, rk);
  return cudaGetLastError();
}

cudaError_t launch_batch_bwd(const BCase *cases, const BCols *cols, int ncols, size_t smem, int threads,
                             cudaStream_t st) {
  if (ncols == 0) return cudaSuccess;
  k_b_bwd<<<ncols, threads, smem, st>>>(cases, cols);
  return cudaGetLastError();
}

size_t batch_tri_smem(int nmax, int modes_per_block) {
  return 128 + (size_t)modes_per_block * (48 * (size_t)nmax + 8 * (2 * kPcrLevels * kSeg + kSeg));
}

cudaError_t launch_batch_tri(const BCase *cases, const BModes *modes, int nmodes, int modes_per_block, int nmax,
                             unsigned *err, unsigned spin, int stale, cudaStream_t st) {
  if (nmodes == 0) return cudaSuccess;
  k_b_tri<<<nmodes, 32 * modes_per_block, batch_tri_smem(nmax, modes_per_block), st>>>(cases, modes, nmax, err, spin,
                                                                                      stale);
  return cudaGetLastError();
}

// shared memory of the persistent substage launch: the larger of the FFT
// phases' column groups and the tridiagonal phase's line slots
size_t batch_substage_smem(size_t fft_smem, int nmax, int mpb) {
  const int slots = std::max(1, kSubTriWarps / mpb) * mpb;
  return std::max(fft_smem, 128 + (size_t)slots * (48 * (size_t)nmax + 8 * (2 * kPcrLevels * kSeg + kSeg)));
}

cudaError_t launch_batch_substage(BCase *cases, const BTile *tiles, int ntiles, int ntiles_x2, const BCols *cols,
                                  int ncols, const BModes *modes, int nmodes, int rk, int tile_x, int rows, int mpb,
                                  int nmax, size_t smem, unsigned *err, unsigned spin, unsigned *bar, int blocks,
                                  cudaStream_t st) {
  SubstageArgs a{cases, tiles, cols, modes, ntiles, ntiles_x2, ncols, nmodes, rk, tile_x, rows, mpb, nmax,
                 err, spin, bar};
  void *args[] = {&a};
  return cudaLaunchCooperativeKernel((const void *)k_b_substage, dim3(blocks), dim3(256), args, smem, st);
}

int batch_substage_blocks(size_t smem) {
  int dev = 0, sms = 0, per = 0, coop = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) ||
      cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev) || !coop)
    return 0;
  if (cudaFuncSetAttribute(k_b_substage, cudaFuncAttributeMaxDynamicSharedMemorySize, 220 * 1024) != cudaSuccess)
    return 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_b_substage, 256, smem) != cudaSuccess) return 0;
  return per * sms;
}

cudaError_t launch_batch_corr(const BCase *cases, const BTile *tiles, int ntiles, int rk, int tile_x, int rows,
                              cudaStream_t st) {
  if (ntiles == 0) return cudaSuccess;
  k_b_corr<<<ntiles, tile_x, 0, st>>>(const_cast<BCase *>(cases), tiles, rk, rows);
  return cudaGetLastError();
}

cudaError_t launch_batch_dt(BCase *cases, int ncases, const double *rk_a, const double *rk_b, cudaStream_t st) {
  if (ncases == 0) return cudaSuccess;
  RkCoefs rk;
  for (int k = 0; k < 3; ++k) {
    rk.a[k] = rk_a[k];
    rk.b[k] = rk_b[k];
  }
  k_b_dt<<<(ncases + 127) / 128, 128, 0, st>>>(cases, ncases, rk);
  return cudaGetLastError();
}

}  // namespace sns
