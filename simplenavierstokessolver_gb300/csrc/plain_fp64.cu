// Plain FP64 path of the SMR-RK3 step on GB300 (sm_103a).
//
// Compiled with --fmad=false: every expression below is evaluated with the
// same IEEE binary64 operations, in the same order, as the reference's C
// (cited per kernel), so results are bit-identical to it. Divisions by grid
// spacings become multiplications by exact reciprocals only when every such
// spacing is a power of two (DevGrid::rcp), where both give the same
// correctly rounded result.
//
// On GB300 the FP64 pipe (~0.5 Tops/s) rather than HBM bounds this path, so
// the kernels minimise FP64 instructions: y-face quantities are carried from
// row to row by each thread, RHS-independent Thomas factors are precomputed,
// and the implicit-source terms (exactly zero in the explicit scheme) are not
// evaluated.
#include <algorithm>
#include <cfloat>
#include <cstdint>
#include <type_traits>

#include "fft_dev.cuh"
#include "sns_internal.h"

// plain_fp64_contract.cu compiles this file a second time, with fused
// multiply-add contraction, into namespace sns::contract (the parallel form)
#ifdef SNS_PLAIN_CONTRACT
#define SNS_PLAIN_FORM contract
#else
#define SNS_PLAIN_FORM exact
#endif

namespace sns {
#ifdef SNS_PLAIN_CONTRACT
namespace contract {
#else
inline namespace exact {
#endif
namespace {

template <bool RCP>
__device__ __forceinline__ double dv(double a, double d, double rd) {
  if constexpr (RCP) {
    return a * rd;
  } else {
    return a / d;
  }
}

__device__ __forceinline__ int wrap_up(int y, int ny) { return y + 1 == ny ? 0 : y + 1; }
__device__ __forceinline__ int wrap_dn(int y, int ny) { return y == 0 ? ny - 1 : y - 1; }

constexpr int kRows = 8;     // rows marched by one thread in the stencil kernels
constexpr int kBlockX = 64;  // columns per block: ~6-7 blocks per SM at 512 x 1024 for load balance

// ------------------------------------------------- exact power-of-two products
// x * 2^e is exact when x and the product are normal numbers, or x is zero,
// and then equals x with its exponent field moved by e. GB300 issues FP64
// instructions at a small fraction of its integer rate, so on grids whose
// spacings are powers of two (DevGrid::p2: the reciprocal spacings and the
// advective coefficients are then powers of two too) the velocity,
// temperature and correction kernels take those products, and the 1/2 of
// every interpolation, in the integer unit. An operand other than zero whose exponent field lies outside
// [1 + kP2Margin, 0x7fe - kP2Margin] (magnitude below 2^-958 or from 2^958 up,
// subnormals, infinities, NaN), where the moved field could leave the normal
// range, clears the row's flag and the row is recomputed with FP64 products.
constexpr unsigned kP2Margin = 64;  // largest |e| taken this way (checked on the host)
constexpr unsigned kP2Lo = (1u + kP2Margin) << 20;
constexpr unsigned kP2Span = (0x7feu - 2u * kP2Margin) << 20;

// c == 2^e: e in the position of the exponent field of the high word
__device__ __forceinline__ int p2_field(double c) { return (((__double2hiint(c) >> 20) & 0x7ff) - 1023) * (1 << 20); }

template <bool FAST>
struct Mul {
  bool ok = true;
  // x * c where c == 2^e and E == p2_field(c)
  __device__ __forceinline__ double by(double x, double c, int E) {
    if constexpr (FAST) {
      const int hi = __double2hiint(x), lo = __double2loint(x);
      const unsigned m = (unsigned)hi & 0x7fffffffu;
      const bool zero = (m | (unsigned)lo) == 0u;
      ok &= zero | (m - kP2Lo < kP2Span);
      return __hiloint2double(zero ? hi : hi + E, lo);
    } else {
      return x * c;
    }
  }
  __device__ __forceinline__ double half(double x) { return by(x, 0.5, -(1 << 20)); }
};

// ---------------------------------------------------------------- temperature
struct TempArgs {
  DevGrid g;
  StageScalars s;
  const double *t_in;
  double *t_out, *at, *qt;
  const double *ux, *uy;
};

// one row of the temperature update: tc = T(x, y), gym, pym the y-face
// terms between rows y-1 and y; tp, tl, tr, uyp, uxm, uxp this row's loads
struct TempRow {
  double A, q, gyp, pyp;
};

template <int IMPX, int IMPY, bool RCP, bool FAST>
__device__ __forceinline__ bool temp_row(const TempArgs &a, double tc, double gym, double pym, double tp, double tl,
                                         double tr, double uyp, double uxm, double uxp, double atr, double dcm,
                                         double dcp, double df, double rcm, double rcp, double rf, double cm,
                                         double cp, const int *e, TempRow &o) {
  Mul<FAST> m;
  const double dy = a.g.dy, rdy = a.g.rdy, kappa = a.s.kappa;
  auto D = [&](double v, double d, double rd, int E) {
    if constexpr (FAST) {
      return m.by(v, rd, E);
    } else {
      return dv<RCP>(v, d, rd);
    }
  };
  auto Cf = [&](double c, double v, int E) {
    if constexpr (FAST) {
      return m.by(v, c, E);
    } else {
      return c * v;
    }
  };
  // e: exponents of rcm, rcp, rdy, rf, cm, cp
  const double gxm = D(tc - tl, dcm, rcm, e[0]);
  const double gxp = D(tr - tc, dcp, rcp, e[1]);
  const double gyp = D(tp - tc, dy, rdy, e[2]);
  const double pyp = m.half(uyp) * gyp;
  const double adv1 = -(Cf(cm, uxm, e[4]) * gxm) - (Cf(cp, uxp, e[5]) * gxp);
  const double adv2 = -pym - pyp;
  const double dif1 = D(kappa * (gxp - gxm), df, rf, e[3]);
  const double dif2 = D(kappa * (gyp - gym), dy, rdy, e[2]);
  double A = adv1 + adv2;
  if (!IMPX) A = A + dif1;
  if (!IMPY) A = A + dif2;
  double q = a.s.adt * A;
  if (a.s.has_b) q = q + a.s.bdt * atr;
  if (IMPX || IMPY) {
    const double G = (IMPX && IMPY) ? dif1 + dif2 : (IMPX ? dif1 : dif2);
    q = q + a.s.gdt * G;
  }
  o.A = A;
  o.q = q;
  o.gyp = gyp;
  o.pyp = pyp;
  return m.ok;
}

// src/temperature/update.c:11-87 (sources) and :114-122, :221-226 (RK3 update)
// for column x, rows y0 .. y0+kRows-1. FAST: the products by powers of two in
// the integer unit, a row outside their range recomputed with FP64 products.
template <int IMPX, int IMPY, bool RCP, bool FAST>
__device__ __forceinline__ void temp_column(const TempArgs &a, int x, int y0) {
  const int nx = a.g.nx, ny = a.g.ny;
  const int y1 = min(y0 + kRows, ny);
  const double *T = a.t_in;
  const double dcm = a.g.dxc[x], dcp = a.g.dxc[x + 1], df = a.g.dxf[x];
  const double rcm = a.g.rdxc[x], rcp = a.g.rdxc[x + 1], rf = a.g.rdxf[x];
  const double cm = a.g.c_cm[x], cp = a.g.c_cp[x];
  const double dy = a.g.dy, rdy = a.g.rdy;
  int e[6] = {0, 0, 0, 0, 0, 0};
  if constexpr (FAST) {
    e[0] = p2_field(rcm);
    e[1] = p2_field(rcp);
    e[2] = p2_field(rdy);
    e[3] = p2_field(rf);
    e[4] = p2_field(cm);
    e[5] = p2_field(cp);
  }
  const bool left = x == 0, right = x == nx - 1;
  double tc = T[(size_t)y0 * nx + x];
  // y-face between rows y0-1 and y0 (periodic halo, src/temperature/boundary_conditions.c:13-14)
  double gym = dv<RCP>(tc - T[(size_t)wrap_dn(y0, ny) * nx + x], dy, rdy);
  double pym = (0.5 * a.uy[(size_t)y0 * nx + x]) * gym;
  for (int y = y0; y < y1; ++y) {
    const int yp = wrap_up(y, ny);
    const size_t r = (size_t)y * nx + x;
    const double tp = T[(size_t)yp * nx + x];
    const double tl = left ? kTempXm : T[r - 1];
    const double tr = right ? kTempXp : T[r + 1];
    const double uyp = a.uy[(size_t)yp * nx + x];
    const double uxm = a.ux[r];
    const double uxp = right ? 0.0 : a.ux[r + 1];
    const double atr = a.s.has_b ? a.at[r] : 0.0;
    TempRow o;
    if constexpr (FAST) {
      if (!temp_row<IMPX, IMPY, RCP, true>(a, tc, gym, pym, tp, tl, tr, uyp, uxm, uxp, atr, dcm, dcp, df, rcm, rcp, rf,
                                           cm, cp, e, o))
        temp_row<IMPX, IMPY, RCP, false>(a, tc, gym, pym, tp, tl, tr, uyp, uxm, uxp, atr, dcm, dcp, df, rcm, rcp, rf,
                                         cm, cp, e, o);
    } else {
      temp_row<IMPX, IMPY, RCP, false>(a, tc, gym, pym, tp, tl, tr, uyp, uxm, uxp, atr, dcm, dcp, df, rcm, rcp, rf, cm,
                                       cp, e, o);
    }
    a.at[r] = o.A;
    if (IMPX || IMPY) {
      a.qt[r] = o.q;
    } else {
      a.t_out[r] = tc + o.q;
    }
    tc = tp;
    gym = o.gyp;
    pym = o.pyp;
  }
}

template <int IMPX, int IMPY, bool RCP, bool FAST>
__global__ void __launch_bounds__(128) k_temp(const TempArgs a) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  if (x >= a.g.nx) return;
  temp_column<IMPX, IMPY, RCP, FAST>(a, x, blockIdx.y * kRows);
}

// ------------------------------------------------------------------ velocity
struct VelArgs {
  DevGrid g;
  StageScalars s;
  const double *ux, *uy, *p, *tf;  // tf: temperature the buoyancy is taken from (nullptr: none)
  double *ux_out, *uy_out, *aux, *auy, *qx, *qy;
};

// metrics of column x: ux at i = x+1 (DXF(i-1), DXF(i), DXC(i)), uy at
// i = x+1 (DXC(i), DXC(i+1), DXF(i)), with the exponents of the power-of-two
// factors when they are taken in the integer unit
struct VelCol {
  double uf_m, uf_p, uc_c, ruf_m, ruf_p, ruc_c, fm, fp;
  double vc_m, vc_p, vf_c, rvc_m, rvc_p, rvf_c, cm, cp;
  int e_ruf_m, e_ruf_p, e_ruc_c, e_fm, e_fp, e_rvc_m, e_rvc_p, e_rvf_c, e_cm, e_cp, e_rdy;
};

// one row: the values carried from the row below, and this row's loads
struct VelIn {
  double u0, u1, um0, um1, v0, vl, pm;  // ux(x+1..x+2, y), ux(.., y-1), uy(x+1, y), uy(x, y), p(x+1, y-1)
  double gym_u, pym_u, gym_v, pym_v;    // y-face terms between rows y-1 and y
  double u0n, u1n, v0n, vln, vr, pc, ul, pl, tfl, tfr, aux, auy;
};

struct VelOut {
  double ux, ax, qx, uy, ay, qy;
  double gym_u, pym_u, gym_v, pym_v;
};

// src/fluid/update_velocity.c:11-104 (ux sources), :106-192 (uy sources),
// :219-230 / :371-381 (RK3 increments) and :436-441 / :580-585 (update), for
// one row of column x. Returns false when a FAST product was out of range.
template <int IMPX, int IMPY, bool RCP, bool FAST>
__device__ __forceinline__ bool vel_row(const VelArgs &a, const VelCol &k, const VelIn &in, bool has_ux,
                                        VelOut &o) {
  Mul<FAST> m;
  const double dy = a.g.dy, rdy = a.g.rdy, nu = a.s.nu;
  // difference / spacing
  auto D = [&](double v, double d, double rd, int E) {
    if constexpr (FAST) {
      return m.by(v, rd, E);
    } else {
      return dv<RCP>(v, d, rd);
    }
  };
  // coefficient * value
  auto C = [&](double c, double v, int E) {
    if constexpr (FAST) {
      return m.by(v, c, E);
    } else {
      return c * v;
    }
  };
  o.gym_u = in.gym_u;
  o.pym_u = in.pym_u;
  // ---- ux(i, j), i = x+1 >= 2
  if (has_ux) {
    const double gxm = D(in.u0 - in.ul, k.uf_m, k.ruf_m, k.e_ruf_m);
    const double gxp = D(in.u1 - in.u0, k.uf_p, k.ruf_p, k.e_ruf_p);
    const double gyp = D(in.u0n - in.u0, dy, rdy, k.e_rdy);
    const double vxm = m.half(in.ul) + m.half(in.u0);
    const double vxp = m.half(in.u0) + m.half(in.u1);
    const double adv1 = -(C(k.fm, vxm, k.e_fm) * gxm) - (C(k.fp, vxp, k.e_fp) * gxp);
    const double pyp = m.half(C(k.fm, in.vln, k.e_fm) + C(k.fp, in.v0n, k.e_fp)) * gyp;
    const double adv2 = -in.pym_u - pyp;
    const double dif1 = D(nu * (gxp - gxm), k.uc_c, k.ruc_c, k.e_ruc_c);
    const double dif2 = D(nu * (gyp - in.gym_u), dy, rdy, k.e_rdy);
    const double pre = -D(in.pc - in.pl, k.uc_c, k.ruc_c, k.e_ruc_c);
    double A = adv1 + adv2;
    if (!IMPX) A = A + dif1;
    if (!IMPY) A = A + dif2;
    if (a.tf) A = A + (m.half(in.tfl) + m.half(in.tfr));
    double G;
    if (IMPX && IMPY) {
      G = (dif1 + dif2) + pre;
    } else if (IMPX) {
      G = dif1 + pre;
    } else if (IMPY) {
      G = dif2 + pre;
    } else {
      G = pre;
    }
    double q = a.s.adt * A;
    if (a.s.has_b) q = q + a.s.bdt * in.aux;
    q = q + a.s.gdt * G;
    o.ax = A;
    o.qx = q;
    o.ux = in.u0 + q;
    o.gym_u = gyp;
    o.pym_u = pyp;
  }
  // ---- uy(i, j), i = x+1 >= 1
  {
    const double gxm = D(in.v0 - in.vl, k.vc_m, k.rvc_m, k.e_rvc_m);
    const double gxp = D(in.vr - in.v0, k.vc_p, k.rvc_p, k.e_rvc_p);
    const double gyp = D(in.v0n - in.v0, dy, rdy, k.e_rdy);
    const double wxm = m.half(in.um0) + m.half(in.u0);
    const double wxp = m.half(in.um1) + m.half(in.u1);
    const double adv1 = -(C(k.cm, wxm, k.e_cm) * gxm) - (C(k.cp, wxp, k.e_cp) * gxp);
    const double pyp = m.half(m.half(in.v0) + m.half(in.v0n)) * gyp;
    const double adv2 = -in.pym_v - pyp;
    const double dif1 = D(nu * (gxp - gxm), k.vf_c, k.rvf_c, k.e_rvf_c);
    const double dif2 = D(nu * (gyp - in.gym_v), dy, rdy, k.e_rdy);
    const double pre = -D(in.pc - in.pm, dy, rdy, k.e_rdy);
    double A = adv1 + adv2;
    if (!IMPX) A = A + dif1;
    if (!IMPY) A = A + dif2;
    double G;
    if (IMPX && IMPY) {
      G = (dif1 + dif2) + pre;
    } else if (IMPX) {
      G = dif1 + pre;
    } else if (IMPY) {
      G = dif2 + pre;
    } else {
      G = pre;
    }
    double q = a.s.adt * A;
    if (a.s.has_b) q = q + a.s.bdt * in.auy;
    q = q + a.s.gdt * G;
    o.ay = A;
    o.qy = q;
    o.uy = in.v0 + q;
    o.gym_v = gyp;
    o.pym_v = pyp;
  }
  return m.ok;
}

template <int IMPX, int IMPY, bool RCP, bool FAST>
__global__ void __launch_bounds__(128) k_vel(const VelArgs a) {
  const int nx = a.g.nx, ny = a.g.ny;
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  if (x >= nx) return;
  const int y0 = blockIdx.y * kRows;
  const int y1 = min(y0 + kRows, ny);
  const bool left = x == 0, right = x == nx - 1;
  const bool has_ux = x >= 1;  // ux is updated for i = 2..itot
  const double dy = a.g.dy, rdy = a.g.rdy;
  VelCol k;
  k.uf_m = has_ux ? a.g.dxf[x - 1] : 1.0;
  k.uf_p = a.g.dxf[x];
  k.uc_c = a.g.dxc[x];
  k.ruf_m = has_ux ? a.g.rdxf[x - 1] : 1.0;
  k.ruf_p = a.g.rdxf[x];
  k.ruc_c = a.g.rdxc[x];
  k.fm = a.g.c_fm[x];
  k.fp = a.g.c_fp[x];
  k.vc_m = a.g.dxc[x];
  k.vc_p = a.g.dxc[x + 1];
  k.vf_c = a.g.dxf[x];
  k.rvc_m = a.g.rdxc[x];
  k.rvc_p = a.g.rdxc[x + 1];
  k.rvf_c = a.g.rdxf[x];
  k.cm = a.g.c_cm[x];
  k.cp = a.g.c_cp[x];
  if constexpr (FAST) {
    k.e_ruf_m = p2_field(k.ruf_m);
    k.e_ruf_p = p2_field(k.ruf_p);
    k.e_ruc_c = p2_field(k.ruc_c);
    k.e_fm = p2_field(k.fm);
    k.e_fp = p2_field(k.fp);
    k.e_rvc_m = p2_field(k.rvc_m);
    k.e_rvc_p = p2_field(k.rvc_p);
    k.e_rvf_c = p2_field(k.rvf_c);
    k.e_cm = p2_field(k.cm);
    k.e_cp = p2_field(k.cp);
    k.e_rdy = p2_field(rdy);
  } else {
    k.e_ruf_m = k.e_ruf_p = k.e_ruc_c = k.e_fm = k.e_fp = k.e_rvc_m = k.e_rvc_p = k.e_rvf_c = k.e_cm = k.e_cp =
        k.e_rdy = 0;
  }
  const double *ux = a.ux, *uy = a.uy, *p = a.p;

  VelIn in;
  const int ym = wrap_dn(y0, ny);
  const size_t r0 = (size_t)y0 * nx + x, rm = (size_t)ym * nx + x;
  in.u0 = ux[r0];
  in.u1 = right ? 0.0 : ux[r0 + 1];
  in.um0 = ux[rm];
  in.um1 = right ? 0.0 : ux[rm + 1];
  in.v0 = uy[r0];
  in.vl = left ? 0.0 : uy[r0 - 1];
  in.pm = p[rm];
  // y-faces between rows y0-1 and y0
  in.gym_u = dv<RCP>(in.u0 - in.um0, dy, rdy);
  in.pym_u = 0.0;
  if (has_ux) in.pym_u = (0.5 * (k.fm * in.vl + k.fp * in.v0)) * in.gym_u;
  const double vm = uy[rm];
  in.gym_v = dv<RCP>(in.v0 - vm, dy, rdy);
  in.pym_v = (0.5 * (0.5 * vm + 0.5 * in.v0)) * in.gym_v;
  in.ul = in.pl = in.tfl = in.tfr = in.aux = in.auy = 0.0;

  for (int y = y0; y < y1; ++y) {
    const int yp = wrap_up(y, ny);
    const size_t r = (size_t)y * nx + x, rp = (size_t)yp * nx + x;
    in.u0n = ux[rp];
    in.u1n = right ? 0.0 : ux[rp + 1];
    in.v0n = uy[rp];
    in.vln = left ? 0.0 : uy[rp - 1];
    in.vr = right ? 0.0 : uy[r + 1];
    in.pc = p[r];
    if (has_ux) {
      in.ul = ux[r - 1];
      in.pl = p[r - 1];
      if (a.tf) {
        in.tfl = a.tf[r - 1];
        in.tfr = a.tf[r];
      }
      if (a.s.has_b) in.aux = a.aux[r];
    }
    if (a.s.has_b) in.auy = a.auy[r];
    VelOut o;
    if constexpr (FAST) {
      if (!vel_row<IMPX, IMPY, RCP, true>(a, k, in, has_ux, o)) vel_row<IMPX, IMPY, RCP, false>(a, k, in, has_ux, o);
    } else {
      vel_row<IMPX, IMPY, RCP, false>(a, k, in, has_ux, o);
    }
    if (has_ux) {
      a.aux[r] = o.ax;
      if (IMPX || IMPY) {
        a.qx[r] = o.qx;
      } else {
        a.ux_out[r] = o.ux;
      }
    }
    a.auy[r] = o.ay;
    if (IMPX || IMPY) {
      a.qy[r] = o.qy;
    } else {
      a.uy_out[r] = o.uy;
    }
    in.gym_u = o.gym_u;
    in.pym_u = o.pym_u;
    in.gym_v = o.gym_v;
    in.pym_v = o.pym_v;
    in.um0 = in.u0;
    in.um1 = in.u1;
    in.u0 = in.u0n;
    in.u1 = in.u1n;
    in.v0 = in.v0n;
    in.vl = in.vln;
    in.pm = in.pc;
  }
}

// ------------------------------------------------------- line recurrences
// The recurrences below read each element once, in order, from memory that
// only the same thread writes: the next chunk of kLineChunk elements (and
// their factors, uniform across the warp) is loaded into registers while the
// current chunk is eliminated, so the loads stay off the dependent chain.
constexpr int kLineChunk = 8;
// elements per chunk of the row-wise solve along x: its lanes walk 32
// different rows, so every load touches 32 cache lines and the prefetch
// distance sets the pace (2048 x 4096: chunks of 8 / 10 / 16 take 1015 /
// 585 / 547 us per launch, 12 to 20 alike); the column-wise solve along y is
// coalesced and fastest with kLineChunk
constexpr int kSolveXChunk = 16;
// elements per chunk of the periodic solve's final pass (no recurrence: the
// next chunk's loads are issued before the current chunk's stores)
constexpr int kFixChunk = 16;

__device__ __forceinline__ bool is_zero_bits(double v) { return (__double_as_longlong(v) << 1) == 0; }

// forward elimination (src/linalg.c:14-23) over e = e0..e1-1 with element
// stride s; prev is the eliminated value at e0-1. Returns the value at e1-1.
template <int CH>
__device__ __forceinline__ double line_forward(double *q, size_t s, const double *inv, const double *l, int e0, int e1,
                                               double prev) {
  double cq[CH], ci[CH], cl[CH];
#pragma unroll
  for (int k = 0; k < CH; ++k) {
    const int e = e0 + k;
    cq[k] = e < e1 ? q[(size_t)e * s] : 0.0;
    ci[k] = e < e1 ? __ldg(inv + e) : 0.0;
    cl[k] = e < e1 ? __ldg(l + e) : 0.0;
  }
#pragma unroll 1
  for (int b = e0; b < e1; b += CH) {
    double nq[CH], ni[CH], nl[CH];
#pragma unroll
    for (int k = 0; k < CH; ++k) {
      const int e = b + CH + k;
      nq[k] = e < e1 ? q[(size_t)e * s] : 0.0;
      ni[k] = e < e1 ? __ldg(inv + e) : 0.0;
      nl[k] = e < e1 ? __ldg(l + e) : 0.0;
    }
#pragma unroll
    for (int k = 0; k < CH; ++k) {
      const int e = b + k;
      if (e < e1) {
        const double v = is_zero_bits(ci[k]) ? 0.0 : ci[k] * (cq[k] - cl[k] * prev);
        q[(size_t)e * s] = v;
        prev = v;
      }
    }
#pragma unroll
    for (int k = 0; k < CH; ++k) {
      cq[k] = nq[k];
      ci[k] = ni[k];
      cl[k] = nl[k];
    }
  }
  return prev;
}

// back substitution (src/linalg.c:25-27) over e = hi down to lo; next is the
// value at hi+1.
template <int CH>
__device__ __forceinline__ void line_backward(double *q, size_t s, const double *up, int hi, int lo, double next) {
  double cq[CH], cu[CH];
#pragma unroll
  for (int k = 0; k < CH; ++k) {
    const int e = hi - k;
    cq[k] = e >= lo ? q[(size_t)e * s] : 0.0;
    cu[k] = e >= lo ? __ldg(up + e) : 0.0;
  }
#pragma unroll 1
  for (int b = hi; b >= lo; b -= CH) {
    double nq[CH], nu[CH];
#pragma unroll
    for (int k = 0; k < CH; ++k) {
      const int e = b - CH - k;
      nq[k] = e >= lo ? q[(size_t)e * s] : 0.0;
      nu[k] = e >= lo ? __ldg(up + e) : 0.0;
    }
#pragma unroll
    for (int k = 0; k < CH; ++k) {
      const int e = b - k;
      if (e >= lo) {
        const double v = cq[k] - cu[k] * next;
        q[(size_t)e * s] = v;
        next = v;
      }
    }
#pragma unroll
    for (int k = 0; k < CH; ++k) {
      cq[k] = nq[k];
      cu[k] = nu[k];
    }
  }
}

// ------------------------------------------------------- Crank-Nicolson solves
// src/linalg.c:9-30 applied per row along x; factors are shared by all rows.
// mode 0: rows x = 0..nx-1, first row divides by d0 (T: update.c:150-157, uy:
//         update_velocity.c:509-516)
// mode 1: ux rows x = 1..nx-1 of the (itot+1)-system whose rows 0 and itot are
//         identity rows with zero right-hand side (update_velocity.c:249-253)
__global__ void __launch_bounds__(32) k_solve_x(int nx, int ny, const SolveXSet set) {
  const int y = blockIdx.x * blockDim.x + threadIdx.x;
  if (y >= ny) return;
  const LineFactors &f = set.f[blockIdx.y];
  const int mode = set.mode[blockIdx.y];
  double *row = set.q[blockIdx.y] + (size_t)y * nx;
  double prev = 0.0;
  if (mode == 0) {
    prev = row[0] / f.d0;
    row[0] = prev;
  }
  prev = line_forward<kSolveXChunk>(row, 1, f.inv, f.l, 1, nx, prev);
  // mode 1: the identity row itot+1 is zero, so row itot-1 is final already
  line_backward<kSolveXChunk>(row, 1, f.up, nx - 2, mode == 0 ? 0 : 1, prev);
}

// src/linalg.c:52-108 applied per column along y (periodic), coalesced across x.
__global__ void __launch_bounds__(32) k_solve_y(int nx, int ny, const SolveYSet set) {
  const int x = set.first_col[blockIdx.y] + blockIdx.x * blockDim.x + threadIdx.x;
  if (x >= nx) return;
  const PeriodicFactors &f = set.f[blockIdx.y];
  const int n = ny;
  double *col = set.q[blockIdx.y] + x;
  const size_t s = (size_t)nx;
  const LineFactors &sub = f.sub;
  double prev = col[0] / sub.d0;
  col[0] = prev;
  prev = line_forward<kLineChunk>(col, s, sub.inv, sub.l, 1, n - 1, prev);
  line_backward<kLineChunk>(col, s, sub.up, n - 3, 0, prev);
  const double q00 = col[0], q0l = col[(size_t)(n - 2) * s];
  const double last = (col[(size_t)(n - 1) * s] - f.u_last * q00 - f.l_last * q0l) / f.den;
  col[(size_t)(n - 1) * s] = last;
  double cq[kFixChunk], c1[kFixChunk];
#pragma unroll
  for (int k = 0; k < kFixChunk; ++k) {
    const int y = k;
    cq[k] = y <= n - 2 ? col[(size_t)y * s] : 0.0;
    c1[k] = y <= n - 2 ? __ldg(f.q1 + y) : 0.0;
  }
#pragma unroll 1
  for (int b = 0; b <= n - 2; b += kFixChunk) {
    double nq[kFixChunk], n1[kFixChunk];
#pragma unroll
    for (int k = 0; k < kFixChunk; ++k) {
      const int y = b + kFixChunk + k;
      nq[k] = y <= n - 2 ? col[(size_t)y * s] : 0.0;
      n1[k] = y <= n - 2 ? __ldg(f.q1 + y) : 0.0;
    }
#pragma unroll
    for (int k = 0; k < kFixChunk; ++k) {
      const int y = b + k;
      if (y <= n - 2) col[(size_t)y * s] = cq[k] + last * c1[k];
    }
#pragma unroll
    for (int k = 0; k < kFixChunk; ++k) {
      cq[k] = nq[k];
      c1[k] = n1[k];
    }
  }
}

__global__ void k_add_increment(int nx, int ny, int kind, const double *in, const double *q, double *out) {
  const size_t n = (size_t)nx * ny;
  for (size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x; k < n; k += (size_t)gridDim.x * blockDim.x) {
    const int x = (int)(k % nx);
    if (kind == 1 && x == 0) continue;
    out[k] = in[k] + q[k];
  }
}

// ------------------------------------------------------------------- Poisson
struct PoissonArgs {
  DevGrid g;
  StageScalars s;
  const double *ux, *uy;
  double2 *spec;
  double *psi;
  int cols;  // x columns per block
};

using fft::fft_slot;
using fft::fft_stages;

// src/fluid/compute_potential.c:69-92: right-hand side (div u*)/(gamma dt)
// and its real DFT along y (forward, FFTW conventions).
// columns x0 .. x0+cols-1 by the whole block, z: cols * ny/2 complex in shared memory
template <bool RCP>
__device__ __forceinline__ void poisson_fwd_cols(const PoissonArgs &a, int x0, double2 *z) {
  const int nx = a.g.nx, ny = a.g.ny, M = ny / 2, C = a.cols;
  double *zd = reinterpret_cast<double *>(z);
  const double dy = a.g.dy, rdy = a.g.rdy;
  for (int e = threadIdx.x; e < C * ny; e += blockDim.x) {
    const int c = e % C, y = e / C, x = x0 + c;
    double d = 0.0;
    if (x < nx) {
      const size_t r = (size_t)y * nx + x;
      const double uxm = a.ux[r];
      const double uxp = x == nx - 1 ? 0.0 : a.ux[r + 1];
      const double uym = a.uy[r];
      const double uyp = a.uy[(size_t)wrap_up(y, ny) * nx + x];
      d = a.s.rgdt * (dv<RCP>(uxp - uxm, a.g.dxf[x], a.g.rdxf[x]) + dv<RCP>(uyp - uym, dy, rdy));
    }
    zd[2 * (c * M + fft_slot(y >> 1, M, a.g.fft_nst, a.g.fft_first2)) + (y & 1)] = d;
  }
  __syncthreads();
  const double2 *tw = reinterpret_cast<const double2 *>(a.g.tw);
  fft_stages<true>(z, C, M, ny, a.g.fft_nst, a.g.fft_first2, tw);
  const int half = M / 2 + 1;
  for (int e = threadIdx.x; e < C * half; e += blockDim.x) {
    const int c = e / half, k = e - c * half, x = x0 + c;
    if (x >= nx) continue;
    fft::rfft_post(z + c * M, a.spec + (size_t)x * a.g.jpitch, M, k, tw);
  }
}

template <bool RCP>
__global__ void __launch_bounds__(256) k_poisson_fwd(const PoissonArgs a) {
  extern __shared__ double2 z[];
  poisson_fwd_cols<RCP>(a, blockIdx.x * a.cols, z);
}

// Thomas sweeps of the Poisson modes. On this GPU an FP64 warp instruction
// occupies the sub-partition's FP64 pipe for the same time whether 1 or 32
// lanes are active, and the recurrence is serial in x, so the sweep is bound
// by the FP64 instructions one warp issues per element. Each warp therefore
// carries one component (real or imaginary) of 32 modes -- 3 FP64
// instructions per element forward, 2 backward -- and the two components of
// a mode run in different blocks (different SMs). The zero-pivot test reads
// the bits of 1/pivot with integer instructions. A per-thread cp.async ring
// keeps kTriDepth chunks of the line in flight; each thread touches only its
// own ring slots.
constexpr int kTriStage = 8;
constexpr int kTriDepth = 8;
constexpr int kTriMaxNx = 16384;  // lower diagonal staged in shared memory (itot limit)

struct TriRing {
  double v[kTriDepth][kTriStage][32];
  double f[kTriDepth][kTriStage][32];
};

__device__ __forceinline__ void cp_async8(void *smem, const void *gmem) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(s), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory");
}

// stage elements x = x0 + dir*k (k < kTriStage) lying in [lo, hi]; always
// commits one group so that the group count stays regular
__device__ __forceinline__ void tri_issue(TriRing &R, int slot, const double *val, const double *fac, int x0,
                                          int dir, int lo, int hi, size_t vs, size_t fs, int lane) {
#pragma unroll
  for (int k = 0; k < kTriStage; ++k) {
    const int x = x0 + dir * k;
    if (x >= lo && x <= hi) {
      cp_async8(&R.v[slot][k][lane], val + (size_t)x * vs);
      cp_async8(&R.f[slot][k][lane], fac + (size_t)x * fs);
    }
  }
  cp_async_commit();
}

// src/fluid/compute_potential.c:109-136 with src/linalg.c:32-50: per Fourier
// mode, Thomas along x with the complex right-hand side; real and imaginary
// parts undergo identical real operations (real matrix), so they are solved
// as independent real lines. blockIdx.y selects the component.
__global__ void __launch_bounds__(32) k_poisson_tri(const DevGrid g, double2 *spec) {
  extern __shared__ double tri_smem[];
  TriRing &R = *reinterpret_cast<TriRing *>(tri_smem);
  double *pl = tri_smem + sizeof(TriRing) / sizeof(double);
  const int lane = threadIdx.x;
  const int nx = g.nx;
  for (int x = lane; x < nx; x += 32) pl[x] = g.pl[x];
  __syncwarp();
  const int J = blockIdx.x * 32 + lane;
  if (J >= g.nh) return;
  const size_t jp = (size_t)g.jpitch;
  double *col = reinterpret_cast<double *>(spec + J) + blockIdx.y;  // stride 2*jp doubles per x
  const size_t vs = 2 * jp;
  const double *inv = g.pinv + J, *up = g.pup + J;
  // ---- forward elimination, x = 1..nx-1 (src/linalg.c:33-45)
  double prev = col[0] / g.pd0[J];
  col[0] = prev;
  const int nel = nx - 1;
  const int nchunk = (nel + kTriStage - 1) / kTriStage;
#pragma unroll 1
  for (int c = 0; c < kTriDepth - 1; ++c) tri_issue(R, c, col, inv, 1 + c * kTriStage, 1, 1, nx - 1, vs, jp, lane);
#pragma unroll 1
  for (int c = 0; c < nchunk; ++c) {
    const int ahead = c + kTriDepth - 1;
    tri_issue(R, ahead % kTriDepth, col, inv, 1 + ahead * kTriStage, 1, 1, nx - 1, vs, jp, lane);
    cp_async_wait<kTriDepth - 1>();
    const int slot = c % kTriDepth;
#pragma unroll
    for (int k = 0; k < kTriStage; ++k) {
      const int x = 1 + c * kTriStage + k;
      if (x < nx) {
        const double iv = R.f[slot][k][lane];
        // |pivot| < DBL_EPSILON rows carry 1/pivot = +0: the reference sets them to 0
        const double v = __double_as_longlong(iv) == 0 ? 0.0 : iv * (R.v[slot][k][lane] - pl[x] * prev);
        col[(size_t)x * vs] = v;
        prev = v;
      }
    }
  }
  cp_async_wait<0>();
  __threadfence_block();  // the back substitution re-reads values stored above
  // ---- back substitution, x = nx-2..0 (src/linalg.c:46-48)
  double next = prev;
#pragma unroll 1
  for (int c = 0; c < kTriDepth - 1; ++c)
    tri_issue(R, c, col, up, nx - 2 - c * kTriStage, -1, 0, nx - 2, vs, jp, lane);
#pragma unroll 1
  for (int c = 0; c < nchunk; ++c) {
    const int ahead = c + kTriDepth - 1;
    tri_issue(R, ahead % kTriDepth, col, up, nx - 2 - ahead * kTriStage, -1, 0, nx - 2, vs, jp, lane);
    cp_async_wait<kTriDepth - 1>();
    const int slot = c % kTriDepth;
#pragma unroll
    for (int k = 0; k < kTriStage; ++k) {
      const int x = nx - 2 - c * kTriStage - k;
      if (x >= 0) {
        const double v = R.v[slot][k][lane] - R.f[slot][k][lane] * next;
        col[(size_t)x * vs] = v;
        next = v;
      }
    }
  }
  cp_async_wait<0>();
}

// src/fluid/compute_potential.c:146-157: inverse real DFT along y and the
// 1/jtot normalisation, psi on the interior (halo and walls implied).
// CG: read the spectrum through L2 (written by other blocks of the same launch)
template <bool CG>
__device__ __forceinline__ void poisson_bwd_cols(const PoissonArgs &a, int x0, double2 *z) {
  const int nx = a.g.nx, ny = a.g.ny, M = ny / 2, C = a.cols;
  const double2 *tw = reinterpret_cast<const double2 *>(a.g.tw);
  const int half = M / 2 + 1;
  for (int e = threadIdx.x; e < C * half; e += blockDim.x) {
    const int c = e / half, k = e - c * half, x = x0 + c;
    double2 *zc = z + c * M;
    if (x >= nx) {
      zc[fft_slot(k, M, a.g.fft_nst, a.g.fft_first2)] = make_double2(0.0, 0.0);
      if (k > 0) zc[fft_slot(M - k, M, a.g.fft_nst, a.g.fft_first2)] = make_double2(0.0, 0.0);
      continue;
    }
    fft::rfft_pre<CG>(a.spec + (size_t)x * a.g.jpitch, zc, M, k, tw, a.g.fft_nst, a.g.fft_first2);
  }
  __syncthreads();
  fft_stages<false>(z, C, M, ny, a.g.fft_nst, a.g.fft_first2, tw);
  const double *zd = reinterpret_cast<const double *>(z);
  for (int e = threadIdx.x; e < C * ny; e += blockDim.x) {
    const int c = e % C, y = e / C, x = x0 + c;
    if (x >= nx) continue;
    a.psi[(size_t)y * nx + x] = zd[2 * (c * M + (y >> 1)) + (y & 1)] * a.s.rny;
  }
}

__global__ void __launch_bounds__(256) k_poisson_bwd(const PoissonArgs a) {
  extern __shared__ double2 z[];
  poisson_bwd_cols<false>(a, blockIdx.x * a.cols, z);
}

// ------------------------------------------- fused Poisson (+ temperature)
// One cooperative launch per substage, one block per SM. The serial Thomas
// sweeps (latency bound, 2 x ceil(nh/32) warps) run on the first blocks, one
// warp per SM sub-partition; every other block is a worker that computes
// forward DFT column groups in ascending x, then (optionally) the explicit
// temperature update, then inverse DFT column groups in descending x. The
// sweep of a mode line consumes spectrum rows as the workers publish them,
// and a worker inverts a column group as soon as every sweep warp has passed
// it on the way back, so the DFTs and the temperature update hide behind the
// sweep. Arithmetic and its order are those of the three separate kernels,
// so the results are identical.
//
// Synchronisation: fwd_done[g] = epoch when group g's spectrum rows are
// written (release: block barrier, fence, store); a sweep warp reads flags
// with relaxed loads and issues one fence before reading the rows it
// verified (acquire). bwd_cnt[s] counts the sweep warps that finished span s
// (span = 2^span_shift x elements), cumulative over launches, so a worker waits
// for epoch * lines. Spectrum reads of data written in this launch go
// through L2 (__ldcg). Every wait polls at most `spin` times (kFusedSpin by
// default, about a second; the host may set fewer); a wait that gives up sets
// *err and its warp or block stops, so the launch always ends.
constexpr int kFusedThreads = 512;
// sweep warps per block, one per SM sub-partition. Dependent FP64 chains run
// ~20% slower with four warps on one SM than with one, but every SM given to
// the sweeps is taken from the DFT workers, whose FP64 throughput bounds the
// launch as much as the sweeps do. Measured on GB300: two per block is the
// fastest while at least kFusedMinWorkers workers remain (512 x 1024: 177 us
// against 183 us with four), four per block beyond (1024 x 2048, 2048 x 4096).
constexpr int kFusedTriWarps = 4;
constexpr int kFusedMinWorkers = 130;
// x elements per span of the back substitution's signals: 128 when the
// workers can invert a whole span at once (the last span starts only when the
// sweeps end), else 64; 512 x 1024: 140.2 us per launch against 143.1 (64)
// and 148.9 (32). The counters are sized for the smaller span.
constexpr int kFusedSpanMin = 64;
constexpr int kFusedSpanShiftMax = 7;
// elements per chunk of the fused forward elimination and back substitution,
// measured at 512 x 1024 (launch, CUDA events): forward 8 / 6 / 10 with back
// 6: 143.1 / 143.9 / 147.3 us; back 6 / 5 / 7 / 8 with forward 8: 143.1 /
// 144.1 / 152.7 / 153.5 us
constexpr int kForwardChunk = 8;
constexpr int kBackChunk = 6;
constexpr unsigned kFusedSpin = 1u << 22;
constexpr int kPoll = 128;  // completion flags read per poll by a sweep warp
constexpr size_t kFusedMinSmem = 116 * 1024;  // above half an SM's shared memory: one block per SM

struct FusedArgs {
  PoissonArgs p;
  TempArgs t;                      // explicit temperature update, when with_temp
  int with_temp;
  unsigned *fwd_done;              // [groups]
  unsigned long long *bwd_cnt;     // [spans]
  unsigned *err;                   // 1: a sweep wait gave up, 2: a worker wait gave up
  unsigned epoch;
  int tri_blocks, tri_warps, lines, groups;
  int span_shift;                  // span = 2^span_shift x elements
  unsigned spin;                   // polls of a wait before it gives up
  unsigned want;                   // the flag value a sweep waits for: epoch (epoch + 1 in tests of the waits)
};

__device__ __forceinline__ unsigned ld_relaxed_u32(const unsigned *p) {
  unsigned v;
  asm volatile("ld.relaxed.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ unsigned long long ld_relaxed_u64(const unsigned long long *p) {
  unsigned long long v;
  asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void st_relaxed_u32(unsigned *p, unsigned v) {
  asm volatile("st.relaxed.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// one component of 32 modes (lines[lg]); false when a wait gave up.
// P2: the lower diagonal pl is 2^e (DevGrid::p2), so pl * prev, one of the
// three dependent FP64 operations per element of the forward elimination,
// is taken in the integer unit (~15 cycles on the chain instead of ~78); a
// chunk with an operand out of range is recomputed with FP64 products.
template <bool P2>
__device__ bool fused_sweep(const FusedArgs &a, const double *pl, int lg) {
  const DevGrid &g = a.p.g;
  const int lane = threadIdx.x & 31, nx = g.nx, C = a.p.cols;
  const int J0 = (lg >> 1) * 32, J = J0 + lane;
  const bool act = J < g.nh;
  const int Jc = act ? J : J0;
  const size_t jp = (size_t)g.jpitch, vs = 2 * jp;
  double *col = reinterpret_cast<double *>(a.p.spec + Jc) + (lg & 1);
  const double *inv = g.pinv + Jc, *up = g.pup + Jc;
  int vg = 0;       // groups 0 .. vg-1 are verified complete
  int ready = 0;    // rows below are readable: vg * C
  // make rows up to x readable: the lanes read the next kPoll
  // completion flags (kPoll / 32 each, relaxed), the leading run of complete
  // groups is taken (polling while x's group is not among them), and one
  // fence then orders the row reads after them. The test on the path taken once per
  // chunk is one comparison (an integer division there cost ~12 us per
  // launch at 512 x 1024: it runs between chunks, outside the latency
  // shadows of the recurrence).
  auto need = [&](int x) -> bool {
    if (x < ready) return true;
    const int gx = x / C;
    unsigned spin = 0;
    while (vg <= gx) {
      bool ok[kPoll / 32];
#pragma unroll
      for (int i = 0; i < kPoll / 32; ++i) {
        const int gi = vg + 32 * i + lane;
        ok[i] = gi >= a.groups || ld_relaxed_u32(a.fwd_done + gi) == a.want;
      }
      int run = kPoll;
#pragma unroll
      for (int i = kPoll / 32 - 1; i >= 0; --i) {
        const unsigned n = __ballot_sync(0xffffffffu, !ok[i]);
        if (n) run = 32 * i + __ffs(n) - 1;
      }
      vg = min(vg + run, a.groups);
      // the warp owns its SM's FP64 work alone: poll back to back (each
      // poll is an L2 round trip; a sleep between them delayed the start)
      if (vg <= gx && ++spin >= a.spin) return false;
    }
    ready = min(vg * C, nx);
    __threadfence();
    return true;
  };
  // while the first spectrum columns are being computed: bring this line's
  // factors into L2 (they come from HBM when the cache was flushed or evicted)
#pragma unroll 1
  for (int x = 0; x < nx; ++x) {
    asm volatile("prefetch.global.L2 [%0];" ::"l"(inv + (size_t)x * jp));
    asm volatile("prefetch.global.L2 [%0];" ::"l"(up + (size_t)x * jp));
  }
  // ---- forward elimination (src/linalg.c:33-45)
  if (!need(0)) return false;
  double prev = __ldcg(col) / g.pd0[Jc];
  if (act) col[0] = prev;
  double cq[kForwardChunk], ci[kForwardChunk];
  if (nx > 1 && !need(min(kForwardChunk, nx - 1))) return false;
#pragma unroll
  for (int k = 0; k < kForwardChunk; ++k) {
    const int e = 1 + k;
    cq[k] = e < nx ? __ldcg(col + (size_t)e * vs) : 0.0;
    ci[k] = e < nx ? __ldg(inv + (size_t)e * jp) : 0.0;
  }
  // one chunk of rows b .. b+kForwardChunk-1; the full chunks run without a
  // per-row guard inside the recurrence, only the last one needs it
  auto forward_chunk = [&](int b, auto guarded) -> bool {
    double nq[kForwardChunk], ni[kForwardChunk];
    const int nb = b + kForwardChunk;
    if (nb < nx && !need(min(nb + kForwardChunk - 1, nx - 1))) return false;
#pragma unroll
    for (int k = 0; k < kForwardChunk; ++k) {
      const int e = nb + k;
      nq[k] = e < nx ? __ldcg(col + (size_t)e * vs) : 0.0;
      ni[k] = e < nx ? __ldg(inv + (size_t)e * jp) : 0.0;
    }
    auto rows = [&](auto fast) -> bool {
      Mul<decltype(fast)::value> m;
#pragma unroll
      for (int k = 0; k < kForwardChunk; ++k) {
        const int x = b + k;
        if (!decltype(guarded)::value || x < nx) {
          const double iv = ci[k], c = pl[x];
          // |pivot| < DBL_EPSILON rows carry 1/pivot = +0: the reference sets them to 0
          const double v = __double_as_longlong(iv) == 0 ? 0.0 : iv * (cq[k] - m.by(prev, c, p2_field(c)));
          if (act) col[(size_t)x * vs] = v;
          prev = v;
        }
      }
      return m.ok;
    };
    if constexpr (P2) {
      const double p0 = prev;
      if (!rows(std::true_type{})) {
        prev = p0;
        rows(std::false_type{});
      }
    } else {
      rows(std::false_type{});
    }
#pragma unroll
    for (int k = 0; k < kForwardChunk; ++k) {
      cq[k] = nq[k];
      ci[k] = ni[k];
    }
    return true;
  };
  int b = 1;
#pragma unroll 1
  for (; b + kForwardChunk <= nx; b += kForwardChunk)
    if (!forward_chunk(b, std::false_type{})) return false;
  if (b < nx && !forward_chunk(b, std::true_type{})) return false;
  // ---- back substitution (src/linalg.c:46-48), x = nx-2 .. 0; span s is
  // final once x passes its lowest element
  auto signal = [&](int s) {
    __threadfence();
    __syncwarp();
    if (lane == 0) atomicAdd(a.bwd_cnt + s, 1ull);
  };
  const int sh = a.span_shift;
  const int top = (nx - 1) >> sh;
  if ((top << sh) > nx - 2) signal(top);  // a top span holding only x = nx-1
  double next = prev;
  double bq[kBackChunk], cu[kBackChunk];
  const int hi = nx - 2;
#pragma unroll
  for (int k = 0; k < kBackChunk; ++k) {
    const int e = hi - k;
    bq[k] = e >= 0 ? __ldcg(col + (size_t)e * vs) : 0.0;
    cu[k] = e >= 0 ? __ldg(up + (size_t)e * jp) : 0.0;
  }
  auto backward_chunk = [&](int b, auto guarded) {
    double nq[kBackChunk], nu[kBackChunk];
#pragma unroll
    for (int k = 0; k < kBackChunk; ++k) {
      const int e = b - kBackChunk - k;
      nq[k] = e >= 0 ? __ldcg(col + (size_t)e * vs) : 0.0;
      nu[k] = e >= 0 ? __ldg(up + (size_t)e * jp) : 0.0;
    }
#pragma unroll
    for (int k = 0; k < kBackChunk; ++k) {
      const int x = b - k;
      if (!decltype(guarded)::value || x >= 0) {
        const double v = bq[k] - cu[k] * next;
        if (act) col[(size_t)x * vs] = v;
        next = v;
      }
    }
    // a span whose lowest element this chunk passed is final: signalled once
    // per chunk, after it, instead of a test inside the recurrence
    const int sb = (b >> sh) << sh;
    if (sb >= max(b - kBackChunk + 1, 0)) signal(sb >> sh);
#pragma unroll
    for (int k = 0; k < kBackChunk; ++k) {
      bq[k] = nq[k];
      cu[k] = nu[k];
    }
  };
  int bb = hi;
#pragma unroll 1
  for (; bb - kBackChunk + 1 >= 0; bb -= kBackChunk) backward_chunk(bb, std::false_type{});
  if (bb >= 0) backward_chunk(bb, std::true_type{});
  return true;
}

template <bool RCP>
__global__ void __launch_bounds__(kFusedThreads, 1) k_poisson_fused(const FusedArgs a) {
  extern __shared__ double2 fz[];
  const DevGrid &g = a.p.g;
  const int nx = g.nx, C = a.p.cols;
  if ((int)blockIdx.x < a.tri_blocks) {
    double *pl = reinterpret_cast<double *>(fz);
    for (int x = threadIdx.x; x < nx; x += blockDim.x) pl[x] = g.pl[x];
    __syncthreads();
    const int w = threadIdx.x >> 5;
    const int lg = blockIdx.x * a.tri_warps + w;
    if (w >= a.tri_warps || lg >= a.lines) return;
    const bool ok = RCP && g.p2 ? fused_sweep<RCP>(a, pl, lg) : fused_sweep<false>(a, pl, lg);
    if (!ok && (threadIdx.x & 31) == 0) atomicOr(a.err, 1u);
    return;
  }
  __shared__ int s_ok;
  const int wk = blockIdx.x - a.tri_blocks, W = gridDim.x - a.tri_blocks;
  // forward DFT column groups, ascending x
  for (int gi = wk; gi < a.groups; gi += W) {
    poisson_fwd_cols<RCP>(a.p, gi * C, fz);
    __syncthreads();
    if (threadIdx.x == 0) {
      __threadfence();
      st_relaxed_u32(a.fwd_done + gi, a.epoch);
    }
  }
  // explicit temperature update, while the sweeps run
  if (a.with_temp) {
    const int xb = (nx + kFusedThreads - 1) / kFusedThreads, yb = (g.ny + kRows - 1) / kRows;
    for (int u = wk; u < xb * yb; u += W) {
      const int x = (u % xb) * kFusedThreads + threadIdx.x;
      if (x < nx) {
        if (RCP && g.p2) {
          temp_column<0, 0, RCP, RCP>(a.t, x, (u / xb) * kRows);
        } else {
          temp_column<0, 0, RCP, false>(a.t, x, (u / xb) * kRows);
        }
      }
    }
  }
  // inverse DFT column groups, descending x, once every sweep warp passed them
  const unsigned long long target = (unsigned long long)a.epoch * (unsigned long long)a.lines;
  for (int k = wk; k < a.groups; k += W) {
    const int gi = a.groups - 1 - k;
    if (threadIdx.x == 0) {
      const int s = (gi * C) >> a.span_shift;
      unsigned spin = 0;
      unsigned long long v;
      while ((v = ld_relaxed_u64(a.bwd_cnt + s)) < target && ++spin < a.spin) {
      }
      s_ok = v >= target;
      if (!s_ok) atomicOr(a.err, 2u);
      __threadfence();
    }
    __syncthreads();
    if (!s_ok) return;
    poisson_bwd_cols<true>(a.p, gi * C, fz);
    __syncthreads();
  }
}

// ------------------------------------------------ correction and pressure
struct CorrArgs {
  DevGrid g;
  StageScalars s;
  const double *psi;
  double *ux, *uy, *p;
  unsigned long long *colmax, *uymax;
};

__device__ __forceinline__ unsigned long long abs_bits(double v) {
  // |v| as an order-preserving key; NaN counts as 0 (fmax(NaN, small) = small
  // in src/param/decide_dt.c:38,46). Integer operations only: an FP64
  // compare would occupy the (slow) FP64 pipe.
  const unsigned long long b = (unsigned long long)__double_as_longlong(v) & 0x7fffffffffffffffull;
  return b > 0x7ff0000000000000ull ? 0ull : b;
}

// NaN or infinity: exponent field all ones (integer test, off the FP64 pipe)
__device__ __forceinline__ bool nonfinite(double v) {
  return (__double2hiint(v) & 0x7ff00000) == 0x7ff00000;
}

constexpr int kCorrRows = 4;  // rows per thread in the (memory-latency bound) correction kernels

__device__ __forceinline__ unsigned long long warp_max_u64(unsigned long long v) {
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) v = max(v, __shfl_xor_sync(0xffffffffu, v, off));
  return v;
}

// src/fluid/correct_velocity.c:6-42 and src/fluid/update_pressure.c:7-60, per
// cell in the reference's order; with colmax set, also max |ux| per column and
// max |uy| for the next src/param/decide_dt.c (exact: division is monotonic).
// Every lane of a block stays alive to the warp reduction (blockDim is a
// multiple of 32); lanes past the last column only contribute zero.
template <int IMPX, int IMPY, bool RCP, bool CORR, bool PRES>
__global__ void __launch_bounds__(128) k_corr(const CorrArgs a) {
  const int nx = a.g.nx, ny = a.g.ny;
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  const bool live = x < nx;
  unsigned long long mx = 0ull, my = 0ull;
  bool nf = false;  // a NaN or infinity among the values written
  if (live) {
    const int y0 = blockIdx.y * kCorrRows;
    int y1 = min(y0 + kCorrRows, ny);
    const double gdt = a.s.gdt, dy = a.g.dy, rdy = a.g.rdy;
    const double dxi = a.g.dxi[x];
    const double dcm = a.g.dxc[x], dcp = a.g.dxc[x + 1], df = a.g.dxf[x];
    const double rcm = a.g.rdxc[x], rcp = a.g.rdxc[x + 1], rf = a.g.rdxf[x];
    const bool left = x == 0, right = x == nx - 1;
    const double *psi = a.psi;
    double sm = psi[(size_t)wrap_dn(y0, ny) * nx + x];
    if constexpr (!IMPX && !IMPY && CORR && PRES) {
      if (y1 - y0 == kCorrRows) {
        // every operand of the rows loaded before the first store (the
        // stores could alias later loads for the compiler): one memory round
        // trip per thread instead of kCorrRows
        double ps[kCorrRows], pw[kCorrRows], u[kCorrRows], v[kCorrRows], pp[kCorrRows];
#pragma unroll
        for (int k = 0; k < kCorrRows; ++k) {
          const size_t r = (size_t)(y0 + k) * nx + x;
          ps[k] = psi[r];
          pw[k] = left ? 0.0 : psi[r - 1];
          u[k] = left ? 0.0 : a.ux[r];
          v[k] = a.uy[r];
          pp[k] = a.p[r];
        }
        // the rows' new values; FAST: the products by 1/dx and 1/dy (powers of
        // two on such grids) in the integer unit, false when out of range
        auto rows = [&](auto fast, double *un, double *vn) -> bool {
          Mul<decltype(fast)::value> m;
          double s0 = sm;
#pragma unroll
          for (int k = 0; k < kCorrRows; ++k) {
            const double sc = ps[k];
            const double sl = left ? sc : pw[k];  // Neumann psi(0) = psi(1)
            if constexpr (decltype(fast)::value) {
              un[k] = u[k] - m.by(gdt * (sc - sl), dxi, p2_field(dxi));
              vn[k] = v[k] - m.by(gdt * (sc - s0), rdy, p2_field(rdy));
            } else {
              un[k] = u[k] - ((gdt * (sc - sl)) * dxi);
              vn[k] = v[k] - dv<RCP>(gdt * (sc - s0), dy, rdy);
            }
            s0 = sc;
          }
          return m.ok;
        };
        double un[kCorrRows], vn[kCorrRows];
        if (!(RCP && a.g.p2 && rows(std::true_type{}, un, vn))) rows(std::false_type{}, un, vn);
#pragma unroll
        for (int k = 0; k < kCorrRows; ++k) {
          const size_t r = (size_t)(y0 + k) * nx + x;
          if (!left) {
            a.ux[r] = un[k];
            mx = max(mx, abs_bits(un[k]));
            nf |= nonfinite(un[k]);
          }
          a.uy[r] = vn[k];
          my = max(my, abs_bits(vn[k]));
          const double pv = pp[k] + ps[k];
          a.p[r] = pv;
          nf |= nonfinite(vn[k]) | nonfinite(pv);
        }
        y1 = y0;  // done: skip the row loop below
      }
    }
    for (int y = y0; y < y1; ++y) {
      const size_t r = (size_t)y * nx + x;
      const double sc = psi[r];
      const double sl = left ? sc : psi[r - 1];  // Neumann psi(0) = psi(1)
      if (CORR) {
        if (!left) {
          const double u = a.ux[r] - ((gdt * (sc - sl)) * dxi);
          a.ux[r] = u;
          mx = max(mx, abs_bits(u));
          nf |= nonfinite(u);
        }
        const double v = a.uy[r] - dv<RCP>(gdt * (sc - sm), dy, rdy);
        a.uy[r] = v;
        my = max(my, abs_bits(v));
        nf |= nonfinite(v);
      }
      if (PRES) {
        double pv = a.p[r] + sc;
        if (IMPX) {
          const double sr = right ? sc : psi[r + 1];  // Neumann psi(nx+1) = psi(nx)
          const double gm = dv<RCP>(sc - sl, dcm, rcm);
          const double gp = dv<RCP>(sr - sc, dcp, rcp);
          pv = pv + a.s.pcorr * dv<RCP>(gp - gm, df, rf);
        }
        if (IMPY) {
          const double sn = psi[(size_t)wrap_up(y, ny) * nx + x];
          const double gm = dv<RCP>(sc - sm, dy, rdy);
          const double gp = dv<RCP>(sn - sc, dy, rdy);
          pv = pv + a.s.pcorr * dv<RCP>(gp - gm, dy, rdy);
        }
        a.p[r] = pv;
        nf |= nonfinite(pv);
      }
      sm = sc;
    }
  }
  if (CORR && a.colmax) {
    if (live && x >= 1) atomicMax(a.colmax + x, mx);
    my = warp_max_u64(my);
    if ((threadIdx.x & 31) == 0) atomicMax(a.uymax, my);
    // word 0 of the column maxima (no ux column 0 exists): non-finite state
    if (__any_sync(0xffffffffu, nf) && (threadIdx.x & 31) == 0) atomicOr(a.colmax, 1ull);
  }
}

__global__ void __launch_bounds__(128) k_umax(int nx, int ny, const double *ux, const double *uy,
                                              unsigned long long *colmax, unsigned long long *uymax) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  unsigned long long mx = 0ull, my = 0ull;
  bool nf = false;
  if (x < nx) {
    const int y0 = blockIdx.y * kRows;
    const int y1 = min(y0 + kRows, ny);
    for (int y = y0; y < y1; ++y) {
      const size_t r = (size_t)y * nx + x;
      const double u = ux[r], v = uy[r];
      if (x >= 1) {
        mx = max(mx, abs_bits(u));
        nf |= nonfinite(u);
      }
      my = max(my, abs_bits(v));
      nf |= nonfinite(v);
    }
    if (x >= 1) atomicMax(colmax + x, mx);
  }
  my = warp_max_u64(my);
  if ((threadIdx.x & 31) == 0) atomicMax(uymax, my);
  if (__any_sync(0xffffffffu, nf) && (threadIdx.x & 31) == 0) atomicOr(colmax, 1ull);
}

dim3 march_grid(const DevGrid &g, int rows = kRows) {
  return dim3((g.nx + kBlockX - 1) / kBlockX, (g.ny + rows - 1) / rows);
}

// one thread per radix-4 butterfly of a stage, 64..256 per block
int poisson_threads(const DevGrid &g, int cols) {
  const int b = cols * (g.ny / 2) / 4;
  return b <= 64 ? 64 : b >= 256 ? 256 : (b + 31) / 32 * 32;
}

int poisson_cols(const DevGrid &g) {
  // enough blocks to cover the SMs at least twice, at most 64 KiB of shared memory each
  int c = 1;
  while (c < 16 && (size_t)(2 * c) * g.ny * sizeof(double) <= 65536 && g.nx / (2 * c) >= 304) c *= 2;
  return c;
}

}  // namespace

// ------------------------------------------------------------------- launches
cudaError_t launch_temp_update(const DevGrid &g, const StageScalars &s, int impx, int impy,
                               const double *t_in, double *t_out, double *at, double *qt,
                               const double *ux, const double *uy, cudaStream_t st) {
  const TempArgs a{g, s, t_in, t_out, at, qt, ux, uy};
  const dim3 grid = march_grid(g), block(kBlockX);
#define SNS_T(X, Y, R, F) k_temp<X, Y, R, F><<<grid, block, 0, st>>>(a)
  if (g.p2) {
    if (impx && impy) SNS_T(1, 1, true, true);
    else if (impx) SNS_T(1, 0, true, true);
    else if (impy) SNS_T(0, 1, true, true);
    else SNS_T(0, 0, true, true);
  } else if (g.rcp) {
    if (impx && impy) SNS_T(1, 1, true, false);
    else if (impx) SNS_T(1, 0, true, false);
    else if (impy) SNS_T(0, 1, true, false);
    else SNS_T(0, 0, true, false);
  } else {
    if (impx && impy) SNS_T(1, 1, false, false);
    else if (impx) SNS_T(1, 0, false, false);
    else if (impy) SNS_T(0, 1, false, false);
    else SNS_T(0, 0, false, false);
  }
#undef SNS_T
  count_launches(1);
  return cudaGetLastError();
}

cudaError_t launch_velocity_update(const DevGrid &g, const StageScalars &s, int impx, int impy,
                                   const double *ux, const double *uy, const double *p, const double *tforce,
                                   double *ux_out, double *uy_out, double *aux, double *auy,
                                   double *qx, double *qy, cudaStream_t st) {
  const VelArgs a{g, s, ux, uy, p, tforce, ux_out, uy_out, aux, auy, qx, qy};
  const dim3 grid = march_grid(g), block(kBlockX);
#define SNS_V(X, Y, R, F) k_vel<X, Y, R, F><<<grid, block, 0, st>>>(a)
  if (g.p2) {
    if (impx && impy) SNS_V(1, 1, true, true);
    else if (impx) SNS_V(1, 0, true, true);
    else if (impy) SNS_V(0, 1, true, true);
    else SNS_V(0, 0, true, true);
  } else if (g.rcp) {
    if (impx && impy) SNS_V(1, 1, true, false);
    else if (impx) SNS_V(1, 0, true, false);
    else if (impy) SNS_V(0, 1, true, false);
    else SNS_V(0, 0, true, false);
  } else {
    if (impx && impy) SNS_V(1, 1, false, false);
    else if (impx) SNS_V(1, 0, false, false);
    else if (impy) SNS_V(0, 1, false, false);
    else SNS_V(0, 0, false, false);
  }
#undef SNS_V
  count_launches(1);
  return cudaGetLastError();
}

cudaError_t launch_solve_x_set(const DevGrid &g, const SolveXSet &set, cudaStream_t st) {
  if (set.n < 1 || set.n > 3) return cudaErrorInvalidValue;
  k_solve_x<<<dim3((g.ny + 31) / 32, set.n), 32, 0, st>>>(g.nx, g.ny, set);
  count_launches(1);
  return cudaGetLastError();
}

cudaError_t launch_solve_y_set(const DevGrid &g, const SolveYSet &set, cudaStream_t st) {
  if (set.n < 1 || set.n > 3) return cudaErrorInvalidValue;
  k_solve_y<<<dim3((g.nx + 31) / 32, set.n), 32, 0, st>>>(g.nx, g.ny, set);
  count_launches(1);
  return cudaGetLastError();
}

cudaError_t launch_solve_x(const DevGrid &g, const LineFactors &f, int mode, double *q, cudaStream_t st) {
  SolveXSet set{};
  set.f[0] = f;
  set.mode[0] = mode;
  set.q[0] = q;
  set.n = 1;
  return SNS_PLAIN_FORM::launch_solve_x_set(g, set, st);
}

cudaError_t launch_solve_y(const DevGrid &g, const PeriodicFactors &f, int first_col, double *q, cudaStream_t st) {
  SolveYSet set{};
  set.f[0] = f;
  set.first_col[0] = first_col;
  set.q[0] = q;
  set.n = 1;
  return SNS_PLAIN_FORM::launch_solve_y_set(g, set, st);
}

cudaError_t launch_add_increment(const DevGrid &g, int kind, const double *in, const double *q, double *out,
                                 cudaStream_t st) {
  const size_t n = (size_t)g.nx * g.ny;
  const int blocks = (int)std::min<size_t>((n + 255) / 256, 152 * 16);
  k_add_increment<<<blocks, 256, 0, st>>>(g.nx, g.ny, kind, in, q, out);
  count_launches(1);
  return cudaGetLastError();
}

// ------------------------------------------------------------- statistics
// UX1 += pow(UX, 1.), UX2 += pow(UX, 2.) etc. per point and sample
// (src/statistics/collect.c:19-24, 38-43, 57-62); pow(v, 1.) is v and
// pow(v, 2.) the correctly rounded square, v * v.
__global__ void __launch_bounds__(256) k_stats(int nx, int ny, const double *ux, const double *uy, const double *t,
                                               double *s) {
  const size_t wu = (size_t)nx + 1, wc = (size_t)nx + 2;
  const size_t nu = wu * ny, nc = wc * ny;
  double *ux1 = s, *ux2 = s + nu, *uy1 = s + 2 * nu, *uy2 = uy1 + nc, *t1 = uy2 + nc, *t2 = t1 + nc;
  for (size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x; k < nc; k += (size_t)gridDim.x * blockDim.x) {
    const int y = (int)(k / wc), i = (int)(k - (size_t)y * wc);  // i = 0..nx+1
    const size_t d = (size_t)y * nx + (i - 1);
    const bool wall = i == 0 || i == nx + 1;
    const double v = wall ? 0.0 : uy[d];
    uy1[k] += v;
    uy2[k] += v * v;
    if (t) {
      const double tv = i == 0 ? kTempXm : i == nx + 1 ? kTempXp : t[d];
      t1[k] += tv;
      t2[k] += tv * tv;
    }
    if (i >= 1) {  // ux at i = 1..nx+1; dense x = i-1 holds the wall i = 1 as zero
      const size_t ku = (size_t)y * wu + (i - 1);
      const double u = i == nx + 1 ? 0.0 : ux[d];
      ux1[ku] += u;
      ux2[ku] += u * u;
    }
  }
}

cudaError_t launch_stats(const DevGrid &g, const double *ux, const double *uy, const double *t, double *s,
                         cudaStream_t st) {
  k_stats<<<2 * 152, 256, 0, st>>>(g.nx, g.ny, ux, uy, t, s);
  count_launches(1);
  return cudaGetLastError();
}

// --------------------------------------------------------- host transfers
// Strided field copies between pinned host arrays (read or written in place
// through their device alias, over the host link) and dense device fields.
// The link's latency is long, so each thread keeps kXferRows loads in flight
// (one column of kXferRows rows) before it stores them; blocks walk row
// groups of one field (blockIdx.y).
constexpr int kXferRows = 8;
constexpr int kXferThreads = 256;

__global__ void __launch_bounds__(kXferThreads) k_xfer(const XferList L) {
  const XferField f = L.f[blockIdx.y];
  const int groups = (L.rows + kXferRows - 1) / kXferRows;
  for (int gi = blockIdx.x; gi < groups; gi += gridDim.x) {
    const int y0 = gi * kXferRows;
    const int ny = min(kXferRows, L.rows - y0);
    for (int x = threadIdx.x; x < f.width; x += kXferThreads) {
      double v[kXferRows];
#pragma unroll
      for (int r = 0; r < kXferRows; ++r)
        if (r < ny) v[r] = __ldcs(f.src + (size_t)(y0 + r) * f.sstride + x);
#pragma unroll
      for (int r = 0; r < kXferRows; ++r)
        if (r < ny) __stcs(f.dst + (size_t)(y0 + r) * f.dstride + x, v[r]);
    }
  }
}

cudaError_t launch_xfer(const XferList &L, cudaStream_t st) {
  if (L.n <= 0) return cudaSuccess;
  int dev = 0, sms = 152;
  if (cudaGetDevice(&dev) == cudaSuccess) cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const int groups = (L.rows + kXferRows - 1) / kXferRows;
  // about four blocks per SM over all fields
  const int per_field = std::max(1, std::min(groups, 4 * sms / L.n));
  k_xfer<<<dim3(per_field, L.n), kXferThreads, 0, st>>>(L);
  count_launches(1);
  return cudaGetLastError();
}

// One entry (row j in 0..ny+1, column c in 0..W-1) of a reference-layout
// array from the dense device field, boundary rules included; false for the
// temperature's corners, which the reference's rules never write.
__device__ __forceinline__ bool lin_entry(const LinField &f, int nx, int ny, int j, int c, double &v) {
  const int jj = j == 0 ? ny : (j == ny + 1 ? 1 : j);  // periodic halo rows
  const double *row = f.dev + (size_t)(jj - 1) * nx;
  switch (f.kind) {
    case LIN_UX:  // c = i - 1; walls i = 1 and i = itot+1 hold 0
      v = (c == 0 || c == nx) ? 0.0 : row[c];
      return true;
    case LIN_UY:  // c = i; walls i = 0 and i = itot+1 hold 0
      v = (c == 0 || c == nx + 1) ? 0.0 : row[c - 1];
      return true;
    case LIN_P:  // Neumann: p(0) = p(1), p(itot+1) = p(itot), halo rows included
      v = row[min(max(c, 1), nx) - 1];
      return true;
    default:  // temperature: wall values on rows 1..jtot only
      if (c == 0 || c == nx + 1) {
        if (j == 0 || j == ny + 1) return false;
        v = c == 0 ? kTempXm : kTempXp;
        return true;
      }
      v = row[c - 1];
      return true;
  }
}

constexpr int kLinPairs = 4;  // 16-byte pairs in flight per thread

__global__ void __launch_bounds__(256) k_lin(const LinList L, int to_host) {
  const LinField f = L.f[blockIdx.y];
  const int nx = L.nx, ny = L.ny, W = f.W;
  const size_t pairs = (size_t)(ny + 2) * W / 2;  // (ny + 2) is even
  const size_t stride = (size_t)gridDim.x * blockDim.x * kLinPairs;
  double2 *host2 = reinterpret_cast<double2 *>(f.host);
  for (size_t base = (size_t)blockIdx.x * blockDim.x * kLinPairs + threadIdx.x; base < pairs; base += stride) {
    if (to_host) {
#pragma unroll
      for (int k = 0; k < kLinPairs; ++k) {
        const size_t t = base + (size_t)k * blockDim.x;
        if (t >= pairs) break;
        const size_t e = 2 * t;
        const int j0 = (int)(e / W), c0 = (int)(e - (size_t)j0 * W);
        const int j1 = c0 + 1 == W ? j0 + 1 : j0, c1 = c0 + 1 == W ? 0 : c0 + 1;
        double v0, v1;
        const bool w0 = lin_entry(f, nx, ny, j0, c0, v0), w1 = lin_entry(f, nx, ny, j1, c1, v1);
        if (w0 && w1) {
          __stcs(host2 + t, make_double2(v0, v1));
        } else {
          if (w0) f.host[e] = v0;
          if (w1) f.host[e + 1] = v1;
        }
      }
    } else {
      double2 v[kLinPairs];
#pragma unroll
      for (int k = 0; k < kLinPairs; ++k) {
        const size_t t = base + (size_t)k * blockDim.x;
        if (t < pairs) v[k] = __ldcs(host2 + t);
      }
#pragma unroll
      for (int k = 0; k < kLinPairs; ++k) {
        const size_t t = base + (size_t)k * blockDim.x;
        if (t >= pairs) break;
        const double vv[2] = {v[k].x, v[k].y};
#pragma unroll
        for (int h = 0; h < 2; ++h) {
          const size_t e = 2 * t + h;
          const int j = (int)(e / W), c = (int)(e - (size_t)j * W);
          if (j < 1 || j > ny) continue;
          // interior columns: ux c = 1..itot-1 (device x = c; x = 0 is the
          // wall i = 1, kept at 0), the others c = 1..itot (x = c - 1)
          if (f.kind == LIN_UX) {
            if (c >= 1 && c <= nx - 1) f.dev[(size_t)(j - 1) * nx + c] = vv[h];
          } else if (c >= 1 && c <= nx) {
            f.dev[(size_t)(j - 1) * nx + c - 1] = vv[h];
          }
        }
      }
    }
  }
}

cudaError_t launch_lin(const LinList &L, int to_host, cudaStream_t st) {
  if (L.n <= 0) return cudaSuccess;
  int dev = 0, sms = 152;
  if (cudaGetDevice(&dev) == cudaSuccess) cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  size_t most = 0;
  for (int k = 0; k < L.n; ++k) most = std::max(most, (size_t)(L.ny + 2) * L.f[k].W / 2);
  const size_t per_block = 256 * (size_t)kLinPairs;
  const int blocks = (int)std::max<size_t>(1, std::min<size_t>((most + per_block - 1) / per_block, 4 * sms / L.n));
  k_lin<<<dim3(blocks, L.n), 256, 0, st>>>(L, to_host);
  count_launches(1);
  return cudaGetLastError();
}

// TEMPFORCEX(i, j) = 0.5*TEMP(i-1, j) + 0.5*TEMP(i, j), i = 2..itot
__global__ void __launch_bounds__(256) k_tempforce(int nx, int ny, const double *t, double *out) {
  const size_t w = (size_t)nx - 1, total = w * ny;
  for (size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x; k < total; k += (size_t)gridDim.x * blockDim.x) {
    const size_t y = k / w, x = k - y * w;
    out[k] = 0.5 * t[y * nx + x] + 0.5 * t[y * nx + x + 1];
  }
}

cudaError_t launch_tempforce_to_host(const DevGrid &g, const double *t, double *host, cudaStream_t st) {
  if (g.nx < 2) return cudaSuccess;
  k_tempforce<<<2 * 152, 256, 0, st>>>(g.nx, g.ny, t, host);
  count_launches(1);
  return cudaGetLastError();
}

static int poisson_setup(const DevGrid &g, size_t *smem) {
  const int C = poisson_cols(g);
  *smem = (size_t)C * g.ny * sizeof(double);
  static bool attr_set = false;
  if (!attr_set) {
    const int lim = 160 * 1024;
    cudaFuncSetAttribute(k_poisson_fwd<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, lim);
    cudaFuncSetAttribute(k_poisson_fwd<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, lim);
    cudaFuncSetAttribute(k_poisson_bwd, cudaFuncAttributeMaxDynamicSharedMemorySize, lim);
    attr_set = true;
  }
  return C;
}

cudaError_t launch_poisson_fwd(const DevGrid &g, const StageScalars &s, const double *ux, const double *uy,
                               double2 *spec, cudaStream_t st) {
  size_t smem;
  const int C = poisson_setup(g, &smem);
  const PoissonArgs a{g, s, ux, uy, spec, nullptr, C};
  const int blocks = (g.nx + C - 1) / C;
  if (g.rcp) {
    k_poisson_fwd<true><<<blocks, poisson_threads(g, C), smem, st>>>(a);
  } else {
    k_poisson_fwd<false><<<blocks, poisson_threads(g, C), smem, st>>>(a);
  }
  count_launches(1);
  return cudaGetLastError();
}

cudaError_t launch_poisson_tri(const DevGrid &g, double2 *spec, cudaStream_t st) {
  static bool attr = false;
  const size_t smem = sizeof(TriRing) + sizeof(double) * (size_t)g.nx;
  if (!attr) {
    cudaFuncSetAttribute(k_poisson_tri, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)(sizeof(TriRing) + sizeof(double) * (size_t)kTriMaxNx));
    attr = true;
  }
  k_poisson_tri<<<dim3((g.nh + 31) / 32, 2), 32, smem, st>>>(g, spec);
  count_launches(1);
  return cudaGetLastError();
}

static int fused_cols(const DevGrid &g) {
  return (g.nx > 1024 && (size_t)2 * g.ny * sizeof(double) <= 160 * 1024) ? 2 : 1;
}

void fused_layout(const DevGrid &g, int *groups, int *spans) {
  const int C = fused_cols(g);
  *groups = (g.nx + C - 1) / C;
  *spans = (g.nx + kFusedSpanMin - 1) / kFusedSpanMin;
}

cudaError_t launch_poisson_fused(const DevGrid &g, const StageScalars &s, const double *ux, const double *uy,
                                 double2 *spec, double *psi, const double *t_in, double *t_out, double *at,
                                 const double *ux_k, const double *uy_k, FusedState &fs, cudaStream_t st) {
  int dev = 0, sms = 0, coop = 0;
  cudaError_t e;
  if ((e = cudaGetDevice(&dev)) != cudaSuccess) return e;
  if ((e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess) return e;
  if ((e = cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev)) != cudaSuccess) return e;
  const int C = fused_cols(g);
  const int lines = 2 * ((g.nh + 31) / 32);
  // two sweep warps per block when that still leaves kFusedMinWorkers workers
  const int tri_warps = sms - (lines + 1) / 2 >= kFusedMinWorkers ? 2 : kFusedTriWarps;
  const int tri_blocks = (lines + tri_warps - 1) / tri_warps;
  const size_t smem = std::max({sizeof(double) * (size_t)g.nx, (size_t)C * g.ny * sizeof(double), kFusedMinSmem});
  if (!coop || g.nx > kTriMaxNx || smem > 200 * 1024 || sms - tri_blocks < 8) return cudaErrorNotSupported;
  static bool attr = false;
  if (!attr) {
    cudaFuncSetAttribute(k_poisson_fused<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
    cudaFuncSetAttribute(k_poisson_fused<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
    attr = true;
  }
  int per_sm = 0;
  if ((e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, g.rcp ? (const void *)k_poisson_fused<true>
                                                                        : (const void *)k_poisson_fused<false>,
                                                         kFusedThreads, smem)) != cudaSuccess)
    return e;
  if (per_sm < 1) return cudaErrorNotSupported;
  FusedArgs a{};
  a.p = PoissonArgs{g, s, ux, uy, spec, psi, C};
  a.t = TempArgs{g, s, t_in, t_out, at, nullptr, ux_k, uy_k};
  a.with_temp = t_out != nullptr;
  a.fwd_done = fs.fwd_done;
  a.bwd_cnt = fs.bwd_cnt;
  a.err = fs.err;
  a.epoch = ++fs.epoch;
  a.spin = fs.spin_limit ? fs.spin_limit : kFusedSpin;
  a.want = a.epoch + (fs.stale ? 1u : 0u);
  fs.stale = 0;  // a test's stale wait applies to one launch
  a.tri_blocks = tri_blocks;
  a.tri_warps = tri_warps;
  a.lines = lines;
  int spans = 0;
  SNS_PLAIN_FORM::fused_layout(g, &a.groups, &spans);
  // the larger span when the workers can take all of its column groups at once
  a.span_shift = ((1 << kFusedSpanShiftMax) / C <= sms - tri_blocks) ? kFusedSpanShiftMax : kFusedSpanShiftMax - 1;
  void *args[] = {&a};
  e = cudaLaunchCooperativeKernel(g.rcp ? (const void *)k_poisson_fused<true> : (const void *)k_poisson_fused<false>,
                                  dim3(sms), dim3(kFusedThreads), args, smem, st);
  if (e != cudaSuccess) {
    --fs.epoch;
    return e;
  }
  count_launches(1);
  return cudaSuccess;
}

cudaError_t launch_poisson_bwd(const DevGrid &g, const StageScalars &s, const double2 *spec, double *psi,
                               cudaStream_t st) {
  size_t smem;
  const int C = poisson_setup(g, &smem);
  const PoissonArgs a{g, s, nullptr, nullptr, const_cast<double2 *>(spec), psi, C};
  const int blocks = (g.nx + C - 1) / C;
  k_poisson_bwd<<<blocks, poisson_threads(g, C), smem, st>>>(a);
  count_launches(1);
  return cudaGetLastError();
}

template <bool CORR, bool PRES>
static cudaError_t launch_corr_t(const DevGrid &g, const StageScalars &s, int impx, int impy, const double *psi,
                                 double *ux, double *uy, double *p, unsigned long long *colmax,
                                 unsigned long long *uymax, cudaStream_t st) {
  const CorrArgs a{g, s, psi, ux, uy, p, colmax, uymax};
  const dim3 grid = march_grid(g, kCorrRows), block(kBlockX);
#define SNS_C(X, Y, R) k_corr<X, Y, R, CORR, PRES><<<grid, block, 0, st>>>(a)
  if (g.rcp) {
    if (impx && impy) SNS_C(1, 1, true);
    else if (impx) SNS_C(1, 0, true);
    else if (impy) SNS_C(0, 1, true);
    else SNS_C(0, 0, true);
  } else {
    if (impx && impy) SNS_C(1, 1, false);
    else if (impx) SNS_C(1, 0, false);
    else if (impy) SNS_C(0, 1, false);
    else SNS_C(0, 0, false);
  }
#undef SNS_C
  count_launches(1);
  return cudaGetLastError();
}

cudaError_t launch_correct(const DevGrid &g, const StageScalars &s, const double *psi, double *ux, double *uy,
                           cudaStream_t st) {
  return launch_corr_t<true, false>(g, s, 0, 0, psi, ux, uy, nullptr, nullptr, nullptr, st);
}

cudaError_t launch_pressure(const DevGrid &g, const StageScalars &s, int impx, int impy, const double *psi,
                            double *p, cudaStream_t st) {
  return launch_corr_t<false, true>(g, s, impx, impy, psi, nullptr, nullptr, p, nullptr, nullptr, st);
}

cudaError_t launch_correct_pressure(const DevGrid &g, const StageScalars &s, int impx, int impy,
                                    const double *psi, double *ux, double *uy, double *p,
                                    unsigned long long *colmax, unsigned long long *uymax, cudaStream_t st) {
  return launch_corr_t<true, true>(g, s, impx, impy, psi, ux, uy, p, colmax, uymax, st);
}

cudaError_t launch_umax(const DevGrid &g, const double *ux, const double *uy, unsigned long long *colmax,
                        unsigned long long *uymax, cudaStream_t st) {
  k_umax<<<march_grid(g), kBlockX, 0, st>>>(g.nx, g.ny, ux, uy, colmax, uymax);
  count_launches(1);
  return cudaGetLastError();
}

}  // namespace SNS_PLAIN_FORM
}  // namespace sns
