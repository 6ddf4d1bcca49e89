// Complex FFT of length M (a power of two, 8 <= M) in shared memory by the
// Stockham autosort algorithm in radix-8 passes (then one radix-4 or radix-2
// pass), for the forms whose Poisson solve is held to a tolerance rather than
// to the reference's operation order. Each thread owns G groups of 8
// complex values per pass: it loads them, applies the pass's twiddles and the
// radix-R butterflies in registers, and after a barrier stores them in their
// sorted positions, so M = 512 takes 3 passes and needs no digit reversal.
// The first pass (span 1) has no twiddles, so the radix-8 passes come first.
//
// Shared memory holds element i of a column at swz(i) = i ^ ((i >> 3) & 7)
// (16-byte elements, 8 per bank row): every pass reads 8 consecutive elements
// of a row or writes one element in each of 8 consecutive rows, and the XOR
// spreads both over all banks.
//
// Twiddles come from the table exp(-2 pi i t / (2 M)), t < 2 M (the real
// FFT's table): w(t) for the length-M transform is entry 2 t.
#pragma once

namespace sns {
namespace fft8 {

__device__ __forceinline__ int swz(int i) { return i ^ ((i >> 3) & 7); }

__device__ __forceinline__ double2 cmul(double2 a, double2 w) {
  return make_double2(a.x * w.x - a.y * w.y, a.x * w.y + a.y * w.x);
}
__device__ __forceinline__ double2 cmulc(double2 a, double2 w) {  // a * conj(w)
  return make_double2(a.x * w.x + a.y * w.y, a.y * w.x - a.x * w.y);
}
__device__ __forceinline__ double2 add(double2 a, double2 b) { return make_double2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ double2 sub(double2 a, double2 b) { return make_double2(a.x - b.x, a.y - b.y); }
// a * (-i) (forward) or a * (+i) (inverse)
template <bool FWD>
__device__ __forceinline__ double2 rot(double2 a) {
  return FWD ? make_double2(a.y, -a.x) : make_double2(-a.y, a.x);
}

template <bool FWD>
__device__ __forceinline__ void dft2(double2 &a, double2 &b) {
  const double2 t = a;
  a = add(t, b);
  b = sub(t, b);
}

// 4-point DFT in place: v0..v3 -> X0..X3
template <bool FWD>
__device__ __forceinline__ void dft4(double2 &v0, double2 &v1, double2 &v2, double2 &v3) {
  const double2 s0 = add(v0, v2), s1 = sub(v0, v2), s2 = add(v1, v3), s3 = rot<FWD>(sub(v1, v3));
  v0 = add(s0, s2);
  v2 = sub(s0, s2);
  v1 = add(s1, s3);
  v3 = sub(s1, s3);
}

// 8-point DFT in place: v[n] -> X[k] = sum_n v[n] w8^(nk), w8 = exp(-+2 pi i / 8).
// Split n = j + 4 m: the even outputs are the 4-point DFT of a_j = v_j + v_j+4,
// the odd ones that of w8^j (v_j - v_j+4).
template <bool FWD>
__device__ __forceinline__ void dft8(double2 *v) {
  constexpr double r = 0.70710678118654752440;  // 1 / sqrt(2), correctly rounded
  double2 a0 = add(v[0], v[4]), a1 = add(v[1], v[5]), a2 = add(v[2], v[6]), a3 = add(v[3], v[7]);
  double2 b0 = sub(v[0], v[4]), b1 = sub(v[1], v[5]), b2 = sub(v[2], v[6]), b3 = sub(v[3], v[7]);
  // b1 *= w8, b2 *= w8^2 = -+i, b3 *= w8^3
  if (FWD) {
    b1 = make_double2((b1.x + b1.y) * r, (b1.y - b1.x) * r);
    b3 = make_double2((b3.y - b3.x) * r, -(b3.x + b3.y) * r);
  } else {
    b1 = make_double2((b1.x - b1.y) * r, (b1.x + b1.y) * r);
    b3 = make_double2(-(b3.x + b3.y) * r, (b3.x - b3.y) * r);
  }
  b2 = rot<FWD>(b2);
  dft4<FWD>(a0, a1, a2, a3);
  dft4<FWD>(b0, b1, b2, b3);
  v[0] = a0;
  v[2] = a1;
  v[4] = a2;
  v[6] = a3;
  v[1] = b0;
  v[3] = b1;
  v[5] = b2;
  v[7] = b3;
}

// One Stockham pass of radix R over `cols` columns of length M at z (column
// c at z + c M, swizzled), span Ns (the length of the sub-transforms already
// done). Thread t handles butterflies t + q blockDim.x, q < G 8 / R (up to G
// groups of 8 values; the block needs at least cols M / (8 G) threads).
// Butterfly j of a column reads elements j + r M / R, multiplies input r by
// w^(r k) with k = j mod Ns and w = exp(-+2 pi i / (Ns R)), and writes
// output r to (j - k) R + k + r Ns.
template <int R, bool FWD, int G>
__device__ __forceinline__ void pass(double2 *z, int cols, int M, int Ns, const double2 *tw) {
  constexpr int per = G * 8 / R;
  const int nb = M / R, total = cols * nb;
  double2 v[8 * G];
  int dst[8 * G];
#pragma unroll
  for (int q = 0; q < per; ++q) {
    const int b = threadIdx.x + q * blockDim.x;
    double2 *u = v + q * R;
    if (b >= total) {
#pragma unroll
      for (int r = 0; r < R; ++r) dst[q * R + r] = -1;
      continue;
    }
    const int c = b / nb, j = b - c * nb;
    const double2 *zc = z + (size_t)c * M;
#pragma unroll
    for (int r = 0; r < R; ++r) u[r] = zc[swz(j + r * nb)];
    const int k = j & (Ns - 1);
    if (Ns > 1) {
      // w^(r k) = exp(-+2 pi i r k / (Ns R)) = table entry 2 r k M / (Ns R)
      const int step = 2 * (M / (Ns * R)) * k;
#pragma unroll
      for (int r = 1; r < R; ++r) {
        const double2 w = tw[r * step];
        u[r] = FWD ? cmul(u[r], w) : cmulc(u[r], w);
      }
    }
    if constexpr (R == 8) {
      dft8<FWD>(u);
    } else if constexpr (R == 4) {
      dft4<FWD>(u[0], u[1], u[2], u[3]);
    } else {
      dft2<FWD>(u[0], u[1]);
    }
    const int base = c * M + (j - k) * R + k;
#pragma unroll
    for (int r = 0; r < R; ++r) dst[q * R + r] = base + r * Ns;
  }
  __syncthreads();
#pragma unroll
  for (int i = 0; i < 8 * G; ++i) {
    const int d = dst[i];
    if (d < 0) continue;
    const int c0 = d & ~(M - 1);  // column base: M is a power of two
    z[c0 + swz(d - c0)] = v[i];
  }
  __syncthreads();
}

// the whole transform of `cols` columns: radix-8 passes, then one radix-4
// or radix-2 pass; the block has at least cols M / (8 G) threads
template <bool FWD, int G>
__device__ __forceinline__ void transform(double2 *z, int cols, int M, const double2 *tw) {
  int Ns = 1, rem = M;
  for (; rem >= 8; rem >>= 3) {
    pass<8, FWD, G>(z, cols, M, Ns, tw);
    Ns <<= 3;
  }
  if (rem == 4) {
    pass<4, FWD, G>(z, cols, M, Ns, tw);
  } else if (rem == 2) {
    pass<2, FWD, G>(z, cols, M, Ns, tw);
  }
}

// split step of the forward real FFT for the bin pair (k, M-k), k in
// [0, M/2]: X[k] (FFTW's unnormalised transform of the 2 M real values
// z[m] = x[2m] + i x[2m+1]) from the column's FFT Z in natural order,
// written to out[J os]; w^k = exp(-2 pi i k / (2 M)) is table entry k
__device__ __forceinline__ void rfft_post(const double2 *zc, double2 *out, int M, int k, const double2 *tw,
                                          size_t os) {
  if (k == 0) {
    const double2 z0 = zc[0];
    out[0] = make_double2(z0.x + z0.y, 0.0);
    out[(size_t)M * os] = make_double2(z0.x - z0.y, 0.0);
  } else {
    const double2 A = zc[swz(k)], B = zc[swz(M - k)];
    const double er = 0.5 * (A.x + B.x), ei = 0.5 * (A.y - B.y);
    const double orr = 0.5 * (A.y + B.y), oi = -(0.5 * (A.x - B.x));
    const double2 w = tw[k];
    const double wor = w.x * orr - w.y * oi;
    const double woi = w.x * oi + w.y * orr;
    out[(size_t)k * os] = make_double2(er + wor, ei + woi);
    if (2 * k != M) out[(size_t)(M - k) * os] = make_double2(er - wor, woi - ei);
  }
}

// inverse split step for the bin pair (k, M-k): 2 Z[k] in natural order from
// X (read at in[J is]); the imaginary parts of X[0] and X[M] are ignored
// (FFTW's c2r convention)
__device__ __forceinline__ void rfft_pre(const double2 *in, double2 *zc, int M, int k, const double2 *tw, size_t is) {
  if (k == 0) {
    const double x0r = in[0].x, xmr = in[(size_t)M * is].x;
    zc[0] = make_double2(x0r + xmr, x0r - xmr);
  } else {
    const double2 A = in[(size_t)k * is], B = in[(size_t)(M - k) * is];
    const double er = A.x + B.x, ei = A.y - B.y, dr = A.x - B.x, di = A.y + B.y;
    const double2 w = tw[k];
    const double orr = dr * w.x + di * w.y;
    const double oi = di * w.x - dr * w.y;
    zc[swz(k)] = make_double2(er - oi, ei + orr);
    if (2 * k != M) zc[swz(M - k)] = make_double2(er + oi, orr - ei);
  }
}

}  // namespace fft8
}  // namespace sns
