// Device real FFT along y shared by the plain FP64 path and the FP32-stencil
// form (same algorithm and operation order as the CPU FFT of the oracle:
// radix-2/4 decimation in time on z[m] = x[2m] + i x[2m+1], in place in
// shared memory, then the real-FFT split step; FFTW's conventions).
// Translation units compiled with --fmad=false reproduce the CPU FFT bit for
// bit; others may contract multiply-adds.
#pragma once

namespace sns {
namespace fft {

// slot of element idx before the in-place decimation-in-time stages: digit
// reversal over the stage radices (2 first when log2(M) is odd, then 4s)
__device__ __forceinline__ int fft_slot(int idx, int M, int nst, int first2) {
  int rest = idx, span = M, slot = 0;
  for (int s = nst - 1; s >= 0; --s) {
    if (s == 0 && first2) {
      span >>= 1;
      slot += (rest & 1) * span;
      rest >>= 1;
    } else {
      span >>= 2;
      slot += (rest & 3) * span;
      rest >>= 2;
    }
  }
  return slot;
}

// One in-place DIT stage on `cols` columns of length M held in shared memory;
// the same floating-point operations as dit_stage() of the CPU FFT.
template <bool FWD>
__device__ __forceinline__ void fft_stages(double2 *z, int cols, int M, int N, int nst, int first2,
                                           const double2 *tw) {
  int L = 1, lg = 0;
  for (int st = 0; st < nst; ++st) {
    const int R = (st == 0 && first2) ? 2 : 4;
    const int span = R * L, tstep = N / span, nb = M / R;
    for (int b = threadIdx.x; b < cols * nb; b += blockDim.x) {
      const int c = b / nb, bb = b - c * nb;
      const int k = bb & (L - 1);
      const int base = c * M + (bb >> lg) * span + k;
      double vr[4], vi[4];
#pragma unroll
      for (int r = 0; r < 4; ++r) {
        if (r < R) {
          const double2 v = z[base + r * L];
          vr[r] = v.x;
          vi[r] = v.y;
        }
      }
      if (L > 1) {
#pragma unroll
        for (int r = 1; r < 4; ++r) {
          if (r < R) {
            const double2 w = tw[r * k * tstep];
            const double xr = vr[r], xi = vi[r];
            if (FWD) {
              vr[r] = xr * w.x - xi * w.y;
              vi[r] = xr * w.y + xi * w.x;
            } else {
              vr[r] = xr * w.x + xi * w.y;
              vi[r] = xi * w.x - xr * w.y;
            }
          }
        }
      }
      if (R == 2) {
        z[base] = make_double2(vr[0] + vr[1], vi[0] + vi[1]);
        z[base + L] = make_double2(vr[0] - vr[1], vi[0] - vi[1]);
      } else {
        const double t0r = vr[0] + vr[2], t0i = vi[0] + vi[2];
        const double t1r = vr[0] - vr[2], t1i = vi[0] - vi[2];
        const double t2r = vr[1] + vr[3], t2i = vi[1] + vi[3];
        const double t3r = vr[1] - vr[3], t3i = vi[1] - vi[3];
        const double sr = FWD ? t3i : -t3i;
        const double si = FWD ? -t3r : t3r;
        z[base] = make_double2(t0r + t2r, t0i + t2i);
        z[base + L] = make_double2(t1r + sr, t1i + si);
        z[base + 2 * L] = make_double2(t0r - t2r, t0i - t2i);
        z[base + 3 * L] = make_double2(t1r - sr, t1i - si);
      }
    }
    __syncthreads();
    L *= R;
    lg += (R == 2) ? 1 : 2;
  }
}


// split step of the forward real FFT for bin pair (k, M-k) of one column,
// k in [0, M/2]: X[k] from the half-length complex spectrum Z (natural order)
// (bins of one column at out[J * os])
__device__ __forceinline__ void rfft_post(const double2 *zc, double2 *out, int M, int k, const double2 *tw,
                                          size_t os = 1) {
  if (k == 0) {
    const double2 z0 = zc[0];
    out[0] = make_double2(z0.x + z0.y, 0.0);
    out[(size_t)M * os] = make_double2(z0.x - z0.y, 0.0);
  } else {
    const double2 A = zc[k], B = zc[M - k];
    const double sre = A.x + B.x, dim = A.y - B.y, dre = A.x - B.x, sim = A.y + B.y;
    const double er = 0.5 * sre, ei = 0.5 * dim;
    const double orr = 0.5 * sim, oi = -(0.5 * dre);
    const double2 w = tw[k];
    const double wor = w.x * orr - w.y * oi;
    const double woi = w.x * oi + w.y * orr;
    out[(size_t)k * os] = make_double2(er + wor, ei + woi);
    if (2 * k != M) out[(size_t)(M - k) * os] = make_double2(er - wor, woi - ei);
  }
}

// inverse split step for bin pair (k, M-k): Z slots (digit-reversed) from X
// (bins of one column at in[J * is]);
// imaginary parts of X[0] and X[M] are ignored (FFTW c2r convention)
// CG: load the input through L2 only (data written by other blocks of the running kernel)
template <bool CG = false>
__device__ __forceinline__ void rfft_pre(const double2 *in, double2 *zc, int M, int k, const double2 *tw, int nst,
                                         int first2, size_t is = 1) {
  auto ld = [](const double2 *p) -> double2 {
    if constexpr (CG) {
      return __ldcg(p);
    } else {
      return *p;
    }
  };
  if (k == 0) {
    const double x0r = ld(in).x, xmr = ld(in + (size_t)M * is).x;
    zc[0] = make_double2(x0r + xmr, x0r - xmr);
  } else {
    const double2 A = ld(in + (size_t)k * is), B = ld(in + (size_t)(M - k) * is);
    const double er = A.x + B.x, ei = A.y - B.y, dr = A.x - B.x, di = A.y + B.y;
    const double2 w = tw[k];
    const double orr = dr * w.x + di * w.y;
    const double oi = di * w.x - dr * w.y;
    zc[fft_slot(k, M, nst, first2)] = make_double2(er - oi, ei + orr);
    if (2 * k != M) zc[fft_slot(M - k, M, nst, first2)] = make_double2(er + oi, orr - ei);
  }
}

}  // namespace fft
}  // namespace sns
