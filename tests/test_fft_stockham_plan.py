"""The radix-8 Stockham FFT of csrc/fft_stockham.cuh, restated in numpy with
the kernels' index formulas, checked on the CPU against numpy's FFT:

* one pass of radix R over a column of M complex values with span Ns:
  butterfly j reads elements j + r M / R, multiplies input r by
  w^(r k) (k = j mod Ns, w = exp(-+2 pi i / (Ns R)), taken from the real
  FFT's twiddle table exp(-2 pi i t / (2 M)) at t = 2 r k M / (Ns R)),
  applies the R-point DFT and writes output r to (j - k) R + k + r Ns;
  radix-8 passes first, then one radix-4 or radix-2 pass;
* the split steps of the parallel form's transform pair (k_par_fwd8 /
  k_par_bwd8 in csrc/plain_parallel.cu): the forward leaves the real FFT's
  halving out (2 X), the inverse rebuilds 2 Z from X, and 1/(2 jtot) at the
  end gives the samples back;
* the shared-memory swizzle i ^ ((i >> 3) & 7) is a bijection within each
  aligned group of 8, so every pass's reads and writes land on distinct
  slots.
"""
import numpy as np
import pytest


def radices(M):
    out, rem = [], M
    while rem >= 8:
        out.append(8)
        rem //= 8
    if rem in (2, 4):
        out.append(rem)
    return out


def stockham(z, fwd):
    M = len(z)
    table = np.exp(-2j * np.pi * np.arange(2 * M) / (2 * M))
    Ns = 1
    for R in radices(M):
        nb = M // R
        out = np.empty_like(z)
        n = np.arange(R)
        dft = np.exp((-1 if fwd else 1) * 2j * np.pi * np.outer(n, n) / R)
        for j in range(nb):
            v = z[j + n * nb].copy()
            k = j & (Ns - 1)
            if Ns > 1:
                w = table[2 * n * k * (M // (Ns * R))]
                v = v * (w if fwd else np.conj(w))
            out[(j - k) * R + k + n * Ns] = dft @ v
        z = out
        Ns *= R
    return z


@pytest.mark.parametrize("M", [8, 16, 32, 64, 128, 256, 512, 1024, 2048])
def test_stockham_passes_equal_the_dft(M):
    rng = np.random.default_rng(M)
    z = rng.standard_normal(M) + 1j * rng.standard_normal(M)
    assert np.allclose(stockham(z, True), np.fft.fft(z), rtol=0, atol=1e-12 * np.sqrt(M))
    assert np.allclose(stockham(z, False), M * np.fft.ifft(z), rtol=0, atol=1e-12 * np.sqrt(M))


@pytest.mark.parametrize("ny", [16, 64, 1024, 4096])
def test_split_steps_and_final_scale(ny):
    M = ny // 2
    x = np.random.default_rng(ny).standard_normal(ny)
    Z = stockham(x[0::2] + 1j * x[1::2], True)
    X2 = np.empty(M + 1, complex)
    X2[0] = 2 * (Z[0].real + Z[0].imag)
    X2[M] = 2 * (Z[0].real - Z[0].imag)
    for k in range(1, M // 2 + 1):
        A, B = Z[k], Z[M - k]
        sre, dim, dre, sim = A.real + B.real, A.imag - B.imag, A.real - B.real, A.imag + B.imag
        w = np.exp(-2j * np.pi * k / ny)
        wor, woi = w.real * sim + w.imag * dre, w.imag * sim - w.real * dre
        X2[k] = complex(sre + wor, dim + woi)
        if 2 * k != M:
            X2[M - k] = complex(sre - wor, woi - dim)
    assert np.allclose(X2, 2 * np.fft.rfft(x), rtol=0, atol=1e-11)
    zc = np.empty(M, complex)
    zc[0] = complex(X2[0].real + X2[M].real, X2[0].real - X2[M].real)
    for k in range(1, M // 2 + 1):
        A, B = X2[k], X2[M - k]
        er, ei, dr, di = A.real + B.real, A.imag - B.imag, A.real - B.real, A.imag + B.imag
        w = np.exp(-2j * np.pi * k / ny)
        orr, oi = dr * w.real + di * w.imag, di * w.real - dr * w.imag
        zc[k] = complex(er - oi, ei + orr)
        if 2 * k != M:
            zc[M - k] = complex(er + oi, orr - ei)
    zz = stockham(zc, False) * (0.5 / ny)
    back = np.empty(ny)
    back[0::2], back[1::2] = zz.real, zz.imag
    assert np.allclose(back, x, rtol=0, atol=1e-12)


@pytest.mark.parametrize("M", [8, 64, 512, 4096])
def test_swizzle_is_a_bijection_per_group_of_eight(M):
    i = np.arange(M)
    s = i ^ ((i >> 3) & 7)
    assert sorted(s) == list(range(M))
    assert np.array_equal(s >> 3, i >> 3)
