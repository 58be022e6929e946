"""The row passes' pairing of real rows (k_row_r2c_r32 / k_row_c2r_r32 in
genfire_gb300/csrc/fft_r32.cuh, and the register and generic row passes),
restated on the CPU: two real rows a, b travel as one complex transform
z = a + i b.  Forward: Xa(q) = (Z(q) + conj Z(-q)) / 2, Xb(q) = (Z(q) - conj Z(-q)) / 2i
for q < h1.  Inverse: Z(q) = Ha(q) + i Hb(q) for q < h1 and Z(N - q) =
conj Ha(q) + i conj Hb(q) where N - q is not a stored point, with the
imaginary parts of q = 0 and q = N/2 dropped, then the real and imaginary
parts of the inverse are the two rows.  Checked against numpy's rfft / irfft
for even and odd lengths and the half-spectrum widths the passes use."""
import numpy as np
import pytest


def forward_pair(a, b, h1):
    N = len(a)
    Z = np.fft.fft(a + 1j * b)
    Xa = np.empty(h1, complex)
    Xb = np.empty(h1, complex)
    for q in range(h1):
        z, zm = Z[q], Z[0 if q == 0 else N - q]
        Xa[q] = 0.5 * (z.real + zm.real) + 0.5j * (z.imag - zm.imag)
        Xb[q] = 0.5 * (z.imag + zm.imag) + 0.5j * (zm.real - z.real)
    return Xa, Xb


def inverse_pair(Ha, Hb, N):
    h1 = len(Ha)
    Z = np.zeros(N, complex)
    for q in range(h1):
        ha, hb = Ha[q], Hb[q]
        if q == 0 or 2 * q == N:
            ha, hb = complex(ha.real, 0.0), complex(hb.real, 0.0)
        Z[q] = complex(ha.real - hb.imag, ha.imag + hb.real)
        if q != 0 and N - q >= h1:
            Z[N - q] = complex(ha.real + hb.imag, hb.real - ha.imag)
    z = np.fft.ifft(Z)
    return z.real, z.imag


@pytest.mark.parametrize("N", [6, 7, 16, 64, 127, 128, 512])
def test_forward_pair_is_two_rffts(N):
    rng = np.random.default_rng(N)
    a, b = rng.standard_normal(N), rng.standard_normal(N)
    h1 = N // 2 + 1
    Xa, Xb = forward_pair(a, b, h1)
    assert np.abs(Xa - np.fft.rfft(a)).max() < 1e-12 * N
    assert np.abs(Xb - np.fft.rfft(b)).max() < 1e-12 * N


@pytest.mark.parametrize("N", [6, 7, 16, 64, 127, 128, 512])
def test_inverse_pair_is_two_irffts(N):
    rng = np.random.default_rng(N + 1)
    a, b = rng.standard_normal(N), rng.standard_normal(N)
    Ha, Hb = np.fft.rfft(a), np.fft.rfft(b)
    # spectra of real rows after a constraint may carry imaginary DC / Nyquist
    # parts; the pass drops them, as the real part of the full inverse would
    Ha[0] += 0.3j
    if N % 2 == 0:
        Hb[-1] -= 0.7j
    ra, rb = inverse_pair(Ha, Hb, N)
    assert np.abs(ra - np.fft.irfft(Ha, N)).max() < 1e-12
    assert np.abs(rb - np.fft.irfft(Hb, N)).max() < 1e-12
