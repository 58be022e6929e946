"""The Fourier constraint and errK on the half spectrum (apply_table in
genfire_gb300/csrc/fft_reg.cuh, with the table of dr.cu), restated on the CPU
against the reference's full-spectrum form (reconstruct.m:133-165):
k = fftn(x); k(C) = M(C); x' = real(ifftn(k)).  On the stored half
(q1 <= n1/2) each point becomes (A + B)/2 with A = M(q) if q is in C (else
k(q)) and B = conj M(-q) if -q is in C (else k(q)), which is the Hermitian
part that real() keeps; errK counts a stored point q if q is in E and its
mirror -q separately when -q is in E but not stored (|k(-q)| = |k(q)|).
Checked for even and odd sizes, symmetric and asymmetric constraint sets."""
import numpy as np
import pytest


def neg_index(n):
    return (-np.arange(n)) % n


@pytest.mark.parametrize("shape", [(6, 5, 4), (7, 7, 7), (8, 6, 9), (5, 4, 6)])
@pytest.mark.parametrize("symmetric", [True, False])
def test_half_spectrum_constraint_equals_full(shape, symmetric):
    n1, n2, n3 = shape
    rng = np.random.default_rng(sum(shape) + symmetric)
    x = rng.standard_normal(shape)
    k = np.fft.fftn(x)
    M = rng.standard_normal(shape) + 1j * rng.standard_normal(shape)
    C = rng.random(shape) < 0.4
    E = rng.random(shape) < 0.5
    i1, i2, i3 = neg_index(n1), neg_index(n2), neg_index(n3)
    mirror = lambda a: a[np.ix_(i1, i2, i3)]
    if symmetric:
        C = C | mirror(C)
        E = E | mirror(E)
        M = 0.5 * (M + np.conj(mirror(M)))          # a Hermitian measured grid
    # the reference, full spectrum
    kf = k.copy()
    kf[C] = M[C]
    x_ref = np.real(np.fft.ifftn(kf))
    errK_ref = np.abs(np.abs(k[E]) - np.abs(M[E])).sum()
    # the half spectrum: q1 = 0 .. n1//2 stored
    h1 = n1 // 2 + 1
    kh = k[:h1]
    Mn = mirror(M)                                   # Mn[q] = M(-q)
    Cn, En = mirror(C), mirror(E)
    out = kh.copy()
    errK = 0.0
    for q1 in range(h1):
        stored_mirror = (-q1) % n1 < h1              # -q is itself a stored point
        for q2 in range(n2):
            for q3 in range(n3):
                kq = kh[q1, q2, q3]
                if E[q1, q2, q3]:
                    errK += abs(abs(kq) - abs(M[q1, q2, q3]))
                if En[q1, q2, q3] and not stored_mirror:
                    errK += abs(abs(kq) - abs(Mn[q1, q2, q3]))
                a = M[q1, q2, q3] if C[q1, q2, q3] else kq
                b = np.conj(Mn[q1, q2, q3]) if Cn[q1, q2, q3] else kq
                if C[q1, q2, q3] or Cn[q1, q2, q3]:
                    out[q1, q2, q3] = 0.5 * (a + b)
    # the stored half of a Hermitian spectrum determines the real object
    full = np.zeros(shape, complex)
    full[:h1] = out
    for q1 in range(h1, n1):
        full[q1] = np.conj(out[(-q1) % n1][np.ix_(i2, i3)])
    x_half = np.real(np.fft.ifftn(full))
    assert np.abs(x_half - x_ref).max() < 1e-12 * max(1.0, np.abs(x_ref).max())
    assert abs(errK - errK_ref) < 1e-10 * max(1.0, errK_ref)
