"""Two more schemes of the CUDA kernels, restated on the CPU.

* Mixed radix (dr_mix.cu): for n = N1 N2 (N1 = 3 or 5), with n = n1 + N1 n2
  and k = k2 + N2 k1, X[k2 + N2 k1] = sum_n1 WN1^(n1 k1) Wn^(n1 k2) Y_n1[k2],
  Y_n1 the N2-point DFT of x[n1::N1]: checked against numpy's FFT.
* Split BF16 (grid_mma.cu): each FP32 operand x becomes hi = bf16(x) and
  lo = bf16(x - hi); a product is hi*hi + hi*lo + lo*hi accumulated in FP32
  (the tensor cores' three MMAs).  Checked: the representation error is at
  most 2^-16 relative, and a K = 256 contraction of unit-modulus phases with
  projection values (the gridding's E_u . P) stays far inside the 1e-4 bar
  against FP64."""
import numpy as np
import pytest


@pytest.mark.parametrize("N1", [3, 5])
@pytest.mark.parametrize("N2", [64, 128, 512])
@pytest.mark.parametrize("inv", [False, True])
def test_mixed_radix_decimation(N1, N2, inv):
    n = N1 * N2
    rng = np.random.default_rng(n + inv)
    x = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    sgn = 1 if inv else -1
    Y = np.stack([(np.fft.ifft(x[n1::N1]) * N2 if inv else np.fft.fft(x[n1::N1])) for n1 in range(N1)])
    X = np.empty(n, complex)
    for k1 in range(N1):
        for k2 in range(N2):
            X[k2 + N2 * k1] = sum(np.exp(sgn * 2j * np.pi * n1 * k1 / N1) * np.exp(sgn * 2j * np.pi * n1 * k2 / n)
                                  * Y[n1, k2] for n1 in range(N1))
    ref = np.fft.ifft(x) * n if inv else np.fft.fft(x)
    assert np.abs(X - ref).max() <= 1e-12 * np.abs(ref).max()


def bf16(x):
    """Round FP32 values to BF16 (nearest, ties to even), returned as FP32."""
    u = np.asarray(x, dtype=np.float32).view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return r.astype(np.uint32).view(np.float32)


def split(x):
    x = np.asarray(x, dtype=np.float32)
    hi = bf16(x)
    lo = bf16((x - hi).astype(np.float32))
    return hi, lo


def test_split_representation_error():
    rng = np.random.default_rng(1)
    x = (rng.standard_normal(100000) * np.exp(rng.uniform(-20, 20, 100000))).astype(np.float32)
    hi, lo = split(x)
    err = np.abs(x.astype(np.float64) - hi.astype(np.float64) - lo.astype(np.float64))
    assert np.all(err <= 2.0 ** -16 * np.abs(x.astype(np.float64)))


def test_split_contraction_error():
    """F = sum_a E(a) P(a) with |E| = 1 and P >= 0 (a projection row), in
    three BF16 products per term with FP32 accumulation."""
    rng = np.random.default_rng(2)
    K, rows = 256, 400
    phase = rng.uniform(0, 1, (rows, K))
    Er = np.cos(2 * np.pi * phase).astype(np.float32)
    Ei = np.sin(2 * np.pi * phase).astype(np.float32)
    P = rng.random(K).astype(np.float32)
    ph, pl = split(P)
    out = []
    for E in (Er, Ei):
        eh, el = split(E)
        acc = np.zeros(rows, np.float32)
        for a in range(K):      # FP32 accumulation term by term
            acc = (acc + (eh[:, a] * ph[a] + eh[:, a] * pl[a] + el[:, a] * ph[a]).astype(np.float32)).astype(np.float32)
        out.append(acc.astype(np.float64))
    got = out[0] + 1j * out[1]
    ref = (Er.astype(np.float64) + 1j * Ei.astype(np.float64)) @ P.astype(np.float64)
    rel = np.linalg.norm(got - ref) / np.linalg.norm(ref)
    assert rel < 1e-5
