"""Two more schemes of the CUDA kernels, restated on the CPU.

* Mixed radix (dr_mix.cu): for n = N1 N2 (N1 = 3 or 5), with n = n1 + N1 n2
  and k = k2 + N2 k1, X[k2 + N2 k1] = sum_n1 WN1^(n1 k1) Wn^(n1 k2) Y_n1[k2],
  Y_n1 the N2-point DFT of x[n1::N1]: checked against numpy's FFT.
* Split BF16 (grid_mma.cu): each FP32 operand x becomes hi = bf16(x) and
  lo = bf16(x - hi); a product is hi*hi + hi*lo + lo*hi accumulated in FP32
  (the tensor cores' three MMAs).  Checked: the representation error is at
  most 2^-16 relative, and a K = 256 contraction of unit-modulus phases with
  projection values (the gridding's E_u . P) stays far inside the 1e-4 bar
  against FP64.
* Split FP16 with per-projection scaling (GENFIRE_PREC_FP16_SCALED): the
  power-of-two scale keeps the hi and lo parts in FP16's normal range for
  amplitudes from 1e-7 to 1e7, and the products needed: one or two FP16
  products miss 1e-4, three are below 1e-6 and well below split BF16."""
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


# ---------------------------------------------------------------------------
# Split FP16 with per-projection scaling (GENFIRE_PREC_FP16_SCALED, grid_mma.cu):
# P is scaled by 2^(14 - e) with max|P| < 2^e, so every hi and lo part stays in
# FP16's normal range; the scale is undone exactly after the contraction.

def fp16_split(x):
    x = np.asarray(x, dtype=np.float32)
    hi = x.astype(np.float16).astype(np.float32)
    lo = (x - hi).astype(np.float32).astype(np.float16).astype(np.float32)
    return hi, lo


def proj_scale(P):
    """The kernel's per-projection scale: 2^(14 - e) with max|P| = f 2^e, f in [0.5, 1)."""
    m = float(np.max(np.abs(P)))
    if m == 0:
        return 1.0
    _, e = np.frexp(np.float32(m))
    return float(np.ldexp(1.0, 14 - int(e)))


@pytest.mark.parametrize("amp", [1e-7, 1.0, 1e7])
def test_fp16_scale_keeps_parts_normal(amp):
    rng = np.random.default_rng(5)
    P = (rng.random(4096) * amp).astype(np.float32)
    s = proj_scale(P)
    hi, lo = fp16_split(P * np.float32(s))
    assert np.max(np.abs(P * s)) < 2.0 ** 14
    assert np.all(np.isfinite(hi)) and np.all(np.isfinite(lo))
    err = np.abs((P * s).astype(np.float64) - hi.astype(np.float64) - lo.astype(np.float64))
    big = np.abs(P * s) >= 2.0 ** -3     # values whose lo part is a normal FP16 number
    assert np.all(err[big] <= 2.0 ** -21 * np.abs(P * s)[big])


def _contract(E_re, E_im, P, split_e, split_p, products):
    out = []
    ph, pl = split_p(P)
    for E in (E_re, E_im):
        eh, el = split_e(E)
        terms = {"hh": eh * ph[None, :], "hl": eh * pl[None, :], "lh": el * ph[None, :]}
        acc = np.zeros(E.shape[0], np.float32)
        for a in range(E.shape[1]):
            t = np.zeros(E.shape[0], np.float32)
            for k in products:
                t = (t + terms[k][:, a]).astype(np.float32)
            acc = (acc + t).astype(np.float32)
        out.append(acc.astype(np.float64))
    return out[0] + 1j * out[1]


def test_fp16_products_error_model():
    """The error study behind three products: on unit-modulus phases against a
    non-negative projection row, one FP16 product misses 1e-4 (each operand's
    rounding alone is ~2e-4 relative), two products still miss it, three are
    far inside it and well below split BF16."""
    rng = np.random.default_rng(6)
    K, rows = 256, 500
    phase = rng.uniform(0, 1, (rows, K))
    Er = np.cos(2 * np.pi * phase).astype(np.float32)
    Ei = np.sin(2 * np.pi * phase).astype(np.float32)
    P = (rng.random(K) * 37.0).astype(np.float32)
    s = np.float32(proj_scale(P))
    Ps = (P * s).astype(np.float32)
    ref = (Er.astype(np.float64) + 1j * Ei.astype(np.float64)) @ P.astype(np.float64)

    def rel(got):
        return np.linalg.norm(got / float(s) - ref) / np.linalg.norm(ref)
    e1 = rel(_contract(Er, Ei, Ps, fp16_split, fp16_split, ["hh"]))
    e2 = rel(_contract(Er, Ei, Ps, fp16_split, fp16_split, ["hh", "hl"]))
    e3 = rel(_contract(Er, Ei, Ps, fp16_split, fp16_split, ["hh", "hl", "lh"]))
    eb = np.linalg.norm(_contract(Er, Ei, P, split, split, ["hh", "hl", "lh"]) - ref) / np.linalg.norm(ref)
    assert e1 > 1e-4 and e2 > 1e-4
    assert e3 < 1e-6 and e3 < 0.2 * eb
