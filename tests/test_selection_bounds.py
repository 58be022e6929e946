"""The selection kernels' candidate interval (row_range in
genfire_gb300/csrc/grid.cu), restated on the CPU in FP32: for a row (K2, K3)
of the half grid, every k1 whose exact FP32 plane test passes
(D = |(k1 h0 + K2 h1) + K3 h2| < cutoff, each operation rounded, as sel_test
evaluates it) must lie inside [k1a, k1b], whichever way the device contracts
K2 h1 + K3 h2 into a fused multiply-add.  Checked against brute force over
random planes, grid sizes up to 2048 and the near-parallel branch
(|h0| < 0.01)."""
import numpy as np
import pytest

f32 = np.float32


def fma32(a, b, c):
    # a * b is exact in double for FP32 inputs; one rounding of the sum
    return f32(np.float64(a) * np.float64(b) + np.float64(c))


def row_range(h, K2, K3, lo, hi, cut_margin, contract):
    """The kernel's interval, with x formed without FMA (0) or with one of the
    two contractions (1: fma(K2, h1, K3 h2), 2: fma(K3, h2, K2 h1))."""
    if contract == 0:
        x = -(f32(K2 * h[1]) + f32(K3 * h[2]))
    elif contract == 1:
        x = -fma32(K2, h[1], f32(K3 * h[2]))
    else:
        x = -fma32(K3, h[2], f32(K2 * h[1]))
    x = f32(x)
    c = cut_margin
    h1 = h[0]
    if abs(h1) >= f32(0.01):
        ih = f32(f32(1.0) / h1)
        b0, b1 = f32(f32(x - c) * ih), f32(f32(x + c) * ih)
        if b0 > b1:
            b0, b1 = b1, b0
        b0 = max(b0, f32(lo) - f32(4))
        b1 = min(b1, f32(hi) + f32(4))
        return max(lo, int(np.floor(b0)) - 1), min(hi, int(np.ceil(b1)) + 1)
    reach = f32(abs(h1) * f32(max(-lo, hi)))
    if abs(x) > f32(c + reach):
        return 1, 0
    return lo, hi


def passing(h, K2, K3, lo, hi, cut_lt):
    k1 = np.arange(lo, hi + 1, dtype=np.float32)
    D = np.abs((k1 * h[0] + f32(K2) * h[1]).astype(np.float32) + f32(K3) * h[2]).astype(np.float32)
    return k1[D < cut_lt].astype(int)


def cut_thresholds(cutoff):
    cut_lt = f32(cutoff)
    if np.float64(cut_lt) < cutoff:
        cut_lt = np.nextafter(cut_lt, f32(np.inf))
    return cut_lt, f32(f32(cutoff) + f32(0.01))


@pytest.mark.parametrize("n", [64, 129, 512, 1024, 2048])
@pytest.mark.parametrize("cutoff", [0.125, 0.7])
def test_candidate_interval_is_conservative(n, cutoff):
    rng = np.random.default_rng(n + int(cutoff * 1000))
    lo, hi = -(n // 2), 0                           # k1 <= 0 half of the centrosymmetric grid
    lo2, hi2 = -(n // 2), n // 2
    cut_lt, margin = cut_thresholds(cutoff)
    checked = 0
    for trial in range(40):
        v = rng.standard_normal(3)
        if trial % 8 == 0:
            v[0] *= 1e-3                            # near-parallel planes: the |h0| < 0.01 branch
        if trial % 8 == 1:
            v[0] = 0.0101 * np.linalg.norm(v[1:])   # just above the branch threshold
        h = (v / np.linalg.norm(v)).astype(np.float32)
        for _ in range(60):
            K2 = int(rng.integers(lo2, hi2 + 1))
            K3 = int(rng.integers(lo2, hi2 + 1))
            hits = passing(h, K2, K3, lo, hi, cut_lt)
            for contract in (0, 1, 2):
                a, b = row_range(h, f32(K2), f32(K3), lo, hi, margin, contract)
                if len(hits):
                    assert a <= hits.min() and hits.max() <= b, (n, h, K2, K3, contract, a, b, hits)
            checked += len(hits)
    assert checked > 0
