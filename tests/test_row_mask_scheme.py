"""The row passes' support mask (k_row_support_mask in genfire_gb300/csrc/dr.cu,
row_pairs_empty / zero_half_rows in genfire_gb300/csrc/fft.cuh), restated on
the CPU.  The mask holds one byte per pair of real rows (rows 2p, 2p + 1 of the
B2 B3 rows of the box, the last pair of an odd count has one row), set when one
of the pair's rows holds a support voxel.  CTA b of every row-pass engine owns
the pairs [b W, (b + 1) W) (W the engine's pairs per CTA, a grid of
ceil(pairs / W) CTAs); it skips when none of its pairs is set.  A skipped
forward pass writes zero half spectra over exactly its rows and q < h1.

Checked: the skip decision equals "no support voxel in the CTA's rows", the
zero writes stay inside the half-spectrum buffer and cover exactly the rows
the skipped CTA owns, and a forward row pass over a supported object (rfft of
each row after the support constraint) is unchanged by the mask."""
import numpy as np
import pytest


def pair_mask(S, B1, nrows):
    """k_row_support_mask with two rows per entry: S is the box-shaped support
    flattened in column-major order (B1 fastest)."""
    rows = S.reshape(nrows, B1)
    npairs = (nrows + 1) // 2
    m = np.zeros(npairs, np.uint8)
    for p in range(npairs):
        m[p] = 1 if rows[2 * p:min(nrows, 2 * p + 2)].any() else 0
    return m


def cta_empty(mask, nrows, W, b):
    """row_pairs_empty for CTA b."""
    npairs = (nrows + 1) // 2
    any_ = 0
    for c in range(W):
        p = b * W + c
        if p < npairs:
            any_ |= int(mask[p])
    return any_ == 0


def zero_writes(nrows, h1, ld1, W, b):
    """The flat indices of Y that zero_half_rows writes for CTA b (its loop
    i = rr h1 + q over 2 W h1 entries, rows below nrows only)."""
    r0 = b * W * 2
    out = []
    for i in range(2 * W * h1):
        rr, q = divmod(i, h1)
        if r0 + rr < nrows:
            out.append((r0 + rr) * ld1 + q)
    return out


@pytest.mark.parametrize("B1,B2,B3", [(8, 6, 5), (7, 9, 3), (16, 16, 16), (5, 1, 1), (12, 10, 7)])
@pytest.mark.parametrize("W", [1, 2, 4, 8])
def test_skip_decision_and_zero_writes(B1, B2, B3, W):
    rng = np.random.default_rng(B1 * 1000 + B2 * 10 + B3 + W)
    nrows = B2 * B3
    N = 2 * B1
    h1 = N // 2 + 1
    ld1 = (h1 + 7) // 8 * 8
    for density in (0.0, 0.02, 0.2, 1.0):
        S = (rng.random(B1 * nrows) < density).astype(np.uint8)
        rows = S.reshape(nrows, B1)
        m = pair_mask(S, B1, nrows)
        npairs = (nrows + 1) // 2
        grid = -(-npairs // W)
        covered = set()
        for b in range(grid):
            own = range(2 * b * W, min(nrows, 2 * (b + 1) * W))
            assert cta_empty(m, nrows, W, b) == (not rows[list(own)].any())
            idx = zero_writes(nrows, h1, ld1, W, b)
            assert all(0 <= i < ld1 * nrows for i in idx)
            assert sorted(idx) == sorted(r * ld1 + q for r in own for q in range(h1))
            covered.update(own)
        assert covered == set(range(nrows))


@pytest.mark.parametrize("W", [1, 2, 8])
def test_masked_forward_pass_is_exact(W):
    """Rows outside the support are zero after the support constraint, so
    writing zero half spectra for them (instead of transforming) gives the same
    half spectrum as the unmasked pass."""
    rng = np.random.default_rng(5 + W)
    B1, B2, B3 = 12, 9, 7
    nrows = B2 * B3
    N = 2 * B1
    h1 = N // 2 + 1
    x = rng.standard_normal((nrows, B1))
    S = np.zeros((nrows, B1), np.uint8)
    S[rng.integers(0, nrows, 6), rng.integers(0, B1, 6)] = 1
    m = pair_mask(S.ravel(), B1, nrows)
    xs = np.zeros((nrows, N))
    xs[:, :B1] = x * S
    full = np.fft.rfft(xs, axis=1)
    Y = np.full((nrows, h1), np.nan + 0j)
    for b in range(-(-((nrows + 1) // 2) // W)):
        own = range(2 * b * W, min(nrows, 2 * (b + 1) * W))
        for r in own:
            Y[r] = 0 if cta_empty(m, nrows, W, b) else np.fft.rfft(xs[r])
    assert np.array_equal(Y, full)
