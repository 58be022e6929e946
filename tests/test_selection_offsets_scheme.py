"""The selection's output offsets (grid.cu: k_sel_count, the CUB scan, k_sel_totals,
k_sel_offsets, k_sel_write), restated on the CPU.

Row counts are uint16 per (projection, row) of a batch; one exclusive scan in
uint32 arithmetic gives every row's offset, which may wrap modulo 2^32 across the
batch.  A projection holds fewer than 2^31 points, so its count and each row's
offset within it are exact as differences modulo 2^32; the global offset is the
projection's first offset (an int64 prefix over the counts) plus that difference.
Checked against int64 arithmetic on a batch whose total exceeds 2^32."""
import numpy as np


def scheme(counts):
    """counts: (P, nrows) uint16 -> (nk int64[P], doff int64[P+1], offsets int64[P, nrows])."""
    P, nrows = counts.shape
    flat = counts.reshape(-1).astype(np.uint64)
    rowoff = ((np.cumsum(flat) - flat) % (1 << 32)).astype(np.uint32)          # the uint32 scan
    last = P * nrows - 1
    end = np.uint32((int(rowoff[last]) + int(flat[last])) % (1 << 32))
    nk = np.empty(P, np.int64)
    for q in range(P):                                                           # k_sel_totals
        b = rowoff[q * nrows]
        e = rowoff[(q + 1) * nrows] if q + 1 < P else end
        nk[q] = (int(e) - int(b)) % (1 << 32)
    doff = np.concatenate([[0], np.cumsum(nk)])                                  # k_sel_offsets
    off = np.empty((P, nrows), np.int64)
    for q in range(P):                                                           # k_sel_write
        first = rowoff[q * nrows]
        off[q] = doff[q] + (rowoff[q * nrows:(q + 1) * nrows] - first).astype(np.uint32).astype(np.int64)
    return nk, doff, off


def test_offsets_exact_when_the_batch_total_wraps():
    rng = np.random.default_rng(3)
    P, nrows = 3, 65000
    counts = rng.integers(30000, 32770, size=(P, nrows)).astype(np.uint16)    # about 2.04e9 points each
    nk, doff, off = scheme(counts)
    exact = np.cumsum(counts.reshape(-1).astype(np.int64)) - counts.reshape(-1).astype(np.int64)
    assert exact[-1] + int(counts[-1, -1]) > (1 << 32)                           # the uint32 scan wrapped
    assert np.array_equal(nk, counts.astype(np.int64).sum(axis=1))
    assert np.array_equal(off.reshape(-1), exact)
    assert all(n < (1 << 31) for n in nk)


def test_offsets_small_and_empty_rows():
    rng = np.random.default_rng(4)
    for P, nrows in ((1, 1), (2, 5), (7, 300)):
        counts = (rng.random((P, nrows)) < 0.2) * rng.integers(0, 300, size=(P, nrows))
        counts = counts.astype(np.uint16)
        nk, doff, off = scheme(counts)
        exact = np.cumsum(counts.reshape(-1).astype(np.int64)) - counts.reshape(-1).astype(np.int64)
        assert np.array_equal(off.reshape(-1), exact) and doff[-1] == counts.sum()
