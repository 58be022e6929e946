"""The mirrored K order of the tensor-core gridding DFT (grid_mma.cu, WsArgs::mirror),
restated on the CPU.

With D1 = 64 H rows and m = D1/2, K runs a = 0 .. m-1 (chunks 0 .. H-1) and then
a = -1 .. -m (chunks H .. 2H-1); the MMAs take the chunk pairs (p, H + p).  A
producer thread holds the split words of 16 consecutive E_u values of its half of
the positive chunk and of one more value; the negative chunk's element k is
conj E_u(32p + k + 1), written as the same words re-paired one element along
(byte permute 0x5432 of neighbouring words) with the sign bits of the imaginary
hi and lo halves flipped.  The projection's B rows are pre-split in the same
order (aa = kabs + m for kabs < m, else 2m - 1 - kabs; rows outside 0 .. D1-1
zero).  Checked: every a in [-m, m-1] appears once with the matching B row, and
the words the scheme writes equal the split of conj E_u at those a bit for bit,
for BF16 and FP16 halves."""
import numpy as np
import pytest

from tests.test_split_and_mixed_radix import bf16


def f16(x):
    return np.asarray(x, dtype=np.float32).astype(np.float16).astype(np.float32)


def split(x, rnd):
    x = np.asarray(x, dtype=np.float32)
    hi = rnd(x)
    lo = rnd((x - hi).astype(np.float32))
    return hi, lo


def halves(v, rnd):
    """16-bit patterns of the values rounded by rnd (bf16 or fp16)."""
    v = rnd(np.asarray(v, np.float32))
    if rnd is bf16:
        return (v.view(np.uint32) >> 16).astype(np.uint32)
    return v.astype(np.float16).view(np.uint16).astype(np.uint32)


def pack(lo_half, hi_half):
    return (lo_half & 0xFFFF) | ((hi_half & 0xFFFF) << 16)


def byte_perm_5432(x, y):
    return ((x >> 16) & 0xFFFF) | ((y & 0xFFFF) << 16)


@pytest.mark.parametrize("rnd", [bf16, f16])
@pytest.mark.parametrize("D1", [64, 128, 192, 256])
def test_mirrored_chunks_equal_the_split_of_the_conjugates(D1, rnd):
    m, H = D1 // 2, D1 // 64
    u = 0.37
    E = lambda a: np.exp(-2j * np.pi * np.asarray(a, np.float64) * u / (2 * D1)).astype(np.complex64)
    covered = []
    for p in range(H):
        for h in range(2):
            a0 = 32 * p + 16 * h
            v = E(a0 + np.arange(17))                                     # the thread's 17 values
            re_hi, re_lo = split(v.real, rnd)
            im_hi, im_lo = split(v.imag, rnd)
            # the positive chunk's words: pairs (2j, 2j+1), plus the 17th value in a low half
            def words(hi):
                w = [pack(halves(hi[2 * j], rnd), halves(hi[2 * j + 1], rnd)) for j in range(8)]
                return w + [pack(halves(hi[16], rnd), 0)]
            rh, rl, ih, il = words(re_hi), words(re_lo), words(im_hi), words(im_lo)
            # the negative chunk by the scheme
            nrh = [byte_perm_5432(rh[j], rh[j + 1]) for j in range(8)]
            nrl = [byte_perm_5432(rl[j], rl[j + 1]) for j in range(8)]
            nih = [byte_perm_5432(ih[j], ih[j + 1]) ^ 0x80008000 for j in range(8)]
            nil = [byte_perm_5432(il[j], il[j + 1]) ^ 0x80008000 for j in range(8)]
            # the same words formed directly from conj E_u at the negative chunk's a
            k = 16 * h + np.arange(16)
            a_neg = -(32 * p + k) - 1
            w = np.conj(E(-a_neg))                                          # E_u(a) = conj E_u(-a)
            assert np.allclose(w, E(a_neg), atol=2e-7)
            d_rh, d_rl = split(w.real, rnd)
            d_ih, d_il = split(w.imag, rnd)
            for got, want in ((nrh, d_rh), (nrl, d_rl), (nih, d_ih), (nil, d_il)):
                ref = [pack(halves(want[2 * j], rnd), halves(want[2 * j + 1], rnd)) for j in range(8)]
                assert [int(x) for x in got] == [int(x) for x in ref]
            covered += list(a0 + np.arange(16)) + list(a_neg)
    assert sorted(covered) == list(range(-m, m))


@pytest.mark.parametrize("D1", [64, 128, 192, 256])
def test_b_rows_follow_the_mirrored_order(D1):
    """B chunk bc, element k: the pre-split's row aa = a + m for the a the A
    chunk of that pair holds; chunks beyond 2H (the block's padding) read no row."""
    m, H = D1 // 2, D1 // 64
    for kc in range(8):                     # all chunks of a 256-row block
        for k in range(32):
            kabs = 32 * kc + k
            aa = kabs + m if kabs < m else 2 * m - 1 - kabs
            if kc < H:
                assert aa - m == 32 * kc + k                      # positive chunk p = kc
            elif kc < 2 * H:
                assert aa - m == -(32 * (kc - H) + k) - 1         # negative chunk of pair kc - H
            else:
                assert not (0 <= aa < D1)                          # padding: zero
    # the MMAs' chunk sequence s -> B chunk
    seq = [(H + (s >> 1)) if s & 1 else (s >> 1) for s in range(2 * H)]
    assert sorted(seq) == list(range(2 * H))
