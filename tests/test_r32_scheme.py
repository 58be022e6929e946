"""The index scheme of the radix-32 FFT engines (genfire_gb300/csrc/fft_r32.cuh),
restated on the CPU: thread t of a column holds the elements t + P m
(P = N/32), stage 1 is a 32-point DFT over m whose output k lands in slot
8 (k & 3) + (k >> 2), the twiddle WN^(t k1), the exchange S[k1][t] with rows
of P + 1 and columns of 32 (P + 1) + 16 / W, stage 2 the P-point DFTs over t,
and the output slot map out_m.  Checked: the scheme computes the DFT (forward
and inverse), every shared-memory index stays inside the CTA's buffer, the
centred-half offsets cover the box exactly, and every half-warp access of
the exchange is free of bank conflicts.  The constants mirror R32<N>."""
import numpy as np
import pytest


def geometry(N):
    P = N // 32
    W = 8 if N <= 512 else 4
    ROW = P + 1
    CS = 32 * ROW + 16 // W
    return P, W, ROW, CS


def out_m(N, s):
    if N == 128:
        return (s >> 2) + 8 * (s & 3)
    if N == 256:
        return (s >> 3) + 4 * (s & 7)
    if N == 512:
        return (s >> 4) + 2 * (((s & 15) >> 2) + 4 * (s & 3))
    return 4 * (s & 7) + (s >> 3)


def half_off(N, m):
    P = N // 32
    return P * m + N // 4 if m < 8 else P * m - 3 * N // 4


def elems(N):
    P, W, ROW, CS = geometry(N)
    return max((N + N // 8) * W, W * CS)  # natural-order tiles and the exchange buffer


def run_scheme(N, x, inv):
    P, W, ROW, CS = geometry(N)
    sgn = 1 if inv else -1
    m = np.arange(32)
    F32 = np.exp(sgn * 2j * np.pi * np.outer(m, m) / 32)   # [k, m]
    slot_of_k = 8 * (m & 3) + (m >> 2)
    S = np.zeros(W * CS, complex)
    for t in range(P):
        y = np.empty(32, complex)
        y[slot_of_k] = F32 @ x[t + P * m]                    # stage 1: output k in slot 8 (k & 3) + (k >> 2)
        for k1 in range(32):
            S[k1 * ROW + t] = y[8 * (k1 & 3) + (k1 >> 2)] * np.exp(sgn * 2j * np.pi * t * k1 / N)
    X = np.empty(N, complex)
    for t in range(P):
        out = np.empty(32, complex)
        if N == 1024:
            out[slot_of_k] = F32 @ np.array([S[t * ROW + tp] for tp in range(32)])
        elif N == 512:
            F16 = np.exp(sgn * 2j * np.pi * np.outer(np.arange(16), np.arange(16)) / 16)
            for h in range(2):
                v = np.array([S[(t + 16 * h) * ROW + tp] for tp in range(16)])
                z = F16 @ v                                     # z[k2], k2 = k2' + 4 k3
                for k2p in range(4):
                    for k3 in range(4):
                        out[16 * h + 4 * k2p + k3] = z[k2p + 4 * k3]
        else:
            FP = np.exp(sgn * 2j * np.pi * np.outer(np.arange(P), np.arange(P)) / P)
            for h in range(32 // P):
                out[P * h:P * h + P] = FP @ np.array([S[(t + P * h) * ROW + tp] for tp in range(P)])
        for s in range(32):
            X[t + P * out_m(N, s)] = out[s]
    return X


@pytest.mark.parametrize("N", [128, 256, 512, 1024])
@pytest.mark.parametrize("inv", [False, True])
def test_scheme_is_the_dft(N, inv):
    rng = np.random.default_rng(N + inv)
    x = rng.standard_normal(N) + 1j * rng.standard_normal(N)
    X = run_scheme(N, x, inv)
    ref = np.fft.ifft(x) * N if inv else np.fft.fft(x)
    assert np.abs(X - ref).max() <= 1e-12 * np.abs(ref).max()


@pytest.mark.parametrize("N", [128, 256, 512, 1024])
def test_slot_maps_and_centred_half(N):
    P = N // 32
    assert sorted(out_m(N, s) for s in range(32)) == list(range(32))
    kept = [m for m in range(32) if m < 8 or m >= 24]
    assert sorted(t + half_off(N, m) for t in range(P) for m in kept) == list(range(N // 2))
    for t in range(P):
        for m in range(32):
            j = (t + P * m + N // 4) % N          # box element held by slot m (box of N/2 at offset N/4)
            if m in kept:
                assert j == t + half_off(N, m)
            else:
                assert j >= N // 2                # outside the box: known zero on input, never stored
    assert sum(1 for s in range(32) if out_m(N, s) in kept) == 16


@pytest.mark.parametrize("N", [128, 256, 512, 1024])
def test_buffer_bounds(N):
    P, W, ROW, CS = geometry(N)
    E = elems(N)
    assert max(c * CS + k1 * ROW + t for c in range(W) for k1 in range(32) for t in range(P)) < E
    assert max((i + (i >> 3)) * W + c for i in range(N) for c in range(W)) < E        # column tile
    assert max(c * (N + N // 8) + i + (i >> 3) for i in range(N) for c in range(W)) < E  # row tile
    assert E * 8 <= 48 * 1024                     # complex64: within the default dynamic shared memory


@pytest.mark.parametrize("N", [128, 256, 512, 1024])
def test_exchange_is_bank_conflict_free(N):
    """8-byte accesses are served per half-warp: the 16 word addresses must
    differ modulo 16.  Column passes put the column fastest (lane -> c = l % W,
    t = l / W)."""
    P, W, ROW, CS = geometry(N)
    nthr = P * W
    groups = 32 // P if N < 1024 else 1
    for base in range(0, nthr, 16):
        lanes = range(base, min(base + 16, nthr))
        for k1 in range(32):
            words = [(l % W) * CS + k1 * ROW + (l // W) for l in lanes]
            assert len({w % 16 for w in words}) == len(words)
        for h in range(groups):
            for tp in range(P):
                words = [(l % W) * CS + ((l // W) + P * h) * ROW + tp for l in lanes]
                assert len({w % 16 for w in words}) == len(words)
