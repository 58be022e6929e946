"""The FFT-gridding restatement of the oracle (fillInFourierGrid.m,
griddingMethod 1) checked against the independent numpy restatement and
against known answers from the mathematics."""
import numpy as np
import pytest

from oracle import np_restate as NR

CASES = [
    # D1, D2, P, os, cutoff, allowMultipleGridMatches
    (12, 12, 3, 2, 0.7, 1), (12, 12, 3, 2, 0.7, 0), (11, 11, 4, 2, 0.9, 1), (10, 12, 2, 3, 0.3, 1),
    (16, 16, 5, 1.5, 1.6, 1), (9, 9, 3, 3, 0.45, 1), (8, 8, 1, 4, 0.7, 1),
]


def _case(seed, D1, D2, P):
    rng = np.random.default_rng(seed)
    projs = rng.random((D1, D2, P))
    angles = np.stack([rng.uniform(0, 360, P), rng.uniform(-70, 70, P), rng.uniform(0, 360, P)], 1)
    angles[0] = (0, 0, 0)
    return projs, angles


@pytest.mark.parametrize("D1,D2,P,os_,cut,am", CASES)
def test_grid_fft_matches_numpy_restatement(oracle, D1, D2, P, os_, cut, am):
    projs, angles = _case(D1 * 100 + P, D1, D2, P)
    prm = oracle.make_params(D1, D2, P, oversamplingRatio=os_, interpolationCutoffDistance=cut)
    M, rec, n = oracle.grid_fft(prm, projs, angles, allow_multiple=am)
    K, rec2, n2 = NR.fill_in_fourier_grid(projs, angles, os_, cut, am)
    assert M.shape == K.shape
    assert n == n2
    assert np.array_equal(M != 0, K != 0)
    assert np.abs(M - K).max() <= 1e-12 * np.abs(K).max()
    assert np.abs(rec - rec2).max() <= 1e-12 * np.abs(rec2).max()


def test_grid_fft_size_rule(oracle):
    # fillInFourierGrid.m:38-42: even Dim2 -> Dim2 * os, odd -> 1 + (Dim2-1) * os
    assert oracle.fft_grid_size(64, 4) == 256
    assert oracle.fft_grid_size(65, 2) == 129
    assert oracle.fft_grid_size(64, 2.5) == 160
    assert oracle.fft_grid_size(63, 2.5) == 156           # 1 + 62 * 2.5
    assert oracle.fft_grid_size(10, 2.25) == -1           # 22.5 is not an integer


def test_grid_fft_zero_angles_is_the_padded_fft_on_the_k3_plane(oracle):
    # phi = theta = psi = 0: every FFT sample sits exactly on a voxel of the
    # kz = 0 plane (distance 0), so with one projection the plane holds the
    # centred FFT of the padded projection, already Hermitian for real input
    D, os_ = 12, 2
    rng = np.random.default_rng(7)
    proj = rng.random((D, D, 1))
    prm = oracle.make_params(D, D, 1, oversamplingRatio=os_, interpolationCutoffDistance=0.3)
    M, _, n = oracle.grid_fft(prm, proj, np.zeros((1, 3)), allow_multiple=1, want_rec=False)
    m = D * os_
    F = np.fft.fftshift(np.fft.fft2(np.fft.ifftshift(NR.paddzero(proj[:, :, 0], (m, m)))))
    assert n == m * m
    plane = M[:, :, m // 2]
    # the first row and column have no mate on the odd-extended grid: the
    # Hermitian average keeps them as they are
    assert np.abs(plane - F).max() <= 1e-12 * np.abs(F).max()
    M[:, :, m // 2] = 0
    assert not M.any()


def test_grid_fft_dc_projection(oracle):
    # a constant projection of value c: its FFT is c * D^2 at k = 0 (and the
    # sinc-like padding pattern elsewhere); the origin voxel averages the k = 0
    # samples of every projection, all equal to c * D^2
    D, os_, P = 8, 2, 4
    c = 0.75
    projs = np.full((D, D, P), c)
    rng = np.random.default_rng(3)
    angles = np.stack([rng.uniform(0, 360, P), rng.uniform(-70, 70, P), rng.uniform(0, 360, P)], 1)
    prm = oracle.make_params(D, D, P, oversamplingRatio=os_, interpolationCutoffDistance=0.7)
    M, _, _ = oracle.grid_fft(prm, projs, angles, allow_multiple=0, want_rec=False)
    m = D * os_
    assert abs(M[m // 2, m // 2, m // 2] - c * D * D) <= 1e-12 * c * D * D


def test_grid_fft_randomized_against_numpy_restatement(oracle):
    """FFT gridding of the C oracle against the numpy restatement over random
    projection shapes, counts, oversampling ratios (integer cube sizes only),
    cutoffs, both match rules and angles, including the zero and right-angle
    poses that put samples exactly on voxels."""
    hyp = pytest.importorskip("hypothesis")
    st = hyp.strategies
    angle = st.one_of(st.floats(-360, 360, allow_nan=False), st.sampled_from([0.0, 90.0, -90.0, 180.0]))

    @hyp.settings(max_examples=30, deadline=None, derandomize=True)
    @hyp.given(D2=st.integers(4, 12), dD1=st.integers(-2, 2), P=st.integers(1, 4), os_=st.sampled_from([1.5, 2.0, 3.0]),
               cut=st.sampled_from([0.3, 0.7, 1.2]), am=st.sampled_from([0, 1]), seed=st.integers(0, 2 ** 16),
               a0=st.tuples(angle, angle, angle))
    def check(D2, dD1, P, os_, cut, am, seed, a0):
        D1 = max(3, D2 + dD1)
        if oracle.fft_grid_size(D2, os_) < 0 or oracle.fft_grid_size(D2, os_) < max(D1, D2):
            return
        rng = np.random.default_rng(seed)
        projs = rng.random((D1, D2, P))
        angles = np.stack([rng.uniform(0, 360, P), rng.uniform(-70, 70, P), rng.uniform(0, 360, P)], 1)
        angles[0] = a0
        prm = oracle.make_params(D1, D2, P, oversamplingRatio=os_, interpolationCutoffDistance=cut)
        M, rec, n = oracle.grid_fft(prm, projs, angles, allow_multiple=am)
        K, rec2, n2 = NR.fill_in_fourier_grid(projs, angles, os_, cut, am)
        assert n == n2
        assert np.array_equal(M != 0, K != 0)
        scale = max(1.0, np.abs(K).max())
        assert np.abs(M - K).max() <= 1e-12 * scale
        assert np.abs(rec - rec2).max() <= 1e-12 * max(1.0, np.abs(rec2).max())

    check()
