"""The Rfree monitor of reconstruct.m (:46-69 selection, :137-146 per
iteration) in the C oracle, against the independent numpy restatement.
Candidates are integer sets (bit-exact); Rfree and errK agree to 1e-12."""
import numpy as np
import pytest

from oracle import np_restate as NR


def _measured(seed, n1, n2, keep=0.5):
    rng = np.random.default_rng(seed)
    M = rng.standard_normal((n1, n2, n1)) + 1j * rng.standard_normal((n1, n2, n1))
    M[rng.random(M.shape) > keep] = 0
    return np.asfortranarray(M)


@pytest.mark.parametrize("n1,n2", [(12, 12), (13, 11), (16, 20), (9, 9)])
@pytest.mark.parametrize("nbins", [1, 4, 10])
def test_candidates_match_numpy(oracle, n1, n2, nbins):
    M = _measured(n1 * 7 + n2, n1, n2)
    total = 0
    for s in range(nbins):
        c = oracle.rfree_candidates(M, nbins, s)
        assert np.array_equal(c, NR.rfree_candidates(M, nbins, s))
        assert np.all(np.diff(c) > 0)
        total += len(c)
    # shells overlap by resRange: every measured point with Q < 1 is in at least one
    Q = NR.make_kspace_indices(M.shape).ravel(order="F")
    assert total >= np.count_nonzero((M.ravel(order="F") != 0) & (Q < 1))


def test_candidates_empty_grid(oracle):
    M = np.zeros((8, 8, 8), dtype=np.complex128, order="F")
    assert len(oracle.rfree_candidates(M, 5, 2)) == 0


def _withhold(M, nbins, frac, seed):
    rng = np.random.default_rng(seed)
    mask = np.asfortranarray(M != 0)
    flat = mask.reshape(-1, order="F")
    shells = []
    for s in range(nbins):
        c = NR.rfree_candidates(M, nbins, s)
        cut = max(int(np.floor(len(c) * frac)), 1)
        sel = c[rng.permutation(len(c))][:cut]
        flat[sel] = False
        shells.append(sel)
    return shells, mask


@pytest.mark.parametrize("D,os_,mode", [(8, 2.0, 3), (7, 2.0, 1), (6, 2.5, 2)])
def test_reconstruct_rfree_matches_numpy(oracle, D, os_, mode):
    n = int(np.floor(D * os_ + 0.5))
    rng = np.random.default_rng(D)
    vol = rng.random((D, D, D))
    M = np.fft.fftshift(np.fft.fftn(np.fft.ifftshift(NR.paddzero(vol, (n, n, n)))))
    M[rng.random(M.shape) > 0.6] = 0
    M = np.asfortranarray(M)
    shells, mask = _withhold(M, 4, 0.1, 5)
    support = np.ones((D, D, D), bool)
    N = 12
    prm = oracle.make_params(D, D, 1, oversamplingRatio=os_, numIterations=N, constraintEnforcementMode=mode)
    rec, errK, Rf = oracle.reconstruct_rfree(prm, M, shells, support=support, mask=mask)
    recn, errKn, Rfn = NR.reconstruct(M, N, support, mode=mode, mask=mask, rfree=shells)
    assert Rf.shape == (4, N)
    assert np.abs(Rf - Rfn).max() < 1e-12
    assert np.abs(errK - errKn).max() < 1e-12
    assert np.abs(rec - recn).max() < 1e-12 * max(1.0, np.abs(recn).max())
    # without shells the extended entry point is the plain one
    rec0, errK0, _, _, _ = oracle.reconstruct(prm, M, support=support, mask=mask)
    assert np.array_equal(rec0, rec) and np.array_equal(errK0, errK)
