"""The Rfree monitor on the GPU (genfire_rfree_candidates,
genfire_recon_set_rfree, genfire_recon_rfree) against the oracle.  Bar:
candidates bit-exact; FP64 Rfree, errK and reconstruction within 1e-10; MIXED
Rfree within 1e-4 absolute."""
import numpy as np
import pytest

from oracle import np_restate as NR
from genfire_gb300 import _lib as L
from tests.conftest import params, rel

pytestmark = pytest.mark.gpu


def _measured(seed, D1, D2, os_, keep=0.5):
    rng = np.random.default_rng(seed)
    n1, n2 = int(np.floor(D1 * os_ + 0.5)), int(np.floor(D2 * os_ + 0.5))
    vol = rng.random((D1, D2, D1))
    M = np.fft.fftshift(np.fft.fftn(np.fft.ifftshift(NR.paddzero(vol, (n1, n2, n1)))))
    M[rng.random(M.shape) > keep] = 0
    return np.asfortranarray(M)


def _withhold(cands, M, frac, seed):
    rng = np.random.default_rng(seed)
    mask = np.asfortranarray(M != 0)
    flat = mask.reshape(-1, order="F")
    shells = []
    for c in cands:
        cut = max(int(np.floor(len(c) * frac)), 1)
        sel = c[rng.permutation(len(c))][:cut]
        flat[sel] = False
        shells.append(sel)
    return shells, mask


@pytest.mark.parametrize("D1,D2,os_", [(8, 8, 2.0), (9, 9, 2.0), (8, 10, 2.5), (12, 12, 2.0), (7, 7, 3.0)])
@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_candidates_bit_exact(lib, ctx, oracle, D1, D2, os_, prec):
    M = _measured(D1 + D2, D1, D2, os_)
    p = params(lib, D1, D2, 1, oversamplingRatio=os_, precision=prec)
    for nb in (1, 3, 10):
        got = ctx.rfree_candidates(p, M, nb)
        assert len(got) == nb
        for s in range(nb):
            assert np.array_equal(got[s], oracle.rfree_candidates(M, nb, s)), (nb, s)


# grid sizes n1 = 16 (power of two), 20 and 24 (mixed radix), 18 and 21 (generic FFT pass)
CASES = [(8, 8, 2.0, 3), (10, 10, 2.0, 1), (12, 12, 2.0, 3), (9, 9, 2.0, 2), (7, 7, 3.0, 3), (8, 10, 2.5, 3)]


@pytest.mark.parametrize("D1,D2,os_,mode", CASES)
def test_rfree_fp64_parity(lib, ctx, oracle, D1, D2, os_, mode):
    M = _measured(3 * D1 + D2, D1, D2, os_)
    nb, N = 5, 14
    kw = dict(oversamplingRatio=os_, numIterations=N, constraintEnforcementMode=mode)
    p = params(lib, D1, D2, 1, **kw)
    shells, mask = _withhold(ctx.rfree_candidates(p, M, nb), M, 0.08, D1)
    r = ctx.recon(p, M, mask=mask)
    r.set_rfree(shells)
    r.iterate(5)
    r.iterate(N - 5)
    rec, errK, _, _, _ = r.result()
    Rf = r.rfree()
    r.close()
    reco, errKo, Rfo = oracle.reconstruct_rfree(oracle.make_params(D1, D2, 1, **kw), M, shells, mask=mask)
    assert Rf.shape == (nb, N)
    assert np.abs(Rf - Rfo).max() < 1e-10
    assert np.abs(errK - errKo).max() < 1e-10
    assert rel(rec, reco) < 1e-10


def test_rfree_mixed(lib, ctx, oracle):
    D, os_, N, nb = 12, 2.0, 12, 4
    M = _measured(11, D, D, os_)
    kw = dict(oversamplingRatio=os_, numIterations=N, constraintEnforcementMode=3)
    p = params(lib, D, D, 1, precision="mixed", **kw)
    shells, mask = _withhold(ctx.rfree_candidates(p, M, nb), M, 0.1, 2)
    r = ctx.recon(p, M.astype(np.complex64), mask=mask)
    r.set_rfree(shells)
    r.iterate(N)
    Rf = r.rfree()
    r.close()
    _, _, Rfo = oracle.reconstruct_rfree(oracle.make_params(D, D, 1, **kw), M, shells, mask=mask)
    assert np.abs(Rf - Rfo).max() < 1e-4


def test_rfree_overlapping_shells_and_mirror_points(lib, ctx, oracle):
    """A point in two shells (the resRange overlap) and points whose stored half
    is the mirror: every centred index of a small grid withheld in one shell."""
    D, os_, N = 6, 2.0, 6
    M = _measured(21, D, D, os_, keep=1.0)
    n = M.shape[0]
    kw = dict(oversamplingRatio=os_, numIterations=N, constraintEnforcementMode=3)
    p = params(lib, D, D, 1, **kw)
    allidx = np.arange(n ** 3, dtype=np.int64)
    shells = [allidx[::7].copy(), allidx[::7][:40].copy()]
    mask = np.asfortranarray(np.ones(M.shape, bool))
    mask.reshape(-1, order="F")[allidx[::7]] = False
    r = ctx.recon(p, M, mask=mask)
    r.set_rfree(shells)
    r.iterate(N)
    Rf = r.rfree()
    r.close()
    _, _, Rfo = oracle.reconstruct_rfree(oracle.make_params(D, D, 1, **kw), M, shells, mask=mask)
    assert np.abs(Rf - Rfo).max() < 1e-10


def test_rfree_errors(lib, ctx):
    D, os_ = 8, 2.0
    M = _measured(1, D, D, os_)
    p = params(lib, D, D, 1, oversamplingRatio=os_, numIterations=4)
    r = ctx.recon(p, M)
    with pytest.raises(lib.GenfireError) as e:
        r.set_rfree([np.array([M.size], dtype=np.int64)])
    assert e.value.status == L.GENFIRE_ERR_ARG
    r.iterate(1)
    with pytest.raises(lib.GenfireError) as e:
        r.set_rfree([np.array([0], dtype=np.int64)])
    assert e.value.status == L.GENFIRE_ERR_STATE
    r.close()
    with pytest.raises(lib.GenfireError):
        ctx.rfree_candidates(p, M, 0)


def test_reconstructor_calculate_rfree(lib, ctx):
    """The class mirror: calculate_Rfree = 1 withholds points per shell,
    reports Rfree_complex (numBinsRfree x numIterations, single) and repeats
    exactly with the same RandomSeed."""
    from genfire_gb300.reconstructor import GENFIRE_Reconstructor
    D, os_ = 8, 2.0
    M = _measured(8, D, D, os_)
    out = []
    for _ in range(2):
        G = GENFIRE_Reconstructor()
        G.Dim1 = G.Dim2 = D
        G.NumProjs = 1
        G.oversamplingRatio = os_
        G.numIterations = 10
        G.constraintEnforcementMode = 3
        G.Support = np.ones((D, D, D), bool)
        G.measuredK = M
        G.measuredK_mask = M != 0
        G.calculate_Rfree = 1
        G.numBinsRfree = 4
        G.percentValuesForRfree = 0.1
        G.RandomSeed = 7
        G = G.reconstruct()
        assert G.Rfree_complex.shape == (4, 10) and G.Rfree_complex.dtype == np.float32
        assert np.all(np.isfinite(G.Rfree_complex)) and np.all(G.Rfree_complex > 0)
        out.append((G.Rfree_complex, G.errK, G.reconstruction))
    assert np.array_equal(out[0][0], out[1][0]) and np.array_equal(out[0][1], out[1][1])


def test_reconstructor_save_temp(lib, ctx, tmp_path):
    """save_temp = 1 writes the best object so far every save_loopLength
    iterations (reconstruct.m:155-158); the last file is the final result, and
    the staged run equals the one-shot run."""
    scipy_io = pytest.importorskip("scipy.io")
    from genfire_gb300.reconstructor import GENFIRE_Reconstructor
    D, os_ = 8, 2.0
    M = _measured(9, D, D, os_)
    outs = []
    for save in (0, 1):
        G = GENFIRE_Reconstructor()
        G.Dim1 = G.Dim2 = D
        G.NumProjs = 1
        G.oversamplingRatio = os_
        G.numIterations = 10
        G.constraintEnforcementMode = 1
        G.Support = np.ones((D, D, D), bool)
        G.measuredK = M
        G.measuredK_mask = M != 0
        G.save_temp = save
        G.save_loopLength = 4
        G.saveFilename = str(tmp_path / "temp_rec")
        G = G.reconstruct()
        outs.append((G.reconstruction, G.errK))
    assert np.array_equal(outs[0][0], outs[1][0]) and np.array_equal(outs[0][1], outs[1][1])
    files = sorted(p.name for p in tmp_path.iterdir())
    assert files == ["temp_rec4.mat", "temp_rec8.mat"]
    t8 = scipy_io.loadmat(str(tmp_path / "temp_rec8.mat"))["temp_reconstruction"]
    # the best object after 8 iterations of the same reconstruction
    p = params(lib, D, D, 1, oversamplingRatio=os_, numIterations=10, constraintEnforcementMode=1)
    r = ctx.recon(p, M, support=np.ones((D, D, D), bool))
    r.iterate(8)
    rec8 = r.result()[0]
    r.close()
    assert np.array_equal(t8, rec8)
