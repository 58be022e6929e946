"""Edge cases of the path against the oracle: zero and one iteration, a single
projection, the smallest projection sizes, odd and non-square sizes through
both gridding methods, and an all-zero measured grid."""
import numpy as np
import pytest

from oracle import np_restate as NR
from tests.conftest import params, rel

pytestmark = pytest.mark.gpu


def _measured(seed, D1, D2, os_, keep=0.5):
    rng = np.random.default_rng(seed)
    n1, n2 = int(np.floor(D1 * os_ + 0.5)), int(np.floor(D2 * os_ + 0.5))
    vol = rng.random((D1, D2, D1))
    M = np.fft.fftshift(np.fft.fftn(np.fft.ifftshift(NR.paddzero(vol, (n1, n2, n1)))))
    M[rng.random(M.shape) > keep] = 0
    return np.asfortranarray(M)


@pytest.mark.parametrize("N", [0, 1, 2])
@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_few_iterations(lib, ctx, oracle, N, prec):
    D, os_ = 8, 2.0
    M = _measured(N + 3, D, D, os_)
    kw = dict(oversamplingRatio=os_, numIterations=N, constraintEnforcementMode=1)
    rec, errK, _, _, _ = ctx.reconstruct(params(lib, D, D, 1, precision=prec, **kw),
                                         M if prec == "fp64" else M.astype(np.complex64))
    reco, errKo, _, _, _ = oracle.reconstruct(oracle.make_params(D, D, 1, **kw), M)
    assert errK.shape == (N,)
    if N == 0:
        assert not rec.any() and not reco.any()   # no best object yet: zeros
        return
    tol = 1e-10 if prec == "fp64" else 1e-4
    assert np.abs(errK - errKo).max() < tol
    assert rel(rec, reco) < tol


def test_all_zero_measured_grid(lib, ctx, oracle):
    """No measured point: errK is 0/0 in the reference (NaN); the object stays zero."""
    D, os_, N = 6, 2.0, 3
    n = int(np.floor(D * os_ + 0.5))
    M = np.zeros((n, n, n), dtype=np.complex128, order="F")
    kw = dict(oversamplingRatio=os_, numIterations=N, constraintEnforcementMode=3)
    rec, errK, _, _, _ = ctx.reconstruct(params(lib, D, D, 1, **kw), M)
    reco, errKo, _, _, _ = oracle.reconstruct(oracle.make_params(D, D, 1, **kw), M)
    assert np.all(np.isnan(errK)) and np.all(np.isnan(errKo))
    assert not rec.any() and not reco.any()


@pytest.mark.parametrize("D1,D2,P,os_,cut", [(2, 2, 1, 2.0, 0.5), (3, 3, 1, 2.0, 0.3), (3, 5, 2, 2.0, 0.4),
                                             (5, 4, 3, 3.0, 0.25), (1, 4, 2, 2.0, 0.5)])
@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_small_projections_dft_gridding(lib, ctx, oracle, D1, D2, P, os_, cut, prec):
    rng = np.random.default_rng(D1 * 10 + D2 + P)
    projs = np.asfortranarray(rng.random((D1, D2, P)))
    angles = np.asfortranarray(np.stack([rng.uniform(0, 360, P), rng.uniform(-70, 70, P),
                                         rng.uniform(0, 360, P)], 1))
    kw = dict(oversamplingRatio=os_, interpolationCutoffDistance=cut)
    p = params(lib, D1, D2, P, precision=prec, **kw)
    if D1 < 2:
        # the grid must hold the projection's own size (oversampled size >= Dim)
        with pytest.raises(lib.GenfireError):
            ctx.grid_dft(p, projs, angles)
        return
    M, rec, nk = ctx.grid_dft(p, projs, angles)
    Mo, reco, nko = oracle.grid_dft(oracle.make_params(D1, D2, P, **kw), projs, angles)
    assert np.array_equal(nk, nko)
    assert np.array_equal(M != 0, Mo != 0)
    tol = 1e-10 if prec == "fp64" else 1e-4
    assert rel(M, Mo) < tol


@pytest.mark.parametrize("D,P,cut,multi", [(3, 1, 0.5, 1), (5, 2, 0.7, 0), (6, 3, 1.5, 1)])
def test_small_fft_gridding(lib, ctx, oracle, D, P, cut, multi):
    rng = np.random.default_rng(D + P)
    projs = np.asfortranarray(rng.random((D, D, P)))
    angles = np.asfortranarray(np.stack([rng.uniform(0, 360, P), rng.uniform(-70, 70, P),
                                         rng.uniform(0, 360, P)], 1))
    kw = dict(oversamplingRatio=2.0, interpolationCutoffDistance=cut)
    p = params(lib, D, D, P, griddingMethod=1, allowMultipleGridMatches=multi, **kw)
    M, rec, npairs = ctx.grid_fft(p, projs, angles)
    Mo, reco, npo = oracle.grid_fft(oracle.make_params(D, D, P, **kw), projs, angles, allow_multiple=multi)
    assert npairs == npo
    assert rel(M, Mo) < 1e-10
