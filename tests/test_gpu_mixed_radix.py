"""The mixed-radix register passes (n = 3 * 2^k or 5 * 2^k, e.g. the grids of
the class-default oversampling 3): FFTs against numpy and the iteration
against the oracle."""
import numpy as np
import pytest

from tests.conftest import params, rel
from tests.test_gpu_recon import _measured, _support

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("shape", [(192, 5, 4), (4, 384, 3), (3, 4, 768), (320, 3, 2), (6, 192, 2)])
def test_fftn_mixed_radix_fp64(lib, ctx, shape):
    rng = np.random.default_rng(sum(shape) + 7)
    a = rng.standard_normal(shape) + 1j * rng.standard_normal(shape)
    assert rel(ctx.fftn(a), np.fft.fftn(a)) < 1e-13
    assert rel(ctx.fftn(a, inverse=True), np.fft.ifftn(a)) < 1e-13


@pytest.mark.parametrize("shape", [(192, 5, 4), (4, 384, 3), (3, 4, 768), (320, 3, 2), (5, 640, 2), (1280, 2, 2),
                                   (1536, 2, 2), (2, 2, 960)])
def test_fftn_mixed_radix_complex64(lib, ctx, shape):
    rng = np.random.default_rng(sum(shape) + 9)
    a = rng.standard_normal(shape) + 1j * rng.standard_normal(shape)
    assert rel(ctx.fftn(a, precision=lib.PREC_MIXED), np.fft.fftn(a)) < 2e-6
    assert rel(ctx.fftn(a, inverse=True, precision=lib.PREC_MIXED), np.fft.ifftn(a)) < 2e-6


@pytest.mark.parametrize("D,os_,prec,N", [(64, 3.0, "fp64", 3), (64, 3.0, "mixed", 4), (64, 5.0, "mixed", 2),
                                          (40, 2.4, "fp64", 3)])
def test_reconstruct_mixed_radix_grid(lib, ctx, oracle, D, os_, prec, N):
    # grids 192 (3 * 64), 320 (5 * 64) and 96 (3 * 32, below the register
    # engine: the generic passes) against the oracle
    support = _support(D, D, shrink=4)
    M, _ = _measured(D + int(os_ * 10), D, D, os_, keep=0.2, support=support)
    kw = dict(oversamplingRatio=os_, numIterations=N, constraintEnforcementMode=3)
    Mg = M.astype(np.complex64) if prec == "mixed" else M
    rec, errK, _, _, _ = ctx.reconstruct(params(lib, D, D, 1, precision=prec, **kw), Mg, support=support)
    reco, errKo, _, _, _ = oracle.reconstruct(oracle.make_params(D, D, 1, **kw), M, support=support)
    tol = 1e-10 if prec == "fp64" else 1e-4
    assert rel(rec, reco) < tol
    assert np.abs(errK - errKo).max() < (1e-10 if prec == "fp64" else 1e-5)


def test_rec_ifft_mixed_radix(lib, ctx, oracle):
    # recIFFT of a DFT gridding on a 3 * 64 grid
    rng = np.random.default_rng(12)
    D, P = 64, 3
    projs = np.asfortranarray(rng.random((D, D, P)))
    angles = np.asfortranarray(np.stack([rng.uniform(0, 360, P), rng.uniform(-70, 70, P), rng.uniform(0, 360, P)], 1))
    kw = dict(oversamplingRatio=3.0, interpolationCutoffDistance=0.3)
    M, rec, _ = ctx.grid_dft(params(lib, D, D, P, **kw), projs, angles)
    assert M.shape == (192, 192, 192)
    assert rel(rec, oracle.rec_ifft(M, D, D)) < 1e-10
