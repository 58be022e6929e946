"""The radix-32 engines (n = 128 .. 1024 as 32 x 4 .. 32 x 32, complex64; one
shared-memory exchange per transform), forced with
GENFIRE_COL_VARIANT=4 wherever they are valid: transforms against numpy, and
the fused dim-3 pass (constraint table, errK, Rfree capture), the dim-2
passes and the row passes of a reconstruction against the oracle.  Bar: 1e-5
relative for single transforms, the MIXED bar 1e-4 for reconstructions."""
import numpy as np
import pytest

from oracle import np_restate as NR
from tests.conftest import params, rel

pytestmark = pytest.mark.gpu


@pytest.fixture
def r32(monkeypatch):
    monkeypatch.setenv("GENFIRE_COL_VARIANT", "4")


@pytest.mark.parametrize("shape", [(8, 4, 512), (6, 512, 3), (512, 3, 5), (16, 512, 512),
                                   (8, 4, 1024), (6, 1024, 3), (1024, 3, 5), (4, 1024, 1024),
                                   (8, 4, 256), (6, 256, 3), (256, 3, 5), (5, 128, 128), (128, 7, 9)])
@pytest.mark.parametrize("inverse", [False, True])
def test_r32_transforms(lib, ctx, r32, shape, inverse):
    rng = np.random.default_rng(sum(shape) + inverse)
    a = (rng.standard_normal(shape) + 1j * rng.standard_normal(shape)).astype(np.complex64)
    got = ctx.fftn(a, inverse=inverse, precision=lib.PREC_MIXED)
    ref = np.fft.ifftn(a.astype(np.complex128)) if inverse else np.fft.fftn(a.astype(np.complex128))
    assert rel(got, ref) < 1e-5


def _measured(seed, D1, D2, os_, keep=0.5):
    rng = np.random.default_rng(seed)
    n1, n2 = int(np.floor(D1 * os_ + 0.5)), int(np.floor(D2 * os_ + 0.5))
    vol = rng.random((D1, D2, D1))
    M = np.fft.fftshift(np.fft.fftn(np.fft.ifftshift(NR.paddzero(vol, (n1, n2, n1)))))
    M[rng.random(M.shape) > keep] = 0
    return np.asfortranarray(M)


@pytest.mark.parametrize("D1,D2,mode,os_", [(256, 4, 3, 2.0), (4, 256, 1, 2.0), (256, 4, 2, 2.0),
                                           (512, 4, 3, 2.0), (4, 512, 1, 2.0), (400, 3, 3, 2.56),
                                           (128, 4, 3, 2.0), (4, 128, 1, 2.0), (64, 5, 3, 2.0), (100, 3, 2, 2.56)])
def test_r32_reconstruct_mixed(lib, ctx, oracle, r32, D1, D2, mode, os_):
    """n1 = 512 or 1024 puts the fused dim-3 pass (forward, constraint, errK,
    inverse) on the engine; n2 = 512 or 1024 the dim-2 forward and inverse
    passes.  A 400 box at oversampling 2.56 (n1 = 1024) takes the unpruned
    variants."""
    N = 4
    M = _measured(D1 + D2 + mode, D1, D2, os_)
    kw = dict(oversamplingRatio=os_, numIterations=N, constraintEnforcementMode=mode)
    p = params(lib, D1, D2, 1, precision="mixed", **kw)
    r = ctx.recon(p, M.astype(np.complex64))
    assert 4 in r.tuning()
    r.iterate(N)
    rec, errK, _, _, _ = r.result()
    r.close()
    reco, errKo, _, _, _ = oracle.reconstruct(oracle.make_params(D1, D2, 1, **kw), M)
    assert np.abs(errK - errKo).max() < 1e-4
    assert rel(rec, reco) < 1e-4


@pytest.mark.parametrize("D1", [64, 128, 256, 512])
def test_r32_rfree_capture(lib, ctx, oracle, r32, D1):
    D2, os_, N, nb = 4, 2.0, 3, 3
    M = _measured(5, D1, D2, os_)
    kw = dict(oversamplingRatio=os_, numIterations=N, constraintEnforcementMode=3)
    p = params(lib, D1, D2, 1, precision="mixed", **kw)
    rng = np.random.default_rng(1)
    mask = np.asfortranarray(M != 0)
    flat = mask.reshape(-1, order="F")
    shells = []
    for c in ctx.rfree_candidates(p, M, nb):
        sel = c[rng.permutation(len(c))][:max(len(c) // 20, 1)]
        flat[sel] = False
        shells.append(sel)
    r = ctx.recon(p, M.astype(np.complex64), mask=mask)
    r.set_rfree(shells)
    r.iterate(N)
    Rf = r.rfree()
    r.close()
    _, _, Rfo = oracle.reconstruct_rfree(oracle.make_params(D1, D2, 1, **kw), M, shells, mask=mask)
    assert np.abs(Rf - Rfo).max() < 1e-4


@pytest.mark.parametrize("D1,D2,mode,pos,sup", [(256, 4, 3, 1, 1), (256, 6, 1, 0, 1), (256, 3, 3, 1, 0),
                                               (512, 3, 3, 1, 1), (512, 2, 1, 0, 1)])
def test_r32_row_passes_reconstruct(lib, ctx, oracle, D1, D2, mode, pos, sup):
    """n1 = 512 or 1024: the dim-1 row passes (real rows to half spectra with
    positivity and support, and back) on the radix-32 engines, the built-in
    choice for 512- and 1024-point complex64 rows; odd row counts leave the
    last pair half empty."""
    os_, N = 2.0, 4
    M = _measured(D1 + 3 * D2 + mode, D1, D2, os_)
    support = np.zeros((D1, D2, D1), bool)
    support[8:D1 - 8, :, 8:D1 - 8] = True
    kw = dict(oversamplingRatio=os_, numIterations=N, constraintEnforcementMode=mode, constraintPositivity=pos,
              constraintSupport=sup)
    rec, errK, _, _, _ = ctx.reconstruct(params(lib, D1, D2, 1, precision="mixed", **kw), M.astype(np.complex64),
                                         support=support)
    reco, errKo, _, _, _ = oracle.reconstruct(oracle.make_params(D1, D2, 1, **kw), M, support=support)
    assert np.abs(errK - errKo).max() < 1e-4
    assert rel(rec, reco) < 1e-4


@pytest.mark.parametrize("D,os_", [(256, 2.0), (200, 2.56)])
def test_r32_box_pruned_passes(lib, ctx, oracle, D, os_):
    """n = 512 grids: a 256 box (oversampling 2) is the centred-half case the
    pruned variants take (the dim-1 forward row pass, the fused dim-3 pass and
    the dim-2 and dim-1 inverses); a 200 box (oversampling 2.56) takes the
    unpruned ones.  20 k random measured points keep the table small."""
    D1 = D2 = D
    N = 2
    n1, n2 = int(np.floor(D1 * os_ + 0.5)), int(np.floor(D2 * os_ + 0.5))
    assert n1 == n2 == 512
    rng = np.random.default_rng(D1 + D2)
    M = np.zeros((n1, n2, n1), dtype=np.complex128, order="F")
    idx = rng.integers(0, [n1, n2, n1], size=(20000, 3))
    M[idx[:, 0], idx[:, 1], idx[:, 2]] = rng.standard_normal(20000) + 1j * rng.standard_normal(20000)
    kw = dict(oversamplingRatio=os_, numIterations=N, constraintEnforcementMode=3)
    rec, errK, _, _, _ = ctx.reconstruct(params(lib, D1, D2, 1, precision="mixed", **kw), M.astype(np.complex64))
    reco, errKo, _, _, _ = oracle.reconstruct(oracle.make_params(D1, D2, 1, **kw), M)
    assert np.abs(errK - errKo).max() < 1e-4
    assert rel(rec, reco) < 1e-4
