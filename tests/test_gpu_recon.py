"""The Fourier-constraint iteration (reconstruct.m) on the GPU, against the
oracle.  Bar: FP64 reconstruction and errK within relative L2 1e-10; MIXED
within 1e-4 relative on the volume."""
import numpy as np
import pytest

from oracle import np_restate as NR
from tests.conftest import params, rel

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-10


def _measured(seed, D1, D2, os_, keep=0.4, support=None):
    """A centred grid from a positive object, with most points left unmeasured."""
    rng = np.random.default_rng(seed)
    n1, n2 = int(np.floor(D1 * os_ + 0.5)), int(np.floor(D2 * os_ + 0.5))
    vol = rng.random((D1, D2, D1))
    if support is not None:
        vol = vol * support
    M = np.fft.fftshift(np.fft.fftn(np.fft.ifftshift(NR.paddzero(vol, (n1, n2, n1)))))
    M[rng.random(M.shape) > keep] = 0
    return np.asfortranarray(M), vol


def _support(D1, D2, shrink=1):
    s = np.zeros((D1, D2, D1), bool)
    s[shrink:D1 - shrink, shrink:D2 - shrink, shrink:D1 - shrink] = True
    return s


CASES = [
    # D1, D2, os, mode, positivity, support-on, N
    (8, 8, 2.0, 3, 1, 1, 12), (8, 8, 2.0, 1, 1, 1, 30), (8, 8, 2.0, 2, 1, 1, 30), (9, 9, 2.0, 3, 1, 1, 10),
    (8, 10, 2.0, 3, 1, 1, 10), (7, 7, 3.0, 3, 0, 1, 10), (8, 8, 2.0, 3, 1, 0, 8), (10, 8, 2.5, 3, 0, 0, 8),
    (16, 16, 2.0, 3, 1, 1, 20), (12, 12, 2.0, 1, 1, 1, 27),
    # the longest transforms: n1 = 1024 (register engine) and 2048 (shared-memory engine) on thin grids
    (512, 4, 2.0, 3, 1, 1, 3), (1024, 3, 2.0, 3, 1, 1, 2),
]


@pytest.mark.parametrize("D1,D2,os_,mode,pos,sup,N", CASES)
def test_reconstruct_fp64_parity(lib, ctx, oracle, D1, D2, os_, mode, pos, sup, N):
    support = _support(D1, D2)
    M, _ = _measured(D1 * 13 + N, D1, D2, os_, support=support)
    kw = dict(oversamplingRatio=os_, numIterations=N, constraintEnforcementMode=mode, constraintPositivity=pos,
              constraintSupport=sup)
    rec, errK, _, _, _ = ctx.reconstruct(params(lib, D1, D2, 1, **kw), M, support=support)
    reco, errKo, _, _, _ = oracle.reconstruct(oracle.make_params(D1, D2, 1, **kw), M, support=support)
    assert rel(rec, reco) < FP64_TOL
    assert np.abs(errK - errKo).max() < FP64_TOL * max(1.0, np.abs(errKo).max())


def test_reconstruct_initial_object_and_mask(lib, ctx, oracle):
    D, os_ = 8, 2.0
    support = _support(D, D)
    M, vol = _measured(3, D, D, os_, support=support)
    rng = np.random.default_rng(4)
    mask = (M != 0) & (rng.random(M.shape) < 0.7)
    init = rng.standard_normal((D, D, D))
    kw = dict(oversamplingRatio=os_, numIterations=15, constraintEnforcementMode=3)
    rec, errK, _, _, _ = ctx.reconstruct(params(lib, D, D, 1, **kw), M, support=support, initial=init, mask=mask)
    reco, errKo, _, _, _ = oracle.reconstruct(oracle.make_params(D, D, 1, **kw), M, support=support, initial=init,
                                              mask=mask)
    assert rel(rec, reco) < FP64_TOL
    assert np.abs(errK - errKo).max() < FP64_TOL


def test_reconstruct_staged_equals_one_shot(lib, ctx):
    D, os_ = 8, 2.0
    M, _ = _measured(5, D, D, os_)
    p = params(lib, D, D, 1, oversamplingRatio=os_, numIterations=20, constraintEnforcementMode=1)
    rec, errK, _, _, _ = ctx.reconstruct(p, M)
    r = ctx.recon(p, M)
    for c in (1, 5, 14):
        r.iterate(c)
    rec2, errK2, _, _, _ = r.result()
    r.close()
    assert np.array_equal(rec, rec2) and np.array_equal(errK, errK2)
    r = ctx.recon(p, M)
    with pytest.raises(lib.GenfireError) as e:
        r.iterate(21)
    assert e.value.status == 6


def test_reconstruct_fixed_point(lib, ctx):
    """All points measured and consistent: the object is returned unchanged."""
    rng = np.random.default_rng(6)
    D, n = 8, 16
    vol = rng.random((D, D, D))
    M = np.fft.fftshift(np.fft.fftn(np.fft.ifftshift(NR.paddzero(vol, (n, n, n)))))
    rec, errK, _, _, _ = ctx.reconstruct(params(lib, D, D, 1, oversamplingRatio=2, numIterations=3,
                                                constraintEnforcementMode=3), M, initial=vol)
    assert np.abs(rec - vol).max() < 1e-12
    assert errK[0] < 1e-13


@pytest.mark.parametrize("D1,D2,os_,mode", [(16, 16, 2.0, 3), (12, 10, 2.0, 1), (15, 15, 2.0, 3)])
def test_reconstruct_mixed_tolerance(lib, ctx, oracle, D1, D2, os_, mode):
    support = _support(D1, D2)
    M, _ = _measured(D1 + 77, D1, D2, os_, support=support)
    M = M.astype(np.complex64)
    kw = dict(oversamplingRatio=os_, numIterations=25, constraintEnforcementMode=mode)
    rec, errK, _, _, _ = ctx.reconstruct(params(lib, D1, D2, 1, precision="mixed", **kw), M, support=support)
    reco, errKo, _, _, _ = oracle.reconstruct(oracle.make_params(D1, D2, 1, **kw), M.astype(np.complex128),
                                              support=support)
    assert rec.dtype == np.float32
    assert rel(rec, reco) < 1e-4
    assert np.abs(errK - errKo).max() < 1e-5


def test_monitor_rfactor_matches_oracle(lib, ctx, oracle):
    rng = np.random.default_rng(8)
    D, P = 10, 4
    vol = rng.random((D, D, D))
    angles = np.asfortranarray(np.stack([rng.uniform(0, 360, P), rng.uniform(-60, 60, P), rng.uniform(0, 360, P)], 1))
    projs = np.asfortranarray(np.stack([oracle.project(vol, *a) for a in angles], 2))
    kw = dict(oversamplingRatio=2.0, interpolationCutoffDistance=0.5, numIterations=6, constraintEnforcementMode=3,
              monitor_R=1, monitorR_loopLength=2, vector3=(0, 0, 1))
    M, _, _ = ctx.grid_dft(params(lib, D, D, P, **kw), projs, angles)
    rec, errK, errR, Rarr, Rarr2 = ctx.reconstruct(params(lib, D, D, P, **kw), M, projections=projs, angles=angles)
    op = oracle.make_params(D, D, P, **kw)
    Mo, _, _ = oracle.grid_dft(op, projs, angles)
    reco, errKo, errRo, Rarro, Rarr2o = oracle.reconstruct(op, Mo, projs=projs, angles=angles)
    assert errR.shape == (3,) and Rarr.shape == (P, 3)
    assert np.abs(errR - errRo).max() < 1e-9
    assert np.abs(Rarr - Rarro).max() < 1e-9 and np.abs(Rarr2 - Rarr2o).max() < 1e-9


def test_reconstruct_rejects_bad_mode(lib, ctx):
    M, _ = _measured(1, 8, 8, 2.0)
    with pytest.raises(lib.GenfireError) as e:
        ctx.reconstruct(params(lib, 8, 8, 1, oversamplingRatio=2, constraintEnforcementMode=4), M)
    assert e.value.status == 1 and "not understood" in str(e.value)


@pytest.mark.parametrize("pinned", [False, True])
def test_large_host_buffers_page_locked_or_not(lib, ctx, pinned):
    """Host buffers of 64 MB and more are page-locked for their copy (cudaHostRegister,
    released before the call returns); a buffer the caller has already page-locked
    makes the registration fail and the copy runs as given.  Both give the results
    of the same data copied from device memory: a 128^3 object on a 256^3 grid
    (the complex64 measured grid is 134 MB)."""
    torch = pytest.importorskip("torch")
    D, os_ = 128, 2.0
    rng = np.random.default_rng(11)
    n = 256
    M = np.zeros((n, n, n), np.complex64, order="F")
    idx = rng.integers(0, n, size=(3, 20000))
    M[idx[0], idx[1], idx[2]] = (rng.standard_normal(20000) + 1j * rng.standard_normal(20000)).astype(np.complex64)
    M = np.asfortranarray(M)
    p = params(lib, D, D, 1, oversamplingRatio=os_, numIterations=3, constraintEnforcementMode=1,
               precision="mixed")
    d_M = torch.from_numpy(M.reshape(-1, order="F").view(np.float32)).cuda()
    r = ctx.recon(p, d_M.data_ptr(), on_device=True)
    r.iterate(3)
    ref, errK_ref, _, _, _ = r.result()
    r.close()
    if pinned:
        t = torch.empty(M.size * 2, dtype=torch.float32, pin_memory=True)
        host = t.numpy().view(np.complex64).reshape(M.shape, order="F")
        host[...] = M
    else:
        host = M
    assert host.nbytes >= 64 << 20
    rec, errK, _, _, _ = ctx.reconstruct(p, host)
    assert np.array_equal(rec, ref) and np.array_equal(errK, errK_ref)
    # the caller's buffer is left as it was: registrable again (not left page-locked by the call)
    rec2, _, _, _, _ = ctx.reconstruct(p, host)
    assert np.array_equal(rec2, ref)


@pytest.mark.parametrize("n,prec", [(512, "mixed"), (128, "mixed"), (128, "fp64"), (192, "mixed"), (100, "mixed")])
def test_support_masks_leave_the_reconstruction_unchanged(lib, ctx, n, prec):
    """A sparse support lets F1 write zero half spectra for the box's row pairs
    without support voxels and I1 skip them, in every row-pass engine (radix-32
    at 512^3, the register passes at 128^3 in FP32 and FP64, the mixed-radix
    passes at 192^3, the generic passes at 100^3); at 512^3 the dim-2 passes
    do the same for empty slabs.
    Only the R-factor monitor, which projects the raw iterate, turns the
    inverse skipping off.  The reconstruction and errK with the monitor on and
    off are identical, and the monitor's R-factors are finite."""
    D, P = n // 2, 2
    rng = np.random.default_rng(21)
    M = np.zeros((n, n, n), np.complex64 if prec == "mixed" else np.complex128, order="F")
    nk, w = 40000 * n // 512, 60 * n // 512
    k = rng.integers(n // 2 - w, n // 2 + w, size=(3, nk))
    M[k[0], k[1], k[2]] = rng.standard_normal(nk) + 1j * rng.standard_normal(nk)
    g = np.indices((D, D, D)) - D // 2
    support = np.asfortranarray((g[0] ** 2 + g[1] ** 2 + (1.6 * g[2]) ** 2) <= (100 * D // 256) ** 2)
    projs = np.asfortranarray(rng.random((D, D, P)))
    angles = np.asfortranarray([[10.0, 20.0, 30.0], [50.0, -40.0, 70.0]])
    out = {}
    for mon in (0, 1):
        p = params(lib, D, D, P, oversamplingRatio=2.0, numIterations=6, constraintEnforcementMode=3,
                   monitor_R=mon, monitorR_loopLength=3, vector3=(0, 0, 1), precision=prec)
        out[mon] = ctx.reconstruct(p, M, support=support, projections=projs, angles=angles)
    rec0, errK0 = out[0][0], out[0][1]
    rec1, errK1, errR1 = out[1][0], out[1][1], out[1][2]
    assert np.array_equal(rec0, rec1) and np.array_equal(errK0, errK1)
    assert errR1.shape == (2,) and np.all(np.isfinite(errR1))
    assert np.abs(rec0).max() > 0
