"""FFT gridding (fillInFourierGrid.m, griddingMethod 1) on the GPU through the
C ABI, against the CPU oracle.

Bar: the number of gridded (voxel, value) pairs and the set of filled voxels
equal (the FP32 slice geometry is evaluated in the same operation order);
FP64 measuredK and recIFFT within relative L2 1e-10 (the GPU sums with FP64
atomics, so only the order of the additions differs); MIXED (FP32 projection
FFTs) within 1e-5."""
import numpy as np
import pytest

from tests.conftest import params, rel

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-10
MIXED_TOL = 1e-5

CASES = [
    # D1, D2, P, os, cutoff, allowMultipleGridMatches
    # (cube sizes 32, 32, 36, 28, 25, 36, 25, 64, 64: lengths with factors 2, 3, 5, 7)
    (16, 16, 6, 2.0, 0.7, 1), (16, 16, 6, 2.0, 0.7, 0), (15, 15, 5, 2.5, 0.5, 1), (12, 14, 4, 2.0, 0.4, 1),
    (10, 10, 4, 2.5, 1.6, 1), (11, 11, 3, 3.5, 0.9, 1), (9, 9, 5, 3.0, 0.125, 1), (16, 16, 1, 4.0, 0.7, 1),
    (32, 32, 12, 2.0, 0.7, 1),
]


def _case(seed, D1, D2, P):
    rng = np.random.default_rng(seed)
    projs = np.asfortranarray(rng.random((D1, D2, P)))
    angles = np.asfortranarray(np.stack([rng.uniform(0, 360, P), rng.uniform(-75, 75, P),
                                         rng.uniform(0, 360, P)], 1))
    angles[0] = (0, 0, 0)
    return projs, angles


def _kw(os_, cut, am):
    return dict(oversamplingRatio=os_, interpolationCutoffDistance=cut, allowMultipleGridMatches=am)


@pytest.mark.parametrize("D1,D2,P,os_,cut,am", CASES)
def test_grid_fft_fp64_parity(lib, ctx, oracle, D1, D2, P, os_, cut, am):
    projs, angles = _case(D1 * 13 + P, D1, D2, P)
    M, rec, n = ctx.grid_fft(params(lib, D1, D2, P, **_kw(os_, cut, am)), projs, angles)
    Mo, reco, no = oracle.grid_fft(oracle.make_params(D1, D2, P, oversamplingRatio=os_,
                                                      interpolationCutoffDistance=cut), projs, angles,
                                   allow_multiple=am)
    assert n == no
    assert M.shape == Mo.shape
    assert np.array_equal(M != 0, Mo != 0)
    assert rel(M, Mo) < FP64_TOL
    assert rel(rec, reco) < FP64_TOL


@pytest.mark.parametrize("D1,D2,P,os_,cut,am", CASES[:5])
def test_grid_fft_mixed_tolerance(lib, ctx, oracle, D1, D2, P, os_, cut, am):
    projs, angles = _case(D1 * 17 + P, D1, D2, P)
    M, rec, n = ctx.grid_fft(params(lib, D1, D2, P, precision="mixed", **_kw(os_, cut, am)), projs, angles)
    Mo, reco, no = oracle.grid_fft(oracle.make_params(D1, D2, P, oversamplingRatio=os_,
                                                      interpolationCutoffDistance=cut), projs, angles,
                                   allow_multiple=am)
    assert M.dtype == np.complex64 and rec.dtype == np.float32
    assert n == no
    assert rel(M, Mo) < MIXED_TOL
    assert rel(rec, reco) < MIXED_TOL


def test_grid_fft_device_entry_matches_host_entry(lib, ctx):
    import torch
    D, P = 16, 5
    projs, angles = _case(5, D, D, P)
    p = params(lib, D, D, P, **_kw(2.0, 0.7, 1))
    M, rec, n = ctx.grid_fft(p, projs, angles)
    m = M.shape[0]
    d_proj = torch.from_numpy(np.ascontiguousarray(projs.reshape(-1, order="F"))).cuda()
    d_M = torch.zeros(m ** 3, dtype=torch.complex128, device="cuda")
    d_rec = torch.zeros(D ** 3, dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    n2 = ctx.grid_fft_device(p, d_proj.data_ptr(), angles, d_M.data_ptr(), d_rec.data_ptr())
    torch.cuda.synchronize()
    assert n2 == n
    assert rel(d_M.cpu().numpy().reshape((m, m, m), order="F"), M) < 1e-13
    assert rel(d_rec.cpu().numpy().reshape((D, D, D), order="F"), rec) < 1e-13


@pytest.mark.parametrize("field,value", [("oversamplingRatio", 2.25), ("Dim1", 40)])
def test_grid_fft_rejects_bad_sizes(lib, ctx, field, value):
    # 16 * 2.25 = 36 is fine but 10 * 2.25 is not; Dim1 larger than the cube
    D = 10
    projs, angles = _case(1, D, D, 2)
    p = params(lib, D, D, 2, **_kw(2.0, 0.7, 1))
    setattr(p, field, value)
    if field == "Dim1":
        projs = np.zeros((value, D, 2))
    with pytest.raises(lib.GenfireError) as e:
        ctx.grid_fft(p, projs, angles)
    assert e.value.status == lib._lib.GENFIRE_ERR_ARG


def test_reconstructor_fft_gridding_end_to_end(lib, ctx, oracle, tmp_path):
    # GENFIRE_Reconstructor with its default griddingMethod = 1: readFiles ->
    # CheckPrepareData -> runGridding -> reconstruct, against the oracle chain
    from genfire_gb300 import GENFIRE_Reconstructor
    D, P, os_, cut, iters = 16, 8, 2, 0.7, 12
    projs, angles = _case(11, D, D, P)
    np.save(tmp_path / "pj.npy", projs)
    np.save(tmp_path / "ang.npy", angles)
    G = GENFIRE_Reconstructor(filename_Projections=str(tmp_path / "pj.npy"),
                              filename_Angles=str(tmp_path / "ang.npy"), oversamplingRatio=os_,
                              interpolationCutoffDistance=cut, numIterations=iters, constraintEnforcementMode=1)
    assert G.griddingMethod == 1
    G = G.readFiles().CheckPrepareData().runGridding().reconstruct()
    prm = oracle.make_params(D, D, P, oversamplingRatio=os_, interpolationCutoffDistance=cut,
                             numIterations=iters, constraintEnforcementMode=1)
    Mo, reco, _ = oracle.grid_fft(prm, projs, angles, allow_multiple=1)
    assert rel(G.measuredK, Mo) < FP64_TOL
    assert rel(G.recIFFT, reco) < FP64_TOL
    reco_o, errK_o = oracle.reconstruct(prm, Mo)[:2]
    assert rel(G.reconstruction, reco_o) < 1e-9
    assert np.abs(np.asarray(G.errK).ravel() - np.asarray(errK_o).ravel()).max() < 1e-9
