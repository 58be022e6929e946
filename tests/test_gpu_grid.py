"""DFT gridding on the GPU through the C ABI, against the CPU oracle.

Bar: K-point index sets, distances and in-plane coordinates bit-exact; FP64
gridded values and recIFFT within relative L2 1e-10; MIXED within 1e-4."""
import hashlib

import numpy as np
import pytest

from tests.conftest import params, rel

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-10
MIXED_TOL = 1e-4


def _sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


SEL_CASES = [
    # D, os, cutoff, centro, vectors
    (8, 2, 0.125, 1, "zyx"), (9, 2, 0.3, 1, "zyz"), (10, 3, 0.7, 1, "zyx"), (7, 2.5, 0.5, 0, "zyx"),
    (8, 2, 0.125, 0, "zyz"), (16, 4, 0.125, 1, "zyx"), (13, 3, 1.2, 1, "zyz"), (12, 1.5, 0.25, 0, "zyx"),
]
VEC = {"zyx": ((0, 0, 1), (0, 1, 0), (1, 0, 0)), "zyz": ((0, 0, 1), (0, 1, 0), (0, 0, 1))}


@pytest.mark.parametrize("D,os_,cut,centro,vec", SEL_CASES)
def test_selection_bit_exact(lib, ctx, oracle, D, os_, cut, centro, vec):
    rng = np.random.default_rng(100 + D)
    v1, v2, v3 = VEC[vec]
    p = params(lib, D, D, 1, oversamplingRatio=os_, interpolationCutoffDistance=cut, DFT_CentroSymmetricity=centro,
               vector1=v1, vector2=v2, vector3=v3)
    op = oracle.make_params(D, D, 1, oversamplingRatio=os_, interpolationCutoffDistance=cut,
                            DFT_CentroSymmetricity=centro, vector1=v1, vector2=v2, vector3=v3)
    n1, n2 = lib.grid_size(p)
    angles = [(0, 0, 0), (0, 90, 0), (90, 45, 0), (0, -70, 0), (45, 45, 45)]
    angles += [tuple(x) for x in np.stack([rng.uniform(0, 360, 6), rng.uniform(-80, 80, 6),
                                           rng.uniform(0, 360, 6)], 1)]
    for ang in angles:
        g = ctx.select(p, *ang)
        Rf, nrm = oracle.proj_geometry(op, *ang)
        o = oracle.select(n1, n2, centro, cut, Rf, nrm)
        for a, b in zip(g, o[:4]):
            assert np.array_equal(a, b), ang


def _random_case(seed, D1, D2, P):
    rng = np.random.default_rng(seed)
    projs = np.asfortranarray(rng.random((D1, D2, P)))
    angles = np.asfortranarray(np.stack([rng.uniform(0, 360, P), rng.uniform(-75, 75, P), rng.uniform(0, 360, P)], 1))
    return projs, angles


GRID_CASES = [
    # D1, D2, P, os, cutoff, centro
    (16, 16, 6, 2.0, 0.3, 1), (15, 15, 5, 2.0, 0.5, 1), (16, 16, 4, 3.0, 0.125, 1), (12, 14, 5, 2.0, 0.4, 1),
    (10, 10, 4, 2.5, 0.7, 1), (11, 11, 3, 2.5, 0.5, 0), (16, 16, 3, 2.0, 0.3, 0), (9, 10, 4, 3.0, 0.6, 1),
]


@pytest.mark.parametrize("D1,D2,P,os_,cut,centro", GRID_CASES)
def test_grid_dft_fp64_parity(lib, ctx, oracle, D1, D2, P, os_, cut, centro):
    projs, angles = _random_case(D1 * 7 + P, D1, D2, P)
    kw = dict(oversamplingRatio=os_, interpolationCutoffDistance=cut, DFT_CentroSymmetricity=centro)
    M, rec, nk = ctx.grid_dft(params(lib, D1, D2, P, **kw), projs, angles)
    Mo, reco, nko = oracle.grid_dft(oracle.make_params(D1, D2, P, **kw), projs, angles)
    assert np.array_equal(nk, nko)
    assert np.array_equal(M != 0, Mo != 0)
    assert rel(M, Mo) < FP64_TOL
    assert rel(rec, reco) < FP64_TOL


@pytest.mark.parametrize("prec", ["mixed", "fp16"])
@pytest.mark.parametrize("D1,D2,P,os_,cut,centro", GRID_CASES[:5])
def test_grid_dft_mixed_tolerance(lib, ctx, oracle, D1, D2, P, os_, cut, centro, prec):
    projs, angles = _random_case(D1 * 11 + P, D1, D2, P)
    kw = dict(oversamplingRatio=os_, interpolationCutoffDistance=cut, DFT_CentroSymmetricity=centro)
    M, rec, nk = ctx.grid_dft(params(lib, D1, D2, P, precision=prec, **kw), projs, angles)
    Mo, reco, nko = oracle.grid_dft(oracle.make_params(D1, D2, P, **kw), projs, angles)
    assert M.dtype == np.complex64 and rec.dtype == np.float32
    assert np.array_equal(nk, nko)
    assert rel(M, Mo) < MIXED_TOL
    assert rel(rec, reco) < MIXED_TOL


def test_exact_hits_last_projection_wins(lib, ctx):
    """Every plane contains k = 0 with D = 0: measuredK(0) is the last projection's sum."""
    projs, angles = _random_case(5, 12, 12, 4)
    M, _, _ = ctx.grid_dft(params(lib, 12, 12, 4, oversamplingRatio=2, interpolationCutoffDistance=0.3), projs, angles)
    c = 12
    assert M[c, c, c].imag == 0
    assert M[c, c, c].real == pytest.approx(projs[:, :, -1].sum(), rel=1e-13)


def test_theta0_plane_equals_padded_fft(lib, ctx):
    """A single untilted projection fills exactly the k3 = 0 plane with its padded FFT."""
    rng = np.random.default_rng(9)
    D, n = 8, 16
    proj = np.asfortranarray(rng.random((D, D, 1)))
    M, _, nk = ctx.grid_dft(params(lib, D, D, 1, oversamplingRatio=2, interpolationCutoffDistance=0.125), proj,
                            np.zeros((1, 3)))
    pad = np.zeros((n, n)); pad[4:12, 4:12] = proj[:, :, 0]
    ref = np.fft.fftshift(np.fft.fft2(np.fft.ifftshift(pad)))
    assert nk[0] == 9 * 17
    assert np.abs(M[:, :, 8] - ref).max() < 1e-12 * np.abs(ref).max()
    M[:, :, 8] = 0
    assert not M.any()


def test_tiny_cutoff_keeps_only_exact_hits(lib, ctx, oracle):
    projs, angles = _random_case(3, 8, 8, 3)
    kw = dict(oversamplingRatio=2, interpolationCutoffDistance=1e-12)
    M, _, nk = ctx.grid_dft(params(lib, 8, 8, 3, **kw), projs, angles)
    Mo, _, nko = oracle.grid_dft(oracle.make_params(8, 8, 3, **kw), projs, angles)
    assert np.array_equal(nk, nko)
    assert rel(M, Mo) < FP64_TOL


def test_golden_turb3_on_gpu(lib, ctx, golden):
    from tests.golden.make_golden import TURB3_PARAMS
    projs, angles = golden["subset"]["projections"], golden["subset"]["angles"]
    g = golden["oracle"]
    kw = {k: v for k, v in TURB3_PARAMS.items()}
    p = params(lib, projs.shape[0], projs.shape[1], projs.shape[2], **kw)
    for i in range(projs.shape[2]):
        ind, dist, u, v = ctx.select(p, *angles[i])
        assert [_sha(ind.astype(np.int64)), _sha(dist), _sha(u), _sha(v)] == list(g["digests"][i])
    M, rec, nk = ctx.grid_dft(p, projs, angles)
    assert np.array_equal(nk, g["nk"])
    flat = M.reshape(-1, order="F")
    assert np.count_nonzero(flat) == int(g["nnz"])
    assert rel(flat[g["sample_idx"]], g["sample_val"]) < FP64_TOL
    assert rel(rec[:, :, p.Dim1 // 2], g["rec_slice"]) < FP64_TOL


@pytest.mark.parametrize("field,value,status", [
    ("oversamplingRatio", 0.5, 1), ("interpolationCutoffDistance", 0.0, 1), ("precision", 9, 1),
    ("Dim1", 1, 1), ("oversamplingRatio", 11.0 / 8.0, 5),
])
def test_grid_dft_rejects_bad_parameters(lib, ctx, field, value, status):
    projs, angles = _random_case(1, 8, 8, 2)
    p = params(lib, 8, 8, 2, oversamplingRatio=2)
    setattr(p, field, value)
    if field == "oversamplingRatio" and status == 5:
        p.interpolationCutoffDistance = 0.3  # n = 11: prime factor 11 is outside the FFT's radix set
    with pytest.raises(lib.GenfireError) as e:
        ctx.grid_dft(p, projs, angles)
    assert e.value.status == status
    assert str(e.value).startswith("GENFIRE:")


@pytest.mark.parametrize("form", ["n128", "n256"])
@pytest.mark.parametrize("prec", ["mixed", "fp16"])
@pytest.mark.parametrize("D1,D2,P,os_,cut", [(64, 64, 12, 2.0, 0.125), (40, 300, 3, 2.0, 0.3), (100, 72, 4, 2.0, 0.2),
                                             (128, 128, 3, 2.0, 0.125), (300, 40, 2, 2.0, 0.3),
                                             (280, 144, 2, 2.0, 0.2)])
def test_grid_dft_mixed_tensor_core_shapes(lib, ctx, oracle, monkeypatch, D1, D2, P, os_, cut, prec, form):
    """Tensor-core DFT (split BF16 and split FP16), both forms (N = 128 with
    128-point tiles, the default; N = 256 with Re and Im stacked in rows and
    64-point tiles): several tiles, K (D1) not a multiple of 32 and above one
    block's rows (256 or 128), N (D2) not a multiple of 16 and above one
    block's columns (128 or 256), a non-power-of-two grid (FP64 phase
    reduction)."""
    monkeypatch.setenv("GENFIRE_DFT_KERNEL", form)
    projs, angles = _random_case(D1 + D2 + P, D1, D2, P)
    kw = dict(oversamplingRatio=os_, interpolationCutoffDistance=cut, vector3=(0, 0, 1))
    M, rec, nk = ctx.grid_dft(params(lib, D1, D2, P, precision=prec, **kw), projs, angles)
    Mo, reco, nko = oracle.grid_dft(oracle.make_params(D1, D2, P, **kw), projs, angles)
    assert np.array_equal(nk, nko)
    assert np.array_equal(M != 0, Mo != 0)
    assert rel(M, Mo) < MIXED_TOL
    assert rel(rec, reco) < MIXED_TOL


def test_fp16_scaled_is_more_accurate_than_bf16(lib, ctx, oracle):
    """Split FP16 keeps ~22 bits per operand against split BF16's ~16: on the same
    projections its gridding error is well below the BF16 one (both below 1e-4)."""
    D, P = 64, 8
    projs, angles = _random_case(4242, D, D, P)
    kw = dict(oversamplingRatio=2.0, interpolationCutoffDistance=0.125)
    Mo, _, _ = oracle.grid_dft(oracle.make_params(D, D, P, **kw), projs, angles, want_rec=False)
    e = {}
    for prec in ("mixed", "fp16"):
        M, _, _ = ctx.grid_dft(params(lib, D, D, P, precision=prec, **kw), projs, angles, want_rec=False)
        e[prec] = rel(M, Mo)
    assert e["mixed"] < MIXED_TOL and e["fp16"] < 1e-5
    assert e["fp16"] < 0.25 * e["mixed"], e


@pytest.mark.parametrize("amp", [1e-7, 1e7])
def test_fp16_scaled_per_projection_scaling(lib, ctx, oracle, amp):
    """Amplitudes far outside FP16's range (1e-7 would underflow, 1e7 overflow)
    grid within 1e-5 of the oracle: each projection is scaled by a power of two
    before the split and the scale is undone exactly."""
    D, P = 32, 3
    projs, angles = _random_case(99, D, D, P)
    projs = np.asfortranarray(projs * amp * np.array([1.0, 3.0, 0.5]))
    kw = dict(oversamplingRatio=2.0, interpolationCutoffDistance=0.3)
    M, _, nk = ctx.grid_dft(params(lib, D, D, P, precision="fp16", **kw), projs, angles, want_rec=False)
    Mo, _, nko = oracle.grid_dft(oracle.make_params(D, D, P, **kw), projs, angles, want_rec=False)
    assert np.array_equal(nk, nko)
    assert np.all(np.isfinite(M))
    assert rel(M, Mo) < 1e-5


def test_reconstructor_fp16_scaled_dft_gridding(lib, ctx, oracle, tmp_path):
    """GENFIRE_Reconstructor(precision='fp16_scaled', griddingMethod=2): readFiles ->
    CheckPrepareData -> runGridding (split-FP16 tensor-core DFT, single measuredK)
    -> reconstruct, against the oracle's FP64 chain."""
    from genfire_gb300 import GENFIRE_Reconstructor
    D, P, iters = 32, 10, 20
    projs, angles = _random_case(515, D, D, P)
    np.save(tmp_path / "pj.npy", projs)
    np.save(tmp_path / "ang.npy", angles)
    G = GENFIRE_Reconstructor(filename_Projections=str(tmp_path / "pj.npy"), filename_Angles=str(tmp_path / "ang.npy"),
                              oversamplingRatio=2, interpolationCutoffDistance=0.3, numIterations=iters,
                              griddingMethod=2, constraintEnforcementMode=3, precision="fp16_scaled")
    G = G.readFiles().CheckPrepareData().runGridding().reconstruct()
    assert G.measuredK.dtype == np.complex64
    prm = oracle.make_params(D, D, P, oversamplingRatio=2, interpolationCutoffDistance=0.3, numIterations=iters,
                             constraintEnforcementMode=3)
    Mo, _, _ = oracle.grid_dft(prm, projs, angles, want_rec=False)
    assert rel(G.measuredK, Mo) < 1e-5
    reco, errKo = oracle.reconstruct(prm, Mo)[:2]
    assert rel(G.reconstruction, reco) < 1e-4
    assert np.abs(np.asarray(G.errK).ravel() - np.asarray(errKo).ravel()).max() < 1e-4
