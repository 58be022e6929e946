"""Host-side logic on the CPU: the GENFIRE_Reconstructor mirror (properties,
checks, error messages of GENFIRE_Reconstructor.m) and the synthetic
workload generator."""
import os

import numpy as np
import pytest

from genfire_gb300 import synth
from genfire_gb300.reconstructor import GENFIRE_Reconstructor, GenfireError


def test_defaults_match_reference_class():
    G = GENFIRE_Reconstructor()
    assert G.numIterations == 50 and G.oversamplingRatio == 3 and G.interpolationCutoffDistance == .7
    assert G.griddingMethod == 1 and G.constraintEnforcementMode == 1
    assert tuple(G.vector1) == (0, 0, 1) and tuple(G.vector2) == (0, 1, 0) and tuple(G.vector3) == (1, 0, 0)
    assert G.monitor_R == 0 and G.monitorR_loopLength == 10 and G.DFT_CentroSymmetricity == 1


def _prepared(P=3, D=8, **kw):
    G = GENFIRE_Reconstructor(**kw)
    G.InputProjections = np.zeros((D, D, P))
    G.InputAngles = np.zeros((P, 3))
    return G


def test_check_prepare_data_sizes_and_delays():
    G = _prepared(oversamplingRatio=2.5, constraintEnforcementMode=3).CheckPrepareData()
    assert (G.NumProjs, G.Dim1, G.Dim2) == (3, 8, 8)
    assert G.n1_oversampled == 20 and G.n2_oversampled == 20
    assert G.Support.shape == (8, 8, 8) and G.Support.all()
    assert list(G.constraintEnforcementDelayIndicators) == [-999] * 5
    G = _prepared(constraintEnforcementMode=1).CheckPrepareData()
    assert len(G.constraintEnforcementDelayIndicators) == 27
    G = _prepared(constraintEnforcementMode=2).CheckPrepareData()
    assert len(G.constraintEnforcementDelayIndicators) == 14


@pytest.mark.parametrize("mut,msg", [
    (lambda G: setattr(G, "InputAngles", np.zeros((2, 3))), "Number of projections and Angles does not match"),
    (lambda G: setattr(G, "InputAngles", np.zeros((3, 4))), "Input Angle 2nd dimenstions larger than three"),
    (lambda G: setattr(G, "constraintEnforcementMode", 7), "constraintEnforcementMode value 7 not understood"),
    (lambda G: setattr(G, "griddingMethod", 3), "Unrecognized gridding method"),
    (lambda G: setattr(G, "initialObject", np.zeros((4, 4, 4))), "Initial Model size does not match"),
])
def test_check_prepare_data_errors(mut, msg):
    G = _prepared()
    mut(G)
    with pytest.raises(GenfireError) as e:
        G.CheckPrepareData()
    assert msg in str(e.value) and str(e.value).startswith("GENFIRE:")


def test_single_angle_column_is_theta():
    G = _prepared(P=4)
    G.InputAngles = np.arange(4.0)[:, None]
    G.CheckPrepareData()
    assert np.array_equal(G.InputAngles[:, 1], np.arange(4.0))
    assert not G.InputAngles[:, [0, 2]].any()


def test_set_parameters():
    G = GENFIRE_Reconstructor()
    G.set_parameters("numIterations", 7, "oversamplingRatio", 2)
    assert G.numIterations == 7 and G.oversamplingRatio == 2
    with pytest.raises(GenfireError, match="not divisible by 2"):
        G.set_parameters("numIterations")
    with pytest.raises(GenfireError, match="Invalid option bogus"):
        G.set_parameters("bogus", 1)


def test_read_files(tmp_path):
    P = np.random.default_rng(0).random((6, 6, 2))
    A = np.zeros((2, 3))
    np.save(tmp_path / "p.npy", P)
    np.save(tmp_path / "a.npy", A)
    G = GENFIRE_Reconstructor(filename_Projections=str(tmp_path / "p.npy"), filename_Angles=str(tmp_path / "a.npy"))
    G.readFiles()
    assert np.array_equal(G.InputProjections, P)
    G.filename_Angles = str(tmp_path / "missing.npy")
    with pytest.raises(GenfireError, match="Angles file does not exist"):
        G.readFiles()


def test_params_mapping():
    G = _prepared(oversamplingRatio=2, interpolationCutoffDistance=.125, numIterations=9,
                  constraintEnforcementMode=3, precision="mixed", vector3=(0, 0, 1)).CheckPrepareData()
    from genfire_gb300 import _lib
    if not os.path.exists(_lib.LIB_PATH):
        pytest.skip("library not built")
    p = G.params()
    assert (p.Dim1, p.NumProjs, p.numIterations, p.constraintEnforcementMode) == (8, 3, 9, 3)
    assert p.precision == _lib.PREC_MIXED and list(p.vector3) == [0, 0, 1]


def test_synthetic_workload_is_seeded(oracle):
    def proj(vol, angles, vectors):
        v = np.asarray(vectors, dtype=float).reshape(-1)
        return np.stack([oracle.project(vol, *a, vectors=v) for a in angles], axis=2)
    a = synth.make_workload("euler128", proj, D=16, n_proj=4, atoms=5)
    b = synth.make_workload("euler128", proj, D=16, n_proj=4, atoms=5)
    assert np.array_equal(a["projections"], b["projections"]) and np.array_equal(a["angles"], b["angles"])
    assert a["projections"].shape == (16, 16, 4)
    assert a["support"].shape == (16, 16, 16) and a["support"].any()
    assert a["vol"].max() > 0
    t = synth.make_workload("tilt64", proj, D=16, n_proj=5, atoms=3)
    assert np.all(t["angles"][:, [0, 2]] == 0)


def test_gaussian_volume_is_analytic():
    v = synth.gaussian_volume(16, np.array([[0.0, 0.0, 0.0]]), [1.0], 1.5, dtype=np.float64)
    assert v[8, 8, 8] == pytest.approx(1.0)
    assert v[9, 8, 8] == pytest.approx(np.exp(-1 / (2 * 1.5 ** 2)))


def test_product_path_fails_loudly_without_the_library(monkeypatch, tmp_path):
    """Without libgenfire.so the package raises; it has no CPU fallback (the
    oracle is never imported by the package)."""
    from genfire_gb300 import _lib
    monkeypatch.setattr(_lib, "_lib", None)
    monkeypatch.setattr(_lib, "LIB_PATH", str(tmp_path / "libgenfire.so"))
    monkeypatch.setattr(GENFIRE_Reconstructor, "_ctx_cache", {})
    with pytest.raises(RuntimeError, match="not built"):
        _lib.Context(0)
    G = _prepared(oversamplingRatio=2, DFT_doGPU=1).CheckPrepareData()
    with pytest.raises(RuntimeError, match="not built"):
        G.runGridding()


def test_package_never_imports_the_oracle():
    import re
    root = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "genfire_gb300")
    for dirpath, _, files in os.walk(root):
        for f in files:
            if f.endswith(".py"):
                src = open(os.path.join(dirpath, f)).read()
                assert not re.search(r"^\s*(from|import)\s+oracle\b", src, flags=re.M), f
                assert "genfire_oracle" not in src and "oracle/" not in src, f
