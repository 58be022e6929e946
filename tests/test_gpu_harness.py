"""The standalone C harness in file mode (Genfire_test.m without MATLAB): MAT
inputs written by scipy, gridding + reconstruct + Tian R-factor through the C
ABI, results saved to a MAT file.  Its outputs equal the same ABI calls made
from Python (DFT gridding is deterministic: bit-equal; FFT gridding sums
with FP64 atomics: within 1e-12)."""
import subprocess

import numpy as np
import pytest

from tests.conftest import params, rel

pytestmark = pytest.mark.gpu
scipy_io = pytest.importorskip("scipy.io")


def _inputs(ctx, tmp_path, D=16, P=7, seed=2):
    rng = np.random.default_rng(seed)
    vol = np.zeros((D, D, D))
    g = np.indices((D, D, D)) - D // 2
    for _ in range(4):
        c = (rng.random(3) - 0.5) * D * 0.4
        vol += np.exp(-((g[0] - c[0]) ** 2 + (g[1] - c[1]) ** 2 + (g[2] - c[2]) ** 2) / 6.0)
    ang = np.asfortranarray(np.stack([rng.uniform(0, 360, P), rng.uniform(-60, 60, P), rng.uniform(0, 360, P)], 1))
    pj = ctx.project(vol, ang)
    fp, fa = str(tmp_path / "pj.mat"), str(tmp_path / "angles.mat")
    scipy_io.savemat(fp, {"pj": pj}, do_compression=True)
    scipy_io.savemat(fa, {"angles": ang}, do_compression=False)
    return pj, ang, fp, fa


def _run(harness, args):
    r = subprocess.run([harness] + args, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    return r.stdout


@pytest.fixture(scope="module")
def harness(lib):
    from genfire_gb300 import build
    return build.HARNESS


@pytest.mark.parametrize("prec", ["fp64", "mixed", "fp16"])
def test_harness_dft_equals_python(lib, ctx, harness, tmp_path, prec):
    pj, ang, fp, fa = _inputs(ctx, tmp_path)
    D, P, N = pj.shape[0], pj.shape[2], 12
    out = str(tmp_path / "res.mat")
    _run(harness, ["--projections", fp, "--angles", fa, "--results", out, "--gridding", "2", "--oversampling", "2",
                   "--cutoff", "0.3", "--iterations", str(N), "--mode", "3", "--vector3", "0,0,1",
                   "--precision", {"fp16": "fp16_scaled"}.get(prec, prec)])
    res = scipy_io.loadmat(out)
    p = params(lib, D, D, P, oversamplingRatio=2.0, interpolationCutoffDistance=0.3, numIterations=N,
               constraintEnforcementMode=3, vector3=(0, 0, 1), precision=prec)
    M, _, _ = ctx.grid_dft(p, pj, ang)
    rec, errK, _, _, _ = ctx.reconstruct(p, M, support=np.ones((D, D, D), bool))
    assert res["final_Rec"].dtype == (np.float64 if prec == "fp64" else np.float32)
    assert np.array_equal(res["final_Rec"], rec)
    assert np.array_equal(res["final_errK"].ravel(), errK)
    assert res["final_Kfactor"].item() == errK.min()
    Rt, Rarr, simu = ctx.rfactor_realspace(rec.astype(np.float64), pj, ang)
    assert res["final_Rfactor"].item() == Rt
    assert np.array_equal(res["final_Rarray"].ravel(), Rarr)
    assert np.array_equal(res["final_simuProjs"], simu)


def test_harness_fft_gridding_and_single_angle_column(lib, ctx, harness, tmp_path):
    """griddingMethod 1 (the class default) and a one-column angle file, which
    CheckPrepareData turns into [0, theta, 0]."""
    pj, ang, fp, _ = _inputs(ctx, tmp_path, D=12, P=5, seed=4)
    theta = np.asfortranarray(ang[:, 1:2])
    fa = str(tmp_path / "theta.mat")
    scipy_io.savemat(fa, {"theta": theta})
    D, P, N = 12, 5, 8
    out = str(tmp_path / "res.mat")
    _run(harness, ["--projections", fp, "--angles", fa, "--results", out, "--oversampling", "2", "--cutoff", "0.5",
                   "--iterations", str(N), "--mode", "3", "--no-rfactor"])
    res = scipy_io.loadmat(out)
    full = np.asfortranarray(np.concatenate([np.zeros((P, 1)), theta, np.zeros((P, 1))], 1))
    p = params(lib, D, D, P, oversamplingRatio=2.0, interpolationCutoffDistance=0.5, numIterations=N,
               constraintEnforcementMode=3, griddingMethod=1)
    M, _, _ = ctx.grid_fft(p, pj, full)
    rec, errK, _, _, _ = ctx.reconstruct(p, M, support=np.ones((D, D, D), bool))
    assert "final_Rfactor" not in res
    assert rel(res["final_Rec"], rec) < 1e-12
    assert np.abs(res["final_errK"].ravel() - errK).max() < 1e-12


def test_harness_input_errors(harness, tmp_path):
    fp = str(tmp_path / "pj.mat")
    fa = str(tmp_path / "a.mat")
    scipy_io.savemat(fp, {"pj": np.ones((8, 8, 3))})
    scipy_io.savemat(fa, {"a": np.ones((4, 3))})
    r = subprocess.run([harness, "--projections", fp, "--angles", fa], capture_output=True, text=True, timeout=60)
    assert r.returncode == 1 and "Number of projections and Angles does not match" in r.stderr
    r = subprocess.run([harness, "--projections", str(tmp_path / "none.mat"), "--angles", fa], capture_output=True,
                       text=True, timeout=60)
    assert r.returncode == 1 and "cannot open" in r.stderr


def test_harness_save_temp_and_rfree(lib, ctx, harness, tmp_path):
    """--save-temp writes temp_reconstruction every L iterations without
    changing the result; --rfree withholds points per shell (seeded, so
    repeatable) and saves final_Rfree (shells x iterations)."""
    pj, ang, fp, fa = _inputs(ctx, tmp_path, D=12, P=6, seed=7)
    N = 10
    base = ["--projections", fp, "--angles", fa, "--gridding", "2", "--oversampling", "2", "--cutoff", "0.4",
            "--iterations", str(N), "--mode", "1", "--no-rfactor"]
    plain, saved = str(tmp_path / "plain.mat"), str(tmp_path / "saved.mat")
    _run(harness, base + ["--results", plain])
    _run(harness, base + ["--results", saved, "--save-temp", "4", "--save-prefix", str(tmp_path / "tmp_")])
    a, b = scipy_io.loadmat(plain), scipy_io.loadmat(saved)
    assert np.array_equal(a["final_Rec"], b["final_Rec"]) and np.array_equal(a["final_errK"], b["final_errK"])
    assert sorted(p.name for p in tmp_path.glob("tmp_*.mat")) == ["tmp_4.mat", "tmp_8.mat"]
    assert scipy_io.loadmat(str(tmp_path / "tmp_8.mat"))["temp_reconstruction"].shape == (12, 12, 12)
    outs = []
    for k in range(2):
        f = str(tmp_path / ("rf%d.mat" % k))
        _run(harness, base + ["--results", f, "--rfree", "4", "--rfree-percent", "0.1", "--seed", "3"])
        outs.append(scipy_io.loadmat(f))
    rf = outs[0]["final_Rfree"]
    assert rf.shape == (4, N) and np.all(np.isfinite(rf)) and np.all(rf > 0)
    assert np.array_equal(rf, outs[1]["final_Rfree"])
    assert not np.array_equal(outs[0]["final_errK"], a["final_errK"])  # the withheld points left errK
