"""Cubic projector (interp3 'cubic' read as Keys' cubic convolution) and
Tian_calc_Rfactor_realspace on the GPU, against the oracle.  The cubic tests
use their own context so the session context stays trilinear."""
import numpy as np
import pytest

from tests.conftest import rel

pytestmark = pytest.mark.gpu


@pytest.fixture
def cubic_ctx(lib):
    c = lib.Context(0)
    c.set_projector_interpolation(lib._lib.INTERP_CUBIC)
    yield c
    c.close()


ANGLES = np.array([[0, 0, 0], [30, 40, 50], [10, -60, 200], [90, 90, 0], [123.4, 71.3, 300.2]])


@pytest.mark.parametrize("shape", [(9, 10, 11), (16, 16, 16), (33, 31, 20), (4, 5, 6)])
def test_cubic_project_fp64(lib, cubic_ctx, oracle, shape):
    rng = np.random.default_rng(sum(shape) + 1)
    vol = rng.random(shape)
    out = cubic_ctx.project(vol, ANGLES)
    for i, a in enumerate(ANGLES):
        assert rel(out[:, :, i], oracle.project_interp(vol, *a, cubic=True)) < 1e-12
    vecs = np.array([[0, 0, 1], [0, 1, 0], [1, 0, 0]], dtype=float)
    out = cubic_ctx.project(vol, ANGLES, vectors=vecs)
    for i, a in enumerate(ANGLES):
        assert rel(out[:, :, i], oracle.project_interp(vol, *a, vectors=vecs.reshape(-1), cubic=True)) < 1e-12


def test_cubic_project_mixed(lib, cubic_ctx, oracle):
    rng = np.random.default_rng(8)
    vol = rng.random((32, 32, 32))
    out = cubic_ctx.project(vol, ANGLES[:3], precision=lib.PREC_MIXED)
    assert out.dtype == np.float32
    for i, a in enumerate(ANGLES[:3]):
        assert rel(out[:, :, i], oracle.project_interp(vol, *a, cubic=True)) < 1e-5


def test_cubic_rfactor_matches_projections(lib, cubic_ctx, oracle):
    rng = np.random.default_rng(9)
    vol = rng.random((20, 20, 20))
    angles = ANGLES[1:]
    meas = np.stack([oracle.project_interp(vol, *a, cubic=True) for a in angles], 2) + rng.standard_normal((20, 20, 4))
    errR, R1, R2 = cubic_ctx.rfactor(vol, angles, meas)
    for i, a in enumerate(angles):
        bp = oracle.project_interp(vol, *a, cubic=True)
        r1, r2 = oracle.rfactor(bp, meas[:, :, i])
        assert abs(R1[i] - r1) <= 1e-12 * r1 and abs(R2[i] - r2) <= 1e-12 * r2
    assert abs(errR - R1.mean()) <= 1e-15


def test_interpolation_argument_checks(lib, ctx, cubic_ctx):
    with pytest.raises(lib.GenfireError) as e:
        ctx.set_projector_interpolation(7)
    assert e.value.status == lib._lib.GENFIRE_ERR_ARG
    with pytest.raises(lib.GenfireError) as e:
        cubic_ctx.project(np.ones((3, 8, 8)), ANGLES[:1])   # cubic needs 4 samples per dimension
    assert e.value.status == lib._lib.GENFIRE_ERR_ARG


@pytest.mark.parametrize("precision_name,interp", [("fp64", 0), ("mixed", 0), ("fp64", 1)])
def test_rfactor_realspace(lib, oracle, precision_name, interp):
    c = lib.Context(0)
    try:
        c.set_projector_interpolation(interp)
        prec = lib.PREC_FP64 if precision_name == "fp64" else lib.PREC_MIXED
        rng = np.random.default_rng(10 + interp)
        model = rng.random((24, 22, 20))
        P = 5
        angles = np.stack([rng.uniform(0, 360, P), rng.uniform(-60, 60, P), rng.uniform(0, 360, P)], 1)
        projs = rng.random((16, 15, P)) * 8
        tot, R, simu = c.rfactor_realspace(model, projs, angles, precision=prec)
        tot_o, R_o, simu_o = oracle.rfactor_realspace(model, projs, angles, cubic=bool(interp))
        tol = 1e-12 if prec == lib.PREC_FP64 else 1e-5
        assert np.abs(R - R_o).max() <= tol * R_o.max()
        assert abs(tot - tot_o) <= tol * tot_o
        assert simu.dtype == np.float32
        assert rel(simu, simu_o) < (1e-7 if prec == lib.PREC_FP64 else 1e-5)
    finally:
        c.close()
