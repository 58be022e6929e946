"""The real-space projector and R-factors on the GPU, against the oracle."""
import numpy as np
import pytest

from tests.conftest import rel

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("shape", [(9, 10, 11), (16, 16, 16), (33, 31, 20), (64, 64, 64)])
def test_project_fp64(lib, ctx, oracle, shape):
    rng = np.random.default_rng(sum(shape))
    vol = rng.random(shape)
    angles = np.array([[0, 0, 0], [30, 40, 50], [10, -60, 200], [90, 90, 0], [123.4, 71.3, 300.2]])
    out = ctx.project(vol, angles)
    for i, a in enumerate(angles):
        assert rel(out[:, :, i], oracle.project(vol, *a)) < 1e-12
    vecs = np.array([[0, 0, 1], [0, 1, 0], [1, 0, 0]], dtype=float)
    out = ctx.project(vol, angles, vectors=vecs)
    for i, a in enumerate(angles):
        assert rel(out[:, :, i], oracle.project(vol, *a, vectors=vecs.reshape(-1))) < 1e-12


def test_project_mixed(lib, ctx, oracle):
    rng = np.random.default_rng(3)
    vol = rng.random((32, 32, 32))
    angles = np.array([[0, 0, 0], [30, 40, 50], [250, -70, 10]])
    out = ctx.project(vol, angles, precision=lib.PREC_MIXED)
    assert out.dtype == np.float32
    for i, a in enumerate(angles):
        assert rel(out[:, :, i], oracle.project(vol, *a)) < 1e-5


def test_rfactor(lib, ctx, oracle):
    rng = np.random.default_rng(4)
    vol = rng.random((20, 20, 20))
    angles = np.stack([rng.uniform(0, 360, 5), rng.uniform(-70, 70, 5), rng.uniform(0, 360, 5)], 1)
    meas = np.stack([oracle.project(vol, *a) for a in angles], 2) + rng.standard_normal((20, 20, 5))
    errR, R1, R2 = ctx.rfactor(vol, angles, meas)
    for i, a in enumerate(angles):
        r1, r2 = oracle.rfactor(oracle.project(vol, *a), meas[:, :, i])
        assert R1[i] == pytest.approx(r1, rel=1e-12) and R2[i] == pytest.approx(r2, rel=1e-12)
    assert errR == pytest.approx(R1.mean(), rel=1e-14)
