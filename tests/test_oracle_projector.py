"""The oracle's cubic projector (interp3 'cubic' read as Keys' cubic
convolution) and its Tian_calc_Rfactor_realspace, against an independent
numpy restatement and known answers."""
import numpy as np
import pytest

from oracle import np_restate as NR


def _rot(oracle, phi, theta, psi):
    R = np.zeros(9)
    import ctypes as C
    oracle.lib().orc_rot_zyz(phi, theta, psi, R.ctypes.data_as(C.POINTER(C.c_double)))
    return R.reshape(3, 3, order="F")


@pytest.mark.parametrize("shape,ang", [((6, 7, 5), (30, 20, 10)), ((5, 5, 6), (0, 90, 0)), ((8, 6, 4), (123, -40, 71))])
def test_cubic_projector_matches_numpy(oracle, shape, ang):
    rng = np.random.default_rng(4)
    vol = rng.random(shape)
    got = oracle.project_interp(vol, *ang, cubic=True)
    want = NR.project_cubic(vol, _rot(oracle, *ang))
    assert np.abs(got - want).max() <= 1e-12 * np.abs(want).max()


def test_cubic_reproduces_quadratics(oracle):
    # Keys' kernel with a = -1/2 and Keys' boundary rule reproduce polynomials
    # of degree <= 2 exactly: the projection of a quadratic volume is the sum
    # of the quadratic at the rotated sample points inside the volume
    n1, n2, n3 = 9, 8, 10
    q = lambda x, y, z: 1.0 + 0.3 * x - 0.2 * y + 0.05 * z + 0.01 * x * x - 0.02 * y * z + 0.015 * z * z
    I, J, K = np.meshgrid(np.arange(n1), np.arange(n2), np.arange(n3), indexing="ij")
    vol = q(I, J, K).astype(np.float64)
    phi, theta, psi = 17.0, 33.0, -21.0
    R = _rot(oracle, phi, theta, psi)
    c = np.array([n1 // 2, n2 // 2, n3 // 2])
    want = np.zeros((n1, n2))
    for i in range(n1):
        for j in range(n2):
            for k in range(n3):
                r = R @ (np.array([i, j, k]) - c) + c
                if 0 <= r[0] <= n1 - 1 and 0 <= r[1] <= n2 - 1 and 0 <= r[2] <= n3 - 1:
                    want[i, j] += q(*r)
    got = oracle.project_interp(vol, phi, theta, psi, cubic=True)
    assert np.abs(got - want).max() <= 1e-11 * np.abs(want).max()
    # trilinear does not (the quadratic terms), which the check can tell apart
    lin = oracle.project_interp(vol, phi, theta, psi, cubic=False)
    assert np.abs(lin - want).max() > 1e-6


def test_cubic_identity_is_axis_sum(oracle):
    rng = np.random.default_rng(5)
    vol = rng.random((6, 5, 7))
    got = oracle.project_interp(vol, 0, 0, 0, cubic=True)
    assert np.abs(got - vol.sum(axis=2)).max() <= 1e-12


def test_rfactor_realspace(oracle):
    # Tian_calc_Rfactor_realspace: ZYX projections cropped to the measured size
    rng = np.random.default_rng(6)
    model = rng.random((12, 12, 12))
    P = 3
    angles = np.stack([rng.uniform(0, 360, P), rng.uniform(-60, 60, P), rng.uniform(0, 360, P)], 1)
    projs = rng.random((8, 10, P)) * 5
    tot, R, simu = oracle.rfactor_realspace(model, projs, angles)
    zyx = ((0, 0, 1), (0, 1, 0), (1, 0, 0))
    for q in range(P):
        bp = oracle.project_interp(model, *angles[q], vectors=zyx)
        crop = NR.stripzero(bp, (8, 10))
        want = np.abs(np.abs(crop) - np.abs(projs[:, :, q])).sum() / np.abs(projs[:, :, q]).sum()
        assert abs(R[q] - want) <= 1e-13 * want
        assert np.array_equal(simu[:, :, q], crop)
    assert abs(tot - R.mean()) <= 1e-15


def test_projectors_randomized_against_numpy(oracle):
    """Trilinear and cubic projectors of the C oracle against the numpy
    restatements over random volume shapes (odd and even sides) and angles,
    including right angles where samples fall on voxel faces."""
    hyp = pytest.importorskip("hypothesis")
    st = hyp.strategies
    angle = st.one_of(st.floats(-360, 360, allow_nan=False), st.sampled_from([0.0, 90.0, -90.0, 180.0]))

    @hyp.settings(max_examples=30, deadline=None, derandomize=True)
    @hyp.given(shape=st.tuples(st.integers(3, 9), st.integers(3, 9), st.integers(3, 9)), ang=st.tuples(angle, angle, angle),
               seed=st.integers(0, 2 ** 16))
    def check(shape, ang, seed):
        vol = np.random.default_rng(seed).random(shape)
        R = _rot(oracle, *ang)
        for cubic, ref in ((False, NR.project), (True, NR.project_cubic)):
            got = oracle.project_interp(vol, *ang, cubic=cubic)
            want = ref(vol, R)
            assert np.abs(got - want).max() <= 1e-12 * max(1.0, np.abs(want).max())

    check()
