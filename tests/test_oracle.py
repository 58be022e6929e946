"""The CPU oracle pinned against the mathematics, an independent numpy
restatement, and the golden fixtures.  The reference itself ships no golden
outputs (MATLAB only, not runnable here), so its own results are unpinned."""
import hashlib

import numpy as np
import pytest

from oracle import np_restate as NR


def _sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


# ---------------------------------------------------------------- FFT
@pytest.mark.parametrize("shape", [(8, 6, 10), (12, 15, 7), (16, 16, 16), (9, 25, 14), (5, 1, 3), (1, 1, 1)])
def test_fftn_matches_numpy(oracle, shape):
    rng = np.random.default_rng(1)
    a = rng.standard_normal(shape) + 1j * rng.standard_normal(shape)
    f = oracle.fftn(a)
    assert np.abs(f - np.fft.fftn(a)).max() <= 1e-12 * max(1, np.abs(f).max())
    i = oracle.fftn(a, inverse=True)
    assert np.abs(i - np.fft.ifftn(a)).max() <= 1e-12 * max(1, np.abs(i).max())


# ---------------------------------------------------------------- geometry
def test_rotation_matches_numpy(oracle):
    rng = np.random.default_rng(2)
    for _ in range(20):
        ang = rng.uniform(-180, 360, 3)
        R = oracle.euler_rot((0, 0, 1), (0, 1, 0), (1, 0, 0), *ang)
        Rn = NR.rotmat((0, 0, 1), (0, 1, 0), (1, 0, 0), *ang)
        assert np.abs(R - Rn).max() < 1e-15
        assert np.abs(R @ R.T - np.eye(3)).max() < 1e-14


def test_zyz_closed_form_equals_quaternion_product(oracle):
    """calculate3Dprojection_RealSpaceinterp.m:3-15: the closed form is Q(z,phi)Q(y,theta)Q(z,psi)."""
    rng = np.random.default_rng(3)
    for _ in range(20):
        ang = rng.uniform(0, 360, 3)
        assert np.abs(oracle.rot_zyz(*ang) - oracle.euler_rot((0, 0, 1), (0, 1, 0), (0, 0, 1), *ang)).max() < 1e-14


def test_zyz_exact_at_right_angles(oracle):
    R = oracle.rot_zyz(90, 90, 0)
    assert set(np.unique(R)) <= {-1.0, 0.0, 1.0}


# ---------------------------------------------------------------- selection
@pytest.mark.parametrize("D,os_,cut,centro", [(8, 2, 0.125, 1), (9, 2, 0.3, 1), (10, 3, 0.7, 1), (7, 2.5, 0.5, 0),
                                              (8, 2, 0.125, 0), (6, 4, 0.125, 1)])
def test_selection_matches_numpy_restatement(oracle, D, os_, cut, centro):
    rng = np.random.default_rng(4)
    n = oracle.oversampled(D, os_)
    prm = oracle.make_params(D, D, 1, oversamplingRatio=os_, interpolationCutoffDistance=cut,
                             DFT_CentroSymmetricity=centro)
    for _ in range(6):
        ang = (rng.uniform(0, 360), rng.uniform(-70, 70), rng.uniform(0, 360))
        Rf, nrm = oracle.proj_geometry(prm, *ang)
        a = oracle.select(n, n, centro, cut, Rf, nrm)
        b = NR.select(n, n, centro, cut, Rf, nrm)
        for x, y in zip(a[:4], b):
            assert np.array_equal(x, y)


def test_selection_theta0_is_k3_plane(oracle):
    """phi = theta = psi = 0: the plane is k3 = 0 and every point is an exact hit."""
    prm = oracle.make_params(8, 8, 1, oversamplingRatio=2, interpolationCutoffDistance=0.125)
    Rf, nrm = oracle.proj_geometry(prm, 0, 0, 0)
    ind, dist, u, v, off = oracle.select(16, 16, 1, 0.125, Rf, nrm)
    ext = oracle.grid_extent(16, 16, 1)
    assert len(ind) == ext[3] * ext[4]
    assert np.all(dist == 0) and off == 0
    l1, l2 = ext[3], ext[4]
    assert np.all(ind // (l1 * l2) == 8)      # k3 index of k3 = 0
    assert np.array_equal(u, (ind % l1 - 8).astype(np.float32))
    assert np.array_equal(v, ((ind // l1) % l2 - 8).astype(np.float32))


# ---------------------------------------------------------------- DFT known answers
def test_dft_dirichlet_kernel(oracle):
    """Constant projection: F = c * D_1(u) D_2(v) with Dirichlet kernels."""
    rng = np.random.default_rng(5)
    D1, D2, n1, n2 = 10, 7, 20, 15
    u = rng.uniform(-10, 10, 50).astype(np.float32)
    v = rng.uniform(-7, 7, 50).astype(np.float32)
    F = oracle.dft(np.full((D1, D2), 2.5), n1, n2, u, v)

    def dirichlet(D, w, n):
        a = np.arange(D) - D // 2
        return np.exp(-2j * np.pi * np.outer(w.astype(np.float64), a) / n).sum(axis=1)
    ref = 2.5 * dirichlet(D1, u, n1) * dirichlet(D2, v, n2)
    assert np.abs(F - ref).max() < 1e-11 * np.abs(ref).max()


def test_dft_single_pixel_is_pure_phase(oracle):
    D1, D2, n1, n2 = 8, 8, 16, 16
    P = np.zeros((D1, D2)); P[5, 2] = 1.0
    rng = np.random.default_rng(6)
    u = rng.uniform(-8, 8, 30).astype(np.float32); v = rng.uniform(-8, 8, 30).astype(np.float32)
    F = oracle.dft(P, n1, n2, u, v)
    ref = np.exp(-2j * np.pi * ((5 - 4) * u.astype(float) / n1 + (2 - 4) * v.astype(float) / n2))
    assert np.abs(F - ref).max() < 1e-14


def test_dft_integer_points_equal_padded_fft(oracle):
    """At integer (u, v) the DFT equals the FFT of the zero-padded projection."""
    rng = np.random.default_rng(7)
    D, n = 8, 16
    P = rng.random((D, D))
    k = np.arange(-8, 8)
    U, V = np.meshgrid(k, k, indexing="ij")
    F = oracle.dft(P, n, n, U.ravel().astype(np.float32), V.ravel().astype(np.float32)).reshape(n, n)
    pad = NR.paddzero(P[:, :, None], (n, n, 1))[:, :, 0]
    ref = np.fft.fftshift(np.fft.fft2(np.fft.ifftshift(pad)))
    assert np.abs(F - ref).max() < 1e-12 * np.abs(ref).max()


# ---------------------------------------------------------------- symmetry and index helpers
@pytest.mark.parametrize("n1,n2", [(8, 8), (9, 8), (8, 9), (9, 9), (6, 10), (7, 5)])
def test_centro_all_parity_branches(oracle, n1, n2):
    rng = np.random.default_rng(8)
    ext = oracle.grid_extent(n1, n2, 1)
    FS = rng.standard_normal(tuple(ext[3:])) + 1j * rng.standard_normal(tuple(ext[3:]))
    assert np.array_equal(oracle.centro(FS, n1, n1 // 2, n2), NR.centro(FS, n1, n1 // 2, n2))


@pytest.mark.parametrize("shape", [(4, 6, 8), (5, 7, 9), (4, 5, 6), (1, 3, 2)])
def test_hermitian_symmetrize(oracle, shape):
    rng = np.random.default_rng(9)
    x = rng.standard_normal(shape) + 1j * rng.standard_normal(shape)
    x[rng.random(shape) < 0.3] = 0
    assert np.allclose(oracle.hermitian_symmetrize(x), NR.hermitian_symmetrize(x), rtol=0, atol=1e-15)


@pytest.mark.parametrize("shape", [(8, 8, 8), (9, 6, 7), (1, 4, 5)])
def test_make_kspace_indices(oracle, shape):
    assert np.allclose(oracle.make_kspace_indices(shape), NR.make_kspace_indices(shape), rtol=0, atol=1e-15)


@pytest.mark.parametrize("big,ori", [((16, 16, 16), (8, 8, 8)), ((17, 16, 15), (8, 9, 7)), ((10, 11, 12), (10, 11, 12))])
def test_volumn_index_pad_strip(oracle, big, ori):
    vi = oracle.volumn_index(big, ori)
    for i in range(3):
        assert (vi[i, 0], vi[i, 1]) == NR.crop_range(big[i], ori[i])
    rng = np.random.default_rng(10)
    v = rng.random(ori)
    pad = oracle.paddzero(v, big)
    assert np.array_equal(pad, NR.paddzero(v, big))
    assert np.array_equal(oracle.stripzero(pad, ori), v)


def test_iffshift3_ind(oracle):
    rng = np.random.default_rng(11)
    for size in [(8, 8, 8), (9, 6, 7)]:
        a = rng.random(size)
        inds = np.arange(1, a.size + 1)
        sh = oracle.iffshift3_ind(size, inds)
        b = np.fft.ifftshift(a)
        assert np.array_equal(b.reshape(-1, order="F")[sh - 1], a.reshape(-1, order="F")[inds - 1])


def test_delays_and_change_points(oracle):
    for mode in (1, 2, 3):
        assert np.allclose(oracle.delay_indicators(mode), NR.delay_indicators(mode), atol=1e-15)
    # reconstruct.m:103 for Genfire_test.m's 200 iterations in mode 3
    assert list(oracle.change_points(200, 5)) == [1, 51, 101, 150, 200]
    assert list(oracle.change_points(1000, 5)) == [1, 251, 501, 750, 1000]
    assert list(oracle.change_points(1, 5)) == [1, 1, 1, 1, 1]


# ---------------------------------------------------------------- gridding end to end
def test_measuredK_hermitian_and_exact_hits(oracle):
    """CentroSymmetricity makes M(k) = conj(M(-k)) for k1 > 0; theta = 0 points are exact."""
    rng = np.random.default_rng(12)
    D, P = 8, 3
    projs = rng.random((D, D, P))
    angles = np.array([[0, 0, 0], [10, 30, 40], [200, -50, 100]], dtype=float)
    prm = oracle.make_params(D, D, P, oversamplingRatio=2, interpolationCutoffDistance=0.3)
    M, rec, nk = oracle.grid_dft(prm, projs, angles)
    n = 16
    c = n // 2
    for i1 in range(c + 1, n):
        for i2 in range(1, n):
            for i3 in range(1, n):
                m = M[2 * c - i1, 2 * c - i2, 2 * c - i3]
                assert M[i1, i2, i3] == np.conj(m)
    # every plane passes through k = 0 with D = 0 exactly: the last projection's
    # exact hit wins (fillInFourierGrid_DFT.m:291), so M(0) is its pixel sum
    assert M[c, c, c].imag == 0
    assert M[c, c, c].real == pytest.approx(projs[:, :, -1].sum(), rel=1e-14)


def test_rec_ifft_matches_numpy(oracle):
    rng = np.random.default_rng(13)
    n, D = 12, 6
    M = rng.standard_normal((n, n, n)) + 1j * rng.standard_normal((n, n, n))
    rec = oracle.rec_ifft(M, D, D)
    ref = NR.stripzero(np.real(np.fft.fftshift(np.fft.ifftn(np.fft.ifftshift(M)))), (D, D, D))
    assert np.abs(rec - ref).max() < 1e-14


@pytest.mark.parametrize("mode", [1, 2, 3])
def test_reconstruct_matches_numpy_restatement(oracle, mode):
    rng = np.random.default_rng(14)
    D, n = 8, 16
    sup = np.zeros((D, D, D), bool); sup[1:7, 1:7, 1:7] = True
    vol = rng.random((D, D, D)) * sup
    M = np.fft.fftshift(np.fft.fftn(np.fft.ifftshift(NR.paddzero(vol, (n, n, n)))))
    M[rng.random(M.shape) < 0.6] = 0
    prm = oracle.make_params(D, D, 1, oversamplingRatio=2, numIterations=23, constraintEnforcementMode=mode)
    r1, e1, _, _, _ = oracle.reconstruct(prm, M, support=sup)
    r2, e2 = NR.reconstruct(M, 23, sup, mode=mode)
    assert np.abs(r1 - r2).max() <= 1e-13 * np.abs(r2).max()
    assert np.abs(e1 - e2).max() <= 1e-13


def test_reconstruct_full_data_is_a_fixed_point(oracle):
    """All measured and consistent: the true object is returned unchanged."""
    rng = np.random.default_rng(15)
    D, n = 6, 12
    vol = rng.random((D, D, D))
    M = np.fft.fftshift(np.fft.fftn(np.fft.ifftshift(NR.paddzero(vol, (n, n, n)))))
    prm = oracle.make_params(D, D, 1, oversamplingRatio=2, numIterations=3, constraintEnforcementMode=3)
    r, errK, _, _, _ = oracle.reconstruct(prm, M, initial=vol)
    assert np.abs(r - vol).max() < 1e-12
    assert errK[0] < 1e-13


# ---------------------------------------------------------------- projector
def test_projector_matches_numpy(oracle):
    rng = np.random.default_rng(16)
    vol = rng.random((9, 10, 11))
    for ang in [(0, 0, 0), (30, 40, 50), (10, -60, 200)]:
        assert np.abs(oracle.project(vol, *ang) - NR.project(vol, oracle.rot_zyz(*ang))).max() < 1e-12


def test_projector_identity_is_axis_sum(oracle):
    rng = np.random.default_rng(17)
    vol = rng.random((7, 8, 9))
    assert np.abs(oracle.project(vol, 0, 0, 0) - vol.sum(axis=2)).max() < 1e-12


def test_projector_gaussian_line_integral(oracle):
    """A centred Gaussian projects to sqrt(2 pi) sigma times a 2-D Gaussian in any direction."""
    n, s = 48, 3.0
    x = np.arange(n) - n // 2
    X, Y, Z = np.meshgrid(x, x, x, indexing="ij")
    vol = np.exp(-(X ** 2 + Y ** 2 + Z ** 2) / (2 * s * s))
    A, B = np.meshgrid(x, x, indexing="ij")
    ref = np.sqrt(2 * np.pi) * s * np.exp(-(A ** 2 + B ** 2) / (2 * s * s))
    for ang in [(0, 0, 0), (20, 35, 70), (100, -60, 10)]:
        p = oracle.project(vol, *ang)
        assert np.abs(p - ref).max() < 0.05 * ref.max()


def test_rfactor(oracle):
    a = np.array([1.0, 2.0, -3.0]); b = np.array([1.0, 1.0, -1.0])
    r1, r2 = oracle.rfactor(a, b)
    assert r1 == pytest.approx(3.0 / 3.0) and r2 == pytest.approx(np.sqrt(5.0) / np.sqrt(3.0))


# ---------------------------------------------------------------- golden fixtures (data_turb3 subset)
def test_golden_turb3(oracle, golden):
    from tests.golden.make_golden import TURB3_PARAMS
    projs, angles = golden["subset"]["projections"], golden["subset"]["angles"]
    g = golden["oracle"]
    prm = oracle.make_params(projs.shape[0], projs.shape[1], projs.shape[2], **TURB3_PARAMS)
    n1 = oracle.oversampled(prm.Dim1, prm.oversamplingRatio)
    for p in range(projs.shape[2]):
        Rf, nrm = oracle.proj_geometry(prm, *angles[p])
        ind, dist, u, v, _ = oracle.select(n1, n1, 1, prm.interpolationCutoffDistance, Rf, nrm)
        assert [_sha(ind.astype(np.int64)), _sha(dist), _sha(u), _sha(v)] == list(g["digests"][p])
    M, rec, nk = oracle.grid_dft(prm, projs, angles)
    assert np.array_equal(nk, g["nk"])
    flat = M.reshape(-1, order="F")
    assert np.abs(flat[g["sample_idx"]] - g["sample_val"]).max() <= 1e-12 * np.abs(g["sample_val"]).max()
    assert np.count_nonzero(flat) == int(g["nnz"])
    assert np.allclose(rec[:, :, prm.Dim1 // 2], g["rec_slice"], rtol=0, atol=1e-12 * np.abs(g["rec_slice"]).max())


def test_selection_randomized_against_numpy_restatement(oracle):
    """Selection (plane distance, closest point, R \\ CP, box filter) of the C
    oracle against the independent numpy restatement over random sizes,
    oversampling ratios, cutoffs, both gridding extents, axis conventions and
    angles, including right angles and the poles."""
    hyp = pytest.importorskip("hypothesis")
    st = hyp.strategies
    angle = st.one_of(st.floats(-360, 360, allow_nan=False), st.sampled_from([0.0, 90.0, -90.0, 180.0, 45.0]))

    @hyp.settings(max_examples=60, deadline=None, derandomize=True)
    @hyp.given(D1=st.integers(3, 12), D2=st.integers(3, 12), os_=st.sampled_from([1.5, 2.0, 2.5, 3.0]),
               cut=st.sampled_from([0.125, 0.3, 0.5, 0.7]), centro=st.sampled_from([0, 1]),
               zyx=st.booleans(), phi=angle, theta=angle, psi=angle)
    def check(D1, D2, os_, cut, centro, zyx, phi, theta, psi):
        v3 = (1, 0, 0) if zyx else (0, 0, 1)
        prm = oracle.make_params(D1, D2, 1, oversamplingRatio=os_, interpolationCutoffDistance=cut,
                                 DFT_CentroSymmetricity=centro, vector3=v3)
        n1, n2 = oracle.oversampled(D1, os_), oracle.oversampled(D2, os_)
        Rf, nrm = oracle.proj_geometry(prm, phi, theta, psi)
        a = oracle.select(n1, n2, centro, cut, Rf, nrm)
        b = NR.select(n1, n2, centro, cut, Rf, nrm)
        for x, y in zip(a[:4], b):
            assert np.array_equal(x, y)

    check()


def test_reconstruct_randomized_against_numpy_restatement(oracle):
    """The loop of reconstruct.m in the C oracle against the numpy restatement
    over random box shapes (odd and even, Dim1 != Dim2), oversampling ratios,
    schedules, positivity and support switches, measured fractions and
    iteration counts crossing the schedule's change points."""
    hyp = pytest.importorskip("hypothesis")
    st = hyp.strategies

    @hyp.settings(max_examples=25, deadline=None, derandomize=True)
    @hyp.given(D1=st.integers(3, 9), D2=st.integers(3, 9), os_=st.sampled_from([2.0, 2.5, 3.0]),
               mode=st.sampled_from([1, 2, 3]), pos=st.booleans(), sup_on=st.booleans(),
               keep=st.sampled_from([0.2, 0.5, 0.9]), N=st.integers(1, 25), seed=st.integers(0, 2 ** 16))
    def check(D1, D2, os_, mode, pos, sup_on, keep, N, seed):
        rng = np.random.default_rng(seed)
        n1, n2 = oracle.oversampled(D1, os_), oracle.oversampled(D2, os_)
        sup = rng.random((D1, D2, D1)) < 0.8
        vol = rng.random((D1, D2, D1)) * sup
        M = np.fft.fftshift(np.fft.fftn(np.fft.ifftshift(NR.paddzero(vol, (n1, n2, n1)))))
        M[rng.random(M.shape) > keep] = 0
        M = np.asfortranarray(M)
        prm = oracle.make_params(D1, D2, 1, oversamplingRatio=os_, numIterations=N, constraintEnforcementMode=mode,
                                 constraintPositivity=int(pos), constraintSupport=int(sup_on))
        r1, e1, _, _, _ = oracle.reconstruct(prm, M, support=sup)
        r2, e2 = NR.reconstruct(M, N, sup, mode=mode, positivity=pos, use_support=sup_on)
        scale = max(1.0, np.abs(r2).max())
        assert np.abs(r1 - r2).max() <= 1e-12 * scale
        assert np.allclose(e1, e2, rtol=0, atol=1e-12, equal_nan=True)

    check()


def test_symmetry_and_index_helpers_randomized(oracle):
    """CentroSymmetricity, hermitianSymmetrize, make_Kspace_indices and the
    pad / crop index ranges of the oracle against the numpy restatement over
    random sizes of both parities."""
    hyp = pytest.importorskip("hypothesis")
    st = hyp.strategies

    @hyp.settings(max_examples=40, deadline=None, derandomize=True)
    @hyp.given(n1=st.integers(2, 13), n2=st.integers(2, 13), n3=st.integers(1, 11), seed=st.integers(0, 2 ** 16),
               o=st.tuples(st.integers(1, 13), st.integers(1, 13), st.integers(1, 13)))
    def check(n1, n2, n3, seed, o):
        rng = np.random.default_rng(seed)
        ext = oracle.grid_extent(n1, n2, 1)
        FS = rng.standard_normal(tuple(ext[3:])) + 1j * rng.standard_normal(tuple(ext[3:]))
        assert np.array_equal(oracle.centro(FS, n1, n1 // 2, n2), NR.centro(FS, n1, n1 // 2, n2))
        x = rng.standard_normal((n1, n2, n3)) + 1j * rng.standard_normal((n1, n2, n3))
        x[rng.random(x.shape) < 0.3] = 0
        assert np.allclose(oracle.hermitian_symmetrize(x), NR.hermitian_symmetrize(x), rtol=0, atol=1e-15)
        assert np.allclose(oracle.make_kspace_indices((n1, n2, n3)), NR.make_kspace_indices((n1, n2, n3)),
                           rtol=0, atol=1e-15)
        big = (n1, n2, n3)
        ori = tuple(min(a, b) for a, b in zip(o, big))
        vi = oracle.volumn_index(big, ori)
        for i in range(3):
            assert (vi[i, 0], vi[i, 1]) == NR.crop_range(big[i], ori[i])
        v = rng.random(ori)
        assert np.array_equal(oracle.stripzero(oracle.paddzero(v, big), ori), v)

    check()


def test_loop_timer_after_warmup(oracle):
    """The reference arm times the iterations after its warm-up ones: the time
    from iteration `first` on is positive, shrinks as `first` grows, never
    exceeds the whole loop's, and is 0 for an out-of-range start."""
    prm = oracle.make_params(16, 16, 1, oversamplingRatio=2, numIterations=6)
    M = np.zeros((32, 32, 32), complex, order="F")
    M[16, 16, 16], M[17, 16, 16] = 1.0, 0.5
    oracle.reconstruct(prm, M)
    total = oracle.last_loop_seconds()
    t = [oracle.last_loop_seconds_from(k) for k in range(6)]
    assert all(x > 0 for x in t)
    assert all(a >= b for a, b in zip(t, t[1:]))
    assert t[0] <= total
    assert oracle.last_loop_seconds_from(6) == 0 and oracle.last_loop_seconds_from(-1) == 0
