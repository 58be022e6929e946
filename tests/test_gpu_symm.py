"""Index and symmetry kernels and the FFT on the GPU, against the oracle."""
import numpy as np
import pytest

from tests.conftest import rel

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("n1,n2", [(8, 8), (9, 8), (8, 9), (9, 9), (6, 10), (7, 5), (64, 48)])
def test_centro_symmetricity_exact(ctx, oracle, n1, n2):
    rng = np.random.default_rng(n1 * 100 + n2)
    ext = oracle.grid_extent(n1, n2, 1)
    FS = rng.standard_normal(tuple(ext[3:])) + 1j * rng.standard_normal(tuple(ext[3:]))
    assert np.array_equal(ctx.centro_symmetricity(FS, n1, n1 // 2, n2), oracle.centro(FS, n1, n1 // 2, n2))


@pytest.mark.parametrize("shape", [(4, 6, 8), (5, 7, 9), (4, 5, 6), (1, 3, 2), (32, 33, 31)])
def test_hermitian_symmetrize_exact(ctx, oracle, shape):
    rng = np.random.default_rng(sum(shape))
    x = rng.standard_normal(shape) + 1j * rng.standard_normal(shape)
    x[rng.random(shape) < 0.3] = 0
    assert np.array_equal(ctx.hermitian_symmetrize(x), oracle.hermitian_symmetrize(x))


@pytest.mark.parametrize("shape", [(8, 8, 8), (9, 6, 7), (1, 4, 5), (64, 64, 64)])
def test_make_kspace_indices_exact(ctx, oracle, shape):
    assert np.array_equal(ctx.make_kspace_indices(shape), oracle.make_kspace_indices(shape))


@pytest.mark.parametrize("size", [(8, 8, 8), (9, 6, 7), (33, 32, 31)])
def test_iffshift3_ind_exact(ctx, oracle, size):
    inds = np.arange(1, int(np.prod(size)) + 1, dtype=np.int64)
    assert np.array_equal(ctx.iffshift3_ind(size, inds), oracle.iffshift3_ind(size, inds))


@pytest.mark.parametrize("shape", [(8, 6, 10), (12, 15, 7), (16, 16, 16), (9, 25, 14), (64, 1, 3), (96, 40, 28),
                                   (512, 2, 2), (1, 1, 7), (1024, 2, 3), (2, 2048, 2)])
def test_fftn_fp64(lib, ctx, shape):
    rng = np.random.default_rng(sum(shape))
    a = rng.standard_normal(shape) + 1j * rng.standard_normal(shape)
    assert rel(ctx.fftn(a), np.fft.fftn(a)) < 1e-13
    assert rel(ctx.fftn(a, inverse=True), np.fft.ifftn(a)) < 1e-13


@pytest.mark.parametrize("shape", [(8, 6, 10), (16, 16, 16), (9, 25, 14), (96, 40, 28), (1024, 2, 2), (2048, 2, 2),
                                   (2, 2048, 3), (3, 2, 2048)])
def test_fftn_complex64(lib, ctx, shape):
    rng = np.random.default_rng(sum(shape))
    a = rng.standard_normal(shape) + 1j * rng.standard_normal(shape)
    assert rel(ctx.fftn(a, precision=lib.PREC_MIXED), np.fft.fftn(a)) < 2e-6
    assert rel(ctx.fftn(a, inverse=True, precision=lib.PREC_MIXED), np.fft.ifftn(a)) < 2e-6


def test_fft_rejects_large_prime(lib, ctx):
    with pytest.raises(lib.GenfireError) as e:
        ctx.fftn(np.ones((11, 2, 2)))
    assert e.value.status == 5
