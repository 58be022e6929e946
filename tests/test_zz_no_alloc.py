"""genfire_rfactor_noalloc: the R-factors computed without allocating device
memory, for callers that work on device buffers they do not own and may not
call cudaMalloc (a MEX function on gpuArray data, a service with its own
memory pool).  Checked through the C ABI against genfire_rfactor on the same
inputs, twice in a row (the static scratch keeps the previous call's
contents, which must not leak into the next result).

This file is collected last so that a failure here leaves every other test
already run."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = 1e-12


def _call(lib, ctx, precision, d_vol, shape, angles, d_meas, vectors=None):
    from genfire_gb300 import _lib
    L = _lib.load()
    P = angles.shape[0]
    A = np.asfortranarray(angles, dtype=np.float64)
    vec = None if vectors is None else np.ascontiguousarray(np.asarray(vectors, dtype=np.float64).reshape(9))
    R1 = np.zeros(P)
    R2 = np.zeros(P)
    eR = C.c_double()
    st = L.genfire_rfactor_noalloc(ctx.handle, precision, C.c_void_p(d_vol), shape[0], shape[1], shape[2], P,
                                   A.ctypes.data_as(C.POINTER(C.c_double)),
                                   None if vec is None else vec.ctypes.data_as(C.POINTER(C.c_double)),
                                   C.c_void_p(d_meas), R1.ctypes.data_as(C.POINTER(C.c_double)),
                                   R2.ctypes.data_as(C.POINTER(C.c_double)), C.byref(eR))
    return st, eR.value, R1, R2


def _case(seed, shape, P):
    rng = np.random.default_rng(seed)
    vol = rng.random(shape)
    angles = np.stack([rng.uniform(0, 360, P), rng.uniform(-70, 70, P), rng.uniform(0, 360, P)], 1)
    meas = np.asfortranarray(rng.random((shape[0], shape[1], P)) * shape[2] * 0.5)
    return vol, angles, meas


def _dev(a, dtype):
    import torch
    flat = np.ascontiguousarray(np.asfortranarray(a, dtype=dtype).reshape(-1, order="F"))
    return torch.from_numpy(flat).cuda()


CASES = [
    (1, (40, 36, 32), 7, None),
    (2, (24, 24, 24), 13, ((0, 0, 1), (0, 1, 0), (1, 0, 0))),
    # more than one 64-projection chunk of the host-side staging (rotations up, sums back)
    (4, (40, 36, 20), 100, None),
]


def _check_twice(lib, ctx, precision, cases):
    import torch
    rdt = np.float64 if precision == lib.PREC_FP64 else np.float32
    for seed, shape, P, vectors in cases:
        vol, angles, meas = _case(seed, shape, P)
        d_vol, d_meas = _dev(vol, rdt), _dev(meas, np.float64)
        torch.cuda.synchronize()
        ref_errR, ref_R1, ref_R2 = ctx.rfactor(vol.astype(rdt), angles, meas, vectors=vectors, precision=precision)
        for call in range(2):
            # the second call must not change the device's free memory: the
            # first one has loaded everything the call needs
            free0 = torch.cuda.mem_get_info()[0] if call == 1 else None
            st, errR, R1, R2 = _call(lib, ctx, precision, d_vol.data_ptr(), shape, angles, d_meas.data_ptr(), vectors)
            if call == 1:
                assert torch.cuda.mem_get_info()[0] == free0
            assert st == 0, lib._lib.load().genfire_last_error(ctx.handle)
            assert abs(errR - ref_errR) <= TOL * abs(ref_errR)
            assert np.abs(R1 - ref_R1).max() <= TOL * np.abs(ref_R1).max()
            assert np.abs(R2 - ref_R2).max() <= TOL * np.abs(ref_R2).max()


@pytest.mark.parametrize("precision_name", ["fp64", "mixed"])
def test_noalloc_matches_rfactor_twice(lib, ctx, precision_name):
    precision = lib.PREC_FP64 if precision_name == "fp64" else lib.PREC_MIXED
    _check_twice(lib, ctx, precision, CASES)


def test_noalloc_cubic_matches_rfactor_twice(lib, ctx):
    # the cubic-convolution projector through the same static scratch
    assert lib._lib.load().genfire_set_projector_interpolation(ctx.handle, lib.INTERP_CUBIC) == 0
    try:
        _check_twice(lib, ctx, lib.PREC_FP64, [CASES[0], CASES[2]])
    finally:
        lib._lib.load().genfire_set_projector_interpolation(ctx.handle, lib.INTERP_TRILINEAR)


def test_noalloc_rejects_oversized_inputs(lib, ctx):
    # 140 projections of 512 x 512 need about 4.6 MB of partial sums; the buffers are
    # full size, so nothing would be read out of bounds even if the check were missing
    vol, angles, meas = _case(3, (512, 512, 2), 140)
    d_vol, d_meas = _dev(vol, np.float64), _dev(meas, np.float64)
    st, _, _, _ = _call(lib, ctx, lib.PREC_FP64, d_vol.data_ptr(), vol.shape, angles, d_meas.data_ptr())
    assert st == 1
    assert b"4 MiB" in lib._lib.load().genfire_last_error(ctx.handle)
