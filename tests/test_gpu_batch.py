"""Batched reconstructions (genfire_recon_batch_*): one graph launch iterates
several independent problems of different sizes, precisions and schedules.
Each member's result must be bit-identical to the same problem iterated on
its own, and the oracle still holds for the FP64 members."""
import numpy as np
import pytest

from tests.conftest import params, rel
from tests.test_gpu_recon import _measured, _support

pytestmark = pytest.mark.gpu

PROBLEMS = [
    # D, os, precision, mode, N (grids 32, 30, 24, 64: the generic and the register FFT engines)
    (16, 2.0, "fp64", 3, 12), (12, 2.5, "mixed", 1, 27), (8, 3.0, "fp64", 2, 30), (32, 2.0, "mixed", 3, 16),
]


def _make(lib, ctx, D, os_, prec, mode, N, seed):
    support = _support(D, D)
    M, _ = _measured(seed, D, D, os_, support=support)
    if prec == "mixed":
        M = M.astype(np.complex64)
    p = params(lib, D, D, 1, oversamplingRatio=os_, numIterations=N, constraintEnforcementMode=mode,
               precision=prec)
    return lib._lib.Recon(ctx, p, M, support=support), p, M, support


def test_batch_matches_members_run_alone(lib, ctx, oracle):
    alone, batched = [], []
    for i, pr in enumerate(PROBLEMS):
        alone.append(_make(lib, ctx, *pr, seed=40 + i))
        batched.append(_make(lib, ctx, *pr, seed=40 + i))
    k = min(pr[4] for pr in PROBLEMS)
    for r, _, _, _ in alone:
        r.iterate(k)
    b = lib.ReconBatch(ctx, [r for r, _, _, _ in batched])
    b.iterate(k - 2)
    b.iterate(2)
    b.close()
    for (ra, p, M, sup), (rb, _, _, _) in zip(alone, batched):
        reca, errKa = ra.result()[:2]
        recb, errKb = rb.result()[:2]
        assert np.array_equal(reca, recb)
        assert np.array_equal(errKa, errKb)
    # members finish on their own after the batch is gone; FP64 members still match the oracle
    for (ra, p, M, sup), (rb, _, _, _) in zip(alone, batched):
        rb.iterate(p.numIterations - k)
        if p.precision == lib.PREC_FP64:
            rec = rb.result()[0]
            kw = dict(oversamplingRatio=p.oversamplingRatio, numIterations=p.numIterations,
                      constraintEnforcementMode=p.constraintEnforcementMode)
            reco = oracle.reconstruct(oracle.make_params(p.Dim1, p.Dim2, 1, **kw), M, support=sup)[0]
            assert rel(rec, reco) < 1e-10
    for r, _, _, _ in alone + batched:
        r.close()


def test_batch_refuses_overrun_and_foreign_members(lib, ctx):
    r1 = _make(lib, ctx, 8, 2.0, "fp64", 3, 5, seed=1)[0]
    r2 = _make(lib, ctx, 8, 2.0, "fp64", 3, 9, seed=2)[0]
    b = lib.ReconBatch(ctx, [r1, r2])
    with pytest.raises(lib.GenfireError) as e:
        b.iterate(6)
    assert e.value.status == lib._lib.GENFIRE_ERR_STATE
    b.iterate(5)
    b.close()
    with pytest.raises(lib.GenfireError) as e:
        lib.ReconBatch(ctx, [r1, r1])
    assert e.value.status == lib._lib.GENFIRE_ERR_ARG
    other = lib.Context(0)
    r3 = _make(lib, other, 8, 2.0, "fp64", 3, 5, seed=3)[0]
    with pytest.raises(lib.GenfireError) as e:
        lib.ReconBatch(ctx, [r1, r3])
    assert e.value.status == lib._lib.GENFIRE_ERR_ARG
    for r in (r1, r2, r3):
        r.close()
    other.close()


def test_handle_lifetimes(lib, ctx):
    """A member of a live batch cannot be destroyed (GENFIRE_ERR_STATE, nothing
    freed), and genfire_destroy frees the reconstructions and batches still
    alive on the context before its stream: their Python objects may be
    collected afterwards without touching freed memory."""
    r, _, _, _ = _make(lib, ctx, *PROBLEMS[0], seed=70)
    b = lib.ReconBatch(ctx, [r])
    assert lib._lib.load().genfire_recon_destroy(r._h) == 6
    r.iterate(1)  # still usable
    b.close()
    r.close()
    c2 = lib.Context(0)
    r2, _, _, _ = _make(lib, c2, *PROBLEMS[3], seed=71)
    b2 = lib.ReconBatch(c2, [r2])
    b2.iterate(1)
    c2._children.discard(r2)  # left to genfire_destroy
    c2._children.discard(b2)
    c2.close()
    b2.close()  # no C call: the context freed them
    r2.close()
    assert r2._h is None and b2._h is None
