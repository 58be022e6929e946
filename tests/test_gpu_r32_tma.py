"""The persistent, TMA-fed fused 512-point pass (k_col_r32_tma, column-pass
variant 5): the same tile arithmetic as the radix-32 fused pass, with each
tile's input brought into shared memory by a tensor copy one tile ahead.
Forced with GENFIRE_COL_VARIANT=5 (valid for the fused dim-3 pass only; the
other passes keep their engine), a reconstruction must equal the one with
variant 4 bit for bit (reconstruction and errK), with and without Rfree
monitoring, and stay within the MIXED bar of the oracle."""
import numpy as np
import pytest

from tests.conftest import params, rel
from tests.test_gpu_r32 import _measured

pytestmark = pytest.mark.gpu


def _run(lib, ctx, monkeypatch, variant, D1, D2, N, mode, seed, rfree=False):
    monkeypatch.setenv("GENFIRE_COL_VARIANT", str(variant))
    M = _measured(seed, D1, D2, 2.0)
    p = params(lib, D1, D2, 1, oversamplingRatio=2.0, numIterations=N, constraintEnforcementMode=mode,
               precision="mixed")
    r = ctx.recon(p, M.astype(np.complex64))
    out = []
    if rfree:
        cand = ctx.rfree_candidates(p, M.astype(np.complex64), 4)
        shells = [c[::7][:50] for c in cand]
        r.set_rfree(shells)
    r.iterate(N)
    rec, errK, _, _, _ = r.result()
    if rfree:
        out.append(r.rfree())
    r.close()
    return rec, errK, out, M, p


@pytest.mark.parametrize("D1,D2,N,mode", [(256, 4, 6, 3), (256, 8, 5, 1), (256, 3, 4, 2)])
def test_tma_fused_pass_equals_r32(lib, ctx, oracle, monkeypatch, D1, D2, N, mode):
    rec4, err4, _, M, _ = _run(lib, ctx, monkeypatch, 4, D1, D2, N, mode, seed=D1 + D2 + mode)
    rec5, err5, _, _, _ = _run(lib, ctx, monkeypatch, 5, D1, D2, N, mode, seed=D1 + D2 + mode)
    assert np.array_equal(rec4, rec5)
    assert np.array_equal(err4, err5)
    op = oracle.make_params(D1, D2, 1, oversamplingRatio=2.0, numIterations=N, constraintEnforcementMode=mode)
    reco, errKo, _, _, _ = oracle.reconstruct(op, M)
    assert rel(rec5, reco) < 1e-4
    assert np.abs(err5 - errKo).max() < 1e-4 * np.abs(errKo).max()


def test_tma_fused_pass_rfree_equals_r32(lib, ctx, monkeypatch):
    a = _run(lib, ctx, monkeypatch, 4, 256, 4, 5, 3, seed=91, rfree=True)
    b = _run(lib, ctx, monkeypatch, 5, 256, 4, 5, 3, seed=91, rfree=True)
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])
    assert np.array_equal(a[2][0], b[2][0])
