"""The tensor-core gridding kernels' bounded waits, made to expire on real work.

Every mbarrier wait of k_dft_tcgen05 (and of its N = 256 form,
k_dft_tcgen05_w, selected by GENFIRE_DFT_KERNEL=n256) has a clock limit.  GENFIRE_DEBUG_DFT_WAIT_CYCLES
shortens the main loop's limit to one cycle (polled with the non-blocking
mbarrier.test_wait), so a wait for a bulk copy or for the MMAs just issued
expires while they are still in flight.  The kernel must
then stop at one barrier for the whole CTA, wait (with the full limit) for
everything in flight, free its TMEM and return; the call reports
GENFIRE_ERR_TIMEOUT.  The same context must then grid normally and match the
oracle.  No fault is provoked: the copies and MMAs the drain waits for are
ordinary in-bounds work that completes."""
import numpy as np
import pytest

from tests.conftest import params, rel

pytestmark = pytest.mark.gpu

ENV = "GENFIRE_DEBUG_DFT_WAIT_CYCLES"


def _case(lib, oracle):
    rng = np.random.default_rng(77)
    D, P = 32, 4
    projs = np.asfortranarray(rng.random((D, D, P)))
    angles = np.asfortranarray(np.stack([rng.uniform(0, 360, P), rng.uniform(-70, 70, P), rng.uniform(0, 360, P)], 1))
    kw = dict(oversamplingRatio=2.0, interpolationCutoffDistance=0.3)
    return (params(lib, D, D, P, precision="mixed", **kw), oracle.make_params(D, D, P, **kw), projs, angles)


@pytest.mark.parametrize("form", ["n128", "n256"])
def test_expired_wait_reports_timeout_and_context_recovers(lib, ctx, oracle, monkeypatch, form):
    monkeypatch.setenv("GENFIRE_DFT_KERNEL", form)
    p, op, projs, angles = _case(lib, oracle)
    Mo, _, nko = oracle.grid_dft(op, projs, angles)
    for _ in range(2):
        monkeypatch.setenv(ENV, "1")
        with pytest.raises(lib.GenfireError) as e:
            ctx.grid_dft(p, projs, angles, want_rec=False)
        assert e.value.status == 4, str(e.value)  # GENFIRE_ERR_TIMEOUT
        assert "bounded wait" in str(e.value)
        monkeypatch.delenv(ENV)
        M, _, nk = ctx.grid_dft(p, projs, angles, want_rec=False)
        assert np.array_equal(nk, nko)
        assert rel(M, Mo) < 1e-4
