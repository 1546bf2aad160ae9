"""Failure handling on the GPU without a GPU fault.

The one-pass hypercube allocation (k3_alloc) is the only kernel that waits on
other blocks: each block reads its predecessors' published look-back words.
Every such wait is bounded.  Here one chunk is made to withhold its word (a
flag that nothing sets: CVG_TEST_LB_WITHHOLD) and the poll limit is cut to a
few thousand (CVG_LB_SPIN_LIMIT), so its successors' waits run out: the kernel
must return, set its timeout status bit, and the run must report
CVG_ERR_KERNEL, while the context stays usable for the next run.
"""
import numpy as np
import pytest

from cuvegas_gb300 import _lib as L, integrands as I, runtime

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("prec", [L.PREC_FP64, L.PREC_FP32])
def test_lookback_wait_runs_out_and_is_reported(ctx, monkeypatch, prec):
    dim, n_it = 4, 400_000          # 12^4 = 20736 hypercubes: 11 chunks of 2048
    f = ctx.integrand(I.GAUSS, dim)
    p = runtime.make_params(dim, n_it * 4, 4, skip=0, n_intervals=64, seed=3, precision=prec)
    monkeypatch.setenv("CVG_LB_SPIN_LIMIT", "4096")
    monkeypatch.setenv("CVG_TEST_LB_WITHHOLD", "4")      # chunk 3 never publishes
    with runtime.Run(f, p) as r:
        assert r.info.n_cubes > 8 * 2048
        # a valid fill (the initial allocation is not affected), then the
        # reallocation whose waits run out; no fill runs on its prefix
        r.step(L.STAGE_FILL | L.STAGE_REALLOC)
        with pytest.raises(L.CuvegasError) as e:
            r.result()
        assert e.value.status == L.ERR_KERNEL
        assert "look-back" in str(e.value)
    # the same context, without the test knob: a whole run is valid again
    monkeypatch.delenv("CVG_TEST_LB_WITHHOLD")
    monkeypatch.delenv("CVG_LB_SPIN_LIMIT")
    with runtime.Run(f, p) as r:
        r.iterate(4)
        res, it_res, _ = r.result()
    assert np.all(np.isfinite(it_res))
    assert abs(res.result - 1.0) < 5 * res.error


def test_short_spin_limit_alone_changes_nothing(ctx, monkeypatch):
    """A small poll limit with every word published: the waits end long
    before it, and results equal a run with the default limit."""
    dim, n_it = 4, 400_000
    f = ctx.integrand(I.GAUSS, dim)
    p = runtime.make_params(dim, n_it * 3, 3, skip=0, n_intervals=64, seed=4,
                            precision=L.PREC_FP64)
    with runtime.Run(f, p) as r:
        r.iterate(3)
        want = r.result()[1]
    monkeypatch.setenv("CVG_LB_SPIN_LIMIT", "1000000")
    with runtime.Run(f, p) as r:
        r.iterate(3)
        got = r.result()[1]
    np.testing.assert_allclose(got, want, rtol=1e-12)
