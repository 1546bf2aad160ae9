"""Full-size benchmark configurations against their analytic integrals
(estimate within 4 combined sigma, chi^2/dof reported and finite)."""
import numpy as np
import pytest

from cuvegas_gb300 import _lib as L, integrands as I, runtime
from cuvegas_gb300 import analytic as A

pytestmark = pytest.mark.gpu


def _run(ctx, src, dim, n_it, iters, prec, theta=None, P=0, seed=0, flags=L.FLAG_GRAPH):
    f = ctx.integrand(src, dim, n_params=P)
    p = runtime.make_params(dim, n_it * iters, iters, skip=5, n_intervals=1024, seed=seed,
                            precision=prec, flags=flags)
    with runtime.Run(f, p, theta) as r:
        r.iterate(iters)
        return r.result()


def test_c2_gauss_d8_fp32(ctx):
    res, it_res, it_sig = _run(ctx, I.GAUSS, 8, 100_000_000, 20, L.PREC_FP32)
    exact = A.gauss_normalised(8)
    assert abs(res.result - exact) < 4 * res.error, (res.result, exact, res.error)
    assert res.error / exact < 2e-5 and np.isfinite(res.chi2_dof)


def test_c5_corner_d16_fp32(ctx):
    """d=16 corner peak, 1e9 evaluations per iteration, 43M hypercubes."""
    c = I.corner_theta(0, 16)
    res, it_res, it_sig = _run(ctx, I.CORNER, 16, 1_000_000_000, 20, L.PREC_FP32, theta=c, P=16)
    exact = A.corner_peak(c)
    assert res.n_cubes == 3 ** 16
    assert abs(res.result - exact) < 4 * res.error, (res.result, exact, res.error)
    assert np.isfinite(res.chi2_dof)
    # each cube gets max(2, floor(share * N)): the floors drop a few samples
    assert 0.99 * 20e9 <= res.tot_nevals <= 20e9 + 2 * 20 * 3 ** 16


def test_c4_product_peak_instances(ctx):
    """A few instances of the batched family one by one (d from 2 to 12)."""
    for inst in I.batch_instances(0, 512)[:12]:
        d, th = inst["dim"], inst["theta"]
        res, _, _ = _run(ctx, I.PRODPEAK, d, max(inst["n_eval_it"], 10000), 10, L.PREC_FP32,
                         theta=th, P=2 * d)
        exact = A.product_peak(inst["c"], inst["u"])
        assert abs(res.result - exact) < 5 * res.error, (d, res.result, exact, res.error)
