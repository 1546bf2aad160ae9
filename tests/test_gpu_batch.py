"""Batched integration (one persistent fill launch per iteration for the whole
batch, batched refinement and reallocation, CUDA graph) against
single-instance runs with the same Philox streams, and the C4 family against
its analytic integrals."""
import numpy as np
import pytest

from cuvegas_gb300 import _lib as L, autotune, batch as B, integrands as I, runtime
from cuvegas_gb300 import analytic as A

pytestmark = pytest.mark.gpu
PPD = [2 * d for d in range(17)]


def _instances(n, seed, lo=4, hi=5):
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n):
        d = 2 + i % 11
        c = rng.uniform(5, 25, size=d)
        u = rng.uniform(0, 1, size=d)
        out.append(dict(dim=d, n_eval_it=int(10 ** rng.uniform(lo, hi)), c=c, u=u,
                        theta=I.prodpeak_theta(c, u)))
    return out


@pytest.mark.parametrize("graph", [False, True])
def test_batch_equals_single_runs_fp64(ctx, graph):
    insts = _instances(16, 1)
    with B.Batch(ctx, I.PRODPEAK, insts, PPD, max_it=6, skip=2, n_intervals=128, seed=9,
                 precision=L.PREC_FP64, graph=graph) as b:
        b.iterate(6)
        res, it_res, _ = b.results()
    for i, inst in enumerate(insts):
        d = inst["dim"]
        f = ctx.integrand(I.PRODPEAK, d, n_params=2 * d)
        p = runtime.make_params(d, inst["n_eval_it"] * 6, 6, skip=2, n_intervals=128, seed=9,
                                precision=L.PREC_FP64, instance=i)
        with runtime.Run(f, p, inst["theta"]) as r:
            r.iterate(6)
            rs, ir, _ = r.result()
        assert res[i].tot_nevals == rs.tot_nevals, i
        np.testing.assert_allclose(it_res[i], ir, rtol=1e-9)
        assert abs(res[i].result - rs.result) <= 1e-10 * abs(rs.result)


def test_batch_beyond_one_scan_block(ctx):
    """1500 small instances: the tile numbering and the fill's work ranges
    scan the instances in blocks of 1024 (the carry between blocks), the
    block-to-instance table and the claims span them all.  FP64: instances on
    both sides of the 1024 boundary equal their single runs (to 1e-10).  FP32
    (same Philox streams): every instance within 3 combined sigma of its FP64
    estimate."""
    rng = np.random.default_rng(11)
    insts = []
    for i in range(1500):
        d = 2 + i % 3
        c = rng.uniform(5, 25, size=d)
        u = rng.uniform(0, 1, size=d)
        insts.append(dict(dim=d, n_eval_it=int(rng.integers(2000, 6000)), c=c, u=u,
                          theta=I.prodpeak_theta(c, u)))
    out = {}
    for prec in (L.PREC_FP64, L.PREC_FP32):
        with B.Batch(ctx, I.PRODPEAK, insts, PPD, max_it=4, skip=1, n_intervals=64, seed=4,
                     precision=prec, graph=True) as b:
            b.iterate(4)
            out[prec] = b.results()[0]
    r64, r32 = out[L.PREC_FP64], out[L.PREC_FP32]
    for i in (0, 1, 1022, 1023, 1024, 1025, 1499):
        inst = insts[i]
        d = inst["dim"]
        f = ctx.integrand(I.PRODPEAK, d, n_params=2 * d)
        p = runtime.make_params(d, inst["n_eval_it"] * 4, 4, skip=1, n_intervals=64, seed=4,
                                precision=L.PREC_FP64, instance=i)
        with runtime.Run(f, p, inst["theta"]) as r:
            r.iterate(4)
            rs, _, _ = r.result()
        assert r64[i].tot_nevals == rs.tot_nevals, i
        assert abs(r64[i].result - rs.result) <= 1e-10 * abs(rs.result), i
    dev = np.array([abs(a.result - b.result) / np.hypot(a.error, b.error)
                    for a, b in zip(r32, r64)])
    assert np.all(np.isfinite(dev))
    assert np.mean(dev < 3) >= 0.98, np.sort(dev)[-10:]


def test_batch_fp32_family_against_analytic(ctx):
    """C4 family (64 instances, d in 2..12, 1e4..1e6 evaluations/iteration),
    FP32 compensated, CUDA graph, autotuned tiles, 10 iterations."""
    insts = _instances(64, 2, lo=4, hi=6)
    block, spt = autotune.tune_batch(ctx, I.PRODPEAK, insts, PPD, L.PREC_FP32)
    assert (block, spt) in autotune.BATCH_CANDIDATES
    with B.Batch(ctx, I.PRODPEAK, insts, PPD, max_it=10, skip=5, seed=3,
                 precision=L.PREC_FP32, graph=True, block=block, spt=spt) as b:
        b.iterate(10)
        res, _, _ = b.results()
    pulls = []
    for i, inst in enumerate(insts):
        exact = A.product_peak(inst["c"], inst["u"])
        pulls.append((res[i].result - exact) / res[i].error)
        assert np.isfinite(res[i].chi2_dof)
    pulls = np.abs(np.array(pulls))
    # VEGAS error estimates at low statistics on peaked 10-12 d integrands run
    # small (the FP64 oracle shows the same); most must be within 4 sigma
    assert np.mean(pulls < 4) >= 0.85 and pulls.max() < 10, pulls


def test_batch_rejects_bad_instances(ctx):
    with pytest.raises(L.CuvegasError):
        B.Batch(ctx, I.PRODPEAK, [dict(dim=0, n_eval_it=1000, theta=np.zeros(0))], PPD,
                max_it=2)
