"""Loop state export/import: a run resumed from a checkpoint ends where an
uninterrupted run ends, and a trained map integrates without adaptation."""
import numpy as np
import pytest

from cuvegas_gb300 import _lib as L, analytic as A, integrands as I, runtime

pytestmark = pytest.mark.gpu


def _params(n_it, max_it, prec, flags=0, seed=11):
    return runtime.make_params(4, n_it * max_it, max_it, skip=2, n_intervals=256, seed=seed,
                               precision=prec, flags=flags)


@pytest.mark.parametrize("prec", [L.PREC_FP64, L.PREC_FP32])
def test_resume_from_checkpoint_equals_one_run(ctx, prec, tmp_path):
    """A run checkpointed after 6 of 10 iterations and continued, and a new
    run resumed from the checkpoint, end in the same place."""
    f = ctx.integrand(I.GAUSS, 4)
    with runtime.Run(f, _params(200000, 10, prec)) as r:
        r.iterate(6)
        r.save_state(tmp_path / "ckpt.npz")
        r.iterate(4)
        ref, ref_it, _ = r.result()
        ref_edges = r.get(L.BUF_X_EDGES)
    st = runtime.Run.load_state(tmp_path / "ckpt.npz")
    assert st["iteration"] == 6
    with runtime.Run(f, _params(200000, 10, prec)) as r:
        r.import_state(st)
        r.iterate(4)
        res, it_res, _ = r.result()
        edges = r.get(L.BUF_X_EDGES)
    # same Philox words, grids and allocations: equal up to the summation order
    # of the FP64 atomics (which can move a sample across a bin edge after a
    # few iterations: ~1e-6 of an estimate; a wrong resume differs by ~1e-3)
    np.testing.assert_allclose(it_res, ref_it, rtol=2e-5)
    np.testing.assert_allclose(edges, ref_edges, rtol=1e-6, atol=1e-8)
    assert abs(res.result - ref.result) <= 2e-5 * abs(ref.result)
    # the same rounding can move a hypercube's n_h = floor(...) by one
    assert abs(res.tot_nevals - ref.tot_nevals) <= max(8, 1e-5 * ref.tot_nevals)


def test_trained_map_without_adaptation(ctx):
    f = ctx.integrand(I.GAUSS, 4)
    with runtime.Run(f, _params(300000, 8, L.PREC_FP32)) as r:
        r.iterate(8)
        st = r.export_state()
    with runtime.Run(f, _params(300000, 5, L.PREC_FP32, flags=L.FLAG_NO_ADAPT, seed=99)) as r:
        r.import_state(st, resume=False)
        r.iterate(5)
        res, it_res, it_sig = r.result()
        assert np.array_equal(r.get(L.BUF_X_EDGES), st["x_edges"])   # the map is kept
        assert np.array_equal(r.get(L.BUF_NH), st["nh"])
    exact = A.gauss_normalised(4)
    assert abs(res.result - exact) < 5 * res.error
    assert res.chi2_dof < 5.0


def test_state_of_another_shape_is_rejected(ctx):
    f = ctx.integrand(I.GAUSS, 4)
    with runtime.Run(f, _params(200000, 4, L.PREC_FP64)) as r:
        st = r.export_state()
    with runtime.Run(f, runtime.make_params(4, 200000 * 4, 4, n_intervals=128)) as r:
        with pytest.raises(ValueError):
            r.import_state(st)
