"""The CUDA path against golden vectors of the reference's own kernels:
replaying the reference's curand uniforms through the C ABI, the fused fill,
the reallocation and the refinement must reproduce what the reference's
vegasFill / results / updateNh / refinement kernels produced (bin counts and
nh exactly, sums and grid to 1e-9; the parity bound is 1e-6)."""
import numpy as np
import pytest

from cuvegas_gb300 import _lib as L, runtime
from golden_cases import GAUSS_W02, cases

pytestmark = pytest.mark.gpu
CASES = cases()


@pytest.mark.parametrize("name,meta,z", CASES, ids=[c[0] for c in CASES])
def test_cuda_reproduces_reference(ctx, name, meta, z):
    dim, N, iters = meta["dim"], meta["n_intervals"], meta["iters"]
    f = ctx.integrand(GAUSS_W02, dim)
    p = runtime.make_params(dim, meta["n_eval_it"] * iters, iters, skip=0, n_intervals=N,
                            precision=L.PREC_FP64)
    with runtime.Run(f, p) as r:
        assert r.info.n_strat == meta["n_strat"] and r.info.n_cubes == meta["n_cubes"]
        assert np.array_equal(r.get(L.BUF_X_EDGES).ravel(), z["x_edges_in_0"])
        assert np.array_equal(r.get(L.BUF_NH).astype(np.int64), z["nh_0"])
        for it in range(iters):
            r.set(L.BUF_X_EDGES, z["x_edges_in_%d" % it])
            r.set(L.BUF_NH, z["nh_%d" % it].astype(np.uint32))
            r.set(L.BUF_ITERATION, np.array([it], dtype=np.uint32))
            r.set(L.BUF_UNIFORMS, z["u_%d" % it].reshape(-1, dim))
            r.step(L.STAGE_FILL)
            assert np.array_equal(r.get(L.BUF_COUNTS).ravel().astype(np.int64),
                                  z["counts_%d" % it].astype(np.int64))
            np.testing.assert_allclose(r.get(L.BUF_JF), z["JF_%d" % it], rtol=1e-9, atol=1e-300)
            np.testing.assert_allclose(r.get(L.BUF_JF2), z["JF2_%d" % it], rtol=1e-9, atol=1e-300)
            np.testing.assert_allclose(r.get(L.BUF_WEIGHTS).ravel(), z["weights_%d" % it],
                                       rtol=1e-9)
            # reallocation from the reference's own per-cube sums
            r.set(L.BUF_JF, z["JF_%d" % it])
            r.set(L.BUF_JF2, z["JF2_%d" % it])
            r.step(L.STAGE_REALLOC)
            # dh cancels (v^2 JF2/n - (v JF/n)^2): 1-ulp differences grow ~1e8-fold
            np.testing.assert_allclose(r.get(L.BUF_DH), z["dh_%d" % it], rtol=1e-7, atol=1e-300)
            assert np.array_equal(r.get(L.BUF_NH).astype(np.int64), z["nh_next_%d" % it])
            st = r.get(L.BUF_STATS)
            np.testing.assert_allclose([st[0, it], st[1, it]],
                                       [z["res_%d" % it][0], z["sig_%d" % it][0]], rtol=1e-11)
            r.step(L.STAGE_REFINE)
            np.testing.assert_allclose(r.get(L.BUF_X_EDGES).ravel(), z["x_edges_out_%d" % it],
                                       rtol=1e-9, atol=1e-15)
        r.set(L.BUF_UNIFORMS, None)
