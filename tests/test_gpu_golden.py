"""The CUDA path against golden vectors of the reference's own kernels:
replaying the reference's curand uniforms through the C ABI, the fused fill,
the reallocation and the refinement must reproduce what the reference's
vegasFill / results / updateNh / refinement kernels produced (bin counts and
nh exactly, sums and grid to 1e-9; the parity bound is 1e-6)."""
import numpy as np
import pytest

from cuvegas_gb300 import _lib as L, runtime
from golden_cases import GAUSS_W02, bench_shape_cases, cases, expand_uniforms, gauss_source, kept_cubes
from oracle import pyoracle as P

pytestmark = pytest.mark.gpu
CASES = cases()
BENCH = bench_shape_cases()


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


@pytest.mark.parametrize("name,meta,z,kept", BENCH, ids=[c[0] for c in BENCH])
def test_cuda_reproduces_reference_at_benchmark_shape(ctx, name, meta, z, kept):
    """C1 exactly (d=4, 1e6 evals/iteration, 1024 bins, width 0.1; iterations
    0, 1, 9) and the d=8 / width 0.1 / 1024-bin shape (2e6 evals/iteration),
    FP64 form: replaying the reference's uniforms of every stride-th
    hypercube (0.5 for the other samples), the fill reproduces those
    hypercubes' sums (1e-9) and matches the oracle on the same buffer in every
    hypercube and bin (counts exactly, sums 5e-11); the reallocation gives
    the reference's damped variances from its sums (1e-7); the refinement
    gives the reference's grid from its whole histograms (1e-9)."""
    dim, N, iters = meta["dim"], meta["n_intervals"], meta["iters"]
    f = ctx.integrand(gauss_source(meta["width"]), dim)
    p = runtime.make_params(dim, meta["n_eval_it"] * iters, iters, skip=0, n_intervals=N,
                            precision=L.PREC_FP64)
    cubes = kept_cubes(meta)
    o = P.OracleRun(dim, meta["n_eval_it"] * iters, iters, n_intervals=N)
    theta = np.array([0.5, meta["width"]])
    with runtime.Run(f, p) as r:
        assert r.info.n_strat == meta["n_strat"] and r.info.n_cubes == meta["n_cubes"]
        assert np.array_equal(r.get(L.BUF_X_EDGES).ravel(), z["x_edges_in_0"])
        assert np.array_equal(r.get(L.BUF_NH), z["nh_0"].astype(np.uint32))
        for it in kept:
            ub = expand_uniforms(meta, z, it)
            r.set(L.BUF_X_EDGES, z["x_edges_in_%d" % it])
            r.set(L.BUF_NH, z["nh_%d" % it].astype(np.uint32))
            r.set(L.BUF_ITERATION, np.array([it], dtype=np.uint32))
            r.set(L.BUF_UNIFORMS, ub)
            r.step(L.STAGE_FILL)
            JF, JF2 = r.get(L.BUF_JF), r.get(L.BUF_JF2)
            W, Cn = r.get(L.BUF_WEIGHTS), r.get(L.BUF_COUNTS)
            np.testing.assert_allclose(JF[cubes], z["JF_%d" % it], rtol=1e-9, atol=1e-300)
            np.testing.assert_allclose(JF2[cubes], z["JF2_%d" % it], rtol=1e-9, atol=1e-300)
            o.set_x_edges(z["x_edges_in_%d" % it])
            o.set_nh(z["nh_%d" % it].astype(np.int64))
            u, keep = P.uniforms(P.U_BUFFER, ubuf=ub)
            o.fill(P.F_GAUSS, theta, u, it=it)
            assert np.array_equal(Cn.astype(np.int64), o.counts)
            # the filler rows put every sample of a non-kept hypercube on one
            # point: the oracle's sequential sum of thousands of equal terms
            # in the central hypercubes drifts by up to ~1e-11 from the
            # fill's per-thread runs
            np.testing.assert_allclose(JF, o.JF, rtol=5e-11, atol=1e-300)
            np.testing.assert_allclose(JF2, o.JF2, rtol=5e-11, atol=1e-300)
            np.testing.assert_allclose(W, o.weights, rtol=5e-11, atol=1e-300)
            JF[cubes], JF2[cubes] = z["JF_%d" % it], z["JF2_%d" % it]
            r.set(L.BUF_JF, JF)
            r.set(L.BUF_JF2, JF2)
            r.step(L.STAGE_REALLOC)
            np.testing.assert_allclose(r.get(L.BUF_DH)[cubes], z["dh_%d" % it], rtol=1e-7,
                                       atol=1e-300)
            r.set(L.BUF_WEIGHTS, z["weights_%d" % it])
            r.set(L.BUF_COUNTS, z["counts_%d" % it].astype(np.uint32))
            r.step(L.STAGE_REFINE)
            np.testing.assert_allclose(r.get(L.BUF_X_EDGES).ravel(), z["x_edges_out_%d" % it],
                                       rtol=1e-9, atol=1e-15)
        r.set(L.BUF_UNIFORMS, None)
