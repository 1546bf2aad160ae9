"""The CPU oracle against golden vectors of the reference's own kernels.

Pins the restatement: with the reference's curand uniforms replayed, the
oracle must reproduce the reference's per-cube and per-bin sums (bin counts
exactly), its reallocation (nh exactly) and its refined grid, to 1e-9
relative (the bound stated for parity is 1e-6)."""
import numpy as np
import pytest

from golden_cases import THETA, bench_shape_cases, cases, expand_uniforms, kept_cubes
from oracle import pyoracle as P

CASES = cases()
BENCH = bench_shape_cases()


@pytest.mark.parametrize("name,meta,z", CASES, ids=[c[0] for c in CASES])
def test_oracle_reproduces_reference(name, meta, z):
    dim, N, iters = meta["dim"], meta["n_intervals"], meta["iters"]
    r = P.OracleRun(dim, meta["n_eval_it"] * iters, iters, n_intervals=N)
    assert r.sz.n_strat == meta["n_strat"] and r.sz.n_cubes == meta["n_cubes"]
    assert abs(r.sz.v_cubes - meta["v_cubes"]) <= 1e-15 * meta["v_cubes"]
    for it in range(iters):
        if it == 0:   # the oracle's own initial state must equal the reference's
            assert np.array_equal(r.x_edges.ravel(), z["x_edges_in_0"])
            assert np.array_equal(r.nh, z["nh_0"])
        r.set_x_edges(z["x_edges_in_%d" % it])
        r.set_nh(z["nh_%d" % it])
        u, keep = P.uniforms(P.U_BUFFER, ubuf=z["u_%d" % it].reshape(-1, dim))
        S = r.fill(P.F_GAUSS, THETA, u, it=it)
        assert S == meta["samples_%d" % it]
        assert np.array_equal(r.counts.ravel(), z["counts_%d" % it].astype(np.int64))
        np.testing.assert_allclose(r.JF, z["JF_%d" % it], rtol=1e-9, atol=1e-300)
        np.testing.assert_allclose(r.JF2, z["JF2_%d" % it], rtol=1e-9, atol=1e-300)
        np.testing.assert_allclose(r.weights.ravel(), z["weights_%d" % it], rtol=1e-9)
        # dh = (v^2 JF2/n - (v JF/n)^2)^beta cancels: 1e-15 differences in JF
        # (the reference accumulates with atomics in arbitrary order) grow to
        # ~1e-7 here, inside the 1e-6 bound.  From the reference's own JF the
        # restatement must agree to rounding: CUDA's pow(x, 2) / pow(t, beta)
        # and glibc's differ by an ulp, which the same cancellation lifts to
        # ~1e-9, hence 1e-8.
        dsum, res, sig = r.results()
        np.testing.assert_allclose(r.dh, z["dh_%d" % it], rtol=1e-6, atol=1e-300)
        np.testing.assert_allclose([res, sig], [z["res_%d" % it][0], z["sig_%d" % it][0]],
                                   rtol=1e-9)
        r.set_cube_sums(z["JF_%d" % it], z["JF2_%d" % it])
        dsum, res, sig = r.results()
        np.testing.assert_allclose(r.dh, z["dh_%d" % it], rtol=1e-8, atol=1e-300)
        np.testing.assert_allclose([res, sig, dsum], [z["res_%d" % it][0], z["sig_%d" % it][0],
                                                      z["dh_sum_%d" % it][0]], rtol=1e-11)
        r.refine()
        np.testing.assert_allclose(r.x_edges.ravel(), z["x_edges_out_%d" % it], rtol=1e-9,
                                   atol=1e-15)
        r.update_nh(dsum)
        assert np.array_equal(r.nh, z["nh_next_%d" % it])
        if it + 1 < iters:   # the reference's own chaining
            assert np.array_equal(z["nh_next_%d" % it], z["nh_%d" % (it + 1)])
            assert np.array_equal(z["x_edges_out_%d" % it], z["x_edges_in_%d" % (it + 1)])


@pytest.mark.parametrize("name,meta,z,kept", BENCH, ids=[c[0] for c in BENCH])
def test_oracle_reproduces_reference_at_benchmark_shape(name, meta, z, kept):
    """C1 exactly (d=4, 1e6 evals/iteration, 1024 bins, width 0.1, iterations
    0, 1 and 9 of 10) and the d=8 / width 0.1 / 1024-bin shape at 2e6
    evals/iteration: with the reference's uniforms of every stride-th
    hypercube replayed, the oracle reproduces those hypercubes' sums (1e-9),
    damped variances (1e-7 from the reference's own sums) and next counts
    (exactly), and from the reference's whole per-bin histograms its refined
    grid (1e-9)."""
    dim, N, iters = meta["dim"], meta["n_intervals"], meta["iters"]
    r = P.OracleRun(dim, meta["n_eval_it"] * iters, iters, n_intervals=N)
    assert r.sz.n_strat == meta["n_strat"] and r.sz.n_cubes == meta["n_cubes"]
    assert abs(r.sz.v_cubes - meta["v_cubes"]) <= 1e-15 * meta["v_cubes"]
    theta = np.array([0.5, meta["width"]])
    cubes = kept_cubes(meta)
    for it in kept:
        if it == 0:
            assert np.array_equal(r.x_edges.ravel(), z["x_edges_in_0"])
            assert np.array_equal(r.nh, z["nh_0"].astype(np.int64))
        r.set_x_edges(z["x_edges_in_%d" % it])
        r.set_nh(z["nh_%d" % it].astype(np.int64))
        u, keep = P.uniforms(P.U_BUFFER, ubuf=expand_uniforms(meta, z, it))
        assert r.fill(P.F_GAUSS, theta, u, it=it) == meta["samples_%d" % it]
        JF, JF2 = r.JF, r.JF2
        np.testing.assert_allclose(JF[cubes], z["JF_%d" % it], rtol=1e-9, atol=1e-300)
        np.testing.assert_allclose(JF2[cubes], z["JF2_%d" % it], rtol=1e-9, atol=1e-300)
        JF[cubes], JF2[cubes] = z["JF_%d" % it], z["JF2_%d" % it]
        r.set_cube_sums(JF, JF2)
        r.results()
        # the cancellation in d_h lifts pow's last-ulp differences (CUDA vs
        # glibc) to ~2e-8 in the worst of these 3661 cubes
        np.testing.assert_allclose(r.dh[cubes], z["dh_%d" % it], rtol=1e-7, atol=1e-300)
        r.update_nh(z["dh_sum_%d" % it][0])
        assert np.array_equal(r.nh[cubes], z["nh_next_%d" % it].astype(np.int64))
        r.set_hist(z["weights_%d" % it], z["counts_%d" % it])
        assert int(z["counts_%d" % it].astype(np.int64).sum()) == dim * meta["samples_%d" % it]
        r.refine()
        np.testing.assert_allclose(r.x_edges.ravel(), z["x_edges_out_%d" % it], rtol=1e-9,
                                   atol=1e-15)
        if it + 1 in kept:   # the reference's own chaining
            assert np.array_equal(z["x_edges_out_%d" % it], z["x_edges_in_%d" % (it + 1)])
