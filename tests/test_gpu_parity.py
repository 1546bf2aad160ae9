"""GPU parity: the CUDA path (through the C ABI) against the CPU oracle on the
same inputs.  FP64 map arithmetic is identical by construction (same explicit
fma sequence, same Philox words), so bin counts must match exactly and float
sums to summation-order rounding."""
import numpy as np
import pytest

from cuvegas_gb300 import _lib as L, integrands as I, runtime
from cuvegas_gb300 import analytic as A
from oracle import pyoracle as P

pytestmark = pytest.mark.gpu

GAUSS_TH = np.array([0.5, 0.1])


def make_run(ctx, src, dim, n_it, max_it, N=64, prec=L.PREC_FP64, seed=1, theta=None, P_=0,
             grad=False, **kw):
    f = ctx.integrand(src, dim, n_params=P_, has_grad=grad)
    p = runtime.make_params(dim, n_it * max_it, max_it, n_intervals=N, seed=seed, precision=prec,
                            **kw)
    return runtime.Run(f, p, theta)


def force_fixed_point(r):
    """Next fill of an FP32 run with fixed-point bin sums (the first fill of a
    run keeps float sums; its exponent table is the pilot's)."""
    r.set(L.BUF_HIST_STATE, np.array([1, 0], dtype=np.uint32))


def oracle_run(dim, n_it, max_it, N=64):
    return P.OracleRun(dim, n_it * max_it, max_it, n_intervals=N)


def relerr(a, b):
    a, b = np.asarray(a, float), np.asarray(b, float)
    return np.max(np.abs(a - b) / np.maximum(np.abs(b), 1e-300))


@pytest.mark.parametrize("dim,n_it,N", [(3, 30000, 64), (1, 5000, 16), (5, 20000, 128),
                                        (2, 999, 2), (8, 60000, 1024), (12, 30000, 100),
                                        (16, 40000, 37)])
def test_fill_fp64_matches_oracle(ctx, dim, n_it, N):
    with make_run(ctx, I.GAUSS, dim, n_it, 4, N=N, seed=5) as r:
        r.step(L.STAGE_FILL)
        JF, JF2 = r.get(L.BUF_JF), r.get(L.BUF_JF2)
        W, Cn = r.get(L.BUF_WEIGHTS), r.get(L.BUF_COUNTS)
    o = oracle_run(dim, n_it, 4, N)
    u, _ = P.uniforms(P.U_PHILOX_F64, seed=5)
    S = o.fill(P.F_GAUSS, GAUSS_TH, u, it=0)
    assert Cn.sum() == S * dim
    assert np.array_equal(Cn.astype(np.int64), o.counts)
    np.testing.assert_allclose(JF, o.JF, rtol=1e-12, atol=1e-300)
    np.testing.assert_allclose(JF2, o.JF2, rtol=1e-12, atol=1e-300)
    np.testing.assert_allclose(W, o.weights, rtol=1e-11, atol=1e-300)


def test_fill_fp32_histograms_against_oracle(ctx):
    """FP32 form: per-bin sums of (f*jac)^2 (fixed point in shared memory,
    wraps and large weights in FP64) against the FP64 oracle on the same
    Philox words.  The FP32 map may put a sample in the neighbouring bin when
    y*N lies within FP32 rounding of an integer."""
    dim, n_it, N = 3, 200000, 64
    with make_run(ctx, I.GAUSS, dim, n_it, 4, N=N, seed=5, prec=L.PREC_FP32) as r:
        k = int(r.get(L.BUF_SCALE_EXP)[0])
        force_fixed_point(r)
        r.step(L.STAGE_FILL)
        JF, W, Cn = r.get(L.BUF_JF), r.get(L.BUF_WEIGHTS), r.get(L.BUF_COUNTS)
    W = W * 4.0 ** k
    o = oracle_run(dim, n_it, 4, N)
    u, _ = P.uniforms(P.U_PHILOX_F32, seed=5)
    S = o.fill(P.F_GAUSS, GAUSS_TH, u, it=0)
    assert Cn.sum() == S * dim
    assert np.abs(Cn.astype(np.int64) - o.counts).sum() <= 2e-4 * S * dim
    np.testing.assert_allclose(W.sum(axis=1), o.weights.sum(axis=1), rtol=2e-5)
    # every bin to its own relative precision, also the tail bins whose sums
    # are ~1e-20 of the central ones (the refinement's damping weighs them)
    assert o.weights.min() < 1e-15 * o.weights.max()
    np.testing.assert_allclose(W, o.weights, rtol=2e-3, atol=0)
    np.testing.assert_allclose(JF.sum(), o.JF.sum(), rtol=1e-5)


@pytest.mark.parametrize("dim,n_it,N,fixed", [(2, 50000, 64, True), (5, 100000, 64, True),
                                              (7, 100000, 64, True), (8, 100000, 1024, True),
                                              (12, 60000, 64, True), (16, 60000, 64, False),
                                              (8, 100000, 1024, False)])
def test_fill_fp32_histograms_every_dimension(ctx, dim, n_it, N, fixed):
    """FP32 form at dimensions whose fixed-point histogram updates split into
    groups of 8, 4, 2 and 1: every dimension's counts and per-dimension sums
    against the FP64 oracle on the same Philox words.  The d=16 Gaussian's
    pilot table is too coarse for fixed point (a bin's pilot mean 2^26 above
    its fill weights), which is why a run's first fill keeps float sums."""
    with make_run(ctx, I.GAUSS, dim, n_it, 4, N=N, seed=7, prec=L.PREC_FP32) as r:
        k = int(r.get(L.BUF_SCALE_EXP)[0])
        if fixed:
            force_fixed_point(r)
        r.step(L.STAGE_FILL)
        JF, W, Cn = r.get(L.BUF_JF), r.get(L.BUF_WEIGHTS), r.get(L.BUF_COUNTS)
    W = W * 4.0 ** k
    o = oracle_run(dim, n_it, 4, N)
    u, _ = P.uniforms(P.U_PHILOX_F32, seed=7)
    S = o.fill(P.F_GAUSS, GAUSS_TH, u, it=0)
    assert np.array_equal(Cn.astype(np.int64).sum(axis=1), np.full(dim, S))
    assert np.abs(Cn.astype(np.int64) - o.counts).sum() <= 2e-4 * S * dim
    np.testing.assert_allclose(W.sum(axis=1), o.weights.sum(axis=1), rtol=2e-5)
    np.testing.assert_allclose(JF.sum(), o.JF.sum(), rtol=1e-5)


@pytest.mark.parametrize("wt", ["1", "0"])
@pytest.mark.parametrize("prec", [L.PREC_FP64, L.PREC_FP32])
def test_warp_and_block_tiles(ctx, monkeypatch, wt, prec):
    """The fill's two tile shapes (a warp's 32*spt samples claimed from a
    counter, or the CTA's block*spt samples): the first fill's per-bin counts
    against the oracle's, and for FP64 whole iterations against the oracle's."""
    monkeypatch.setenv("CVG_FILL_WARP_TILES", wt)
    # 2e6 samples in warp tiles of 32 x 8: more tiles than the grid's warps,
    # so warps also claim tiles from the counter
    dim, n_it, N, it = 5, 2000000, 128, 4
    kind = P.U_PHILOX_F64 if prec == L.PREC_FP64 else P.U_PHILOX_F32
    with make_run(ctx, I.GAUSS, dim, n_it, it, N=N, seed=3, prec=prec, skip=1,
                  block=512, spt=8) as r:
        if wt == "1":
            assert n_it // r.info.tile_samples > r.info.grid * r.info.block // 32
        assert r.info.warp_tiles == int(wt)
        assert r.info.tile_samples == (32 if wt == "1" else r.info.block) * r.info.spt
        r.step(L.STAGE_FILL)
        Cn = r.get(L.BUF_COUNTS)
        r.step(L.STAGE_REALLOC | L.STAGE_REFINE)
        r.iterate(it - 1)
        res, it_res, _ = r.result()
    o = oracle_run(dim, n_it, it, N)
    u, _ = P.uniforms(kind, seed=3)
    S = o.fill(P.F_GAUSS, GAUSS_TH, u, it=0)
    assert Cn.astype(np.int64).sum() == S * dim
    if prec == L.PREC_FP64:
        assert np.array_equal(Cn.astype(np.int64), o.counts)
        u, _ = P.uniforms(P.U_PHILOX_F64, seed=3)
        ref = P.integrate(P.F_GAUSS, dim, n_it * it, it, theta=GAUSS_TH, skip=1, n_intervals=N, u=u)
        assert relerr(it_res, ref["it_res"]) < 1e-9
    else:
        assert np.abs(Cn.astype(np.int64) - o.counts).sum() <= 2e-4 * S * dim
        assert abs(res.result - 1.0) < 5 * res.error


def test_fp32_bin_exponent_table(ctx):
    """The pilot's table of per-bin weight exponents follows the integrand:
    central bins of the Gaussian far above the tails; each refinement
    replaces it with one for the new bins."""
    dim, n_it, N = 3, 200000, 64
    with make_run(ctx, I.GAUSS, dim, n_it, 4, N=N, seed=5, prec=L.PREC_FP32) as r:
        t0 = r.get(L.BUF_BIN_EXP)
        r.iterate(2)
        t1 = r.get(L.BUF_BIN_EXP)
        k = int(r.get(L.BUF_SCALE_EXP)[0])
    e0 = t0[:-1].reshape(dim, N)
    assert t0[-1] == 0                                   # pilot sums are unscaled
    assert np.all(e0[:, N // 2] > e0[:, 0] + 40)         # exp(-2*25) ~ 2^-72 at the edge
    assert np.all(np.abs(e0[:, N // 2] - e0[:, N // 2 - 1]) < 4)
    e1 = t1[:-1].reshape(dim, N)
    assert not np.array_equal(e0, e1)
    # after adaptation the bins are far closer in expected weight
    assert np.ptp(e1) < np.ptp(e0)
    assert abs(int(t1[-1]) - k) <= 4


def test_fill_fp32_histogram_word_wraps(ctx):
    """f = 1 on the uniform grid: every sample adds weight 1 (2^16 fixed-point
    units) to its bin.  Each CTA takes ~2.6e5 of the 4e7 samples, more than
    2^16 per bin of its two, so its shared-memory words wrap (2^32 units)
    at least once; the bin sums must still equal the counts exactly."""
    n_it = 40_000_000
    with make_run(ctx, I.CONST_ONE, 1, n_it, 2, N=2, seed=1, prec=L.PREC_FP32,
                  block=1024, spt=64) as r:
        assert int(r.get(L.BUF_SCALE_EXP)[0]) == 0
        assert r.info.grid <= 2 * 152
        assert n_it / r.info.grid / 2 > 2 ** 16
        force_fixed_point(r)
        r.step(L.STAGE_FILL)
        W, Cn = r.get(L.BUF_WEIGHTS), r.get(L.BUF_COUNTS)
        r.step(L.STAGE_REALLOC | L.STAGE_REFINE)
        res, it_res, _ = r.result()
    assert Cn.sum() == n_it
    assert np.array_equal(W, Cn.astype(np.float64))
    assert it_res[0] == 1.0


def test_fill_replay_uniforms_matches_oracle(ctx):
    dim, n_it, N = 3, 20000, 32
    o = oracle_run(dim, n_it, 2, N)
    S = int(o.nh_sum[-1])
    ub = np.random.default_rng(9).uniform(0, 1, size=(S, dim)).astype(np.float32)
    ub[::97, 0] = 1.0                    # curand_uniform may return exactly 1
    with make_run(ctx, I.GAUSS, dim, n_it, 2, N=N) as r:
        r.set(L.BUF_UNIFORMS, ub)
        r.step(L.STAGE_FILL)
        JF, JF2 = r.get(L.BUF_JF), r.get(L.BUF_JF2)
        W, Cn = r.get(L.BUF_WEIGHTS), r.get(L.BUF_COUNTS)
    u, keep = P.uniforms(P.U_BUFFER, ubuf=ub)
    o.fill(P.F_GAUSS, GAUSS_TH, u, it=0)
    assert np.array_equal(Cn.astype(np.int64), o.counts)
    np.testing.assert_allclose(JF, o.JF, rtol=1e-12)
    np.testing.assert_allclose(JF2, o.JF2, rtol=1e-12)
    np.testing.assert_allclose(W, o.weights, rtol=1e-11)


def test_realloc_matches_oracle(ctx):
    dim, n_it, N = 3, 30000, 64
    o = oracle_run(dim, n_it, 4, N)
    u, _ = P.uniforms(P.U_PHILOX_F64, seed=2)
    o.fill(P.F_GAUSS, GAUSS_TH, u, it=0)
    with make_run(ctx, I.GAUSS, dim, n_it, 4, N=N, seed=2) as r:
        r.set(L.BUF_JF, o.JF)
        r.set(L.BUF_JF2, o.JF2)
        r.step(L.STAGE_REALLOC)
        nh, dh = r.get(L.BUF_NH), r.get(L.BUF_DH)
        nh_sum = r.get(L.BUF_NH_SUM)
        res, it_res, it_sig = r.result()
        assert r.get(L.BUF_ITERATION)[0] == 1
        assert not r.get(L.BUF_JF).any()      # consumed and cleared
    dsum, ri, si = o.results()
    # dh cancels; CUDA's and glibc's pow differ by an ulp, lifted to ~1e-13..1e-10
    np.testing.assert_allclose(dh, o.dh, rtol=1e-9)
    np.testing.assert_allclose([it_res[0], it_sig[0]], [ri, si], rtol=1e-12)
    o.update_nh(dsum)
    assert np.array_equal(nh.astype(np.int64), o.nh)
    assert np.array_equal(nh_sum.astype(np.int64), o.nh_sum)


def test_realloc_fp32_form_against_fp64_oracle(ctx):
    """FP32 form: per-cube mean/variance in compensated FP32, sums in FP64.
    Iteration estimate to 1e-10, variance to 1e-6, allocation within 1e-5."""
    dim, n_it, N = 4, 200000, 64
    o = oracle_run(dim, n_it, 4, N)
    u, _ = P.uniforms(P.U_PHILOX_F64, seed=12)
    o.fill(P.F_GAUSS, GAUSS_TH, u, it=0)
    with make_run(ctx, I.GAUSS, dim, n_it, 4, N=N, seed=12, prec=L.PREC_FP32) as r:
        r.set(L.BUF_JF, o.JF)
        r.set(L.BUF_JF2, o.JF2)
        r.step(L.STAGE_REALLOC)
        nh = r.get(L.BUF_NH).astype(np.int64)
        st = r.get(L.BUF_STATS)
    dsum, ri, si = o.results()
    assert abs(st[0, 0] - ri) <= 1e-10 * abs(ri)
    assert abs(st[1, 0] - si) <= 1e-6 * abs(si)
    o.update_nh(dsum)
    assert np.all(np.abs(nh - o.nh) <= 1 + 1e-5 * o.nh)
    assert nh.sum() <= o.sz.n_eval_it + 2 * o.sz.n_cubes


@pytest.mark.parametrize("dim,N", [(4, 256), (1, 2), (2, 3), (3, 100), (2, 1000), (1, 4096)])
def test_refine_matches_oracle(ctx, dim, N):
    """Grid refinement (8-CTA clusters per dimension) against the oracle for
    bin counts that do and do not divide among the cluster's CTAs."""
    rng = np.random.default_rng(4)
    w = rng.gamma(1.5, 2.0, size=(dim, N))
    c = rng.integers(0, 40, size=(dim, N))
    w[c == 0] = 0.0
    o = oracle_run(dim, 50000, 3, N)
    xe = o.x_edges
    xe[:, 1:-1] = np.sort(rng.uniform(0, 1, size=(dim, N - 1)), axis=1)
    o.set_x_edges(xe)
    o.set_hist(w, c)
    o.refine()
    with make_run(ctx, I.GAUSS, dim, 50000, 3, N=N) as r:
        r.set(L.BUF_X_EDGES, xe)
        r.set(L.BUF_WEIGHTS, w)
        r.set(L.BUF_COUNTS, c.astype(np.uint32))
        r.step(L.STAGE_REFINE)
        got = r.get(L.BUF_X_EDGES)
        assert not r.get(L.BUF_WEIGHTS).any() and not r.get(L.BUF_COUNTS).any()
    np.testing.assert_allclose(got, o.x_edges, rtol=1e-12, atol=1e-15)
    assert np.all(np.diff(got, axis=1) > 0)


@pytest.mark.parametrize("graph", [False, True])
def test_full_run_fp64_matches_oracle(ctx, graph):
    dim, n_it, max_it, N = 3, 40000, 6, 128
    with make_run(ctx, I.GAUSS, dim, n_it, max_it, N=N, seed=3, skip=2,
                  flags=L.FLAG_GRAPH if graph else 0) as r:
        r.iterate(max_it)
        res, it_res, it_sig = r.result()
        xe = r.get(L.BUF_X_EDGES)
    u, _ = P.uniforms(P.U_PHILOX_F64, seed=3)
    o = P.integrate(P.F_GAUSS, dim, n_it * max_it, max_it, theta=GAUSS_TH, skip=2,
                    n_intervals=N, u=u)
    assert res.tot_nevals == o["tot_nevals"]
    assert relerr(it_res, o["it_res"]) < 1e-9
    assert relerr(it_sig, o["it_sig"]) < 1e-8
    assert abs(res.result - o["result"]) / abs(o["result"]) < 1e-10
    assert abs(res.error - o["error"]) / o["error"] < 1e-8
    np.testing.assert_allclose(xe, o["x_edges"], rtol=1e-9, atol=1e-12)


@pytest.mark.parametrize("dim,n_it,max_it,skip", [(4, 1_000_000, 10, 5), (8, 2_000_000, 4, 1)],
                         ids=["c1_d4_1e6x10", "c2shape_d8_2e6x4"])
def test_benchmark_shape_full_run_fp64_matches_oracle(ctx, dim, n_it, max_it, skip):
    """C1 exactly (d=4, 1e6 evals/iteration, 10 iterations, 1024 bins, alpha
    0.5, beta 0.75, seed 0) and the d=8 / 1024-bin shape of the headline at
    2e6 evals/iteration, FP64 form, through the C ABI against the oracle on
    the same Philox stream: identical evaluation totals, every iteration's
    estimate to 1e-9, the result to 1e-10 and the final grid to 1e-9."""
    N = 1024
    with make_run(ctx, I.GAUSS, dim, n_it, max_it, N=N, seed=0, skip=skip) as r:
        r.iterate(max_it)
        res, it_res, it_sig = r.result()
        xe = r.get(L.BUF_X_EDGES)
    u, _ = P.uniforms(P.U_PHILOX_F64, seed=0)
    o = P.integrate(P.F_GAUSS, dim, n_it * max_it, max_it, theta=GAUSS_TH, skip=skip,
                    n_intervals=N, u=u)
    assert res.tot_nevals == o["tot_nevals"]
    assert relerr(it_res, o["it_res"]) < 1e-9
    assert relerr(it_sig, o["it_sig"]) < 1e-8
    assert abs(res.result - o["result"]) / abs(o["result"]) < 1e-10
    assert abs(res.error - o["error"]) / o["error"] < 1e-8
    np.testing.assert_allclose(xe, o["x_edges"], rtol=1e-9, atol=1e-12)


def _quantiles(a):
    a = np.asarray(a, dtype=np.float64)
    return {"p50": float(np.median(a)), "p99": float(np.quantile(a, 0.99)),
            "p999": float(np.quantile(a, 0.999)), "max": float(a.max()), "n": int(a.size)}


@pytest.mark.parametrize("dim,n_it,pre", [(4, 1_000_000, 3), (4, 1_000_000, 9), (8, 2_000_000, 3)],
                         ids=["c1_it3", "c1_it9", "c2shape_it3"])
def test_fp32_elementwise_against_fp64_oracle(ctx, record_property, dim, n_it, pre):
    """Chosen (FP32-compensated) form against the FP64 oracle, element by
    element, on the same Philox samples: the FP32 loop adapts for `pre`
    iterations, then its next fill (fixed-point bin sums) is compared with the
    oracle's fill of the same iteration on the same grid and n_h.

    Measured on GB300 at these shapes: per-hypercube JF and JF2 agree to a
    median of ~5e-5 / 1e-4 and a 99.9th percentile of ~6e-4 / 1.2e-3 relative;
    per-bin weights to a median of ~7e-5 and a 99th percentile of ~1e-3.
    The FP32 map takes bin widths from FP32 edges (for the narrowest adapted
    bins the width differs from the FP64 width by ~3e-4 relative; the map and
    its Jacobian stay consistent, so the estimate stays unbiased), and a
    sample whose y*N lies within FP32 rounding of a bin edge lands in the
    neighbouring bin (the largest per-cube differences, up to ~0.2 in a cube
    of few samples).  Hypercubes whose per-sample (f*jac*2^-k)^2 fall below
    the FP32 range (JF2/n < 2^-80 after scaling) flush to zero in the FP32
    sums; together they hold less than 1e-12 of the integral and are
    excluded from the per-cube figures.  Bounds asserted: JF median 3e-4,
    99.9th percentile 3e-3, max 0.5; JF2 median 6e-4, 99.9th percentile 6e-3,
    max 0.5; weights median 3e-4, 99th percentile 5e-3, max 0.05 over bins
    above 1e-20 of the largest; bin counts within 2e-4 of all updates; sum
    of JF within 2e-6."""
    N = 1024
    with make_run(ctx, I.GAUSS, dim, n_it, 10, N=N, seed=0, prec=L.PREC_FP32, skip=0) as r:
        r.iterate(pre)
        xe, nh = r.get(L.BUF_X_EDGES), r.get(L.BUF_NH)
        assert r.get(L.BUF_HIST_STATE)[0] == 1          # fixed-point bin sums
        r.step(L.STAGE_FILL)
        JF, JF2 = r.get(L.BUF_JF), r.get(L.BUF_JF2)
        W, Cn = r.get(L.BUF_WEIGHTS), r.get(L.BUF_COUNTS)
        k = int(r.get(L.BUF_BIN_EXP)[-1])
    W = W * 4.0 ** k
    o = P.OracleRun(dim, n_it * 10, 10, n_intervals=N)
    o.set_x_edges(xe)
    o.set_nh(nh.astype(np.int64))
    u, _ = P.uniforms(P.U_PHILOX_F32, seed=0)
    S = o.fill(P.F_GAUSS, GAUSS_TH, u, it=pre)
    oJF, oJF2, oW = o.JF, o.JF2, o.weights
    in_range = oJF2 / nh * 4.0 ** -k >= 2.0 ** -80
    assert oJF[~in_range].sum() < 1e-12 * oJF.sum()
    eJF = np.abs(JF - oJF)[in_range] / oJF[in_range]
    eJF2 = np.abs(JF2 - oJF2)[in_range] / oJF2[in_range]
    big = oW >= 1e-20 * oW.max()
    eW = np.abs(W - oW)[big] / oW[big]
    qJF, qJF2, qW = _quantiles(eJF), _quantiles(eJF2), _quantiles(eW)
    record_property("fp32_vs_fp64", {"JF": qJF, "JF2": qJF2, "weights": qW})
    print("fp32 vs fp64 oracle", dim, n_it, pre, qJF, qJF2, qW)
    assert qJF["p50"] <= 3e-4 and qJF["p999"] <= 3e-3 and qJF["max"] <= 0.5, qJF
    assert qJF2["p50"] <= 6e-4 and qJF2["p999"] <= 6e-3 and qJF2["max"] <= 0.5, qJF2
    assert qW["p50"] <= 3e-4 and qW["p99"] <= 5e-3 and qW["max"] <= 0.05, qW
    assert np.abs(Cn.astype(np.int64) - o.counts).sum() <= 2e-4 * S * dim
    assert abs(JF.sum() - oJF.sum()) <= 2e-6 * oJF.sum()


def test_single_cube_and_fp32_against_fp64_oracle(ctx):
    """n_strat = 1 (d=12, 1e4 evals/iteration): one hypercube holds every sample;
    the reference maps this case on the CPU, here it stays on the GPU."""
    dim, n_it, max_it = 12, 10000, 5
    c, uu = np.full(dim, 8.0), np.full(dim, 0.4)
    u, _ = P.uniforms(P.U_PHILOX_F64, seed=8)
    o = P.integrate(P.F_PRODPEAK, dim, n_it * max_it, max_it, theta=np.concatenate([c, uu]),
                    skip=1, n_intervals=64, u=u)
    th = I.prodpeak_theta(c, uu)
    with make_run(ctx, I.PRODPEAK, dim, n_it, max_it, N=64, seed=8, theta=th, P_=2 * dim,
                  skip=1) as r:
        assert r.info.n_cubes == 1
        r.iterate(max_it)
        res, _, _ = r.result()
    assert res.tot_nevals == o["tot_nevals"]
    assert abs(res.result - o["result"]) / abs(o["result"]) < 1e-9
    with make_run(ctx, I.PRODPEAK, dim, n_it, max_it, N=64, seed=8, theta=th, P_=2 * dim,
                  skip=1, prec=L.PREC_FP32) as r:
        r.iterate(max_it)
        r32, _, _ = r.result()
    assert abs(r32.result - o["result"]) < 0.2 * o["error"]


def test_global_histogram_path(ctx):
    """d=16 with 4096 bins in FP64 does not fit shared memory: grid and bin
    sums go through global memory; results must not change."""
    dim, n_it, N = 16, 200000, 4096
    th = np.linspace(0.1, 1.0, dim)
    with make_run(ctx, I.CORNER, dim, n_it, 2, N=N, seed=4, theta=th, P_=dim) as r:
        assert r.info.hist_smem == 0
        r.step(L.STAGE_FILL)
        JF, Cn = r.get(L.BUF_JF), r.get(L.BUF_COUNTS)
    o = oracle_run(dim, n_it, 2, N)
    u, _ = P.uniforms(P.U_PHILOX_F64, seed=4)
    o.fill(P.F_CORNER, th, u, it=0)
    assert np.array_equal(Cn.astype(np.int64), o.counts)
    np.testing.assert_allclose(JF, o.JF, rtol=1e-12)


def test_c1_fp64_and_fp32_against_analytic(ctx):
    """C1 shape: d=4, 1e6 evals/iteration, 10 iterations, 1024 bins."""
    exact = A.gauss_normalised(4)
    out = {}
    for prec in (L.PREC_FP64, L.PREC_FP32):
        with make_run(ctx, I.GAUSS, 4, 1_000_000, 10, N=1024, seed=0, prec=prec,
                      flags=L.FLAG_GRAPH) as r:
            r.iterate(10)
            res, _, _ = r.result()
        out[prec] = res
        assert abs(res.result - exact) < 4 * res.error, (prec, res.result, exact, res.error)
        assert np.isfinite(res.chi2_dof)
        assert res.error / exact < 1e-4
    # same Philox stream: FP32 and FP64 estimates agree far inside the error
    assert abs(out[0].result - out[1].result) < 0.5 * out[0].error


def test_gradient_matches_oracle(ctx):
    dim = 6
    th = I.mixture_theta(0, dim)
    with make_run(ctx, I.MIXTURE, dim, 50000, 3, N=128, seed=6, theta=th, P_=16,
                  grad=True) as r:
        r.step(L.STAGE_FILL | L.STAGE_REFINE | L.STAGE_REALLOC)   # adapt once
        xe, nh = r.get(L.BUF_X_EDGES), r.get(L.BUF_NH)
        g = r.grad()                       # iteration 1 samples, current grid/nh
    o = oracle_run(dim, 50000, 3, 128)
    o.set_x_edges(xe)
    o.set_nh(nh.astype(np.int64))
    u, _ = P.uniforms(P.U_PHILOX_F64, seed=6)
    go = o.grad(P.F_MIXTURE, th, 16, u, it=1)
    np.testing.assert_allclose(g, go, rtol=1e-9, atol=1e-14)


def test_state_checks(ctx):
    with make_run(ctx, I.GAUSS, 2, 1000, 2, N=16) as r:
        with pytest.raises(L.CuvegasError):
            r.set(L.BUF_NH, np.ones(r.info.n_cubes, dtype=np.uint32))   # nh < 2
        r.iterate(2)
        with pytest.raises(L.CuvegasError) as e:
            r.iterate(1)
        assert e.value.status == L.ERR_STATE


def test_reused_arena_gives_identical_runs(monkeypatch):
    """Destroyed runs leave their device arena to the context and the next run
    of a similar size takes it over.  With CVG_ARENA_POISON every arena handed
    out is filled with 0xFF bytes (NaN doubles), so a buffer a run reads
    without initialising it shows up as NaN or as a different result.  Runs
    agree to summation order (FP64 atomics add shared runs in any order)."""
    monkeypatch.setenv("CVG_ARENA_POISON", "1")
    pctx = runtime.Context(0)

    def once(n_it, prec):
        with make_run(pctx, I.GAUSS, 4, n_it, 5, N=256, seed=9, prec=prec) as r:
            r.iterate(5)
            res, it_res, it_sig = r.result()
            return np.concatenate([it_res, it_sig, [res.result, res.error]]), r.get(L.BUF_X_EDGES)
    try:
        for prec in (L.PREC_FP64, L.PREC_FP32):
            a = once(300000, prec)            # fresh, poisoned allocation
            once(500000, prec)                # other data left in the cached arena
            b = once(300000, prec)            # reuses it, poisoned again
            assert np.all(np.isfinite(a[0])) and np.all(np.isfinite(a[1]))
            assert np.all(np.isfinite(b[0])) and np.all(np.isfinite(b[1]))
            if prec == L.PREC_FP64:
                np.testing.assert_allclose(b[0], a[0], rtol=1e-12)
                np.testing.assert_allclose(b[1], a[1], rtol=1e-12, atol=1e-15)
            else:
                # the FP32 form's second fill keeps its bin sums with float
                # atomics (order-dependent rounding), so grids and estimates
                # agree to statistical precision, not bit for bit
                it_a, sig_a, it_b = a[0][:5], a[0][5:10], b[0][:5]
                assert np.all(np.abs(it_b - it_a) < 5 * np.sqrt(sig_a))
                np.testing.assert_allclose(b[1], a[1], rtol=1e-4, atol=1e-6)
    finally:
        pctx.close()
