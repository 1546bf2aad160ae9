"""CPU tests of the oracle (the checker): known answers and self-consistency."""
import ctypes
import math

import numpy as np
import pytest

from cuvegas_gb300 import analytic as A
from oracle import pyoracle as P

# Published Philox4x32-10 known-answer vectors (Random123 kat_vectors).
KAT = [
    ((0, 0, 0, 0), (0, 0), (0x6627e8d5, 0xe169c58d, 0xbc57ac4c, 0x9b00dbd8)),
    ((0xffffffff,) * 4, (0xffffffff,) * 2, (0x408f276d, 0x41c83b0e, 0xa20bc7c6, 0x6d5451fd)),
    ((0x243f6a88, 0x85a308d3, 0x13198a2e, 0x03707344), (0xa4093822, 0x299f31d0),
     (0xd16cfe09, 0x94fdcceb, 0x5001e420, 0x24126ea1)),
]


@pytest.mark.parametrize("ctr,key,want", KAT)
def test_philox_kat(ctr, key, want):
    assert tuple(P.philox(ctr, key)) == want


def test_philox_matches_curand_host_generator():
    """First block of curand's host Philox4_32_10 generator = philox(ctr=0, key=seed)."""
    try:
        cr = ctypes.CDLL("libcurand.so")
    except OSError:
        try:
            cr = ctypes.CDLL("/usr/local/cuda/lib64/libcurand.so")
        except OSError:
            pytest.skip("libcurand not available")
    gen = ctypes.c_void_p()
    assert cr.curandCreateGeneratorHost(ctypes.byref(gen), 161) == 0  # CURAND_RNG_PSEUDO_PHILOX4_32_10
    for seed in (0, 1, 0x1234567890abcdef):
        assert cr.curandSetPseudoRandomGeneratorSeed(gen, ctypes.c_uint64(seed)) == 0
        assert cr.curandSetGeneratorOffset(gen, ctypes.c_uint64(0)) == 0
        out = (ctypes.c_uint32 * 4)()
        assert cr.curandGenerate(gen, out, 4) == 0
        want = P.philox((0, 0, 0, 0), (seed & 0xffffffff, seed >> 32))
        assert list(out) == want
    cr.curandDestroyGenerator(gen)


def test_sizes_follow_reference():
    # main.cu:304, 329-331, 444-445 for the configs' shapes
    s = P.sizes(10 * 1_000_000, 10, 4)
    assert (s.n_eval_it, s.n_strat, s.n_cubes, s.nh_init) == (1_000_000, 22, 234256, 4)
    s = P.sizes(20 * 100_000_000, 20, 8)
    assert (s.n_strat, s.n_cubes, s.nh_init) == (8, 16777216, 5)
    s = P.sizes(15 * 10_000_000, 15, 6)
    assert (s.n_strat, s.n_cubes, s.nh_init) == (11, 1771561, 5)
    s = P.sizes(20 * 1_000_000_000, 20, 16)
    assert (s.n_strat, s.n_cubes, s.nh_init) == (3, 43046721, 23)
    s = P.sizes(10 * 10_000, 10, 12)
    assert (s.n_strat, s.n_cubes, s.nh_init) == (1, 1, 10000)
    with pytest.raises(ValueError):
        P.sizes(10, 10, 4)        # fewer than 4 evals per iteration -> no stratum


def test_uniform_grid_and_nh_init():
    r = P.OracleRun(3, 3 * 4000, 3, n_intervals=16)
    xe = r.x_edges
    assert np.array_equal(xe[1], np.arange(17) / 16)
    assert np.all(r.nh == r.sz.nh_init)
    assert r.nh_sum[-1] == r.sz.nh_init * r.sz.n_cubes


def _py_refine(weights, counts, x_edges, alpha):
    """Second, literal restatement of src/main.cu:106-145, 189-246 for one dim."""
    N = len(weights)
    w = [weights[i] / counts[i] if counts[i] != 0 else weights[i] for i in range(N)]
    dsum = sum(w)
    sm = []
    for i in range(N):
        if i == 0:
            t = (7.0 * w[0] + w[1]) / (8.0 * dsum)
        elif i == N - 1:
            t = (w[i - 1] + 7.0 * w[i]) / (8.0 * dsum)
        else:
            t = (w[i - 1] + 6.0 * w[i] + w[i + 1]) / (8.0 * dsum)
        if t != 0:
            t = ((t - 1.0) / math.log(t)) ** alpha
        sm.append(t)
    ssum = sum(sm)
    cs = np.cumsum(sm)
    delta = ssum / N
    old = [N - 1] * N
    for i in range(N):
        div = int(cs[i] / delta)
        off = int(cs[i - 1] / delta) if i > 0 else 0
        for j in range(div - off):
            old[off + j] = i
    xn = list(x_edges)
    for k in range(N - 1):
        o = old[k]
        acc = (k + 1) * delta - (cs[o - 1] if o > 0 else 0)
        xn[k + 1] = x_edges[o] + acc / sm[o] * (x_edges[o + 1] - x_edges[o])
    return np.array(xn)


def test_refine_matches_literal_restatement():
    rng = np.random.default_rng(3)
    r = P.OracleRun(2, 2 * 4000, 2, n_intervals=32)
    w = rng.gamma(2.0, 1.0, size=(2, 32))
    c = rng.integers(0, 50, size=(2, 32))
    w[c == 0] = 0
    xe0 = r.x_edges
    r.set_hist(w, c)
    r.refine()
    xe = r.x_edges
    for d in range(2):
        want = _py_refine(w[d], c[d], xe0[d], 0.5)
        np.testing.assert_allclose(xe[d], want, rtol=1e-13, atol=1e-15)
        assert np.all(np.diff(xe[d]) > 0)
        assert xe[d][0] == 0.0 and xe[d][-1] == 1.0


def test_refine_zero_weights_keeps_grid():
    r = P.OracleRun(2, 2 * 4000, 2, n_intervals=8)
    xe0 = r.x_edges
    r.set_hist(np.zeros((2, 8)), np.zeros((2, 8), dtype=np.int64))
    r.refine()
    assert np.array_equal(r.x_edges, xe0)


def test_results_and_nh_formulas():
    """results (main.cu:81-104) and updateNh (main.cu:173-187) restated in numpy."""
    rng = np.random.default_rng(5)
    r = P.OracleRun(2, 2 * 40000, 2, n_intervals=8)
    nc = r.sz.n_cubes
    nh = rng.integers(2, 9, size=nc)
    r.set_nh(nh)
    JF = rng.normal(1.0, 0.2, size=nc)
    JF2 = JF ** 2 * nh + rng.uniform(0, 0.5, size=nc)
    r.set_cube_sums(JF, JF2)
    dsum, res, sig = r.results()
    v = r.sz.v_cubes
    Ih = JF / nh * v
    S2 = (JF2 / nh * v * v) - Ih * Ih
    t = np.maximum(v * v * JF2 / nh - (v * JF / nh) ** 2, 0)
    dh = t ** 0.75
    np.testing.assert_allclose(r.dh, dh, rtol=1e-13)
    np.testing.assert_allclose([dsum, res, sig], [dh.sum(), Ih.sum(), (S2 / nh).sum()], rtol=1e-12)
    r.update_nh(dsum)
    want = np.maximum(2, (dh / dsum * r.sz.n_eval_it).astype(np.int64))
    assert np.array_equal(r.nh, want)
    assert np.array_equal(r.nh_sum, np.concatenate([[0], np.cumsum(want)]))


def test_fill_replay_buffer_equals_philox():
    """Buffer replay of the Philox FP64 uniforms reproduces the Philox fill."""
    dim = 3
    r1 = P.OracleRun(dim, 3 * 2000, 3, n_intervals=16)
    u1, _ = P.uniforms(P.U_PHILOX_F64, seed=11)
    r1.fill(P.F_GAUSS, np.array([0.5, 0.2]), u1, it=0)
    # build the same uniforms in sample order
    nh_sum = r1.nh_sum
    S = nh_sum[-1]
    ub = np.zeros((S, dim), dtype=np.float64)
    for c in range(r1.sz.n_cubes):
        for j in range(nh_sum[c + 1] - nh_sum[c]):
            w = P.philox((j, c, 0, 0), (11, 0))
            ub[nh_sum[c] + j] = (np.array(w[:dim], dtype=np.float64) + 0.5) * 2.0 ** -32
    # float32 replay differs from the FP64 uniforms by rounding: compare loosely
    r2 = P.OracleRun(dim, 3 * 2000, 3, n_intervals=16)
    u2, keep = P.uniforms(P.U_BUFFER, ubuf=ub.astype(np.float32))
    r2.fill(P.F_GAUSS, np.array([0.5, 0.2]), u2, it=0)
    np.testing.assert_allclose(r2.JF, r1.JF, rtol=1e-5)
    assert abs(r2.counts.sum() - r1.counts.sum()) == 0


def test_oracle_c1_small_against_analytic():
    u, _ = P.uniforms(P.U_PHILOX_F64, seed=0)
    o = P.integrate(P.F_GAUSS, 4, 8 * 200_000, 8, theta=np.array([0.5, 0.1]), skip=3, u=u)
    exact = A.gauss_normalised(4)
    assert abs(o["result"] - exact) < 4 * o["error"], (o["result"], exact, o["error"])
    assert o["error"] / exact < 3e-4


def test_analytic_values():
    assert abs(A.gauss_normalised(4) - math.erf(5) ** 4) < 1e-15
    # corner peak, d=1: (1/c)(1 - 1/(1+c))
    assert abs(A.corner_peak([0.5]) - (1 / 0.5) * (1 - 1 / 1.5)) < 1e-14
    # product peak, d=1, numerical check
    c, u = 7.0, 0.3
    x = (np.arange(200000) + 0.5) / 200000
    num = np.mean(1 / (c ** -2 + (x - u) ** 2))
    assert abs(A.product_peak([c], [u]) - num) / num < 1e-6
    # mixture gradient vs central differences of the closed form
    from cuvegas_gb300 import integrands as I
    th = I.mixture_theta(0)
    g = A.mixture_grad(th, 6)
    h = 1e-6
    for i in range(len(th)):
        tp, tm = th.copy(), th.copy()
        tp[i] += h
        tm[i] -= h
        fd = (A.mixture(tp, 6) - A.mixture(tm, 6)) / (2 * h)
        assert abs(fd - g[i]) <= 1e-6 * max(1.0, abs(g[i]))


def test_corner_peak_exact_small():
    # d=2 closed form: 1/(2 c1 c2) [1 - 1/(1+c1) - 1/(1+c2) + 1/(1+c1+c2)]
    c1, c2 = 0.3, 0.8
    want = (1 - 1 / (1 + c1) - 1 / (1 + c2) + 1 / (1 + c1 + c2)) / (2 * c1 * c2)
    assert abs(A.corner_peak([c1, c2]) - want) < 1e-14
