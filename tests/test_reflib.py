"""The reference's integrand library (src/commons/functions.cu:5-111) on the
GPU: fill parity with the oracle's restatement on the same Philox words,
and integrals against closed forms in both precision forms."""
import math

import numpy as np
import pytest

from cuvegas_gb300 import _lib as L, integrands as I, runtime
from oracle import pyoracle as P

DIM = 3


def closed_form(name, d=DIM):
    """Integral over [0,1]^d (None where there is no simple closed form)."""
    if name == "linear":
        return d / 2.0
    if name in ("roosarnold", "morokoffcalfisch", "one"):
        return 1.0
    if name == "hellekalek":
        return 0.0
    if name == "ridge":
        g = lambda x0: math.sqrt(math.pi) / 20.0 * (math.erf(10.0 * (1.0 - x0)) + math.erf(10.0 * x0))
        return (100.0 / math.pi) ** 2 / 1000.0 * sum(g(i / 999.0) ** d for i in range(1000))
    if name == "expon":
        return (math.sqrt(math.pi) / 2.0 * math.erf(1.0)) ** d
    if name == "cosin":
        return math.sin(1.0) ** d
    if name == "dirichlet":
        return math.gamma(5.0 * d) / (math.gamma(5.0) ** d * 5.0 ** d)
    if name == "gaussian":
        return math.erf(0.5 / math.sqrt(2e-4)) ** d
    if name == "sinexp":
        return (1.0 - math.cos(1.0)) + (math.e - 1.0)
    return None


def test_oracle_reflib_against_closed_forms():
    """The oracle's restatement integrates to the closed forms (CPU)."""
    for k, name in enumerate(I.REFLIB_NAMES):
        if name == "one":
            continue                     # zero variance: the reference's weights give NaN
        o = P.integrate(P.F_REFLIB, DIM, 60000 * 6, 6, theta=np.array([float(k)]), skip=2,
                        n_intervals=64, u=P.uniforms(P.U_PHILOX_F64, seed=2)[0])
        ex = closed_form(name)
        assert abs(o["result"] - ex) < 6 * o["error"] + 1e-12, (name, o["result"], ex, o["error"])


@pytest.mark.gpu
@pytest.mark.parametrize("k,name", list(enumerate(I.REFLIB_NAMES)))
def test_reflib_fill_matches_oracle(ctx, k, name):
    n_it, N = 20000, 64
    f = ctx.integrand(I.reflib_source(name), DIM)
    p = runtime.make_params(DIM, n_it * 3, 3, n_intervals=N, seed=6)
    with runtime.Run(f, p) as r:
        r.step(L.STAGE_FILL)
        JF, JF2 = r.get(L.BUF_JF), r.get(L.BUF_JF2)
        W, Cn = r.get(L.BUF_WEIGHTS), r.get(L.BUF_COUNTS)
    o = P.OracleRun(DIM, n_it * 3, 3, n_intervals=N)
    u, _ = P.uniforms(P.U_PHILOX_F64, seed=6)
    o.fill(P.F_REFLIB, np.array([float(k)]), u, it=0)
    assert np.array_equal(Cn.astype(np.int64), o.counts)
    # CUDA's and glibc's pow/exp/cos/tgamma may differ in the last place
    np.testing.assert_allclose(JF, o.JF, rtol=1e-11, atol=1e-300)
    np.testing.assert_allclose(JF2, o.JF2, rtol=1e-11, atol=1e-300)
    np.testing.assert_allclose(W, o.weights, rtol=1e-11, atol=1e-300)


@pytest.mark.gpu
@pytest.mark.parametrize("prec", [L.PREC_FP64, L.PREC_FP32])
@pytest.mark.parametrize("name", I.REFLIB_NAMES)
def test_reflib_integrals(ctx, name, prec):
    f = ctx.integrand(I.reflib_source(name), DIM)
    p = runtime.make_params(DIM, 200000 * 8, 8, skip=3, n_intervals=256, seed=4, precision=prec)
    with runtime.Run(f, p) as r:
        r.iterate(8)
        res, _, _ = r.result()
    ex = closed_form(name)
    if name == "one":                    # every iteration exact (zero variance)
        assert res.error == 0.0 and abs(res.result - 1.0) < 1e-12
        return
    tol = 5 * res.error + (1e-6 * abs(ex) if prec == L.PREC_FP32 else 0.0)
    assert abs(res.result - ex) < tol, (name, res.result, ex, res.error)
