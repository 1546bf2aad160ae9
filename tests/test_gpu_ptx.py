"""Integrands given as PTX with numba's ABI (the device ABI the reference
links), JIT-linked into the fill: same fill as the equivalent CUDA source,
closed-form integral, the reference's Python call."""
import os

import numpy as np
import pytest

from cuvegas_gb300 import _lib as L, python_wrapper as W, runtime

pytestmark = pytest.mark.gpu

PTX = open(os.path.join(os.path.dirname(__file__), "golden", "ptx", "sumsq3.ptx")).read()
SRC = ('extern "C" __device__ int integrand(double* ret, double* x) '
       '{ *ret = fma(x[2], x[2], fma(x[1], x[1], x[0] * x[0])); return 0; }\n')


def _fill(f):
    p = runtime.make_params(3, 60000 * 3, 3, n_intervals=64, seed=3)
    with runtime.Run(f, p) as r:
        r.step(L.STAGE_FILL)
        return [r.get(b) for b in (L.BUF_JF, L.BUF_JF2, L.BUF_WEIGHTS, L.BUF_COUNTS)]


def test_ptx_fill_equals_source_fill(ctx):
    a = _fill(ctx.integrand_ptx(PTX, 3))
    b = _fill(ctx.integrand(SRC, 3, abi=L.ABI_NUMBA))
    assert np.array_equal(a[3], b[3])
    for x, y in zip(a[:3], b[:3]):
        np.testing.assert_allclose(x, y, rtol=1e-14, atol=1e-300)


def test_ptx_integral_and_python_call(ctx):
    res, info = W.integrate(PTX, 3, n_evals=2_000_000, max_it=10, skip=4, seed=1)
    assert abs(res - 1.0) < 5 * info["error"]
    with pytest.raises(ValueError):
        W.integrate(PTX, 3, domain=[[0, 2]] * 3, n_evals=100000, max_it=4)
    with pytest.raises(ValueError):
        W.integrate(PTX, 3, n_evals=100000, max_it=4, precision="fp32")


def test_numba_function_when_numba_is_present():
    numba = pytest.importorskip("numba")
    from numba import cuda

    @cuda.jit(device=True)
    def f(x):
        return x[0] * x[0] + x[1] * x[1] + x[2] * x[2]

    res, info = W.integrate(f, 3, n_evals=1_000_000, max_it=8, skip=3, seed=2)
    assert abs(res - 1.0) < 5 * info["error"]
    res2, info2 = W.integrate(f, 3, domain=[[0, 2]] * 3, n_evals=1_000_000, max_it=8, skip=3,
                              seed=2)
    assert abs(res2 - 32.0) < 5 * info2["error"]        # 8 * 3 * (8/3) / 2 ... = 32
