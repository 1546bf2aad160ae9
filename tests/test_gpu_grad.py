"""Backward kernel: dI/dtheta of the two-Gaussian mixture (d=6, 16 parameters,
C3 shape) against same-seed central finite differences (h=1e-4) of the
frozen-state estimator and against the analytic gradient."""
import numpy as np
import pytest

from cuvegas_gb300 import _lib as L, autograd as AG, integrands as I, runtime
from cuvegas_gb300 import analytic as A

pytestmark = pytest.mark.gpu
DIM = 6


def _params(prec, n_it, iters, skip):
    return runtime.make_params(DIM, n_it * iters, iters, skip=skip, n_intervals=1024, seed=3,
                               precision=prec)


@pytest.mark.parametrize("prec", [L.PREC_FP64, L.PREC_FP32])
def test_grad_vs_finite_differences(ctx, prec):
    th = I.mixture_theta(0, DIM)
    f = ctx.integrand(I.MIXTURE, DIM, n_params=16, has_grad=True)
    p = _params(prec, 200000, 6, 3)
    Ival, err, G, _, recs, _ = AG.forward_with_grad(f, p, th, record=True)
    I0, _ = AG.replay_estimates(f, p, th, recs)
    # the replay reproduces the forward estimate (same samples, grids, counts)
    assert abs(I0 - Ival) <= 1e-12 * abs(Ival)
    h = 1e-4
    for k in range(16):
        tp, tm = th.copy(), th.copy()
        tp[k] += h
        tm[k] -= h
        fd = (AG.replay_estimates(f, p, tp, recs)[0] - AG.replay_estimates(f, p, tm, recs)[0]) / (2 * h)
        tol = 1e-3 * max(abs(fd), 1e-3 * np.abs(G).max())
        assert abs(G[k] - fd) <= tol, (k, G[k], fd)


def test_grad_vs_analytic_c3(ctx):
    """C3 shape: 15 iterations x 1e7 evaluations, FP32 form."""
    th = I.mixture_theta(0, DIM)
    f = ctx.integrand(I.MIXTURE, DIM, n_params=16, has_grad=True)
    p = _params(L.PREC_FP32, 10_000_000, 15, 5)
    Ival, err, G, g_it, _, res = AG.forward_with_grad(f, p, th)
    exact = A.mixture(th, DIM)
    gex = A.mixture_grad(th, DIM)
    assert abs(Ival - exact) < 4 * err, (Ival, exact, err)
    # statistical error of each gradient component from the spread over iterations
    sg = g_it.std(axis=0, ddof=1) / np.sqrt(len(g_it))
    for k in range(16):
        assert abs(G[k] - gex[k]) <= 5 * sg[k] + 1e-3 * abs(gex[k]), (k, G[k], gex[k], sg[k])


def test_autograd_function(ctx):
    torch = pytest.importorskip("torch")
    th = torch.tensor(I.mixture_theta(1, DIM), dtype=torch.float64, requires_grad=True)
    out = AG.integrate_diff(I.MIXTURE, DIM, th, n_evals=6 * 200000, max_it=6, skip=2, seed=5)
    out.backward()
    assert th.grad is not None and th.grad.shape == (16,)
    gex = A.mixture_grad(th.detach().numpy(), DIM)
    assert np.all(np.isfinite(th.grad.numpy()))
    assert np.corrcoef(th.grad.numpy(), gex)[0, 1] > 0.99
