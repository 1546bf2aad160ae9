"""Differentiable VEGAS+ integrals: I(theta) and dI/dtheta.

The forward pass runs the iteration loop step by step on the GPU.  For every
iteration that enters the weighted mean, the gradient kernel re-draws the
same Philox samples of that iteration with its grid and hypercube counts held
fixed and accumulates sum_h (V/n_h) sum_j J * df/dtheta (the derivative of
that iteration's estimate).  The iteration gradients are combined with the
same inverse-variance weights as the estimate (weights held constant), and
``backward`` returns grad_output * dI/dtheta.

The integrand source must define ``integrand(T* x, const T* theta)`` and
``integrand_grad(T* x, const T* theta, T* g)``.

``replay_estimates`` re-evaluates recorded iterations at other parameters
with the same samples, grids and counts (the frozen-state estimator whose
finite differences the gradient kernel reproduces).
"""
import numpy as np
import torch

from . import _lib as L
from . import runtime


class IterationRecord:
    """Grid, counts and weight of one iteration that entered the mean."""

    def __init__(self, it, x_edges, nh, res, sig2):
        self.it, self.x_edges, self.nh, self.res, self.sig2 = it, x_edges, nh, res, sig2


def forward_with_grad(integrand, params, theta, record=False):
    """Run the loop; returns (I, sigma, dI/dtheta, per-iteration grads, records, result)."""
    th = np.ascontiguousarray(theta, dtype=np.float64)
    grads, recs = {}, []
    with runtime.Run(integrand, params, th) as r:
        for it in range(params.max_it):
            if record and it >= params.skip:
                xe, nh = r.get(L.BUF_X_EDGES), r.get(L.BUF_NH)
            r.step(L.STAGE_FILL)
            if it >= params.skip:
                grads[it] = r.grad()          # same samples, grid and nh as this fill
            r.step(L.STAGE_REALLOC | L.STAGE_REFINE)
            if record and it >= params.skip:
                recs.append(IterationRecord(it, xe, nh, None, None))
        res, it_res, it_sig = r.result()
    used = list(range(params.skip, params.max_it))
    w = np.array([1.0 / it_sig[i] for i in used])
    g_it = np.array([grads[i] for i in used])
    G = (w[:, None] * g_it).sum(0) / w.sum()
    for rec in recs:
        rec.res, rec.sig2 = it_res[rec.it], it_sig[rec.it]
    return res.result, res.error, G, g_it, recs, res


def replay_estimates(integrand, params, theta, records):
    """Estimates I_i(theta) of recorded iterations with their samples, grids and
    counts held fixed; returns the mean with the recorded weights."""
    p = runtime.make_params(params.n_dim, params.tot_eval, params.max_it, skip=0,
                            n_intervals=params.n_intervals, n_strat=params.n_strat,
                            alpha=params.alpha, beta=params.beta, seed=params.seed,
                            precision=params.precision, flags=L.FLAG_NO_ADAPT,
                            block=params.block, spt=params.spt, instance=params.instance)
    vals = []
    with runtime.Run(integrand, p, np.ascontiguousarray(theta, dtype=np.float64)) as r:
        for rec in records:
            r.set(L.BUF_X_EDGES, rec.x_edges)
            r.set(L.BUF_NH, rec.nh)
            r.set(L.BUF_ITERATION, np.array([rec.it], dtype=np.uint32))
            r.step(L.STAGE_FILL | L.STAGE_REALLOC)
            vals.append(r.get(L.BUF_STATS)[0, rec.it])
    w = np.array([1.0 / rec.sig2 for rec in records])
    return float((w * np.array(vals)).sum() / w.sum()), np.array(vals)


class VegasIntegral(torch.autograd.Function):
    """I = integral of f(x; theta) over [0,1]^d by VEGAS+, differentiable in theta."""

    @staticmethod
    def forward(ctx, theta, integrand, params):
        I, err, G, _, _, _ = forward_with_grad(integrand, params,
                                               theta.detach().cpu().double().numpy())
        ctx.save_for_backward(torch.as_tensor(G, dtype=theta.dtype, device=theta.device))
        ctx.error = err
        return torch.as_tensor(I, dtype=theta.dtype, device=theta.device)

    @staticmethod
    def backward(ctx, grad_out):
        (G,) = ctx.saved_tensors
        return grad_out * G, None, None


def integrate_diff(source, n_dim, theta, n_evals=1000000, max_it=20, skip=5, n_intervals=1024,
                   n_strat=None, alpha=0.5, beta=0.75, seed=0, precision="fp32", device=None):
    """Differentiable integral: returns a 0-d tensor I(theta) with grad_fn."""
    theta = torch.as_tensor(theta)
    ctx = runtime.default_context(device)
    f = ctx.integrand(source, n_dim, n_params=theta.numel(), has_grad=True)
    p = runtime.make_params(n_dim, n_evals, max_it, skip=skip, n_intervals=n_intervals,
                            n_strat=n_strat or 0, alpha=alpha, beta=beta, seed=seed,
                            precision={"fp64": L.PREC_FP64, "fp32": L.PREC_FP32}[precision])
    return VegasIntegral.apply(theta, f, p)
