"""Batched integration: many integrals of one integrand family advanced
together on the GPU (cvg_batch_* of include/cuvegas.h).

Instances differ in dimension, evaluations per iteration and parameters
theta.  Per iteration the whole batch costs one persistent fill launch, one
batched refinement and one batched reallocation; with ``graph=True`` the
iteration is captured once as a CUDA graph and replayed.
"""
import ctypes as C
import time

import numpy as np

from . import _lib as L
from . import runtime


class Batch:
    def __init__(self, ctx, source, instances, params_per_dim, max_it=10, skip=5,
                 n_intervals=1024, alpha=0.5, beta=0.75, seed=0, precision=L.PREC_FP32,
                 graph=True, block=0, spt=0, first_instance=0):
        """instances: list of dicts with keys dim, n_eval_it (evaluations per
        iteration) or tot_eval, theta (n_params(dim) values), optional n_strat
        and instance (Philox stream id; default first_instance + index)."""
        self._lib = ctx._lib
        self.ctx = ctx
        self.n = len(instances)
        self.max_it = max_it
        arr = (L.Instance * self.n)()
        thetas = []
        for i, inst in enumerate(instances):
            arr[i].n_dim = int(inst["dim"])
            arr[i].n_strat = int(inst.get("n_strat", 0))
            arr[i].tot_eval = int(inst.get("tot_eval", int(inst.get("n_eval_it", 0)) * max_it))
            arr[i].instance = int(inst.get("instance", first_instance + i))
            th = np.asarray(inst.get("theta", []), dtype=np.float64)
            if th.size != params_per_dim[arr[i].n_dim]:
                raise ValueError("instance %d: %d parameters expected" %
                                 (i, params_per_dim[arr[i].n_dim]))
            thetas.append(th)
        self.theta = np.ascontiguousarray(np.concatenate(thetas) if thetas else np.zeros(1))
        ppd = (C.c_int32 * 17)(*[int(params_per_dim[d]) for d in range(17)])
        p = runtime.make_params(1, 1, max_it, skip=skip, n_intervals=n_intervals, alpha=alpha,
                                beta=beta, seed=seed, precision=precision,
                                flags=L.FLAG_GRAPH if graph else 0, block=block, spt=spt)
        h = C.c_void_p()
        L.check(self._lib.cvg_batch_create(ctx.handle, source.encode(), L.ABI_NATIVE, self.n, arr,
                                           ppd, self.theta.ctypes.data_as(C.c_void_p),
                                           C.byref(p), C.byref(h)))
        self.handle = h

    def close(self):
        if getattr(self, "handle", None):
            self._lib.cvg_batch_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def iterate(self, n):
        L.check(self._lib.cvg_batch_iterate(self.handle, int(n)))

    def info(self):
        b, s, g = C.c_int32(), C.c_int32(), C.c_int32()
        sm, ns = C.c_int64(), C.c_int64()
        L.check(self._lib.cvg_batch_info_get(self.handle, C.byref(b), C.byref(s), C.byref(g),
                                             C.byref(sm), C.byref(ns)))
        return dict(block=b.value, spt=s.value, grid=g.value, fill_smem=sm.value,
                    next_samples=ns.value)

    def results(self):
        out = (L.Result * self.n)()
        it_res = np.zeros((self.n, self.max_it))
        it_sig = np.zeros((self.n, self.max_it))
        L.check(self._lib.cvg_batch_results(self.handle, out, it_res.ctypes.data_as(C.c_void_p),
                                            it_sig.ctypes.data_as(C.c_void_p)))
        return list(out), it_res, it_sig


def integrate_batch(source, instances, params_per_dim, max_it=10, skip=5, n_intervals=1024,
                    alpha=0.5, beta=0.75, seed=0, precision="fp32", graph=True, device=None,
                    tune=True):
    """Integrate every instance; returns a list of (result, error, chi2_dof)."""
    from . import autotune
    prec = {"fp64": L.PREC_FP64, "fp32": L.PREC_FP32}[precision]
    ctx = runtime.default_context(device)
    block = spt = 0
    if tune:
        block, spt = autotune.tune_batch(ctx, source, instances, params_per_dim, prec,
                                         n_intervals=n_intervals)
    with Batch(ctx, source, instances, params_per_dim, max_it=max_it, skip=skip,
               n_intervals=n_intervals, alpha=alpha, beta=beta, seed=seed, precision=prec,
               graph=graph, block=block, spt=spt) as b:
        b.iterate(max_it)
        res, _, _ = b.results()
    return [(r.result, r.error, r.chi2_dof) for r in res]
