"""Object layer over the C ABI: contexts, compiled integrands, runs.

All work happens in libcuvegas.so on the GPU; this module only moves
parameters and host arrays across the boundary.
"""
import ctypes as C

import numpy as np

from . import _lib as L

_contexts = {}


class Context:
    """One device + stream (include/cuvegas.h: cvg_context_create)."""

    def __init__(self, device=0, stream=None):
        self._lib = L.load()
        h = C.c_void_p()
        L.check(self._lib.cvg_context_create(int(device), stream, C.byref(h)))
        self.handle = h
        self.device = device
        self._integrands = {}

    def close(self):
        if self.handle:
            for f in list(self._integrands.values()):
                f.close()
            self._integrands.clear()
            self._lib.cvg_context_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def trim(self):
        """Free the device arenas kept from destroyed runs and batches."""
        L.check(self._lib.cvg_context_trim(self.handle))

    def measure_peak(self, kind):
        v = C.c_double()
        L.check(self._lib.cvg_measure_peak(self.handle, int(kind), C.byref(v)))
        return v.value

    def integrand(self, source, n_dim, n_params=0, has_grad=False, abi=L.ABI_NATIVE):
        key = (source, int(n_dim), int(n_params), bool(has_grad), int(abi))
        f = self._integrands.get(key)
        if f is None:
            f = Integrand(self, source, n_dim, n_params, has_grad, abi)
            self._integrands[key] = f
        return f

    def integrand_ptx(self, ptx, n_dim, source=None):
        """Integrand given as PTX with the numba ABI (cvg_compile_integrand_ptx)."""
        key = ("ptx", ptx, source, int(n_dim))
        f = self._integrands.get(key)
        if f is None:
            f = Integrand(self, source or "", n_dim, abi=L.ABI_NUMBA, ptx=ptx)
            self._integrands[key] = f
        return f


def default_context(device=None):
    if device is None:
        device = 0
        try:
            import torch
            if torch.cuda.is_available():
                device = torch.cuda.current_device()
        except Exception:
            pass
    ctx = _contexts.get(device)
    if ctx is None or not ctx.handle:
        ctx = Context(device)
        _contexts[device] = ctx
    return ctx


class Integrand:
    """A JIT-compiled integrand (cvg_compile_integrand)."""

    def __init__(self, ctx, source, n_dim, n_params=0, has_grad=False, abi=L.ABI_NATIVE, ptx=None):
        self.ctx = ctx
        self.source = source + (ptx or "")
        self.n_dim = int(n_dim)
        self.n_params = int(n_params)
        self.has_grad = bool(has_grad)
        h = C.c_void_p()
        if ptx is not None:
            L.check(ctx._lib.cvg_compile_integrand_ptx(ctx.handle, source.encode() if source else None,
                                                       ptx.encode(), self.n_dim, C.byref(h)))
        else:
            L.check(ctx._lib.cvg_compile_integrand(ctx.handle, source.encode(), self.n_dim, int(abi),
                                                   self.n_params, int(self.has_grad), C.byref(h)))
        self.handle = h

    def close(self):
        if self.handle:
            self.ctx._lib.cvg_integrand_release(self.handle)
            self.handle = None


def make_params(n_dim, tot_eval, max_it, skip=5, n_intervals=1024, n_strat=0, alpha=0.5,
                beta=0.75, seed=0, precision=L.PREC_FP64, flags=0, block=0, spt=0, instance=0,
                max_batch_size=1048576, gpu_thr=0.1):
    p = L.Params()
    p.tot_eval = int(tot_eval)
    p.max_it = int(max_it)
    p.skip = int(skip)
    p.max_batch_size = int(max_batch_size)
    p.n_intervals = int(n_intervals)
    p.n_strat = int(n_strat or 0)
    p.n_dim = int(n_dim)
    p.precision = int(precision)
    p.alpha = float(alpha)
    p.beta = float(beta)
    p.seed = int(seed) & 0xFFFFFFFFFFFFFFFF
    p.gpu_thr = float(gpu_thr)
    p.flags = int(flags)
    p.block = int(block)
    p.spt = int(spt)
    p.instance = int(instance)
    return p


def _theta_ptr(theta, n_params):
    if n_params == 0:
        return None, None
    th = np.ascontiguousarray(theta, dtype=np.float64)
    if th.size != n_params:
        raise ValueError("theta must have %d values" % n_params)
    return th, th.ctypes.data_as(C.c_void_p)


def integrate_once(integrand, params, theta=None):
    """cvg_integrate: one whole integration; returns (Result, it_res, it_sig2)."""
    lib = integrand.ctx._lib
    th, thp = _theta_ptr(theta, integrand.n_params)
    res = L.Result()
    it_res = np.zeros(params.max_it)
    it_sig = np.zeros(params.max_it)
    L.check(lib.cvg_integrate(integrand.ctx.handle, integrand.handle, C.byref(params), thp,
                              C.byref(res), it_res.ctypes.data_as(C.c_void_p),
                              it_sig.ctypes.data_as(C.c_void_p)))
    return res, it_res, it_sig


_BUF_DTYPES = {
    L.BUF_X_EDGES: np.float64, L.BUF_NH: np.uint32, L.BUF_NH_SUM: np.uint64,
    L.BUF_JF: np.float64, L.BUF_JF2: np.float64, L.BUF_WEIGHTS: np.float64,
    L.BUF_COUNTS: np.uint32, L.BUF_DH: np.float64, L.BUF_THETA: np.float64,
    L.BUF_ITERATION: np.uint32, L.BUF_STATS: np.float64, L.BUF_SCALE_EXP: np.int32, L.BUF_BIN_EXP: np.int32,
    L.BUF_HIST_STATE: np.uint32, L.BUF_TILE_CUBE: np.uint32,
}


class Run:
    """Persistent device state of one integration (cvg_run_*)."""

    def __init__(self, integrand, params, theta=None):
        self.f = integrand
        self.params = params
        self._lib = integrand.ctx._lib
        th, thp = _theta_ptr(theta, integrand.n_params)
        h = C.c_void_p()
        L.check(self._lib.cvg_run_create(integrand.ctx.handle, integrand.handle, C.byref(params),
                                         thp, C.byref(h)))
        self.handle = h
        self.info = self.get_info()

    def close(self):
        if getattr(self, "handle", None):
            self._lib.cvg_run_destroy(self.handle)
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

    def get_info(self):
        info = L.RunInfo()
        L.check(self._lib.cvg_run_info_get(self.handle, C.byref(info)))
        return info

    def iterate(self, n):
        L.check(self._lib.cvg_run_iterate(self.handle, int(n)))

    def step(self, stages):
        L.check(self._lib.cvg_run_step(self.handle, int(stages)))

    def sync(self):
        L.check(self._lib.cvg_run_sync(self.handle))

    def result(self):
        res = L.Result()
        M = self.params.max_it
        it_res = np.zeros(M)
        it_sig = np.zeros(M)
        L.check(self._lib.cvg_run_result(self.handle, C.byref(res),
                                         it_res.ctypes.data_as(C.c_void_p),
                                         it_sig.ctypes.data_as(C.c_void_p)))
        return res, it_res, it_sig

    def _count(self, buf):
        info = self.get_info()
        D, N, nc = info.n_dim, info.n_intervals, info.n_cubes
        return {L.BUF_X_EDGES: D * (N + 1), L.BUF_NH: nc, L.BUF_NH_SUM: nc + 1, L.BUF_JF: nc,
                L.BUF_JF2: nc, L.BUF_WEIGHTS: D * N, L.BUF_COUNTS: D * N, L.BUF_DH: nc,
                L.BUF_THETA: self.f.n_params, L.BUF_ITERATION: 1,
                L.BUF_STATS: 3 * self.params.max_it, L.BUF_SCALE_EXP: 1,
                L.BUF_BIN_EXP: D * N + 1, L.BUF_HIST_STATE: 2,
                L.BUF_TILE_CUBE: info.max_tiles}[buf]

    def get(self, buf):
        dt = _BUF_DTYPES[buf]
        out = np.zeros(self._count(buf), dtype=dt)
        L.check(self._lib.cvg_run_get(self.handle, int(buf), out.ctypes.data_as(C.c_void_p),
                                      out.nbytes))
        if buf in (L.BUF_X_EDGES,):
            out = out.reshape(self.info.n_dim, self.info.n_intervals + 1)
        elif buf in (L.BUF_WEIGHTS, L.BUF_COUNTS):
            out = out.reshape(self.info.n_dim, self.info.n_intervals)
        elif buf == L.BUF_STATS:
            out = out.reshape(3, self.params.max_it)
        return out

    def set(self, buf, arr):
        if buf == L.BUF_UNIFORMS:
            if arr is None:
                L.check(self._lib.cvg_run_set(self.handle, int(buf), None, 0))
                return
            a = np.ascontiguousarray(arr, dtype=np.float32)
        else:
            a = np.ascontiguousarray(arr, dtype=_BUF_DTYPES[buf]).ravel()
        L.check(self._lib.cvg_run_set(self.handle, int(buf), a.ctypes.data_as(C.c_void_p),
                                      a.nbytes))

    # ---- state export / import (checkpoint, resume, warm start) ----------
    def export_state(self):
        """The loop's state between iterations: grid, hypercube allocation,
        iteration counter and per-iteration estimates (plus, in the FP32 form,
        the f*jac scale and the per-bin exponent table).  A run created with
        the same dimension, bins and hypercubes continues from it with
        import_state; with FLAG_NO_ADAPT it integrates on the trained map."""
        self.sync()
        st = {"n_dim": self.info.n_dim, "n_intervals": self.info.n_intervals,
              "n_cubes": self.info.n_cubes, "precision": self.params.precision,
              "max_it": self.params.max_it,
              "x_edges": self.get(L.BUF_X_EDGES), "nh": self.get(L.BUF_NH),
              "iteration": int(self.get(L.BUF_ITERATION)[0]), "stats": self.get(L.BUF_STATS)}
        if self.params.precision == L.PREC_FP32:
            st["scale_exp"] = int(self.get(L.BUF_SCALE_EXP)[0])
            st["bin_exp"] = self.get(L.BUF_BIN_EXP)
            st["hist_state"] = self.get(L.BUF_HIST_STATE)
        return st

    def import_state(self, st, resume=True):
        """Load a state from export_state.  resume=True also takes over the
        iteration counter and the estimates, so the weighted mean continues
        over the earlier iterations (the Philox stream continues too);
        resume=False keeps this run's own counter and estimates (a warm start
        on the trained map)."""
        info = self.info
        if (int(st["n_dim"]), int(st["n_intervals"]), int(st["n_cubes"])) != \
                (info.n_dim, info.n_intervals, info.n_cubes):
            raise ValueError("state of a run with another dimension, bin count or hypercubes")
        self.set(L.BUF_X_EDGES, st["x_edges"])
        self.set(L.BUF_NH, st["nh"])
        if self.params.precision == L.PREC_FP32 and "bin_exp" in st:
            self.set(L.BUF_SCALE_EXP, np.array([st["scale_exp"]], dtype=np.int32))
            self.set(L.BUF_BIN_EXP, st["bin_exp"])
            if "hist_state" in st:
                self.set(L.BUF_HIST_STATE, st["hist_state"])
        if resume:
            it = int(st["iteration"])
            if it > self.params.max_it:
                raise ValueError("state is at iteration %d, this run has max_it %d"
                                 % (it, self.params.max_it))
            old = np.asarray(st["stats"], dtype=np.float64).reshape(3, -1)
            stats = np.zeros((3, self.params.max_it))
            stats[:, :it] = old[:, :it]
            self.set(L.BUF_STATS, stats)
            self.set(L.BUF_ITERATION, np.array([it], dtype=np.uint32))

    def save_state(self, path):
        st = self.export_state()
        np.savez(path, **{k: np.asarray(v) for k, v in st.items()})

    @staticmethod
    def load_state(path):
        with np.load(path) as z:
            return {k: (z[k] if z[k].ndim else z[k].item()) for k in z.files}

    # ---- sample split across ranks (cvg_run_set_shard / cvg_run_buffer) ----
    def set_shard(self, shard, shards):
        """Fill only tiles [T*shard/shards, T*(shard+1)/shards) of each
        iteration (see cuvegas_gb300.shard)."""
        L.check(self._lib.cvg_run_set_shard(self.handle, int(shard), int(shards)))

    def buffer(self, buf):
        """(device address, bytes) of one of the run's buffers."""
        ptr, n = C.c_void_p(), C.c_size_t()
        L.check(self._lib.cvg_run_buffer(self.handle, int(buf), C.byref(ptr), C.byref(n)))
        return ptr.value, n.value

    def grad(self, it=L.IT_CURRENT):
        g = np.zeros(self.f.n_params)
        L.check(self._lib.cvg_run_grad(self.handle, int(it), g.ctypes.data_as(C.c_void_p)))
        return g

    def fill_times(self, cap=4096):
        ms = (C.c_float * cap)()
        n = C.c_int32()
        L.check(self._lib.cvg_run_fill_times(self.handle, ms, cap, C.byref(n)))
        return np.array(ms[:min(n.value, cap)], dtype=np.float64)

    def last_fill_ms(self):
        ms = C.c_float()
        L.check(self._lib.cvg_run_last_fill_ms(self.handle, C.byref(ms)))
        return ms.value
