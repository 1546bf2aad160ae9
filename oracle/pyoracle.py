"""ctypes front-end of the CPU oracle (test infrastructure only).

Mirrors the calls of ``oracle/vegas_oracle.h``; every function there cites the
reference lines it restates.
"""
import ctypes as C
import numpy as np

from . import build_oracle

F_GAUSS, F_MIXTURE, F_PRODPEAK, F_CORNER, F_CONST, F_REFLIB = range(6)
U_PHILOX_F64, U_PHILOX_F32, U_BUFFER = range(3)

_lib = None


class Sizes(C.Structure):
    _fields_ = [("n_eval_it", C.c_int64), ("n_strat", C.c_int32), ("n_cubes", C.c_int64),
                ("v_cubes", C.c_double), ("nh_init", C.c_int64)]


class State(C.Structure):
    _fields_ = [("dim", C.c_int), ("n_intervals", C.c_int), ("n_strat", C.c_int),
                ("n_cubes", C.c_int64), ("n_eval_it", C.c_int64),
                ("v_cubes", C.c_double), ("alpha", C.c_double), ("beta", C.c_double),
                ("x_edges", C.POINTER(C.c_double)), ("weights", C.POINTER(C.c_double)),
                ("counts", C.POINTER(C.c_int64)), ("JF", C.POINTER(C.c_double)),
                ("JF2", C.POINTER(C.c_double)), ("nh", C.POINTER(C.c_int64)),
                ("nh_sum", C.POINTER(C.c_int64)), ("dh", C.POINTER(C.c_double))]


class Uniforms(C.Structure):
    _fields_ = [("kind", C.c_int), ("seed", C.c_uint64), ("instance", C.c_uint32),
                ("ubuf", C.POINTER(C.c_float))]


class Result(C.Structure):
    _fields_ = [("result", C.c_double), ("error", C.c_double), ("chi2_dof", C.c_double),
                ("tot_nevals", C.c_int64), ("n_it_used", C.c_int)]


def lib():
    global _lib
    if _lib is None:
        path = build_oracle.build()
        L = C.CDLL(path)
        dp = C.POINTER(C.c_double)
        L.orc_philox4x32_10.argtypes = [C.POINTER(C.c_uint32)] * 3
        L.orc_eval.restype = C.c_double
        L.orc_eval.argtypes = [C.c_int, dp, C.c_int, dp]
        L.orc_eval_grad.argtypes = [C.c_int, dp, C.c_int, dp, dp]
        L.orc_compute_sizes.argtypes = [C.c_int64, C.c_int, C.c_int, C.c_int, C.POINTER(Sizes)]
        L.orc_state_init.argtypes = [C.POINTER(State), C.c_int, C.c_int, C.POINTER(Sizes),
                                     C.c_double, C.c_double]
        L.orc_state_free.argtypes = [C.POINTER(State)]
        L.orc_scan_nh.argtypes = [C.POINTER(State)]
        L.orc_fill.restype = C.c_int64
        L.orc_fill.argtypes = [C.POINTER(State), C.c_int, dp, C.POINTER(Uniforms), C.c_uint32,
                               C.c_int]
        L.orc_results.argtypes = [C.POINTER(State), dp, dp, dp]
        L.orc_update_nh.argtypes = [C.POINTER(State), C.c_double]
        L.orc_refine.argtypes = [C.POINTER(State)]
        L.orc_integrate.argtypes = [C.c_int, dp, C.c_int, C.c_int64, C.c_int, C.c_int, C.c_int,
                                    C.c_int, C.c_double, C.c_double, C.POINTER(Uniforms),
                                    C.c_int, C.POINTER(Result), dp, dp, dp]
        L.orc_grad_iteration.argtypes = [C.POINTER(State), C.c_int, dp, C.c_int,
                                         C.POINTER(Uniforms), C.c_uint32, C.c_int, dp]
        _lib = L
    return _lib


def _dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double)) if a is not None else None


def philox(ctr, key):
    c = (C.c_uint32 * 4)(*ctr)
    k = (C.c_uint32 * 2)(*key)
    o = (C.c_uint32 * 4)()
    lib().orc_philox4x32_10(c, k, o)
    return list(o)


def sizes(tot_eval, max_it, dim, n_strat=0):
    s = Sizes()
    rc = lib().orc_compute_sizes(int(tot_eval), int(max_it), int(dim), int(n_strat), C.byref(s))
    if rc:
        raise ValueError("invalid sizes (rc=%d)" % rc)
    return s


def uniforms(kind=U_PHILOX_F64, seed=0, instance=0, ubuf=None):
    u = Uniforms()
    u.kind = kind
    u.seed = seed
    u.instance = instance
    keep = None
    if ubuf is not None:
        keep = np.ascontiguousarray(ubuf, dtype=np.float32)
        u.ubuf = keep.ctypes.data_as(C.POINTER(C.c_float))
    return u, keep


def evaluate(family, x, theta=None):
    x = np.ascontiguousarray(x, dtype=np.float64)
    th = None if theta is None else np.ascontiguousarray(theta, dtype=np.float64)
    return lib().orc_eval(family, _dp(x), x.shape[-1], _dp(th))


class OracleRun:
    """Step-by-step access to one oracle run (fill / results / refine / nh)."""

    def __init__(self, dim, tot_eval, max_it, n_intervals=1024, n_strat=0, alpha=0.5,
                 beta=0.75):
        self.sz = sizes(tot_eval, max_it, dim, n_strat)
        self.st = State()
        if lib().orc_state_init(C.byref(self.st), dim, n_intervals, C.byref(self.sz), alpha,
                                beta):
            raise MemoryError("oracle state")
        self.dim, self.N = dim, n_intervals

    def __del__(self):
        try:
            lib().orc_state_free(C.byref(self.st))
        except Exception:
            pass

    def _arr(self, ptr, n, dt):
        return np.ctypeslib.as_array(ptr, shape=(n,)).astype(dt, copy=True)

    @property
    def x_edges(self):
        return self._arr(self.st.x_edges, self.dim * (self.N + 1), np.float64).reshape(
            self.dim, self.N + 1)

    def set_x_edges(self, xe):
        xe = np.ascontiguousarray(xe, dtype=np.float64).ravel()
        np.ctypeslib.as_array(self.st.x_edges, shape=(xe.size,))[:] = xe

    @property
    def nh(self):
        return self._arr(self.st.nh, self.st.n_cubes, np.int64)

    def set_nh(self, nh):
        np.ctypeslib.as_array(self.st.nh, shape=(self.st.n_cubes,))[:] = nh
        lib().orc_scan_nh(C.byref(self.st))

    @property
    def nh_sum(self):
        return self._arr(self.st.nh_sum, self.st.n_cubes + 1, np.int64)

    @property
    def JF(self):
        return self._arr(self.st.JF, self.st.n_cubes, np.float64)

    @property
    def JF2(self):
        return self._arr(self.st.JF2, self.st.n_cubes, np.float64)

    @property
    def dh(self):
        return self._arr(self.st.dh, self.st.n_cubes, np.float64)

    @property
    def weights(self):
        return self._arr(self.st.weights, self.dim * self.N, np.float64).reshape(self.dim, self.N)

    @property
    def counts(self):
        return self._arr(self.st.counts, self.dim * self.N, np.int64).reshape(self.dim, self.N)

    def set_hist(self, weights, counts):
        np.ctypeslib.as_array(self.st.weights, shape=(self.dim * self.N,))[:] = np.ravel(weights)
        np.ctypeslib.as_array(self.st.counts, shape=(self.dim * self.N,))[:] = np.ravel(counts)

    def set_cube_sums(self, JF, JF2):
        np.ctypeslib.as_array(self.st.JF, shape=(self.st.n_cubes,))[:] = JF
        np.ctypeslib.as_array(self.st.JF2, shape=(self.st.n_cubes,))[:] = JF2

    def fill(self, family, theta=None, u=None, it=0, n_threads=0):
        th = None if theta is None else np.ascontiguousarray(theta, dtype=np.float64)
        if u is None:
            u, _ = uniforms()
        n = lib().orc_fill(C.byref(self.st), family, _dp(th), C.byref(u), it, n_threads)
        if n < 0:
            raise RuntimeError("oracle fill failed")
        return n

    def results(self):
        d, r, s = C.c_double(), C.c_double(), C.c_double()
        lib().orc_results(C.byref(self.st), C.byref(d), C.byref(r), C.byref(s))
        return d.value, r.value, s.value

    def update_nh(self, dh_sum):
        lib().orc_update_nh(C.byref(self.st), dh_sum)
        lib().orc_scan_nh(C.byref(self.st))

    def refine(self):
        lib().orc_refine(C.byref(self.st))

    def grad(self, family, theta, n_params, u, it, n_threads=0):
        th = np.ascontiguousarray(theta, dtype=np.float64)
        g = np.zeros(n_params)
        rc = lib().orc_grad_iteration(C.byref(self.st), family, _dp(th), n_params, C.byref(u),
                                      it, n_threads, _dp(g))
        if rc:
            raise RuntimeError("oracle grad failed")
        return g


def integrate(family, dim, tot_eval, max_it, theta=None, skip=5, n_intervals=1024, n_strat=0,
              alpha=0.5, beta=0.75, u=None, n_threads=0):
    """Whole loop; returns (result, error, chi2_dof, tot_nevals, it_res, it_sig, x_edges)."""
    th = None if theta is None else np.ascontiguousarray(theta, dtype=np.float64)
    if u is None:
        u, _ = uniforms()
    res = Result()
    it_res = np.zeros(max_it)
    it_sig = np.zeros(max_it)
    xe = np.zeros(dim * (n_intervals + 1))
    rc = lib().orc_integrate(family, _dp(th), dim, int(tot_eval), max_it, skip, n_intervals,
                             n_strat, alpha, beta, C.byref(u), n_threads, C.byref(res),
                             _dp(it_res), _dp(it_sig), _dp(xe))
    if rc:
        raise RuntimeError("oracle integrate rc=%d" % rc)
    return dict(result=res.result, error=res.error, chi2_dof=res.chi2_dof,
                tot_nevals=res.tot_nevals, it_res=it_res, it_sig=it_sig,
                x_edges=xe.reshape(dim, n_intervals + 1))
