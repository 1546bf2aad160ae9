"""ctypes binding of libcuvegas.so (the C ABI declared in include/cuvegas.h).

The library is built in-tree by ``cuvegas_gb300._build.build()``.  There is no
fallback: if the library is missing or cannot be loaded, every entry point
raises ``CuvegasError``.
"""
import ctypes as C
import os
import threading

PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG, "_lib", "libcuvegas.so")

OK, ERR_INVALID, ERR_CUDA, ERR_COMPILE, ERR_NOMEM, ERR_KERNEL, ERR_STATE = range(7)
PREC_FP64, PREC_FP32 = 0, 1
ABI_NATIVE, ABI_NUMBA = 0, 1
FLAG_GRAPH, FLAG_NO_ADAPT, FLAG_TIME_FILL = 1, 2, 4
STAGE_FILL, STAGE_REALLOC, STAGE_REFINE = 1, 2, 4
(BUF_X_EDGES, BUF_NH, BUF_NH_SUM, BUF_JF, BUF_JF2, BUF_WEIGHTS, BUF_COUNTS, BUF_DH, BUF_THETA,
 BUF_ITERATION, BUF_UNIFORMS, BUF_STATS, BUF_SCALE_EXP, BUF_BIN_EXP, BUF_HIST_STATE,
 BUF_TILE_CUBE) = range(16)
IT_CURRENT = 0xFFFFFFFF

# every exported symbol of include/cuvegas.h
EXPORTS = (
    "cvg_last_error", "cvg_version", "cvg_context_create", "cvg_context_destroy",
    "cvg_compile_integrand", "cvg_integrand_release", "cvg_integrate", "cvg_run_create",
    "cvg_run_destroy", "cvg_run_iterate", "cvg_run_step", "cvg_run_result", "cvg_run_sync",
    "cvg_run_get", "cvg_run_set", "cvg_run_info_get", "cvg_run_grad", "cvg_compile_check",
    "cvg_run_last_fill_ms", "cvg_run_fill_times", "cvg_measure_peak", "cvg_realloc_noalloc",
    "cvg_batch_create", "cvg_batch_destroy", "cvg_batch_iterate", "cvg_batch_results",
    "cvg_batch_info_get", "cvg_batch_last_fill_ms", "cvg_batch_compile_check",
    "cvg_context_trim", "cvg_compile_integrand_ptx", "cvg_run_set_shard", "cvg_run_buffer",
)
NOALLOC_MAX_CUBES = 262144


class CuvegasError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__("cuvegas error %d: %s" % (status, msg))
        self.status = status


class Params(C.Structure):
    _fields_ = [("tot_eval", C.c_int64), ("max_it", C.c_int32), ("skip", C.c_int32),
                ("max_batch_size", C.c_int64), ("n_intervals", C.c_int32),
                ("n_strat", C.c_int32), ("n_dim", C.c_int32), ("precision", C.c_int32),
                ("alpha", C.c_double), ("beta", C.c_double), ("seed", C.c_uint64),
                ("gpu_thr", C.c_double), ("flags", C.c_int32), ("block", C.c_int32),
                ("spt", C.c_int32), ("instance", C.c_uint32)]


class Result(C.Structure):
    _fields_ = [("result", C.c_double), ("error", C.c_double), ("n_strat", C.c_int32),
                ("n_intervals", C.c_int32), ("n_cubes", C.c_int64), ("tot_nevals", C.c_int64),
                ("tot_time_ms", C.c_double), ("avg_it_time_ms", C.c_double),
                ("seed", C.c_uint64), ("gpu_thr", C.c_double), ("chi2_dof", C.c_double),
                ("n_it_used", C.c_int32), ("n_it_done", C.c_int32), ("precision", C.c_int32),
                ("pad", C.c_int32)]


class Instance(C.Structure):
    _fields_ = [("n_dim", C.c_int32), ("n_strat", C.c_int32), ("tot_eval", C.c_int64),
                ("instance", C.c_uint32), ("pad", C.c_int32)]


class RunInfo(C.Structure):
    _fields_ = [("n_eval_it", C.c_int64), ("n_cubes", C.c_int64), ("next_samples", C.c_int64),
                ("max_tiles", C.c_int64), ("n_strat", C.c_int32), ("n_intervals", C.c_int32),
                ("n_dim", C.c_int32), ("block", C.c_int32), ("spt", C.c_int32),
                ("grid", C.c_int32), ("edges_smem", C.c_int32), ("hist_smem", C.c_int32),
                ("v_cubes", C.c_double), ("fill_smem_bytes", C.c_int64),
                ("tile_samples", C.c_int32), ("warp_tiles", C.c_int32)]


_lib = None
_lock = threading.Lock()


def load():
    """Load libcuvegas.so (raises CuvegasError when it is missing)."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        if not os.path.exists(LIB_PATH):
            raise CuvegasError(ERR_STATE, "libcuvegas.so is not built (%s); run "
                               "cuvegas_gb300._build.build()" % LIB_PATH)
        L = C.CDLL(LIB_PATH)
        vp, sz = C.c_void_p, C.c_size_t
        st = C.c_int
        L.cvg_last_error.restype = C.c_char_p
        L.cvg_version.restype = C.c_char_p
        sig = {
            "cvg_context_create": [C.c_int, vp, C.POINTER(vp)],
            "cvg_context_destroy": [vp],
            "cvg_context_trim": [vp],
            "cvg_compile_integrand_ptx": [vp, C.c_char_p, C.c_char_p, C.c_int32, C.POINTER(vp)],
            "cvg_compile_integrand": [vp, C.c_char_p, C.c_int32, C.c_int32, C.c_int32,
                                      C.c_int32, C.POINTER(vp)],
            "cvg_integrand_release": [vp],
            "cvg_integrate": [vp, vp, C.POINTER(Params), vp, C.POINTER(Result), vp, vp],
            "cvg_run_create": [vp, vp, C.POINTER(Params), vp, C.POINTER(vp)],
            "cvg_run_destroy": [vp],
            "cvg_run_iterate": [vp, C.c_int32],
            "cvg_run_step": [vp, C.c_int32],
            "cvg_run_result": [vp, C.POINTER(Result), vp, vp],
            "cvg_run_sync": [vp],
            "cvg_run_get": [vp, C.c_int32, vp, sz],
            "cvg_run_set": [vp, C.c_int32, vp, sz],
            "cvg_run_set_shard": [vp, C.c_int32, C.c_int32],
            "cvg_run_buffer": [vp, C.c_int32, C.POINTER(vp), C.POINTER(sz)],
            "cvg_run_info_get": [vp, C.POINTER(RunInfo)],
            "cvg_run_grad": [vp, C.c_uint32, vp],
            "cvg_compile_check": [C.c_char_p, C.c_int32, C.c_int32, C.c_int32, C.c_int32,
                                  C.c_int32, C.c_char_p, C.c_char_p, sz],
            "cvg_run_last_fill_ms": [vp, C.POINTER(C.c_float)],
            "cvg_run_fill_times": [vp, C.POINTER(C.c_float), C.c_int32, C.POINTER(C.c_int32)],
            "cvg_measure_peak": [vp, C.c_int32, C.POINTER(C.c_double)],
            "cvg_realloc_noalloc": [vp, vp, vp, C.c_uint32, C.c_double, C.c_double, C.c_int64,
                                    C.c_int32, vp, vp, C.c_uint64, C.c_int32, vp],
            "cvg_batch_create": [vp, C.c_char_p, C.c_int32, C.c_int32, C.POINTER(Instance),
                                 C.POINTER(C.c_int32), vp, C.POINTER(Params), C.POINTER(vp)],
            "cvg_batch_destroy": [vp],
            "cvg_batch_iterate": [vp, C.c_int32],
            "cvg_batch_results": [vp, C.POINTER(Result), vp, vp],
            "cvg_batch_info_get": [vp, C.POINTER(C.c_int32), C.POINTER(C.c_int32),
                                   C.POINTER(C.c_int32), C.POINTER(C.c_int64), C.POINTER(C.c_int64)],
            "cvg_batch_last_fill_ms": [vp, C.POINTER(C.c_float)],
            "cvg_batch_compile_check": [C.c_char_p, C.c_int32, C.POINTER(C.c_int32),
                                        C.POINTER(C.c_int32), C.c_int32, C.c_int32, C.c_char_p,
                                        C.c_char_p, sz],
        }
        for name, args in sig.items():
            fn = getattr(L, name)
            fn.argtypes = args
            fn.restype = st
        _lib = L
        return L


def last_error():
    return load().cvg_last_error().decode(errors="replace")


def check(status):
    if status != OK:
        raise CuvegasError(status, last_error())
    return status


def version():
    return load().cvg_version().decode()


def compile_check(source, n_dim, precision=PREC_FP64, n_params=0, has_grad=False,
                  abi=ABI_NATIVE, arch="sm_103a"):
    """NVRTC-only compile of the fill kernel for `source` (no GPU needed)."""
    L = load()
    log = C.create_string_buffer(1 << 16)
    s = L.cvg_compile_check(source.encode(), n_dim, abi, n_params, int(bool(has_grad)),
                            precision, arch.encode(), log, len(log))
    if s != OK:
        raise CuvegasError(s, last_error())
    return log.value.decode(errors="replace")


def batch_compile_check(source, dims, params_per_dim, precision=PREC_FP32, block=512,
                        arch="sm_103a"):
    """NVRTC-only compile of the batched kernels (no GPU needed)."""
    L = load()
    log = C.create_string_buffer(1 << 16)
    d = (C.c_int32 * len(dims))(*dims)
    ppd = (C.c_int32 * 17)(*params_per_dim)
    s = L.cvg_batch_compile_check(source.encode(), len(dims), d, ppd, precision, block,
                                  arch.encode(), log, len(log))
    if s != OK:
        raise CuvegasError(s, last_error())
    return log.value.decode(errors="replace")
