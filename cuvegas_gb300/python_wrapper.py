"""Python entry point with the reference's call signature.

Mirrors ``integrate`` of vegas_cuda/src/vegas_cuda_extension/python_wrapper.py:9-77:
same keyword arguments with the same meanings and defaults, same result tuple
``(result, dict)`` with the same keys, plus ``chi2_dof``, ``precision``,
``it_res`` and ``it_sigma``.

Differences, by design:
  * ``device_function`` is CUDA C++ source defining ``integrand`` (compiled by
    NVRTC inside libcuvegas); or a numba CUDA device function ``f(x) -> float``
    (needs numba), compiled to PTX with numba's own ABI-naming option and
    linked into the fill; or such PTX text (a function ``integrand`` with
    numba's ABI, ``int integrand(double* ret, double* x)``);
  * ``multi_gpu``, ``multi_cpu``, ``gpu_num``, ``cpu_num`` and ``gpu_thr`` are
    accepted and reported but change nothing: one GPU, no CPU mapping fallback;
  * ``precision='fp32'`` selects the FP32 evaluation with compensated
    accumulation (FP64 mean, variance, chi^2 and grid); ``'fp64'`` is the plain
    form.
"""
import math
import os

import numpy as np

from . import _lib as L
from . import runtime


def _domain_source(source, domain, n_dim, abi):
    """Remap [0,1]^d to `domain` around the user integrand
    (python_wrapper.py:20-46): x_i <- x_i*(b_i-a_i) + a_i, result * volume."""
    start = np.zeros(n_dim)
    rng = np.zeros(n_dim)
    vol = 1.0
    for i in range(n_dim):
        a, b = float(domain[i][0]), float(domain[i][1])
        start[i] = a
        rng[i] = b - a
        vol *= rng[i]
    if not np.any(start) and np.all(rng == 1.0):
        return source
    if abi != L.ABI_NATIVE:
        raise ValueError("domain remapping needs the native integrand ABI")
    fmt = lambda v: ", ".join(repr(float(x)) for x in v)
    return (
        "#define integrand cvg_user_integrand\n" + source + "\n#undef integrand\n"
        "template <typename T> __device__ __forceinline__ T integrand(T* x) {\n"
        "    const double a[] = {%s};\n    const double r[] = {%s};\n"
        "#pragma unroll\n    for (int i = 0; i < cvg_n_dim; ++i) x[i] = x[i] * (T)r[i] + (T)a[i];\n"
        "    return cvg_user_integrand(x) * (T)%r;\n}\n" % (fmt(start), fmt(rng), vol))


def _is_ptx(obj):
    return isinstance(obj, str) and ".version" in obj and ".func" in obj


def _is_numba(obj):
    return type(obj).__module__.startswith("numba") and hasattr(obj, "py_func")


def _numba_ptx(fn, abi_name):
    """PTX of a numba device function f(x: float64*) -> float64 with numba's
    ABI under the given name (numba's abi_info option; the reference renames
    the function by editing the PTX text, python_wrapper.py:48-59)."""
    from numba import cuda, types
    sig = types.float64(types.CPointer(types.float64))
    ptx, _ = cuda.compile(fn.py_func, sig, device=True, abi="numba",
                          abi_info={"abi_name": abi_name}, output="ptx", cc=(10, 3))
    return ptx


def _ptx_domain_source(domain, n_dim, inner):
    """numba-ABI `integrand` that remaps [0,1]^d to `domain` and calls `inner`."""
    start = [float(domain[i][0]) for i in range(n_dim)]
    rng = [float(domain[i][1]) - float(domain[i][0]) for i in range(n_dim)]
    vol = float(np.prod(rng))
    fmt = lambda v: ", ".join(repr(x) for x in v)
    return ('extern "C" __device__ int %s(double* ret, double* x);\n'
            'extern "C" __device__ int integrand(double* ret, double* x) {\n'
            '    const double a[] = {%s};\n    const double r[] = {%s};\n'
            '    double y[cvg_n_dim];\n'
            '    for (int i = 0; i < cvg_n_dim; ++i) y[i] = x[i] * r[i] + a[i];\n'
            '    const int s = %s(ret, y);\n    *ret *= %r;\n    return s;\n}\n'
            % (inner, fmt(start), fmt(rng), inner, vol))


def _trivial_domain(domain, n_dim):
    return domain is None or all(float(domain[i][0]) == 0.0 and float(domain[i][1]) == 1.0
                                 for i in range(n_dim))


def _as_source(device_function):
    if isinstance(device_function, str):
        return device_function, L.ABI_NATIVE
    if isinstance(device_function, tuple) and len(device_function) == 2:
        return device_function[0], int(device_function[1])
    raise TypeError("device_function must be CUDA C++ source text defining `integrand`, "
                    "a numba CUDA device function, or numba-ABI PTX")


def integrate(device_function, n_dim, domain=None, n_evals=1000000, max_it=20, skip=5,
              batch_size=1048576, n_intervals=1024, n_strat=None, alpha=0.5, beta=0.75,
              seed=None, multi_gpu=None, multi_cpu=None, gpu_num=-1, cpu_num=-1, gpu_thr=0.1,
              precision="fp64", theta=None, n_params=0, graph=True, device=None):
    # seed (python_wrapper.py:11-13)
    if seed is None:
        seed = int.from_bytes(os.urandom(4), "big")
    # n_strat (python_wrapper.py:15-18)
    if n_strat is None:
        n_eval_it = n_evals // max_it
        n_strat = int(math.pow((n_eval_it / 4.0), 1.0 / n_dim))
    prec = {"fp64": L.PREC_FP64, "fp32": L.PREC_FP32}[precision]
    if theta is not None and not n_params:
        n_params = len(theta)
    ctx = runtime.default_context(device)
    if _is_numba(device_function) or _is_ptx(device_function):
        if prec != L.PREC_FP64:
            raise ValueError("numba integrands are FP64: precision must be 'fp64'")
        remap = not _trivial_domain(domain, n_dim)
        if _is_numba(device_function):
            inner = "cvg_numba_user" if remap else "integrand"
            ptx = _numba_ptx(device_function, inner)
        else:
            if remap:
                raise ValueError("a PTX `integrand` cannot be wrapped for domain remapping; "
                                 "compile it under another abi_name and pass a numba function")
            ptx = device_function
        f = ctx.integrand_ptx(ptx, n_dim, source=_ptx_domain_source(domain, n_dim, inner)
                              if remap else None)
    else:
        source, abi = _as_source(device_function)
        if domain is not None:
            source = _domain_source(source, domain, n_dim, abi)
        f = ctx.integrand(source, n_dim, n_params=n_params, abi=abi)
    p = runtime.make_params(n_dim, n_evals, max_it, skip=skip, n_intervals=n_intervals,
                            n_strat=n_strat, alpha=alpha, beta=beta, seed=seed, precision=prec,
                            flags=L.FLAG_GRAPH if graph else 0, max_batch_size=batch_size,
                            gpu_thr=gpu_thr)
    res, it_res, it_sig = runtime.integrate_once(f, p, theta)
    info = {
        "error": res.error, "n_strat": res.n_strat, "n_cubes": res.n_cubes,
        "n_intervals": res.n_intervals, "tot_nevals": res.tot_nevals,
        "tot_time": res.tot_time_ms, "avg_it_time": res.avg_it_time_ms, "seed": seed,
        "multi_gpu": False, "multi_cpu": False, "gpu_num": 1, "omp_threads_num": 0,
        "gpu_thr": gpu_thr, "chi2_dof": res.chi2_dof, "precision": precision,
        "it_res": it_res, "it_sigma": np.sqrt(np.abs(it_sig)),
    }
    return res.result, info
