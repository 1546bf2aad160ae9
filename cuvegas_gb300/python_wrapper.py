"""Python entry point with the reference's call signature.

Mirrors ``integrate`` of vegas_cuda/src/vegas_cuda_extension/python_wrapper.py:9-77:
same keyword arguments with the same meanings and defaults, same result tuple
``(result, dict)`` with the same keys, plus ``chi2_dof``, ``precision``,
``it_res`` and ``it_sigma``.

Differences, by design:
  * ``device_function`` is CUDA C++ source defining ``integrand`` (compiled by
    NVRTC inside libcuvegas), or a numba CUDA device function when numba is
    installed (it must then be given as source: numba's PTX is not linked);
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


def _as_source(device_function):
    if isinstance(device_function, str):
        return device_function, L.ABI_NATIVE
    if isinstance(device_function, tuple) and len(device_function) == 2:
        return device_function[0], int(device_function[1])
    raise TypeError("device_function must be CUDA C++ source text defining `integrand` "
                    "(numba device functions are not linked by this build)")


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
    source, abi = _as_source(device_function)
    if domain is not None:
        source = _domain_source(source, domain, n_dim, abi)
    prec = {"fp64": L.PREC_FP64, "fp32": L.PREC_FP32}[precision]
    if theta is not None and not n_params:
        n_params = len(theta)
    ctx = runtime.default_context(device)
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
