"""Tile-shape autotuner for the fill kernels.

The fill's free parameters are the CTA size (``block``) and the number of
consecutive samples each thread owns (``spt``); a tile is block*spt samples.
The tuner times one fill launch (CUDA events on the run's stream) for each
candidate on the live workload, after one untimed iteration, and keeps the
fastest.  Winners are cached in a JSON file keyed by GPU, dimension set,
precision, bins and the evaluations per iteration (rounded to a power of 2),
so a workload is tuned once per machine.
"""
import hashlib
import json
import math
import os
import threading

from . import _lib as L
from . import runtime

CANDIDATES = [(256, 16), (512, 8), (512, 12), (512, 16), (1024, 4), (1024, 8)]
# single runs of large iterations run warp tiles (32 * spt samples per warp),
# where larger tiles and 1024-thread blocks measured faster
RUN_CANDIDATES = CANDIDATES + [(512, 24), (512, 32), (1024, 16), (1024, 24), (1024, 32)]
# batched fills run warp tiles too; their largest dimension's variant holds
# the kernel's registers, so 512- and 768-thread blocks stay in the set
BATCH_CANDIDATES = [(512, 16), (512, 32), (768, 32), (1024, 16), (1024, 32)]
_lock = threading.Lock()


def cache_path():
    base = os.environ.get("CVG_CACHE_DIR") or os.path.join(
        os.environ.get("HOME") or "/tmp", ".cache", "cuvegas_gb300")
    os.makedirs(base, exist_ok=True)
    return os.path.join(base, "autotune.json")


def _gpu_name():
    try:
        import torch
        if torch.cuda.is_available():
            return torch.cuda.get_device_name(0)
    except Exception:
        pass
    return "gpu"


def _load():
    try:
        with open(cache_path()) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def _store(key, value):
    with _lock:
        data = _load()
        data[key] = value
        tmp = cache_path() + ".tmp%d" % os.getpid()
        with open(tmp, "w") as f:
            json.dump(data, f, indent=1, sort_keys=True)
        os.replace(tmp, cache_path())


def _key(kind, dims, prec, n_intervals, evals, source):
    h = hashlib.sha1(source.encode()).hexdigest()[:12]
    return "%s|%s|%s|d%s|p%d|N%d|e2^%d" % (kind, _gpu_name(), h, ",".join(map(str, sorted(dims))),
                                          prec, n_intervals, int(math.log2(max(evals, 1))))


def tune_run(integrand, params, theta=None, candidates=RUN_CANDIDATES):
    """Best (block, spt) for a single-instance run of these parameters."""
    key = _key("run", [params.n_dim], params.precision, params.n_intervals,
               params.tot_eval // params.max_it, integrand_source(integrand))
    hit = _load().get(key)
    if hit:
        return tuple(hit)
    best, best_ms = None, float("inf")
    for block, spt in candidates:
        p = runtime.make_params(params.n_dim, params.tot_eval, params.max_it, skip=params.skip,
                                n_intervals=params.n_intervals, seed=params.seed,
                                precision=params.precision, flags=L.FLAG_TIME_FILL,
                                block=block, spt=spt)
        try:
            with runtime.Run(integrand, p, theta) as r:
                r.iterate(min(2, params.max_it))
                ms = r.fill_times()[-1]
        except L.CuvegasError:
            continue
        if ms < best_ms:
            best, best_ms = (block, spt), ms
    if best is None:
        best = (512, 8)
    _store(key, list(best))
    return best


def integrand_source(integrand):
    return getattr(integrand, "source", "") or str(id(integrand))


def tune_batch(ctx, source, instances, params_per_dim, precision, n_intervals=1024,
               candidates=BATCH_CANDIDATES):
    """Best (block, spt) for a batch: per candidate, the batched fills of
    iterations 1-3 (after the first adaptation; the fill times differ most
    between candidates in these early iterations)."""
    from .batch import Batch
    dims = sorted({int(i["dim"]) for i in instances})
    evals = sum(int(i.get("n_eval_it", 0)) for i in instances)
    key = _key("batchwt3_%d" % len(instances), dims, precision, n_intervals, evals, source)
    hit = _load().get(key)
    if hit:
        return tuple(hit)
    best, best_ms = None, float("inf")
    for block, spt in candidates:
        try:
            with Batch(ctx, source, instances, params_per_dim, max_it=4, skip=0,
                       n_intervals=n_intervals, precision=precision, graph=False, block=block,
                       spt=spt) as b:
                b.iterate(1)            # iteration 0: uniform grid, not timed
                ms = 0.0
                for _ in range(3):      # each eager iteration times its own fill
                    b.iterate(1)
                    ms += _batch_fill_ms(b)
        except L.CuvegasError:
            continue
        if ms < best_ms:
            best, best_ms = (block, spt), ms
    if best is None:
        best = (512, 8)
    _store(key, list(best))
    return best


def _batch_fill_ms(b):
    import ctypes as C
    ms = C.c_float()
    L.check(b._lib.cvg_batch_last_fill_ms(b.handle, C.byref(ms)))
    return ms.value
