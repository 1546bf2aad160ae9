"""Replicas across GPUs: one process per GPU, each running an independent
VEGAS+ integration of the same integral.

The reference spreads one integration over several GPUs and sums the
per-hypercube and per-bin accumulators over them every iteration
(src/main.cu:591-654, peer copies plus sumVals).  Here every rank runs the
whole loop on its own GPU with its own Philox stream (counter word 3 carries
the instance id, so replicas never share a sample); there is no exchange
inside the loop.  Ranks meet only to combine what they produced:

  * ``reduce_timing``: slowest rank's time and total evaluations (the bench's
    whole-job throughput = total evaluations / max time);
  * ``combine``: the replicas' estimates merged by inverse-variance weights,
    the same rule the loop itself applies to its iterations
    (src/main.cu:698-713).

Any ``torch.distributed`` backend works (nccl on GPUs, gloo on CPU).
"""
import math

import numpy as np


def instance_id(rank, base=0):
    """Philox instance id of a rank's replica (24 bits: counter word 3, bits 8..31)."""
    inst = int(base) + int(rank)
    if not 0 <= inst < (1 << 24):
        raise ValueError("instance id %d out of range [0, 2^24)" % inst)
    return inst


def _dist():
    try:
        import torch.distributed as dist
    except ImportError:
        return None
    if dist.is_available() and dist.is_initialized() and dist.get_world_size() > 1:
        return dist
    return None


def reduce_timing(ms, evals, device="cpu"):
    """(max over ranks of ms, sum over ranks of evals); identity on one rank."""
    dist = _dist()
    if dist is None:
        return float(ms), float(evals)
    import torch
    mx = torch.tensor([float(ms)], dtype=torch.float64, device=device)
    tot = torch.tensor([float(evals)], dtype=torch.float64, device=device)
    dist.all_reduce(mx, op=dist.ReduceOp.MAX)
    dist.all_reduce(tot, op=dist.ReduceOp.SUM)
    return float(mx[0]), float(tot[0])


def combine_local(results, errors):
    """Inverse-variance mean of independent estimates: (mean, error, chi2/dof).
    Estimates with a non-positive or non-finite error are left out."""
    r = np.asarray(results, dtype=np.float64)
    e = np.asarray(errors, dtype=np.float64)
    ok = np.isfinite(r) & np.isfinite(e) & (e > 0)
    if not ok.any():
        raise ValueError("no estimate with a positive finite error")
    r, e = r[ok], e[ok]
    w = 1.0 / (e * e)
    mean = float((w * r).sum() / w.sum())
    err = float(1.0 / math.sqrt(w.sum()))
    chi2 = float((w * (r - mean) ** 2).sum() / (len(r) - 1)) if len(r) > 1 else 0.0
    return mean, err, chi2


def combine(result, error, device="cpu"):
    """All ranks' (result, error) gathered and merged; every rank gets the same
    (mean, error, chi2/dof, per-rank results, per-rank errors)."""
    dist = _dist()
    if dist is None:
        m, e, c = combine_local([result], [error])
        return m, e, c, np.array([result]), np.array([error])
    import torch
    world = dist.get_world_size()
    mine = torch.tensor([float(result), float(error)], dtype=torch.float64, device=device)
    allv = [torch.zeros(2, dtype=torch.float64, device=device) for _ in range(world)]
    dist.all_gather(allv, mine)
    rs = np.array([float(t[0]) for t in allv])
    es = np.array([float(t[1]) for t in allv])
    m, e, c = combine_local(rs, es)
    return m, e, c, rs, es
