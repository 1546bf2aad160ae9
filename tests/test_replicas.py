"""Replica path across ranks, on CPU with the gloo backend (world size 2):
timing reduction, the inverse-variance merge of the replicas' estimates and
the Philox instance ids that keep replicas' samples apart."""
import math
import os
import socket

import numpy as np
import pytest
import torch.multiprocessing as mp

from cuvegas_gb300 import replicas


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        ms, ev = replicas.reduce_timing(10.0 + rank, 1e6 * (rank + 1))
        res = [1.0, 1.3][rank]
        err = [0.1, 0.2][rank]
        m, e, c, rs, es = replicas.combine(res, err)
        out[rank] = (ms, ev, m, e, c, list(rs), list(es), replicas.instance_id(rank, base=7))
    finally:
        dist.destroy_process_group()


def test_two_rank_replicas_gloo():
    world = 2
    port = _free_port()
    with mp.Manager() as mgr:
        out = mgr.dict()
        mp.spawn(_worker, args=(world, port, out), nprocs=world, join=True)
        res = dict(out)
    w = np.array([1 / 0.01, 1 / 0.04])
    mean = (w * np.array([1.0, 1.3])).sum() / w.sum()
    for rank in range(world):
        ms, ev, m, e, c, rs, es, inst = res[rank]
        assert ms == 11.0 and ev == 3e6            # slowest rank, total evaluations
        assert rs == [1.0, 1.3] and es == [0.1, 0.2]
        assert m == pytest.approx(mean, rel=1e-15)
        assert e == pytest.approx(1 / math.sqrt(w.sum()), rel=1e-15)
        assert c == pytest.approx((w * (np.array([1.0, 1.3]) - mean) ** 2).sum(), rel=1e-12)
        assert inst == 7 + rank


def test_single_rank_is_identity():
    assert replicas.reduce_timing(3.0, 5.0) == (3.0, 5.0)
    m, e, c, _, _ = replicas.combine(2.0, 0.5)
    assert (m, e, c) == (2.0, 0.5, 0.0)


def test_combine_skips_unusable_estimates():
    m, e, _ = replicas.combine_local([1.0, float("nan"), 3.0], [1.0, 1.0, 0.0])
    assert (m, e) == (1.0, 1.0)
    with pytest.raises(ValueError):
        replicas.combine_local([1.0], [0.0])
    with pytest.raises(ValueError):
        replicas.instance_id(1 << 24)
