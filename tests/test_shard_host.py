"""Host logic of the sample split across ranks (cuvegas_gb300.shard), on CPU
with two gloo ranks: a stand-in run whose "fill" writes rank-dependent sums.
After each fill the ranks must hold the sums over both ranks (per-cube,
per-bin values and counts, and the FP32 form's rare-update count, but not the
histogram-form flag), and every iteration must be fill, all-reduce, then
reallocation + refinement."""
import os
import socket

import numpy as np
import pytest

from cuvegas_gb300 import _lib as L


class FakeRun:
    """Buffers of a run, as numpy arrays; steps record their order."""

    def __init__(self, rank, prec):
        self.rank = rank
        self.params = type("P", (), {"precision": prec})()
        self.buf = {L.BUF_JF: np.zeros(7), L.BUF_JF2: np.zeros(7),
                    L.BUF_WEIGHTS: np.zeros((2, 5)), L.BUF_COUNTS: np.zeros((2, 5), np.uint32),
                    L.BUF_HIST_STATE: np.array([1, 0], np.uint32)}
        self.steps = []
        self.shard = None

    def set_shard(self, s, w):
        self.shard = (s, w)

    def step(self, stages):
        self.steps.append(stages)
        if stages == L.STAGE_FILL:
            k = self.rank + 1
            self.buf[L.BUF_JF][:] = k * np.arange(7) + 0.25
            self.buf[L.BUF_JF2][:] = k * 1e-300 + np.arange(7)   # tiny values survive
            self.buf[L.BUF_WEIGHTS][:] = k * 0.5
            self.buf[L.BUF_COUNTS][:] = k * 3
            self.buf[L.BUF_HIST_STATE][1] = 10 * k

    def get(self, b):
        return self.buf[b].copy()

    def set(self, b, a):
        self.buf[b][...] = np.asarray(a).reshape(self.buf[b].shape)


def _rank(rank, world, port, out, prec):
    import torch.distributed as dist
    from cuvegas_gb300 import shard
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        fr = FakeRun(rank, prec)
        sr = shard.ShardedRun(None, None, run=fr)
        assert sr.reduce is shard.allreduce_host and fr.shard == (rank, world)
        sr.iterate(2)
        np.savez(os.path.join(out, "r%d.npz" % rank), steps=np.array(fr.steps),
                 **{"b%d" % k: v for k, v in fr.buf.items()})
    finally:
        dist.destroy_process_group()


@pytest.mark.parametrize("prec", [L.PREC_FP64, L.PREC_FP32])
def test_two_ranks_hold_the_summed_fill(tmp_path, prec):
    import torch.multiprocessing as mp
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    mp.spawn(_rank, args=(2, port, str(tmp_path), prec), nprocs=2, join=True)
    z = [np.load(os.path.join(tmp_path, "r%d.npz" % k)) for k in range(2)]
    for k, r in enumerate(z):
        assert list(r["steps"]) == [L.STAGE_FILL, L.STAGE_REALLOC | L.STAGE_REFINE] * 2
        np.testing.assert_array_equal(r["b%d" % L.BUF_JF], 3 * np.arange(7) + 0.5)
        np.testing.assert_array_equal(r["b%d" % L.BUF_JF2], 2 * np.arange(7) + 3e-300)
        np.testing.assert_array_equal(r["b%d" % L.BUF_WEIGHTS], np.full((2, 5), 1.5))
        np.testing.assert_array_equal(r["b%d" % L.BUF_COUNTS], np.full((2, 5), 9))
        hs = r["b%d" % L.BUF_HIST_STATE]
        assert hs[0] == 1                                   # the form flag is not summed
        # summed in the FP32 form; FP64 runs have no such count and keep their own
        assert hs[1] == (30 if prec == L.PREC_FP32 else 10 * (k + 1))
