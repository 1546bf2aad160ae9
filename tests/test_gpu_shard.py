"""Sample split of one integral across ranks (the reference's multi-GPU
iteration, src/main.cu:591-654), on the one GPU this test has.

1. In one process: `world` runs of the same integral, each filling its range
   of tiles (cvg_run_set_shard), their sums added on the host and written
   back to every run, against one run that fills everything.  FP64 form,
   every iteration: bin counts exact, per-cube and per-bin sums to 1e-12,
   identical allocation, grid to 1e-12, results to 1e-12; the ranks' grids
   are identical to each other.  FP32 form: the first fill's counts exact,
   per-cube sums 1e-12, bin sums 1e-6 (the first fills keep float bin sums,
   whose rounding depends on the order of the adds), and the ranks identical
   to each other at every iteration.
2. Two processes with a gloo group, both on this GPU, through ShardedRun
   (host-copy all-reduce): the same result as one process.  No kernel of one
   process waits on the other; the exchange is on the host.
"""
import os
import socket

import numpy as np
import pytest

from cuvegas_gb300 import _lib as L, integrands as I, runtime

pytestmark = pytest.mark.gpu

SUMS = (L.BUF_JF, L.BUF_JF2, L.BUF_WEIGHTS, L.BUF_COUNTS)


def _add(parts, buf):
    vals = [r.get(buf) for r in parts]
    dt = vals[0].dtype
    acc = sum(v.astype(np.float64 if dt == np.float64 else np.int64) for v in vals)
    return acc.astype(dt)


@pytest.mark.parametrize("world", [2, 3])
@pytest.mark.parametrize("prec", [L.PREC_FP64, L.PREC_FP32])
def test_split_fills_add_up_to_the_one_rank_fill(ctx, prec, world):
    dim, n_it, N, iters = 5, 600_000, 128, 4
    f = ctx.integrand(I.GAUSS, dim)
    p = runtime.make_params(dim, n_it * iters, iters, skip=1, n_intervals=N, seed=11,
                            precision=prec)
    one = runtime.Run(f, p)
    parts = [runtime.Run(f, p) for _ in range(world)]
    try:
        for s, r in enumerate(parts):
            r.set_shard(s, world)
        assert one.info.next_samples // one.info.tile_samples >= 4 * world
        for it in range(iters):
            one.step(L.STAGE_FILL)
            for r in parts:
                r.step(L.STAGE_FILL)
            sums = {b: _add(parts, b) for b in SUMS}
            # each range is a proper part: no rank filled everything
            assert all(r.get(L.BUF_COUNTS).sum() < sums[L.BUF_COUNTS].sum() for r in parts)
            if prec == L.PREC_FP64 or it == 0:
                assert np.array_equal(sums[L.BUF_COUNTS], one.get(L.BUF_COUNTS))
                np.testing.assert_allclose(sums[L.BUF_JF], one.get(L.BUF_JF), rtol=1e-12, atol=0)
                np.testing.assert_allclose(sums[L.BUF_JF2], one.get(L.BUF_JF2), rtol=1e-12, atol=0)
                np.testing.assert_allclose(sums[L.BUF_WEIGHTS], one.get(L.BUF_WEIGHTS),
                                           rtol=1e-12 if prec == L.PREC_FP64 else 1e-6, atol=0)
            hs = None
            if prec == L.PREC_FP32:
                hs = parts[0].get(L.BUF_HIST_STATE)
                hs[1] = sum(int(r.get(L.BUF_HIST_STATE)[1]) for r in parts)
            for r in parts:
                for b in SUMS:
                    r.set(b, sums[b])
                if hs is not None:
                    r.set(L.BUF_HIST_STATE, hs)
            one.step(L.STAGE_REALLOC | L.STAGE_REFINE)
            for r in parts:
                r.step(L.STAGE_REALLOC | L.STAGE_REFINE)
            xe = [r.get(L.BUF_X_EDGES) for r in parts]
            nh = [r.get(L.BUF_NH) for r in parts]
            for k in range(1, world):     # every rank holds the same state
                assert np.array_equal(xe[k], xe[0]) and np.array_equal(nh[k], nh[0])
            if prec == L.PREC_FP64:
                assert np.array_equal(nh[0], one.get(L.BUF_NH))
                np.testing.assert_allclose(xe[0], one.get(L.BUF_X_EDGES), rtol=1e-12, atol=1e-15)
        res = [r.result() for r in parts]
        ro = one.result()
        for k in range(1, world):
            assert res[k][0].result == res[0][0].result
        if prec == L.PREC_FP64:
            assert res[0][0].tot_nevals == ro[0].tot_nevals
            np.testing.assert_allclose(res[0][1], ro[1], rtol=1e-12)
            assert abs(res[0][0].result - ro[0].result) <= 1e-12 * abs(ro[0].result)
        else:
            assert abs(res[0][0].result - ro[0].result) < 3 * ro[0].error
    finally:
        one.close()
        for r in parts:
            r.close()


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out_dir, prec):
    import torch.distributed as dist
    from cuvegas_gb300 import shard
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        ctx = runtime.Context(0)
        f = ctx.integrand(I.GAUSS, 4)
        p = runtime.make_params(4, 800_000 * 5, 5, skip=1, n_intervals=256, seed=5,
                                precision=prec)
        with shard.ShardedRun(f, p) as sr:
            assert sr.reduce is shard.allreduce_host
            sr.iterate(5)
            res, it_res, it_sig = sr.result()
            xe = sr.get(L.BUF_X_EDGES)
        np.savez(os.path.join(out_dir, "rank%d.npz" % rank), it_res=it_res, it_sig=it_sig,
                 xe=xe, result=res.result, tot=res.tot_nevals)
        ctx.close()
    finally:
        dist.destroy_process_group()


@pytest.mark.parametrize("prec", [L.PREC_FP64, L.PREC_FP32])
def test_two_gloo_ranks_equal_one_process(ctx, tmp_path, prec):
    import torch.multiprocessing as mp
    mp.spawn(_rank_main, args=(2, _free_port(), str(tmp_path), prec), nprocs=2, join=True)
    z = [np.load(os.path.join(tmp_path, "rank%d.npz" % k)) for k in range(2)]
    assert np.array_equal(z[0]["xe"], z[1]["xe"]) and z[0]["result"] == z[1]["result"]
    f = ctx.integrand(I.GAUSS, 4)
    p = runtime.make_params(4, 800_000 * 5, 5, skip=1, n_intervals=256, seed=5, precision=prec)
    with runtime.Run(f, p) as r:
        r.iterate(5)
        res, it_res, _ = r.result()
    if prec == L.PREC_FP64:
        assert int(z[0]["tot"]) == res.tot_nevals
        np.testing.assert_allclose(z[0]["it_res"], it_res, rtol=1e-12)
    else:
        assert abs(float(z[0]["result"]) - res.result) < 3 * res.error
