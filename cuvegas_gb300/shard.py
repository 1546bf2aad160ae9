"""Sample split of one integral across ranks: the reference's multi-GPU mode.

The reference splits each iteration's samples over the GPUs of one process
(src/main.cu:591-628), adds the per-hypercube sums JF/JF2 and the per-bin
weights and counts of all GPUs (src/main.cu:636-654; the Python extension in
vegas_cuda/src/vegas_cuda_extension/cuda_wrapper.cu:646-706), refines the grid
on GPU 0 and copies it to the others (src/main.cu:531-541).

Here one process drives one GPU (torch.distributed ranks).  Every rank creates
the same run (same parameters, seed and instance) and fills a contiguous range
of the iteration's tiles (cvg_run_set_shard); the Philox counter names each
sample by (sample-in-cube, cube, iteration), so the ranks' fills together are
exactly the one-rank fill.  The four sums (and, in the FP32 form, the count
of rare histogram updates) are all-reduced; every rank then runs the same
reallocation and refinement, which are deterministic, so all ranks hold the
same grid and allocation without a broadcast.

Collectives: NCCL all-reduces the run's own device buffers in place
(cvg_run_buffer); any other backend (gloo) goes through host copies.
"""
import numpy as np

from . import _lib as L
from . import runtime

# buffers summed across ranks after each fill: (buffer, element type)
SUM_BUFFERS = ((L.BUF_JF, "<f8"), (L.BUF_JF2, "<f8"), (L.BUF_WEIGHTS, "<f8"),
               (L.BUF_COUNTS, "<i4"))


class _DeviceView:
    """A run's device buffer as a CUDA array (zero copy)."""

    def __init__(self, ptr, n, typestr):
        self.__cuda_array_interface__ = {"shape": (n,), "typestr": typestr,
                                         "data": (ptr, False), "version": 2, "strides": None}


def device_tensor(run, buf, typestr, first=0, count=None):
    """torch tensor over elements [first, first+count) of one of the run's
    device buffers (u32 counts are summed as int32: a bin holds < 2^31)."""
    import torch
    ptr, nbytes = run.buffer(buf)
    item = np.dtype(typestr).itemsize
    n = nbytes // item - first if count is None else count
    return torch.as_tensor(_DeviceView(ptr + first * item, n, typestr), device="cuda")


def allreduce_device(run, group=None):
    """Sum the fill's outputs over the ranks, in place on the device (NCCL)."""
    import torch
    import torch.distributed as dist
    run.sync()                                  # the fill has finished on the run's stream
    for buf, ts in SUM_BUFFERS:
        dist.all_reduce(device_tensor(run, buf, ts), group=group)
    if run.params.precision == L.PREC_FP32:
        dist.all_reduce(device_tensor(run, L.BUF_HIST_STATE, "<i4", first=1, count=1), group=group)
    torch.cuda.current_stream().synchronize()   # before the run's stream reads the sums


def allreduce_host(run, group=None):
    """Sum the fill's outputs over the ranks through host copies (any backend)."""
    import torch
    import torch.distributed as dist
    for buf, ts in SUM_BUFFERS:
        a = run.get(buf)
        t = torch.from_numpy(np.ascontiguousarray(a, dtype=np.float64 if ts == "<f8" else np.int64))
        dist.all_reduce(t, group=group)
        run.set(buf, t.numpy().astype(a.dtype))
    if run.params.precision == L.PREC_FP32:
        hs = run.get(L.BUF_HIST_STATE)
        t = torch.tensor([int(hs[1])], dtype=torch.int64)
        dist.all_reduce(t, group=group)
        hs[1] = int(t.item())
        run.set(L.BUF_HIST_STATE, hs)


class ShardedRun:
    """One integral whose samples are split across the ranks of a process
    group.  Each rank calls iterate() with the same arguments; results,
    grids and allocations come out identical on every rank."""

    def __init__(self, integrand, params, theta=None, rank=None, world=None, group=None,
                 device_collectives=None, run=None):
        import torch.distributed as dist
        if rank is None or world is None:
            rank, world = dist.get_rank(group), dist.get_world_size(group)
        self.rank, self.world, self.group = int(rank), int(world), group
        self.run = run if run is not None else runtime.Run(integrand, params, theta)
        self.params = self.run.params
        self.run.set_shard(self.rank, self.world)
        if device_collectives is None:
            device_collectives = self.world > 1 and dist.get_backend(group) == "nccl"
        self.reduce = allreduce_device if device_collectives else allreduce_host

    def iterate(self, n):
        for _ in range(int(n)):
            self.run.step(L.STAGE_FILL)
            if self.world > 1:
                self.reduce(self.run, self.group)
            self.run.step(L.STAGE_REALLOC | L.STAGE_REFINE)

    def result(self):
        return self.run.result()

    def get(self, buf):
        return self.run.get(buf)

    def sync(self):
        self.run.sync()

    @property
    def info(self):
        return self.run.info

    def close(self):
        self.run.close()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()
