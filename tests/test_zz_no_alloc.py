"""cvg_realloc_noalloc, the allocation-free reallocation step, against the
library's own reallocation step.

Some callers cannot call cudaMalloc: code running inside another framework's
memory pool or allocator, or a process that reserved all device memory up
front.  cvg_realloc_noalloc gives them the hypercube reallocation with every
temporary in a static device array, so they only pass their own inputs and
outputs.  Its results must equal cvg_run_step(CVG_STAGE_REALLOC) on the same
inputs, on two calls in a row (the shared array keeps the previous call's
contents, which must not leak into the next), its tile map must equal the
loop's, device memory must not change across a call, sums of any magnitude
must be taken in the FP32 form, and a non-finite estimate must come back as
CVG_ERR_KERNEL.  This file is collected last.
"""
import ctypes as C

import numpy as np
import pytest

from cuvegas_gb300 import _lib as L, integrands as I, runtime
from oracle import pyoracle as P

pytestmark = pytest.mark.gpu


def _call(lib, torch, JF, JF2, nh_sum, info, prec, est, tile_cube=None, n_eval_it=None):
    stream = torch.cuda.current_stream(JF.device)
    return lib.cvg_realloc_noalloc(
        C.c_void_p(JF.data_ptr()), C.c_void_p(JF2.data_ptr()), C.c_void_p(nh_sum.data_ptr()),
        C.c_uint32(info.n_cubes), C.c_double(info.v_cubes), C.c_double(0.75),
        C.c_int64(info.n_eval_it if n_eval_it is None else n_eval_it), C.c_int32(prec),
        C.c_void_p(est.data_ptr()),
        C.c_void_p(tile_cube.data_ptr()) if tile_cube is not None else None,
        C.c_uint64(tile_cube.numel() if tile_cube is not None else 0),
        C.c_int32(info.tile_samples if tile_cube is not None else 0),
        C.c_void_p(stream.cuda_stream))


def _loop_step(ctx, prec, dim=4, n_it=200000, N=64, seed=21):
    """The loop's own reallocation of the oracle's per-cube sums."""
    o = P.OracleRun(dim, n_it * 4, 4, n_intervals=N)
    u, _ = P.uniforms(P.U_PHILOX_F64, seed=seed)
    o.fill(P.F_GAUSS, np.array([0.5, 0.1]), u, it=0)
    f = ctx.integrand(I.GAUSS, dim)
    p = runtime.make_params(dim, n_it * 4, 4, n_intervals=N, seed=seed, precision=prec)
    with runtime.Run(f, p) as r:
        info = r.info
        assert info.n_cubes <= L.NOALLOC_MAX_CUBES
        nh_sum0 = r.get(L.BUF_NH_SUM)
        # the loop's FP32 form carries its own scale; start it where the
        # entry point's device-side rule puts it for these sums
        if prec == L.PREC_FP32:
            ms = o.JF2.sum() / float(nh_sum0[-1])
            k = int(np.frexp(ms)[1] / 2) if ms > 0 else 0      # C's e / 2 truncates
            r.set(L.BUF_SCALE_EXP, np.array([max(-100, min(100, k))], dtype=np.int32))
        r.set(L.BUF_JF, o.JF)
        r.set(L.BUF_JF2, o.JF2)
        r.step(L.STAGE_REALLOC)
        want = {"nh_sum": r.get(L.BUF_NH_SUM), "est": r.get(L.BUF_STATS)[:, 0],
                "tiles": r.get(L.BUF_TILE_CUBE)}
    return o, info, nh_sum0, want


def _tensors(torch, o, nh_sum0, scale=1.0):
    dev = torch.device("cuda", 0)
    JF = torch.tensor(o.JF * scale, dtype=torch.float64, device=dev)
    JF2 = torch.tensor(o.JF2 * scale * scale, dtype=torch.float64, device=dev)
    nh_sum = torch.tensor(nh_sum0.view(np.int64), dtype=torch.int64, device=dev)
    est = torch.full((3,), -1.0, dtype=torch.float64, device=dev)
    return JF, JF2, nh_sum, est


@pytest.mark.parametrize("prec", [L.PREC_FP64, L.PREC_FP32])
def test_noalloc_matches_run_step_twice(ctx, prec):
    torch = pytest.importorskip("torch")
    o, info, nh_sum0, want = _loop_step(ctx, prec)
    lib = L.load()
    dev = torch.device("cuda", 0)
    n_tiles = int(-(-int(want["nh_sum"][-1]) // info.tile_samples))
    for _ in range(2):
        JF, JF2, nh_sum, est = _tensors(torch, o, nh_sum0)
        tiles = torch.full((info.max_tiles,), -1, dtype=torch.int32, device=dev)
        assert _call(lib, torch, JF, JF2, nh_sum, info, prec, est, tiles) == L.OK, L.last_error()
        torch.cuda.synchronize()
        got = nh_sum.cpu().numpy().view(np.uint64)
        assert np.array_equal(got, want["nh_sum"])
        np.testing.assert_allclose(est.cpu().numpy(), want["est"], rtol=1e-12)
        assert not JF.any().item() and not JF2.any().item()   # consumed, as in the loop
        # tile map of the next fill: the cube of each tile's first sample
        t = tiles.cpu().numpy().view(np.uint32)
        assert np.array_equal(t[:n_tiles], want["tiles"][:n_tiles])


def test_noalloc_allocates_nothing(ctx):
    """After a first call (which looks up the static array and may load the
    module holding it), a call leaves the device's free memory unchanged."""
    torch = pytest.importorskip("torch")
    o, info, nh_sum0, _ = _loop_step(ctx, L.PREC_FP32)
    lib = L.load()
    bufs = [_tensors(torch, o, nh_sum0) for _ in range(2)]
    assert _call(lib, torch, *bufs[0][:3], info, L.PREC_FP32, bufs[0][3]) == L.OK
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info(0)[0]
    assert _call(lib, torch, *bufs[1][:3], info, L.PREC_FP32, bufs[1][3]) == L.OK
    torch.cuda.synchronize()
    assert torch.cuda.mem_get_info(0)[0] == free0


@pytest.mark.parametrize("scale", [2.0 ** -83, 2.0 ** 83, 1e-25, 1e25])
def test_noalloc_fp32_takes_sums_of_any_magnitude(ctx, scale):
    """The integrand scaled by 2^-83, 2^83, 1e-25 or 1e25: the FP32 form scales
    its float splits by a power of two worked out from JF2 on the device, so
    with a power-of-two factor the results are the unscaled ones times the
    factor exactly, and with 1e+-25 the estimate matches the FP64 form to
    1e-10 and the allocation to one sample (+1e-5 relative) per hypercube."""
    torch = pytest.importorskip("torch")
    o, info, nh_sum0, _ = _loop_step(ctx, L.PREC_FP64)
    lib = L.load()

    def run(prec, s):
        JF, JF2, nh_sum, est = _tensors(torch, o, nh_sum0, s)
        assert _call(lib, torch, JF, JF2, nh_sum, info, prec, est) == L.OK, L.last_error()
        torch.cuda.synchronize()
        return nh_sum.cpu().numpy().view(np.uint64).astype(np.int64), est.cpu().numpy()

    ps, es = run(L.PREC_FP32, scale)
    if np.log2(scale) == int(np.log2(scale)):
        p1, e1 = run(L.PREC_FP32, 1.0)
        assert np.array_equal(ps, p1)
        assert es[0] == e1[0] * scale and es[1] == e1[1] * scale * scale and es[2] == e1[2]
    else:
        p64, e64 = run(L.PREC_FP64, scale)
        assert abs(es[0] - e64[0]) <= 1e-10 * abs(e64[0])
        assert abs(es[1] - e64[1]) <= 1e-6 * abs(e64[1])
        n32, n64 = np.diff(ps), np.diff(p64)
        assert np.all(np.abs(n32 - n64) <= 1 + 1e-5 * n64)


def test_noalloc_reports_a_non_finite_estimate(ctx):
    """A non-finite per-cube sum makes the iteration estimate non-finite: the
    kernels set their status bit and the call returns CVG_ERR_KERNEL."""
    torch = pytest.importorskip("torch")
    o, info, nh_sum0, _ = _loop_step(ctx, L.PREC_FP64)
    lib = L.load()
    for prec in (L.PREC_FP64, L.PREC_FP32):
        JF, JF2, nh_sum, est = _tensors(torch, o, nh_sum0)
        JF[5] = float("inf")
        JF2[5] = float("inf")
        assert _call(lib, torch, JF, JF2, nh_sum, info, prec, est) == L.ERR_KERNEL
        assert "not finite" in L.last_error()
    # the next call with finite sums is valid again (the status was cleared)
    JF, JF2, nh_sum, est = _tensors(torch, o, nh_sum0)
    assert _call(lib, torch, JF, JF2, nh_sum, info, L.PREC_FP64, est) == L.OK


def test_noalloc_rejects_sizes_beyond_its_array(ctx):
    torch = pytest.importorskip("torch")
    dev = torch.device("cuda", 0)
    x = torch.zeros(4, dtype=torch.float64, device=dev)
    n = L.NOALLOC_MAX_CUBES + 1
    lib = L.load()
    st = lib.cvg_realloc_noalloc(C.c_void_p(x.data_ptr()), C.c_void_p(x.data_ptr()),
                                 C.c_void_p(x.data_ptr()), C.c_uint32(n), C.c_double(1.0),
                                 C.c_double(0.75), C.c_int64(100), C.c_int32(0),
                                 C.c_void_p(x.data_ptr()), None, C.c_uint64(0), C.c_int32(0), None)
    assert st == L.ERR_INVALID
    assert "preallocated" in L.last_error()
    for n_eval_it in (0, -5, 2 ** 31):
        st = lib.cvg_realloc_noalloc(C.c_void_p(x.data_ptr()), C.c_void_p(x.data_ptr()),
                                     C.c_void_p(x.data_ptr()), C.c_uint32(4), C.c_double(1.0),
                                     C.c_double(0.75), C.c_int64(n_eval_it), C.c_int32(0),
                                     C.c_void_p(x.data_ptr()), None, C.c_uint64(0), C.c_int32(0),
                                     None)
        assert st == L.ERR_INVALID
        assert "n_eval_it" in L.last_error()
