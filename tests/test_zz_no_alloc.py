"""cvg_realloc_noalloc, the allocation-free reallocation step, against the
library's own reallocation step.

Some callers cannot call cudaMalloc: code running inside another framework's
memory pool or allocator, or a process that reserved all device memory up
front.  cvg_realloc_noalloc gives them the hypercube reallocation with every
temporary in a static device array, so they only pass their own inputs and
outputs.  Its results must equal cvg_run_step(CVG_STAGE_REALLOC) on the same
inputs, on two calls in a row (the shared array keeps the previous call's
contents, which must not leak into the next).  This file is collected last.
"""
import ctypes as C

import numpy as np
import pytest

from cuvegas_gb300 import _lib as L, integrands as I, runtime
from oracle import pyoracle as P

pytestmark = pytest.mark.gpu


def _call(lib, torch, JF, JF2, nh_sum, info, prec, est):
    stream = torch.cuda.current_stream(JF.device)
    return lib.cvg_realloc_noalloc(
        C.c_void_p(JF.data_ptr()), C.c_void_p(JF2.data_ptr()), C.c_void_p(nh_sum.data_ptr()),
        C.c_uint32(info.n_cubes), C.c_double(info.v_cubes), C.c_double(0.75),
        C.c_int64(info.n_eval_it), C.c_int32(prec), C.c_void_p(est.data_ptr()), None,
        C.c_uint64(0), C.c_int32(0), C.c_void_p(stream.cuda_stream))


@pytest.mark.parametrize("prec", [L.PREC_FP64, L.PREC_FP32])
def test_noalloc_matches_run_step_twice(ctx, prec):
    torch = pytest.importorskip("torch")
    dim, n_it, N = 4, 200000, 64
    o = P.OracleRun(dim, n_it * 4, 4, n_intervals=N)
    u, _ = P.uniforms(P.U_PHILOX_F64, seed=21)
    o.fill(P.F_GAUSS, np.array([0.5, 0.1]), u, it=0)
    f = ctx.integrand(I.GAUSS, dim)
    p = runtime.make_params(dim, n_it * 4, 4, n_intervals=N, seed=21, precision=prec)
    with runtime.Run(f, p) as r:
        info = r.info
        assert info.n_cubes <= L.NOALLOC_MAX_CUBES
        nh_sum0 = r.get(L.BUF_NH_SUM)
        # the entry point takes JF/JF2 at their own magnitude (scale exponent 0)
        r.set(L.BUF_SCALE_EXP, np.array([0], dtype=np.int32))
        r.set(L.BUF_JF, o.JF)
        r.set(L.BUF_JF2, o.JF2)
        r.step(L.STAGE_REALLOC)
        want_nh_sum = r.get(L.BUF_NH_SUM)
        want_est = r.get(L.BUF_STATS)[:, 0]
    lib = L.load()
    dev = torch.device("cuda", 0)
    for _ in range(2):
        JF = torch.tensor(o.JF, dtype=torch.float64, device=dev)
        JF2 = torch.tensor(o.JF2, dtype=torch.float64, device=dev)
        nh_sum = torch.tensor(nh_sum0.view(np.int64), dtype=torch.int64, device=dev)
        est = torch.full((3,), -1.0, dtype=torch.float64, device=dev)
        assert _call(lib, torch, JF, JF2, nh_sum, info, prec, est) == L.OK, L.last_error()
        torch.cuda.synchronize()
        got = nh_sum.cpu().numpy().view(np.uint64)
        assert np.array_equal(got, want_nh_sum)
        np.testing.assert_allclose(est.cpu().numpy(), want_est, rtol=1e-12)
        assert not JF.any().item() and not JF2.any().item()   # consumed, as in the loop


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
