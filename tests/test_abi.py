"""CPU tests of the C ABI boundary: the library loads, exports every symbol of
include/cuvegas.h, and integrand sources compile with NVRTC (no GPU calls)."""
import os
import re

import pytest

from cuvegas_gb300 import _build, _lib as L, integrands as I

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module", autouse=True)
def built():
    _build.build()


def header_functions():
    src = open(os.path.join(ROOT, "include", "cuvegas.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(cvg_[a-z0-9_]+)\s*\(", src)))


def test_exports_every_declared_symbol():
    lib = L.load()
    names = header_functions()
    assert len(names) >= 19
    for n in names:
        assert hasattr(lib, n), n
    assert set(names) == set(L.EXPORTS)


def test_version_and_error_buffer():
    assert L.version().startswith("cuvegas_gb300")
    assert isinstance(L.last_error(), str)


@pytest.mark.parametrize("name,src,dim,P,g", [
    ("gauss", I.GAUSS, 4, 0, False), ("gauss8", I.GAUSS, 8, 0, False),
    ("mixture", I.MIXTURE, 6, 16, True), ("prodpeak", I.PRODPEAK, 12, 24, False),
    ("corner", I.CORNER, 16, 16, False), ("one", I.CONST_ONE, 1, 0, False)])
@pytest.mark.parametrize("prec", [L.PREC_FP64, L.PREC_FP32])
def test_integrands_compile(name, src, dim, P, g, prec):
    L.compile_check(src, dim, precision=prec, n_params=P, has_grad=g)


@pytest.mark.parametrize("wt", ["0", "1"])
@pytest.mark.parametrize("dim,P", [(3, 0), (8, 0), (16, 16)])
def test_fill_tile_shapes_compile(monkeypatch, wt, dim, P):
    """Both tile shapes of the single-run fill (warp tiles, block tiles)
    compile for FP32 and FP64, with and without the gradient pass."""
    monkeypatch.setenv("CVG_FILL_WARP_TILES", wt)
    src = I.GAUSS if P == 0 else I.CORNER
    for prec in (L.PREC_FP32, L.PREC_FP64):
        L.compile_check(src, dim, precision=prec, n_params=P)
    L.compile_check(I.MIXTURE, 6, precision=L.PREC_FP32, n_params=16, has_grad=True)


def test_numba_abi_compiles():
    src = """extern "C" __device__ int integrand(double* ret, double* x) {
        double s = 0; for (int i = 0; i < cvg_n_dim; ++i) s += x[i]; *ret = s; return 0; }"""
    L.compile_check(src, 3, abi=L.ABI_NUMBA)


def test_compile_error_is_reported():
    with pytest.raises(L.CuvegasError) as e:
        L.compile_check("__device__ double integrand(double* x) { return undefined_thing; }", 2)
    assert e.value.status == L.ERR_COMPILE
    assert "undefined_thing" in str(e.value)


def test_fp32_needs_float_overload():
    src = "__device__ double integrand(double* x) { return x[0]; }"
    L.compile_check(src, 2, precision=L.PREC_FP64)
    with pytest.raises(L.CuvegasError):
        L.compile_check(src, 2, precision=L.PREC_FP32)


def test_bad_arguments_rejected():
    with pytest.raises(L.CuvegasError) as e:
        L.compile_check(I.GAUSS, 0)
    assert e.value.status == L.ERR_INVALID
    with pytest.raises(L.CuvegasError):
        L.compile_check(I.GAUSS, 33)


def test_batch_kernels_compile():
    L.batch_compile_check(I.PRODPEAK, list(range(2, 13)), [2 * d for d in range(17)],
                          precision=L.PREC_FP32)
