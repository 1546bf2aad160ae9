"""Compile the reference's own CUDA kernels to PTX for the golden harness.

Sources stay where they lie (reference src/main.cu); only PTX text is written,
into oracle/_ref/ (git-ignored).  The reference's config.cuh is replaced by
oracle/ref_shim.cuh through `-include` (its include guard makes the
reference's own `#include "config.cuh"` a no-op).  The stock Makefile is not
used (it links -lnvToolsExt, absent on CUDA 13).  Test infrastructure only.
"""
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_ref")
REF = os.environ.get("CVG_REFERENCE", "/root/reference")
DIMS = (2, 3, 4)
# the reference's kernels for the benchmark workloads' Gaussian (width 0.1):
# golden vectors at the d=4 and d=8 benchmark shapes, and the reference-kernel
# timing leg of bench.py
TIMING = ((4, "0.1"), (8, "0.1"))


def build(force=False):
    src = os.path.join(REF, "src", "main.cu")
    if not os.path.exists(src):
        raise FileNotFoundError(src)
    os.makedirs(OUT, exist_ok=True)
    shim = os.path.join(HERE, "ref_shim.cuh")
    outs = []
    for d in DIMS:
        out = os.path.join(OUT, "ref_main_d%d.ptx" % d)
        if not force and os.path.exists(out) and os.path.getmtime(out) >= max(
                os.path.getmtime(shim), os.path.getmtime(__file__)):
            outs.append(out)
            continue
        cmd = ["nvcc", "-ptx", "-arch=sm_103a", "-O3", "-include", shim, "-DCVG_REF_DIM=%d" % d,
               "-Xcompiler", "-fopenmp", src, "-o", out]
        subprocess.run(cmd, check=True, capture_output=True, text=True)
        outs.append(out)
    for d, width in TIMING:
        out = os.path.join(OUT, "ref_main_d%d_w%s.ptx" % (d, width.replace(".", "")))
        if not force and os.path.exists(out) and os.path.getmtime(out) >= max(
                os.path.getmtime(shim), os.path.getmtime(__file__)):
            outs.append(out)
            continue
        cmd = ["nvcc", "-ptx", "-arch=sm_103a", "-O3", "-include", shim, "-DCVG_REF_DIM=%d" % d,
               "-DCVG_REF_WIDTH=%s" % width, "-Xcompiler", "-fopenmp", src, "-o", out]
        subprocess.run(cmd, check=True, capture_output=True, text=True)
        outs.append(out)
    return outs


if __name__ == "__main__":
    print(build(force=True))
