"""Generate the reference golden vectors (run on a GPU machine).

1. oracle/ref_build.py compiled the reference's own kernels (reference
   src/main.cu) to PTX under oracle/_ref/ on a machine holding the reference.
2. This script compiles oracle/ref_harness.cu (our driver of those kernels,
   following the reference's iteration sequence) with nvcc, runs it for each
   case below and packs the dumps into tests/golden/ref_<case>.npz.

Two kinds of case:
  - full cases (small sizes): every uniform, every per-cube sum, every
    iteration;
  - benchmark-shape cases (C1 exactly: d=4, 1e6 evals/iteration, 1024 bins,
    Gaussian width 0.1, 10 iterations; and d=8 / width 0.1 / 1024 bins at 2e6
    evals/iteration): the uniforms and per-cube results of every
    `stride`-th hypercube only (cubes 0, stride, 2*stride, ...), for the
    iterations listed in `keep`, together with the whole grid, the whole
    per-bin histograms, the whole n_h vector and the iteration scalars.  The
    uniforms of all samples would be 15-60 MB per iteration.

Usage: python tests/golden/make_golden.py [out_dir] [case ...]
"""
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
# name, dim, evals/iteration, bins, iterations, Gaussian width, keep, cube stride
CASES = [
    ("d2_n4000_b64", 2, 4000, 64, 3, "0.2", None, 1),
    ("d3_n20000_b256", 3, 20000, 256, 3, "0.2", None, 1),
    ("d4_n40000_b1024", 4, 40000, 1024, 2, "0.2", None, 1),
    ("c1_d4_n1e6_b1024_w01", 4, 1_000_000, 1024, 10, "0.1", (0, 1, 9), 64),
    ("c2shape_d8_n2e6_b1024_w01", 8, 2_000_000, 1024, 3, "0.1", (0, 1, 2), 256),
]
DT = {"u": np.float32, "JF": np.float64, "JF2": np.float64, "weights": np.float64,
      "counts": np.int32, "nh": np.int64, "nh_next": np.int64, "dh": np.float64,
      "x_edges_in": np.float64, "x_edges_out": np.float64, "res": np.float64,
      "sig": np.float64, "dh_sum": np.float64}


def ptx_for(dim, width):
    if width == "0.2":
        return os.path.join(ROOT, "oracle", "_ref", "ref_main_d%d.ptx" % dim)
    return os.path.join(ROOT, "oracle", "_ref", "ref_main_d%d_w%s.ptx" % (dim, width.replace(".", "")))


def subset(meta, arrays_it, dim, stride):
    """Keep the uniforms and per-cube results of cubes 0, stride, 2*stride..."""
    nh = arrays_it["nh"]
    off = np.concatenate([[0], np.cumsum(nh)])
    cubes = np.arange(0, nh.size, stride)
    u = arrays_it["u"].reshape(-1, dim)
    rows = np.concatenate([np.arange(off[c], off[c + 1]) for c in cubes])
    out = dict(arrays_it)
    out["u"] = u[rows]
    for k in ("JF", "JF2", "dh"):
        out[k] = arrays_it[k][cubes]
    out["nh_next"] = arrays_it["nh_next"][cubes].astype(np.uint32)
    out["nh"] = nh.astype(np.uint32)
    return out


def main(out_dir, names=None):
    work = tempfile.mkdtemp(prefix="golden_work_")
    exe = os.path.join(work, "ref_harness")
    subprocess.run(["nvcc", "-O2", "-std=c++17", "-gencode", "arch=compute_103a,code=sm_103a",
                    "-o", exe, os.path.join(ROOT, "oracle", "ref_harness.cu")], check=True)
    os.makedirs(out_dir, exist_ok=True)
    for name, dim, n_it, nb, iters, width, keep, stride in CASES:
        if names and name not in names:
            continue
        cdir = os.path.join(work, name)
        os.makedirs(cdir, exist_ok=True)
        cmd = [exe, ptx_for(dim, width), str(dim), str(n_it), str(nb), str(iters), cdir]
        if keep is not None:
            cmd.append("keep=" + ",".join(str(k) for k in keep))
        subprocess.run(cmd, check=True)
        meta = {}
        for line in open(os.path.join(cdir, "meta.txt")):
            k, v = line.split()
            meta[k] = float(v) if "." in v or "e" in v else int(v)
        meta["width"] = float(width)
        meta["cube_stride"] = stride
        kept = list(range(iters)) if keep is None else list(keep)
        arrays = {"meta_" + k: np.array(v) for k, v in meta.items()}
        arrays["kept"] = np.array(kept)
        for it in kept:
            a = {key: np.fromfile(os.path.join(cdir, "%s_%d.bin" % (key, it)), dtype=dt)
                 for key, dt in DT.items()}
            if stride > 1:
                a = subset(meta, a, dim, stride)
            for key, v in a.items():
                arrays["%s_%d" % (key, it)] = v
        np.savez_compressed(os.path.join(out_dir, "ref_%s.npz" % name), **arrays)
        print("wrote", name, os.path.getsize(os.path.join(out_dir, "ref_%s.npz" % name)), "bytes")


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else HERE, sys.argv[2:] or None)
