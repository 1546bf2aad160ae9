"""Generate the reference golden vectors (run on a GPU machine).

1. oracle/ref_build.py compiled the reference's own kernels (reference
   src/main.cu) to PTX under oracle/_ref/ on a machine holding the reference.
2. This script compiles tests/golden/ref_harness.cu (our driver of those
   kernels, following the reference's iteration sequence) with nvcc, runs it
   for each case below and packs the dumps into tests/golden/ref_<case>.npz.

Usage: python tests/golden/make_golden.py [out_dir]
"""
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
CASES = [  # name, dim, evals/iteration, bins, iterations
    ("d2_n4000_b64", 2, 4000, 64, 3),
    ("d3_n20000_b256", 3, 20000, 256, 3),
    ("d4_n40000_b1024", 4, 40000, 1024, 2),
]
DT = {"u": np.float32, "JF": np.float64, "JF2": np.float64, "weights": np.float64,
      "counts": np.int32, "nh": np.int64, "nh_next": np.int64, "dh": np.float64,
      "x_edges_in": np.float64, "x_edges_out": np.float64, "res": np.float64,
      "sig": np.float64, "dh_sum": np.float64}


def main(out_dir):
    work = os.path.join(out_dir, "golden_work")
    os.makedirs(work, exist_ok=True)
    exe = os.path.join(work, "ref_harness")
    subprocess.run(["nvcc", "-O2", "-std=c++17", "-gencode", "arch=compute_103a,code=sm_103a",
                    "-o", exe, os.path.join(HERE, "ref_harness.cu")], check=True)
    for name, dim, n_it, nb, iters in CASES:
        cdir = os.path.join(work, name)
        os.makedirs(cdir, exist_ok=True)
        ptx = os.path.join(ROOT, "oracle", "_ref", "ref_main_d%d.ptx" % dim)
        subprocess.run([exe, ptx, str(dim), str(n_it), str(nb), str(iters), cdir], check=True)
        meta = {}
        for line in open(os.path.join(cdir, "meta.txt")):
            k, v = line.split()
            meta[k] = float(v) if "." in v or "e" in v else int(v)
        arrays = {"meta_" + k: np.array(v) for k, v in meta.items()}
        for it in range(iters):
            for key, dt in DT.items():
                arrays["%s_%d" % (key, it)] = np.fromfile(
                    os.path.join(cdir, "%s_%d.bin" % (key, it)), dtype=dt)
        np.savez_compressed(os.path.join(out_dir, "ref_%s.npz" % name), **arrays)
        print("wrote", name)


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else HERE)
