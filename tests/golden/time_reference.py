"""Time the reference's own CUDA kernels on this GPU (run on a GPU machine).

The reference's src/main.cu kernels, compiled to PTX by oracle/ref_build.py
with the benchmark workloads' Gaussian (width 0.1), are driven through the
reference's iteration sequence by tests/golden/ref_harness.cu in its "time"
mode: each iteration -- fill, results, reductions, n_h update, map rebuild,
grid refinement and the host reads between them -- is timed with CUDA events.
This is the reference GPU implementation measured beside ours; it is not a
bench.py arm.

Usage: python tests/golden/time_reference.py [out_dir]
"""
import os
import re
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
CASES = [  # name, dim, evals/iteration, bins, iterations
    ("c1_gauss_d4_1e6", 4, 1_000_000, 1024, 10),
    ("c2_gauss_d8_1e8", 8, 100_000_000, 1024, 6),
]


def main(out_dir):
    work = os.path.join(out_dir, "reference_timing")
    os.makedirs(work, exist_ok=True)
    exe = os.path.join(work, "ref_harness")
    subprocess.run(["nvcc", "-O2", "-std=c++17", "-gencode", "arch=compute_103a,code=sm_103a",
                    "-o", exe, os.path.join(HERE, "ref_harness.cu")], check=True)
    for name, dim, n_it, nb, iters in CASES:
        ptx = os.path.join(ROOT, "oracle", "_ref", "ref_main_d%d_w01.ptx" % dim)
        r = subprocess.run([exe, ptx, str(dim), str(n_it), str(nb), str(iters), work, "time"],
                           capture_output=True, text=True)
        if r.returncode != 0:
            sys.exit("%s: harness exited %d\n%s%s" % (name, r.returncode, r.stdout, r.stderr))
        rows = [tuple(float(v) for v in re.findall(r"samples (\d+) ms ([\d.]+)", line)[0])
                for line in r.stdout.splitlines() if line.startswith("iteration")]
        warm = rows[2:] if len(rows) > 3 else rows
        evals = sum(s for s, _ in warm)
        ms = sum(t for _, t in warm)
        print("%s: %d iterations timed (first 2 skipped), %.3f ms per iteration, %.4g evals/s"
              % (name, len(warm), ms / len(warm), evals / (ms * 1e-3)))
        print(r.stdout.strip())


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else os.path.join(ROOT, "gpurun_out"))
