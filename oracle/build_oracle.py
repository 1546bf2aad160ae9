"""Build the CPU oracle shared library (test infrastructure only).

``gcc -O2 -fopenmp -ffp-contract=off`` keeps x86_64 and aarch64 results equal
(no fused multiply-add contraction except the explicit ``fma`` calls).
"""
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "liboracle.so")


def build(force: bool = False) -> str:
    src = [os.path.join(HERE, "vegas_oracle.c")]
    hdr = os.path.join(HERE, "vegas_oracle.h")
    os.makedirs(OUT_DIR, exist_ok=True)
    newest = max(os.path.getmtime(p) for p in src + [hdr])
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= newest:
        return LIB
    tmp = LIB + ".tmp%d" % os.getpid()
    cmd = ["gcc", "-O2", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off",
           "-std=gnu11", "-o", tmp] + src + ["-lm"]
    subprocess.run(cmd, check=True)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force=True))
