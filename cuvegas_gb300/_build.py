"""Build libcuvegas.so in-tree for sm_103a, and the cuvegas command-line driver.

Steps: embed the device headers (for NVRTC) into a generated include, compile
the translation units with nvcc in parallel, link one shared library with
the CUDA runtime linked statically and NVRTC dynamically, then compile the
host-only CLI (cli/cuvegas_cli.cpp) against it.
"""
import concurrent.futures as cf
import os
import shutil
import subprocess

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
BUILD = os.path.join(PKG, "_build")
LIBDIR = os.path.join(PKG, "_lib")
LIB = os.path.join(LIBDIR, "libcuvegas.so")
CLI = os.path.join(LIBDIR, "cuvegas")
CLI_SRC = os.path.join(PKG, "cli", "cuvegas_cli.cpp")
INCLUDE = os.path.join(ROOT, "include")
GENCODE = ["-gencode", "arch=compute_103a,code=sm_103a"]
EMBED = ["cvg_common.cuh", "cvg_fill.cuh"]
UNITS = ["cvg_kernels.cu", "cvg_host.cu", "cvg_noalloc.cu", "cvg_batch.cu"]


def cuda_home():
    env = os.environ.get("CUDA_HOME") or os.environ.get("CUDA_PATH")
    if env:
        return env
    nvcc = shutil.which("nvcc")
    if nvcc:
        return os.path.dirname(os.path.dirname(os.path.realpath(nvcc)))
    return "/usr/local/cuda"


def _embed(out_path):
    parts = ["// generated by cuvegas_gb300/_build.py -- do not edit\n"]
    for name in EMBED:
        with open(os.path.join(CSRC, name)) as f:
            text = f.read()
        assert ")CVGRAW\"" not in text
        var = "cvg_src_" + name.split("_", 1)[1].split(".")[0]
        parts.append('static const char %s[] = R"CVGRAW(%s)CVGRAW";\n' % (var, text))
    data = "".join(parts)
    if os.path.exists(out_path) and open(out_path).read() == data:
        return
    with open(out_path, "w") as f:
        f.write(data)


def _inputs():
    files = [os.path.join(CSRC, n) for n in os.listdir(CSRC)]
    files.append(os.path.join(INCLUDE, "cuvegas.h"))
    files.append(CLI_SRC)
    files.append(os.path.abspath(__file__))
    return files


def build(force=False, verbose=False):
    os.makedirs(BUILD, exist_ok=True)
    os.makedirs(LIBDIR, exist_ok=True)
    gen = os.path.join(BUILD, "cvg_embedded.inc")
    _embed(gen)
    newest = max(os.path.getmtime(p) for p in _inputs())
    if (not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= newest
            and os.path.exists(CLI) and os.path.getmtime(CLI) >= newest):
        return LIB
    nvcc = os.path.join(cuda_home(), "bin", "nvcc")
    if not os.path.exists(nvcc):
        nvcc = "nvcc"
    common = [nvcc] + GENCODE + ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC",
                                 "-I", CSRC, "-I", BUILD, "-I", INCLUDE]

    def compile_unit(name):
        obj = os.path.join(BUILD, name.replace(".cu", ".o"))
        cmd = common + ["-c", os.path.join(CSRC, name), "-o", obj]
        if verbose:
            print(" ".join(cmd))
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed for %s:\n%s%s" % (name, r.stdout, r.stderr))
        return obj

    with cf.ThreadPoolExecutor(len(UNITS)) as ex:
        objs = list(ex.map(compile_unit, UNITS))
    libdir = os.path.join(cuda_home(), "lib64")
    tmp = LIB + ".tmp%d" % os.getpid()
    cmd = [nvcc] + GENCODE + ["-shared", "-o", tmp] + objs + [
        "-L", libdir, "-lnvrtc", "-lnvJitLink", "-Xlinker", "-rpath=" + libdir]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n%s%s" % (r.stdout, r.stderr))
    os.replace(tmp, LIB)
    _build_cli(verbose)
    return LIB


def _build_cli(verbose=False):
    """Host-only C++ driver; finds libcuvegas.so next to itself."""
    cxx = shutil.which("g++") or shutil.which("c++") or "g++"
    tmp = CLI + ".tmp%d" % os.getpid()
    cmd = [cxx, "-O2", "-std=c++17", "-Wall", "-I", INCLUDE, CLI_SRC, "-o", tmp, "-L", LIBDIR,
           "-lcuvegas", "-Wl,-rpath,$ORIGIN"]
    if verbose:
        print(" ".join(cmd))
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("CLI build failed:\n%s%s" % (r.stdout, r.stderr))
    os.replace(tmp, CLI)


if __name__ == "__main__":
    print(build(force=True, verbose=True))
