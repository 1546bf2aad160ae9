"""The cuvegas driver with the reference's config.cuh plug-in contract:
config globals parsed from the header, the header and the linked device
sources expanded and JIT-compiled, output in the reference's line format."""
import math
import os
import re
import subprocess

import pytest

from cuvegas_gb300 import _build
from oracle.ref_build import REF as REF_ROOT

HERE = os.path.dirname(os.path.abspath(__file__))
CFG = os.path.join(HERE, "golden", "cli", "config.cuh")
SRC = os.path.join(HERE, "golden", "cli", "peaks.cu")
REF = os.path.join(REF_ROOT, "src")     # the reference sources, present only on the machine that holds them


def _cli(*args, timeout=600):
    _build.build()
    return subprocess.run([_build.CLI] + list(args), capture_output=True, text=True,
                          timeout=timeout)


def test_check_parses_config_and_compiles():
    r = _cli("--check", CFG, SRC)
    assert r.returncode == 0, r.stderr
    kv = dict(line.split(": ", 1) for line in r.stdout.strip().splitlines())
    assert kv == {"n_dim": "4", "tot_eval": "4000000", "max_it": "10", "skip": "3",
                  "n_intervals": "512", "alpha": "0.5", "beta": "0.75", "precision": "fp64",
                  "compile": "ok"}


def test_missing_definition_and_include_fail_loudly():
    r = _cli("--check", CFG)                   # gauss_peak declared, never defined
    assert r.returncode != 0
    r = _cli("--check", os.path.join(HERE, "golden", "cli", "peaks.cuh"))   # no n_dim
    assert r.returncode != 0 and "n_dim" in r.stderr


def test_dump_source_expands_includes():
    r = _cli("--dump-source", CFG, SRC)
    assert r.returncode == 0
    assert "#include" not in r.stdout
    assert "double gauss_peak(double* x, int n_dim);" in r.stdout     # declaration (header)
    assert "double gauss_peak(double* x, int n_dim) {" in r.stdout    # definition (linked source)
    assert "#define M_PI" in r.stdout


@pytest.mark.skipif(not os.path.isdir(REF), reason="reference sources not present")
def test_reference_config_compiles_unchanged():
    r = _cli("--check", os.path.join(REF, "config.cuh"), os.path.join(REF, "commons", "functions.cu"))
    assert r.returncode == 0, r.stderr
    assert "n_dim: 4" in r.stdout and "compile: ok" in r.stdout


@pytest.mark.gpu
def test_cli_run_prints_reference_lines():
    r = _cli(CFG, SRC)
    assert r.returncode == 0, r.stderr
    pairs = [re.match(r"(.*?):? (-?[0-9][-0-9.e+]*)( ms)?$", line).groups()[:2]
             for line in r.stdout.strip().splitlines()]
    assert [k for k, _ in pairs] == ["GPUs", "Strat", "Cubes", "Intervals", "Result", "Error",
                                     "Total evals", "Time elapsed", "Iteration avg time",
                                     "Nocontext", "Context creation", "Integrand compile",
                                     "Chi2/dof"]
    out = dict(pairs)
    # the reference's meaning: Time elapsed = Context creation + Nocontext,
    # with the JIT compile of the integrand (ahead of time in the reference)
    # on its own line
    parts = float(out["Context creation"]) + float(out["Integrand compile"]) + float(out["Nocontext"])
    assert abs(float(out["Time elapsed"]) - parts) < 1.0
    exact = math.erf(5.0) ** 4
    res, err = float(out["Result"]), float(out["Error"])
    n_strat, n_cubes = int(out["Strat"]), int(out["Cubes"])
    assert n_strat == int((400000 / 4) ** 0.25) and n_cubes == n_strat ** 4
    # n_h >= 2 per cube: an iteration takes up to N_it + 2 n_cubes samples
    assert 0.8 * 4000000 < int(out["Total evals"]) <= 10 * (400000 + 2 * n_cubes)
    assert abs(res - exact) < 5 * err
