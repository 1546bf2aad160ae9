"""The bench's reference arm (the CPU restatement of the reference loop on
the host cores) prints the contract's JSON line; it needs no GPU."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_arm_json_line():
    # the arm runs the headline workload (1e8 evaluations per iteration); here
    # a smaller size keeps the CPU suite short
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference",
                        "--steps", "1", "--warmup", "3", "--evals", "2000000"],
                       capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference"
    assert d["value"] > 0 and d["unit"] == "evals/s" and d["higher_is_better"] is True
    assert d["steps"] == 1 and d["warmup"] >= 3 and d["n_gpus"] == 1
    assert d["cpu_baseline"]["value"] == d["value"]
    assert d["cpu_baseline"]["kind"] in ("port", "reference") and d["cpu_baseline"]["cores"] >= 1
    assert d["e2e"] == {"value": d["value"], "unit": d["unit"], "h2d_bytes_per_step": 0,
                        "d2h_bytes_per_step": 0}
    assert d["config"]["workload"] and d["metric"]
    assert d["config"]["evals_per_iteration"] == 2000000


def test_fill_roofline_binds_the_slowest_ceiling():
    """bench.fill_roofline: each pipe's ceiling and the issue ceiling at the
    algorithmic instruction floor, in evaluations/s; the lowest one binds,
    achieved and frac in that ceiling's units."""
    sys.path.insert(0, ROOT)
    import bench

    class FakeCtx:
        peaks = {0: 70.0, 8: 10.0, 9: 0.4}      # T FMA-flops/s, T ex2/s, T Philox calls/s

        def measure_peak(self, kind):
            return self.peaks[kind]

    bench._PEAKS.clear()
    # 1e8 evaluations in 2 ms = 5e10 evals/s at 2000 MHz
    r = bench.fill_roofline(FakeCtx(), 1e8, 2.0, 2000.0)
    c = r["ceilings_evals_per_s"]
    floor = sum(bench.INSTR_FLOOR.values())
    issue = 152 * 4 * 32 * 2000e6
    assert abs(c["fp32"] - 35e12 / bench.FLOPS_PER_EVAL) < 1 and abs(c["sfu"] - 10e12 / 8) < 1
    assert abs(c["sampler"] - 0.4e12 / 2) < 1
    assert abs(c["issue"] - issue / floor) < 1
    assert r["bound"] == "issue" and r["unit"] == "T thread instructions/s"
    assert abs(r["achieved"] - 5e10 * floor / 1e12) < 1e-9
    assert abs(r["frac"] - 5e10 / (issue / floor)) < 1e-12
    # a slower sampler binds instead
    bench._PEAKS.clear()
    FakeCtx.peaks[9] = 0.2
    r = bench.fill_roofline(FakeCtx(), 1e8, 2.0, 2000.0)
    assert r["bound"] == "sampler" and abs(r["frac"] - 5e10 / 1e11) < 1e-12
    bench._PEAKS.clear()
