#!/usr/bin/env python
"""Benchmark of the VEGAS+ iteration loop on one GB300 (N GPUs: replicas or a
sample split).

Headline workload: Gaussian family, d=8, width 0.1, centre 0.5, 1e8 integrand
evaluations per iteration, 1024 bins per dimension, alpha=0.5, beta=0.75,
seed 0, 20 iterations -- FP32 evaluation with Kahan-compensated f/f^2
accumulation and FP64 mean/variance/grid ("chosen" form).  A step is one
VEGAS+ iteration: fill (sample, map, integrand, accumulate), hypercube
reallocation, grid refinement.

Printed JSON line (rank 0):
  value      evals/s over the K timed iterations, state resident in HBM
  e2e        evals/s of whole integrations through the C ABI with host
             parameters in and host results out (cvg_integrate); the context
             keeps its device arena between calls, and `cold_arena` repeats
             the call with the arena freed first (allocation inside the call,
             as the reference allocates in every call)
  plain      the same workload in the plain FP64 form, with the FP64-pipe
             roofline of its fill
  time_to_1e-4  a sweep over evaluations per iteration (20 iterations, skip
             5) in both forms: the fastest run whose final err/|I| <= 1e-4
             with |I - exact| <= 3 err
  configs    the other benchmark configurations (C1, C3, C4, C5): value,
             ms/step, pull, chi2/dof, clocks
  reference_gpu  the reference's own CUDA kernels (compiled from its sources
             to PTX, driven through its iteration sequence), CUDA events per
             iteration on this GPU, beside `plain` as the matched-precision
             comparison
  roofline   fill kernel against its ceilings: per pipe (FP32 ops, ex2,
             Philox calls, each peak from a live microbenchmark of this GPU)
             and instruction issue (4 warp instructions per SM per clock) at
             the algorithmic instruction floor of an evaluation; the lowest
             ceiling binds
  cpu_baseline  the CPU oracle (FP64, OpenMP, all host cores) on a bounded
             sample of the same workload
`--impl reference` times the reference's computation on the host cores (the
CPU restatement of the reference loop in oracle/, FP64, all cores) on the
same workload (1e8 evaluations per iteration).
`--mode split` (N > 1) splits each iteration's samples across the ranks with
an NCCL all-reduce of the fill's sums (the reference's multi-GPU mode);
the default `replicas` runs independent integrals.
"""
import argparse
import json
import math
import os
import re
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

DIM, N_IT, NBINS, ITERS, SEED = 8, 100_000_000, 1024, 20, 0
SKIP = 5
N_SM = 152


def _measured_peaks():
    """Measured copy bandwidth and clocks of the GB300s (MEASURED_PEAKS.json)."""
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


HBM_GBS = float(_measured_peaks().get("hbm_gbs", 6800.0))   # fallback: one earlier GB300 figure
FLOPS_PER_EVAL = 11 * DIM + 4          # algorithmic FP32 ops per evaluation (map 7/dim, integrand 4/dim, 4)
SFU_PER_EVAL = DIM                     # one exp per dimension
PHILOX_PER_EVAL = (DIM + 3) // 4       # Philox4x32-10 calls per evaluation (4 uniforms per call)
# Algorithmic instruction floor of one FP32 evaluation (thread instructions),
# counted from the operations the formulas need, per phase:
#   sampler   Philox4x32-10: 10 rounds x (2 wide multiplies + 2 three-input
#             XORs) per call, 1 call per 4 dimensions; 1 bit operation per
#             uniform to place its bits in a float significand
#   map       per dimension: stratified z (1 FMA), bin by a round-down add
#             and its bits (2), edge and width (1 paired load), fraction (1),
#             x (1 FMA), Jacobian factor (1)
#   integrand per dimension: x - 0.5 and its square accumulated (2); then one
#             exp (ex2 + its scaling multiply) and the normalisation (1)
#   sums      f*jac, its square, two Kahan updates (4 each)
#   histogram per dimension: the scaled weight (3: exponent, multiply,
#             rounding add), one address, a count and a value atomic (2)
#   loop      sample loop, cube run bookkeeping (~5)
INSTR_FLOOR = {"sampler": 40 * PHILOX_PER_EVAL + DIM, "map": 7 * DIM,
               "integrand": 2 * DIM + 3, "sums": 10, "histogram": 6 * DIM, "loop": 5}
METRIC = "integrand evals/s, VEGAS+ Gaussian d=8, 1e8 evals/iteration (FP32-compensated form)"
WORKLOAD = "gauss-d8-1e8x20-fp32kahan"
LAUNCHES_PER_IT = 4                    # fill, 2 reallocation kernels (results+finish, one-pass allocation), refinement


def _dist():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


class ClockSampler:
    """nvidia-smi samples of SM clock and throttle reasons during a region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.Q,
                 "--format=csv,noheader,nounits", "-lms", "20"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
            # nvidia-smi takes a while to start: let its first sample land
            # before the timed region begins (a region of a few tens of ms
            # would otherwise end before any sample)
            t0 = time.time()
            while not self.lines and time.time() - t0 < 3.0 and self.proc.poll() is None:
                time.sleep(0.005)
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def profile_value(name, key):
    """A `key=value` figure from a committed ncu summary under profiles/ (or None)."""
    try:
        for line in open(os.path.join(ROOT, "profiles", name)):
            if line.startswith(key + "="):
                return float(line.split("=", 1)[1])
    except (OSError, ValueError):
        pass
    return None


_PEAKS = {}


def live_peak(ctx, kind):
    """Live microbenchmark of this GPU (cvg_measure_peak), once per process."""
    if kind not in _PEAKS:
        _PEAKS[kind] = ctx.measure_peak(kind)
    return _PEAKS[kind]


def fill_roofline(ctx, evals_per_launch, mean_ms, sm_mhz):
    """Roofline of the FP32 fill.  Evaluations/s are bounded by each pipe
    alone -- FP32 ops, ex2, the Philox calls of the sampler (peaks measured
    live, cvg_measure_peak kinds 0, 8, 9) -- and by instruction issue: 4 warp
    instructions per SM per clock at the algorithmic instruction floor of an
    evaluation (INSTR_FLOOR).  The lowest ceiling binds; frac = measured
    evals/s / that ceiling.  The instructions the fill actually executes per
    evaluation (ncu, committed summary) give its own issue ceiling beside it."""
    p_fp32 = live_peak(ctx, 0) / 2.0           # T FP32 instructions/s (FMA = 2 flops)
    p_sfu = live_peak(ctx, 8)                  # T ex2/s
    p_philox = live_peak(ctx, 9)               # T Philox calls/s
    clk = (sm_mhz or 2070.0) * 1e6
    issue = N_SM * 4 * 32 * clk / 1e12         # T thread instructions/s
    floor = float(sum(INSTR_FLOOR.values()))
    rate = evals_per_launch / (mean_ms * 1e-3)
    ceil = {"fp32": (p_fp32 * 1e12 / FLOPS_PER_EVAL, FLOPS_PER_EVAL, p_fp32, "T FP32 ops/s"),
            "sfu": (p_sfu * 1e12 / SFU_PER_EVAL, SFU_PER_EVAL, p_sfu, "T ex2/s"),
            "sampler": (p_philox * 1e12 / PHILOX_PER_EVAL, PHILOX_PER_EVAL, p_philox,
                        "T Philox calls/s"),
            "issue": (issue * 1e12 / floor, floor, issue, "T thread instructions/s")}
    bound = min(ceil, key=lambda k: ceil[k][0])
    evals_max, per_eval, peak, unit = ceil[bound]
    achieved = rate * per_eval / 1e12
    out = {"bound": bound, "achieved": achieved, "peak": peak, "unit": unit,
           "frac": achieved / peak, "traffic": None,
           "ceilings_evals_per_s": {k: v[0] for k, v in ceil.items()},
           "evals_per_s_fill": rate, "fill_ms_mean": mean_ms,
           "evals_per_launch": evals_per_launch,
           "per_eval": {"fp32_ops": FLOPS_PER_EVAL, "ex2": SFU_PER_EVAL,
                        "philox_calls": PHILOX_PER_EVAL, "instruction_floor": INSTR_FLOOR},
           "issue_clock_mhz": clk / 1e6,
           "peak_source": "live microbenchmarks of this GPU (cvg_measure_peak kinds 0, 8, 9); issue "
                          "rate = 152 SMs x 4 warp instructions/clock at the sampled SM clock; "
                          "MEASURED_PEAKS.json holds HBM and bf16 figures only"}
    ipe = profile_value("fill_gauss_d8_traffic.txt", "inst_per_eval")
    if ipe:
        out["executed_instructions_per_eval"] = ipe
        out["issue_ceiling_at_executed_evals_per_s"] = issue * 1e12 / ipe
        out["issue_frac_at_executed"] = rate / (issue * 1e12 / ipe)
    return out


def c5_roofline(ctx, evals_per_launch, mean_ms, sm_mhz):
    """C5's fill (corner peak, d=16) against the ceilings the workload names:
    FP32 pipe (FP32 instructions per evaluation, ncu, x evaluations/s against
    the live FP32 FMA peak / 2), SFU (ncu's XU-pipe share of the same
    launch), HBM (DRAM bytes per evaluation of the full 1e9 workload, ncu, x
    evaluations/s against the measured copy bandwidth) and instruction issue
    (instructions per evaluation x evaluations/s against 152 SMs x 4 warp
    instructions per clock), which binds."""
    rate = evals_per_launch / (mean_ms * 1e-3)
    clk = (sm_mhz or 2070.0) * 1e6
    issue = N_SM * 4 * 32 * clk / 1e12
    src = "fill_corner_d16_counts.txt"
    ipe = profile_value(src, "inst_per_eval")
    fpe = profile_value(src, "fp32_inst_per_eval")
    bpe = profile_value(src, "dram_bytes_per_eval")
    out = {"bound": "issue", "evals_per_s_fill": rate, "fill_ms_mean": mean_ms,
           "evals_per_launch": evals_per_launch, "issue_clock_mhz": clk / 1e6,
           "counts_source": "profiles/" + src}
    if ipe:
        out.update({"instructions_per_eval": ipe, "achieved": rate * ipe / 1e12, "peak": issue,
                    "unit": "T thread instructions/s", "frac": rate * ipe / 1e12 / issue})
    if fpe:
        p_fp32 = live_peak(ctx, 0) / 2.0
        out.update({"fp32_inst_per_eval": fpe, "fp32_achieved": rate * fpe / 1e12,
                    "fp32_peak": p_fp32, "fp32_unit": "T FP32 instructions/s",
                    "fp32_pipe_frac": rate * fpe / 1e12 / p_fp32})
    out["sfu_pipe_pct_ncu"] = profile_value(src, "ncu_xu_pipe_pct")
    if bpe:
        out.update({"dram_bytes_per_eval": bpe, "hbm_gbs": rate * bpe / 1e9,
                    "hbm_peak_gbs": HBM_GBS, "hbm_frac": rate * bpe / 1e9 / HBM_GBS})
    return out


def plain_roofline(ctx, evals_per_launch, mean_ms):
    """FP64-pipe roofline of the plain (FP64) fill.  The FP64 pipe executes
    one FMA, add or multiply per lane per issue, so its ceiling is the live
    FP64 FMA peak (cvg_measure_peak kind 1) / 2 in FP64 instructions/s; the
    fill's FP64 instructions per evaluation (DFMA + DADD + DMUL, ncu,
    committed summary -- the FP64 exp is a sequence of them) x evaluations/s
    is the achieved rate."""
    p64 = live_peak(ctx, 1)                    # TFLOP/s (FMA = 2 flops)
    rate = evals_per_launch / (mean_ms * 1e-3)
    out = {"bound": "fp64", "peak": p64 / 2.0, "unit": "T FP64 instructions/s",
           "evals_per_s_fill": rate, "fill_ms_mean": mean_ms,
           "peak_source": "live FP64 FMA microbenchmark (kind 1) / 2"}
    ipe = profile_value("fill_plain_gauss_d8.md", "fp64_inst_per_eval")
    fpe = profile_value("fill_plain_gauss_d8.md", "fp64_flops_per_eval")
    if ipe:
        out.update({"achieved": rate * ipe / 1e12, "fp64_inst_per_eval": ipe,
                    "frac": rate * ipe / 1e12 / (p64 / 2.0),
                    "ncu_fp64_pipe_active_pct": profile_value("fill_plain_gauss_d8.md",
                                                              "fp64_pipe_active_pct")})
    if fpe:
        out.update({"fp64_flops_per_eval": fpe, "tflops": rate * fpe / 1e12,
                    "flops_frac": rate * fpe / 1e12 / p64})
    return out


def cpu_oracle_rate(n_it, iters, threads=0):
    """Oracle (FP64 restatement of the reference loop) on host cores: evals/s."""
    import numpy as np
    from oracle import pyoracle as P
    r = P.OracleRun(DIM, n_it * (iters + 1), iters + 1, n_intervals=NBINS)
    u, _ = P.uniforms(P.U_PHILOX_F64, seed=SEED)
    th = np.array([0.5, 0.1])
    tot, t0 = 0, time.perf_counter()
    for it in range(iters):
        tot += r.fill(P.F_GAUSS, th, u, it=it, n_threads=threads)
        d, _, _ = r.results()
        r.refine()
        r.update_nh(d)
    dt = time.perf_counter() - t0
    return tot / dt, tot, dt


def run_reference(args):
    rank, world, _ = _dist()
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
        if rank != 0:
            dist.destroy_process_group()
            return
    import numpy as np
    from oracle import pyoracle as P
    cores = os.cpu_count() or 1
    n_it = N_IT               # the headline workload's own size per iteration
    steps, warm = args.steps, args.warmup
    r = P.OracleRun(DIM, n_it * (steps + warm + 1), steps + warm + 1, n_intervals=NBINS)
    u, _ = P.uniforms(P.U_PHILOX_F64, seed=SEED)
    th = np.array([0.5, 0.1])
    tot, el = 0, 0.0
    for it in range(warm + steps):
        t0 = time.perf_counter()
        n = r.fill(P.F_GAUSS, th, u, it=it)
        d, _, _ = r.results()
        r.refine()
        r.update_nh(d)
        dt = time.perf_counter() - t0
        if it >= warm:
            tot += n
            el += dt
    v = tot / el
    sample = "%d VEGAS+ iterations (after %d warm-up iterations) of the d=8 Gaussian workload " \
             "at %d evals/iteration, 1024 bins, FP64, all %d host cores" % (steps, warm, n_it, cores)
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": "evals/s",
            "n_gpus": args.gpus, "steps": steps, "warmup": warm,
            "ms_per_step": 1e3 * el / steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": WORKLOAD, "dim": DIM, "evals_per_iteration": n_it,
                       "nbins": NBINS, "alpha": 0.5, "beta": 0.75, "seed": SEED,
                       "implementation": "CPU restatement of the reference VEGAS+ loop "
                                         "(oracle/vegas_oracle.c), OpenMP over hypercubes"},
            "cpu_baseline": {"value": v, "unit": "evals/s", "cores": cores, "kind": "port",
                             "sample": sample},
            "e2e": {"value": v, "unit": "evals/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


def timed_iterations(run, n, stream, torch):
    """Run n iterations with a CUDA event between each; returns per-iteration ms."""
    evs = [torch.cuda.Event(enable_timing=True) for _ in range(n + 1)]
    evs[0].record(stream)
    for i in range(n):
        run.iterate(1)
        evs[i + 1].record(stream)
    stream.synchronize()
    return [evs[i].elapsed_time(evs[i + 1]) for i in range(n)]


def weighted(it_res, it_sig, skip):
    """Weighted mean and error of iterations >= skip (src/main.cu:698-713, 792)."""
    sw = sum(1.0 / s for s in it_sig[skip:])
    swr = sum(r / s for r, s in zip(it_res[skip:], it_sig[skip:]))
    return swr / sw, 1.0 / math.sqrt(sw)


def tt_sweep(f, prec, exact, evals, iters=ITERS, skip=SKIP):
    """time-to-1e-4: whole integrations (cvg_integrate, host parameters in,
    host results out; one untimed call per size first, so JIT and the device
    arena are warm) at each evaluations-per-iteration size, 20 iterations,
    skip 5.  The time is that of the fastest run whose final err/|I| <= 1e-4
    and |I - exact| <= 3 err."""
    from cuvegas_gb300 import _lib as L, runtime
    pts, best = [], None
    for n_it in evals:
        p = runtime.make_params(f.n_dim, n_it * iters, iters, skip=skip, n_intervals=NBINS,
                                seed=SEED, precision=prec, flags=L.FLAG_GRAPH)
        runtime.integrate_once(f, p)
        t0 = time.perf_counter()
        res, _, _ = runtime.integrate_once(f, p)
        wall = time.perf_counter() - t0
        rel = res.error / abs(res.result)
        ok = rel <= 1e-4 and abs(res.result - exact) <= 3 * res.error
        pts.append({"evals_per_iteration": n_it, "wall_s": wall, "rel_err": rel,
                    "pull": (res.result - exact) / res.error, "chi2_dof": res.chi2_dof,
                    "passes": bool(ok)})
        if ok and (best is None or wall < best["wall_s"]):
            best = pts[-1]
    return {"time_s": best["wall_s"] if best else None,
            "at_evals_per_iteration": best["evals_per_iteration"] if best else None,
            "iterations": iters, "skip": skip, "points": pts}


def run_timed(f, dim, n_it, iters, prec, stream, torch, theta=None, skip=SKIP, fill_times=True,
              nh_stats=False):
    """Iterations timed as CUDA-graph replays (CUDA events); fill launch
    times from an eager run of the same workload (events around each fill;
    with nh_stats, also the sample counts of the largest hypercubes of that
    run's last allocation)."""
    import numpy as np
    from cuvegas_gb300 import _lib as L, runtime
    fills, nhs = [], None
    if fill_times:
        p = runtime.make_params(dim, n_it * iters, iters, skip=skip, n_intervals=NBINS, seed=SEED,
                                precision=prec, flags=L.FLAG_TIME_FILL)
        with runtime.Run(f, p, theta) as r:
            r.iterate(iters)
            fills = list(r.fill_times()[1:])
            if nh_stats:
                nh = r.get(L.BUF_NH)
                nhs = {"max": int(nh.max()), "cubes_ge_1e4": int((nh >= 10_000).sum()),
                       "cubes_ge_1e6": int((nh >= 1_000_000).sum()),
                       "share_of_samples_in_cubes_ge_1e4": float(nh[nh >= 10_000].sum() / nh.sum())}
    p = runtime.make_params(dim, n_it * iters, iters, skip=skip, n_intervals=NBINS, seed=SEED,
                            precision=prec, flags=L.FLAG_GRAPH)
    with runtime.Run(f, p, theta) as r:
        r.iterate(1)          # warm (graph capture, first adaptation): not timed
        r.sync()
        with ClockSampler(torch.cuda.current_device()) as clk:
            it_ms = timed_iterations(r, iters - 1, stream, torch)
        res, it_res, it_sig = r.result()
        st = r.get(L.BUF_STATS)
        info = r.info
    ev = float(st[2, 1:iters].sum())
    return dict(res=res, it_res=it_res, it_sig=it_sig, it_ms=it_ms, fills=fills, evals=ev,
                ms=float(sum(it_ms)), clk=clk.summary(), info=info, nh_stats=nhs)


def time_to_rel(it_res, it_sig, it_ms, skip, target=1e-4, exact=None):
    """Time from the first iteration until the running weighted estimate
    reaches err/|I| <= target (and |I-exact| <= 3 err when exact is known)."""
    sw = swr = 0.0
    t = 0.0
    for i in range(len(it_ms)):
        t += it_ms[i]
        if i < skip:
            continue
        sw += 1.0 / it_sig[i]
        swr += it_res[i] / it_sig[i]
        I, err = swr / sw, 1.0 / math.sqrt(sw)
        if err / abs(I) <= target and (exact is None or abs(I - exact) <= 3 * err):
            return t / 1e3, i + 1, I, err
    return None, None, None, None


def _form_summary(m, iters, exact, prec):
    import numpy as np
    from cuvegas_gb300 import _lib as L
    step_ms = m["ms"] / (iters - 1)
    d = {"value": m["evals"] / (m["ms"] / 1e3), "unit": "evals/s", "ms_per_step": step_ms,
         "result": m["res"].result, "error": m["res"].error, "exact": exact,
         "pull": (m["res"].result - exact) / m["res"].error, "chi2_dof": m["res"].chi2_dof,
         "clocks": m["clk"], "n_cubes": m["info"].n_cubes,
         "dtype": "f32" if prec == L.PREC_FP32 else "f64"}
    t, nit, _, _ = time_to_rel(m["it_res"], m["it_sig"], [0.0] + m["it_ms"], SKIP, exact=exact)
    d["time_to_1e-4_s"] = t
    if m["fills"]:
        fill_ms = float(np.mean(m["fills"]))
        d["fill_ms_mean"] = fill_ms
        d["realloc_refine_ms"] = step_ms - fill_ms
    if m.get("nh_stats"):
        d["fill_ms_per_iteration"] = [round(float(x), 4) for x in m["fills"]]
        d["nh_largest_hypercubes"] = m["nh_stats"]
    return d


def summary_c1(ctx, stream, torch, quick=False, evals=None):
    """C1: Gaussian d=4, 1e6 evals/iteration, 10 iterations, 1024 bins."""
    from cuvegas_gb300 import _lib as L, integrands as I, analytic as A
    n_it = evals or 1_000_000
    f = ctx.integrand(I.GAUSS, 4)
    exact = A.gauss_normalised(4)
    out = {"workload": "gauss-d4-%.0ex10" % n_it, "dim": 4, "evals_per_iteration": n_it,
           "iterations": 10}
    for name, prec in (("chosen", L.PREC_FP32), ("plain", L.PREC_FP64)):
        m = run_timed(f, 4, n_it, 10, prec, stream, torch)
        out[name] = _form_summary(m, 10, exact, prec)
    out["speedup_chosen_vs_plain"] = out["chosen"]["value"] / out["plain"]["value"]
    return out


def summary_c5(ctx, stream, torch, quick=False, evals=None):
    """C5: corner peak d=16, 1e9 evals/iteration, 20 iterations, 1024 bins.
    The chosen form also reports every iteration's fill time and the sample
    counts of its largest hypercubes after adaptation (per-hypercube sums of
    runs that share a hypercube go to FP64 atomics; a warp that lies wholly in
    one hypercube combines its runs first)."""
    from cuvegas_gb300 import _lib as L, integrands as I, analytic as A
    n_it = evals or 1_000_000_000
    th = I.corner_theta(0, 16)
    f = ctx.integrand(I.CORNER, 16, n_params=16)
    exact = A.corner_peak(th)
    out = {"workload": "corner-d16-%.0ex20" % n_it, "dim": 16, "evals_per_iteration": n_it,
           "iterations": 20}
    m = run_timed(f, 16, n_it, 20, L.PREC_FP32, stream, torch, th, nh_stats=True)
    out["chosen"] = _form_summary(m, 20, exact, L.PREC_FP32)
    if m["fills"]:
        fills = m["fills"][1:] if len(m["fills"]) > 2 else m["fills"]
        out["chosen"]["roofline"] = c5_roofline(ctx, n_it, sum(fills) / len(fills),
                                                m["clk"].get("sm_mhz"))
    if not quick:
        # plain: graph-replayed iterations only (no separate fill-timed run)
        m = run_timed(f, 16, n_it, 20, L.PREC_FP64, stream, torch, th, fill_times=False)
        out["plain"] = _form_summary(m, 20, exact, L.PREC_FP64)
        out["speedup_chosen_vs_plain"] = out["chosen"]["value"] / out["plain"]["value"]
    return out


def summary_c3(ctx, stream, torch, quick=False):
    """C3: differentiable mixture d=6, 16 parameters, 1e7 evals/iteration x 15,
    forward + backward; gradient against analytic values and same-seed
    central differences (h = 1e-4)."""
    import numpy as np
    from cuvegas_gb300 import _lib as L, integrands as I, analytic as A, runtime
    from cuvegas_gb300 import autograd as AG
    th = I.mixture_theta(0, 6)
    f = ctx.integrand(I.MIXTURE, 6, n_params=16, has_grad=True)
    out = {"workload": "mixture-d6-1e7x15-grad", "dim": 6, "params": 16,
           "evals_per_iteration": 10_000_000, "iterations": 15}
    exact = A.mixture(th, 6)
    gex = A.mixture_grad(th, 6)
    for name, prec in (("chosen", L.PREC_FP32), ("plain", L.PREC_FP64)):
        p = runtime.make_params(6, 10_000_000 * 15, 15, skip=5, n_intervals=NBINS, seed=SEED,
                                precision=prec)
        # warm-up at the timed iteration size: the same fill variants (tile
        # shape included) are compiled before the timed call
        AG.forward_with_grad(f, runtime.make_params(6, 10_000_000 * 2, 2, skip=1,
                                                    n_intervals=NBINS, precision=prec), th)
        torch.cuda.synchronize()
        with ClockSampler(torch.cuda.current_device()) as clk:
            t0 = time.perf_counter()
            Ival, err, G, g_it, _, res = AG.forward_with_grad(f, p, th)
            dt = time.perf_counter() - t0
        sg = g_it.std(axis=0, ddof=1) / np.sqrt(len(g_it))
        out[name] = {"forward_backward_s": dt, "evals": int(res.tot_nevals),
                     "value": res.tot_nevals / dt, "unit": "evals/s (forward + backward)",
                     "result": Ival, "error": err, "exact": exact,
                     "pull": (Ival - exact) / err, "chi2_dof": res.chi2_dof,
                     "grad_max_err_vs_analytic_rel_to_max": float(
                         np.max(np.abs(G - gex)) / np.max(np.abs(gex))),
                     "grad_max_pull_vs_analytic": float(np.max(np.abs(G - gex) / sg)),
                     "clocks": clk.summary(), "dtype": "f32" if prec == L.PREC_FP32 else "f64"}
    out["speedup_chosen_vs_plain"] = out["plain"]["forward_backward_s"] / out["chosen"]["forward_backward_s"]
    # same-seed central differences of the frozen-state estimator, FP32
    p = runtime.make_params(6, 1_000_000 * 6, 6, skip=3, n_intervals=NBINS, seed=1,
                            precision=L.PREC_FP32)
    _, _, G, _, recs, _ = AG.forward_with_grad(f, p, th, record=True)
    h, worst = 1e-4, 0.0
    for k in range(16):
        tp, tm = th.copy(), th.copy()
        tp[k] += h
        tm[k] -= h
        fd = (AG.replay_estimates(f, p, tp, recs)[0] - AG.replay_estimates(f, p, tm, recs)[0]) / (2 * h)
        worst = max(worst, abs(G[k] - fd) / max(abs(fd), 1e-12))
    out["grad_max_rel_err_vs_fd_h1e-4"] = worst
    return out


def summary_c4(ctx, stream, torch, quick=False, n_plain=32):
    """C4: 512 product-peak integrals of dimension 2..12, 1e4..1e7 evals per
    iteration, 10 iterations, one persistent fill launch per iteration for
    all of them, iterations replayed as a CUDA graph, autotuned tiles; plain
    form = FP64, one cvg_integrate call per instance (first `n_plain`)."""
    import numpy as np
    from cuvegas_gb300 import _lib as L, integrands as I, analytic as A, runtime
    from cuvegas_gb300 import autotune, batch as B
    insts = I.batch_instances(0, 512)
    ppd = [2 * d for d in range(17)]
    block, spt = autotune.tune_batch(ctx, I.PRODPEAK, insts, ppd, L.PREC_FP32)
    with B.Batch(ctx, I.PRODPEAK, insts, ppd, max_it=10, skip=5, seed=SEED,
                 precision=L.PREC_FP32, graph=True, block=block, spt=spt) as b:
        b.iterate(1)
        torch.cuda.synchronize()
        evs = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
        with ClockSampler(torch.cuda.current_device()) as clk:
            evs[0].record(stream)
            b.iterate(9)
            evs[1].record(stream)
            stream.synchronize()
        ms = evs[0].elapsed_time(evs[1])
        res, it_res, it_sig = b.results()
    ev = sum(r.tot_nevals for r in res)
    ev_timed = ev * 0.9          # iterations 2..10 (all instances have ~constant counts)
    pulls, chi2 = [], []
    for r, inst in zip(res, insts):
        ex = A.product_peak(inst["c"], inst["u"])
        pulls.append((r.result - ex) / r.error)
        chi2.append(r.chi2_dof)
    pulls = np.abs(np.array(pulls))
    out = {"workload": "prodpeak-batch512-d2..12", "instances": len(insts)}
    out["chosen"] = {"value": ev_timed / (ms / 1e3), "unit": "evals/s", "ms_per_step": ms / 9,
                     "block": block, "spt": spt, "graph": True,
                     "evals_per_iteration": ev / 10, "clocks": clk.summary(),
                     "frac_within_4sigma": float(np.mean(pulls < 4)),
                     "max_pull": float(pulls.max()), "median_chi2_dof": float(np.median(chi2))}
    # plain form: FP64, one integral per call (the reference's interface
    # shape); each instance runs once untimed first (its fill variant is
    # compiled then), then all are timed
    plist = []
    for i, inst in enumerate(insts[:n_plain]):
        d = inst["dim"]
        fi = ctx.integrand(I.PRODPEAK, d, n_params=2 * d)
        p = runtime.make_params(d, inst["n_eval_it"] * 10, 10, skip=5, n_intervals=NBINS,
                                seed=SEED, precision=L.PREC_FP64, instance=i)
        plist.append((fi, p, inst["theta"]))
        runtime.integrate_once(fi, p, inst["theta"])
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    ev_p = 0
    for fi, p, th in plist:
        r, _, _ = runtime.integrate_once(fi, p, th)
        ev_p += r.tot_nevals
    dt = time.perf_counter() - t0
    out["plain"] = {"value": ev_p / dt, "unit": "evals/s", "instances_timed": n_plain,
                    "note": "FP64, cvg_integrate per instance, JIT and arena warm"}
    out["speedup_chosen_vs_plain"] = out["chosen"]["value"] / out["plain"]["value"]
    return out


def reference_gpu(cases):
    """The reference's own CUDA kernels timed on this GPU: its src/main.cu
    compiled to PTX with the benchmark Gaussian (oracle/ref_build.py, where
    the reference sources are present; the PTX travels with the checkout),
    driven through its iteration sequence -- fill, results, CUB reductions and
    scans, n_h update, map rebuild, refinement and its host reads -- by
    oracle/ref_harness.cu, CUDA events around each iteration.  Informational:
    the bench's reference arm is the CPU restatement."""
    ref_dir = os.path.join(ROOT, "oracle", "_ref")
    src = os.path.join(ROOT, "oracle", "ref_harness.cu")
    exe = os.path.join(ref_dir, "ref_harness")
    missing = [d for d, *_ in cases
               if not os.path.exists(os.path.join(ref_dir, "ref_main_d%d_w01.ptx" % d))]
    if missing:
        return {"unavailable": "reference PTX for d=%s not present (built by oracle/ref_build.py "
                               "where the reference sources are)" % missing}
    if not os.path.exists(exe) or os.path.getmtime(exe) < os.path.getmtime(src):
        r = subprocess.run(["nvcc", "-O2", "-std=c++17", "-gencode",
                            "arch=compute_103a,code=sm_103a", "-o", exe, src],
                           capture_output=True, text=True)
        if r.returncode != 0:
            return {"unavailable": "harness build failed: " + r.stderr[-300:]}
    out = {"how": "reference src/main.cu kernels (PTX) driven by oracle/ref_harness.cu, CUDA "
                  "events per iteration (its host reads included), first 2 iterations left out",
           "dtype": "f64"}
    for dim, n_it, iters, name in cases:
        ptx = os.path.join(ref_dir, "ref_main_d%d_w01.ptx" % dim)
        with ClockSampler(0) as clk:
            r = subprocess.run([exe, ptx, str(dim), str(n_it), str(NBINS), str(iters), ref_dir,
                                "time"], capture_output=True, text=True)
        if r.returncode != 0:
            out[name] = {"unavailable": "harness exited %d: %s" % (r.returncode, r.stderr[-300:])}
            continue
        rows = [tuple(float(v) for v in re.findall(r"samples (\d+) ms ([\d.]+)", line)[0])
                for line in r.stdout.splitlines() if line.startswith("iteration")]
        warm = rows[2:] if len(rows) > 3 else rows
        evals = sum(s for s, _ in warm)
        ms = sum(t for _, t in warm)
        out[name] = {"value": evals / (ms * 1e-3), "unit": "evals/s",
                     "ms_per_iteration": ms / len(warm), "iterations_timed": len(warm),
                     "evals_per_iteration": n_it, "clocks": clk.summary()}
    return out


def run_ours(args):
    import numpy as np
    import torch
    rank, world, local = _dist()
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    from cuvegas_gb300 import _build, _lib as L, replicas, runtime, integrands as I
    from cuvegas_gb300 import analytic as A, shard
    _build.build()
    stream = torch.cuda.Stream(device=local)
    torch.cuda.set_stream(stream)
    ctx = runtime.Context(local, stream=C_stream(stream))
    f = ctx.integrand(I.GAUSS, DIM)
    exact = A.gauss_normalised(DIM)
    steps, warm = args.steps, args.warmup
    split = args.mode == "split" and world > 1

    def barrier():
        torch.cuda.synchronize()
        if world > 1:
            torch.distributed.barrier()

    def measure(prec, n_it):
        p = runtime.make_params(DIM, n_it * (warm + steps), warm + steps,
                                skip=min(SKIP, warm + steps - 1), n_intervals=NBINS,
                                seed=SEED + (0 if split else rank), precision=prec,
                                flags=L.FLAG_TIME_FILL,
                                instance=0 if split else replicas.instance_id(rank))
        with runtime.Run(f, p) as r:
            target = r
            if split:
                target = shard.ShardedRun(f, p, run=r)
            target.iterate(warm)
            r.sync()
            r.fill_times()
            barrier()
            with ClockSampler(local) as clk:
                t0 = time.perf_counter()
                it_ms = timed_iterations(target, steps, stream, torch)
                wall = time.perf_counter() - t0
            fills = r.fill_times()
            st = r.get(L.BUF_STATS)
            info = r.info
        # samples of the iterations: in a split run each rank filled its part
        # of these; the whole job's evaluations are counted once
        evals = float(st[2, warm:warm + steps].sum())
        ms = float(sum(it_ms))
        return dict(evals=evals, ms=ms, wall=wall, fills=fills, clk=clk.summary(), info=info,
                    samples=st[2, warm:warm + steps])

    # warm the JIT cache for both forms
    for prec in (L.PREC_FP32, L.PREC_FP64):
        with runtime.Run(f, runtime.make_params(DIM, 4 * 100000, 4, n_intervals=NBINS,
                                                precision=prec)) as r:
            r.iterate(4)
            r.sync()

    chosen = measure(L.PREC_FP64 if args.form == "plain" else L.PREC_FP32, N_IT)
    # slowest rank's timed region; all ranks' evaluations (a split run's
    # evaluations are the job's once, not once per rank)
    ms_all, ev_all = replicas.reduce_timing(chosen["ms"], chosen["evals"], device="cuda")
    if split:
        ev_all = chosen["evals"]
    value = ev_all / (ms_all / 1e3)

    extra = {}
    full = rank == 0 and not args.quick and args.form == "chosen"

    # roofline of the fill kernel (chosen form)
    fills = chosen["fills"]
    roof = None
    if rank == 0 and len(fills) and args.form == "chosen":
        mean_ms = float(np.mean(fills))
        evals_per_launch = float(np.mean(chosen["samples"])) / (world if split else 1)
        roof = fill_roofline(ctx, evals_per_launch, mean_ms, chosen["clk"].get("sm_mhz"))
        roof["kernel"] = "cvg_fill_entry (FP32, d=8, 1024 bins)"
        roof["fill_share_of_step"] = mean_ms / (chosen["ms"] / steps)
        tr = profile_value("fill_gauss_d8_traffic.txt", "dram_bytes_per_eval")
        if tr:
            roof["traffic"] = tr * evals_per_launch   # ncu DRAM bytes per evaluation x evaluations
            roof["traffic_note"] = ("ncu dram__bytes_read+write of the fill at 3e7 evals, per "
                                    "evaluation, scaled to this launch; HBM share %.1f%% of %.0f GB/s"
                                    % (100 * roof["traffic"] / (mean_ms * 1e-3) / 1e9 / HBM_GBS,
                                       HBM_GBS))

    if full:
        plain = measure(L.PREC_FP64, N_IT)
        pf = float(np.mean(plain["fills"])) if len(plain["fills"]) else None
        extra["plain"] = {"value": plain["evals"] / (plain["ms"] / 1e3), "unit": "evals/s",
                          "ms_per_step": plain["ms"] / steps, "dtype": "f64",
                          "fill_ms_mean": pf, "clocks": plain["clk"]}
        if pf:
            extra["plain"]["roofline"] = plain_roofline(ctx, float(np.mean(plain["samples"])), pf)
        sweep = (100_000, 300_000, 1_000_000, 3_000_000, 10_000_000, 30_000_000, 100_000_000)
        t32 = tt_sweep(f, L.PREC_FP32, exact, sweep)
        t64 = tt_sweep(f, L.PREC_FP64, exact, sweep)
        extra["time_to_1e-4"] = {
            "definition": "fastest whole cvg_integrate call (20 iterations, skip 5) over a sweep of "
                          "evaluations per iteration whose final err/|I| <= 1e-4 and "
                          "|I - exact| <= 3 err",
            "chosen_s": t32["time_s"], "plain_s": t64["time_s"], "chosen": t32, "plain": t64}
        extra["speedup_chosen_vs_plain"] = {
            "evals_per_s": value / extra["plain"]["value"],
            "time_to_1e-4": (t64["time_s"] / t32["time_s"]
                             if t32["time_s"] and t64["time_s"] else None)}

    # end to end through the C ABI: host params in, host result out
    e2e = None
    if full:
        p = runtime.make_params(DIM, N_IT * ITERS, ITERS, skip=SKIP, n_intervals=NBINS,
                                seed=SEED, precision=L.PREC_FP32, flags=L.FLAG_GRAPH)
        runtime.integrate_once(f, p)              # JIT and device arena warm
        t0 = time.perf_counter()
        res, _, _ = runtime.integrate_once(f, p)
        dt = time.perf_counter() - t0
        ctx.trim()                                # free the kept arena: this call allocates
        t0 = time.perf_counter()
        res_c, _, _ = runtime.integrate_once(f, p)
        dt_c = time.perf_counter() - t0
        h2d = 8 * DIM * (NBINS + 1)                # initial grid
        d2h = 8 * 3 * ITERS + 64 + 4               # per-iteration stats, sums, status
        e2e = {"value": res.tot_nevals / dt, "unit": "evals/s",
               "h2d_bytes_per_step": h2d / ITERS, "d2h_bytes_per_step": d2h / ITERS,
               "call": "cvg_integrate", "wall_s": dt, "result": res.result, "error": res.error,
               "arena": "warm: the context keeps the device arena of the previous call "
                        "(cvg_context_trim frees it)",
               "cold_arena": {"value": res_c.tot_nevals / dt_c, "wall_s": dt_c,
                              "note": "arena freed before the call: device allocation inside"}}

    cpu = None
    if full and not args.no_cpu:
        n_cpu = N_IT          # the workload's own size per iteration, 3 iterations
        rate, tot, dt = cpu_oracle_rate(n_cpu, 3)
        cpu = {"value": rate, "unit": "evals/s", "cores": os.cpu_count(), "kind": "port",
               "sample": "3 VEGAS+ iterations of the same d=8 Gaussian workload at %d "
                         "evals/iteration, FP64 CPU oracle on all host cores, %d evals in %.1f s"
                         % (n_cpu, tot, dt)}

    if full and not args.no_configs:
        cfgs = {}
        for name, fn in (("c1", summary_c1), ("c3", summary_c3), ("c4", summary_c4),
                         ("c5", summary_c5)):
            try:
                t0 = time.perf_counter()
                cfgs[name] = fn(ctx, stream, torch)
                cfgs[name]["bench_s"] = time.perf_counter() - t0
            except Exception as e:          # report, do not lose the headline line
                cfgs[name] = {"error": "%s: %s" % (type(e).__name__, e)}
        extra["configs"] = cfgs
        extra["reference_gpu"] = reference_gpu([(8, N_IT, 6, "c2"), (4, 1_000_000, 10, "c1")])
        rg = extra["reference_gpu"].get("c2", {})
        if "value" in rg:
            extra["reference_gpu"]["plain_over_reference_c2"] = extra["plain"]["value"] / rg["value"]
            extra["reference_gpu"]["chosen_over_reference_c2"] = value / rg["value"]

    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": "evals/s", "n_gpus": world,
                "steps": steps, "warmup": warm, "ms_per_step": ms_all / steps,
                "higher_is_better": True, "scaling": "strong" if split else "weak",
                "vs_baseline": None, "dtype": "f32", "data": "synthetic",
                "config": {"workload": WORKLOAD, "dim": DIM, "evals_per_iteration": N_IT,
                           "nbins": NBINS, "alpha": 0.5, "beta": 0.75, "seed": SEED,
                           "n_strat": chosen["info"].n_strat, "n_cubes": chosen["info"].n_cubes,
                           "parallelism": ("sample-split" if split else "replicas")
                           if world > 1 else "single",
                           "l2": "per-hypercube state %.0f MB > L2 (129 MB), streamed every "
                                 "iteration" % (chosen["info"].n_cubes * 36 / 1e6)},
                "gpu_launches": LAUNCHES_PER_IT * steps,
                "iteration_samples": [int(x) for x in chosen["samples"]],
                "clocks": chosen["clk"], "roofline": roof, "cpu_baseline": cpu, "e2e": e2e}
        line.update(extra)
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


def run_workload(args):
    """One JSON line for another benchmark configuration."""
    import torch
    from cuvegas_gb300 import _build, runtime
    _build.build()
    torch.cuda.set_device(0)
    stream = torch.cuda.Stream(device=0)
    torch.cuda.set_stream(stream)
    ctx = runtime.Context(0, stream=C_stream(stream))
    fn = {"c1": summary_c1, "c3": summary_c3, "c4": summary_c4, "c5": summary_c5}[args.workload]
    out = {"n_gpus": 1, "data": "synthetic"}
    kw = {"evals": args.evals} if args.workload in ("c1", "c5") and args.evals else {}
    out.update(fn(ctx, stream, torch, quick=args.quick, **kw))
    if args.workload == "c1" and not args.no_cpu:
        import numpy as np
        from oracle import pyoracle as Po
        t0 = time.perf_counter()
        u, _ = Po.uniforms(Po.U_PHILOX_F64, seed=0)
        o = Po.integrate(Po.F_GAUSS, 4, 1_000_000 * 10, 10, theta=np.array([0.5, 0.1]),
                         skip=5, u=u)
        dt = time.perf_counter() - t0
        out["cpu_baseline"] = {"value": o["tot_nevals"] / dt, "unit": "evals/s",
                               "cores": os.cpu_count(), "kind": "port",
                               "sample": "the whole C1 run (10 x 1e6), FP64 oracle",
                               "result": o["result"], "error": o["error"]}
    print(json.dumps(out), flush=True)


def C_stream(stream):
    import ctypes
    return ctypes.c_void_p(stream.cuda_stream)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=17)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--mode", default="replicas", choices=["replicas", "split"],
                    help="N > 1: independent replicas, or one integral split across ranks")
    ap.add_argument("--quick", action="store_true", help="headline number only")
    ap.add_argument("--form", default="chosen", choices=["chosen", "plain"],
                    help="form of the headline measurement (plain: FP64, for profiling)")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-configs", action="store_true",
                    help="leave out the C1/C3/C4/C5 summaries and the reference-kernel timing")
    ap.add_argument("--workload", default="c2", choices=["c1", "c2", "c3", "c4", "c5"],
                    help="c2 is the headline line; the others print their own line")
    ap.add_argument("--evals", type=int, default=0,
                    help="evals/iteration override (profiling runs on a smaller case)")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.evals:
        global N_IT
        N_IT = args.evals
    if args.impl == "reference":
        run_reference(args)
    elif args.workload != "c2":
        run_workload(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
