#!/usr/bin/env python
"""Benchmark of the VEGAS+ iteration loop on one GB300 (replicas on N GPUs).

Workload (default): Gaussian family, d=8, width 0.1, centre 0.5, 1e8 integrand
evaluations per iteration, 1024 bins per dimension, alpha=0.5, beta=0.75,
seed 0, 20 iterations -- FP32 evaluation with Kahan-compensated f/f^2
accumulation and FP64 mean/variance/grid ("chosen" form).  A step is one
VEGAS+ iteration: fill (sample, map, integrand, accumulate), hypercube
reallocation, grid refinement.

Printed JSON line (rank 0):
  value      evals/s over the K timed iterations, state resident in HBM
  e2e        evals/s of whole integrations through the C ABI with host
             parameters in and host results out (cvg_integrate)
  plain      the same workload in the plain FP64 form
  roofline   fill kernel against the lowest of its per-pipe ceilings (FP32
             ops, ex2, Philox4x32-10 calls per evaluation), each peak from a
             live microbenchmark of the same GPU; the sampler binds, so
             achieved = Philox calls per launch / CUDA-event launch time
  cpu_baseline  the CPU oracle (FP64, OpenMP, all host cores) on a bounded
             sample of the same workload
`--impl reference` times the reference's computation on the host cores (the
CPU restatement of the reference loop in oracle/, FP64).
"""
import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

DIM, N_IT, NBINS, ITERS, SEED = 8, 100_000_000, 1024, 20, 0
def _hbm_gbs():
    """Measured copy bandwidth of the GB300s (MEASURED_PEAKS.json)."""
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return float(json.load(f)["hbm_gbs"])
    except (OSError, ValueError, KeyError):
        return 6800.0                      # fallback figure of one earlier GB300 measurement


HBM_GBS = _hbm_gbs()
FLOPS_PER_EVAL = 11 * DIM + 4          # algorithmic FP32 ops per evaluation (map 7/dim, integrand 4/dim, 4)
SFU_PER_EVAL = DIM                     # one exp per dimension
PHILOX_PER_EVAL = (DIM + 3) // 4       # Philox4x32-10 calls per evaluation (4 uniforms per call)
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


def fill_roofline(ctx, evals_per_launch, mean_ms, fp_eval, sfu_eval, philox_eval):
    """Compute roofline of a fill launch: evaluations/s are bounded by each
    pipe alone -- FP32 ops, special-function (exp) ops, Philox calls of the
    sampler -- with peaks measured live on this GPU (cvg_measure_peak).  The
    binding pipe is reported; frac = measured evals/s / that pipe's bound."""
    p_fp32 = ctx.measure_peak(0) / 2.0         # T FP32 instructions/s (FMA = 2 flops)
    p_sfu = ctx.measure_peak(8)                # T ex2/s
    p_philox = ctx.measure_peak(9)             # T Philox calls/s
    rate = evals_per_launch / (mean_ms * 1e-3)
    ceil = {"fp32": (p_fp32 * 1e12 / fp_eval, fp_eval, p_fp32, "T FP32 ops/s"),
            "sfu": (p_sfu * 1e12 / max(sfu_eval, 1e-9), sfu_eval, p_sfu, "T ex2/s"),
            "sampler": (p_philox * 1e12 / philox_eval, philox_eval, p_philox, "T Philox calls/s")}
    bound = min(ceil, key=lambda k: ceil[k][0])
    evals_max, per_eval, peak, unit = ceil[bound]
    achieved = rate * per_eval / 1e12
    return {"bound": bound, "achieved": achieved, "peak": peak, "unit": unit,
            "frac": achieved / peak, "traffic": None,
            "ceilings_evals_per_s": {k: v[0] for k, v in ceil.items()},
            "evals_per_s_fill": rate, "fill_ms_mean": mean_ms,
            "evals_per_launch": evals_per_launch,
            "per_eval": {"fp32_ops": fp_eval, "ex2": sfu_eval, "philox_calls": philox_eval},
            "peak_source": "live microbenchmarks of this GPU (cvg_measure_peak kinds 0, 8, 9); "
                           "MEASURED_PEAKS.json holds HBM and bf16 figures only"}


def _ncu_traffic():
    """DRAM bytes per evaluation of the fill from the committed ncu summary (or None)."""
    p = os.path.join(ROOT, "profiles", "fill_gauss_d8_traffic.txt")
    try:
        for line in open(p):
            if line.startswith("dram_bytes_per_eval="):
                return float(line.split("=", 1)[1])
    except OSError:
        pass
    return None


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
    n_it = 10_000_000         # bounded sample per step (same d, bins, integrand)
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
    sample = "%d VEGAS+ iterations of the d=8 Gaussian workload at %d evals/iteration " \
             "(1024 bins), FP64" % (steps, n_it)
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": "evals/s",
            "n_gpus": args.gpus, "steps": steps, "warmup": warm,
            "ms_per_step": 1e3 * el / steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": WORKLOAD, "dim": DIM, "evals_per_iteration": n_it,
                       "nbins": NBINS, "implementation": "CPU restatement of the reference "
                       "VEGAS+ loop (oracle/vegas_oracle.c), OpenMP over hypercubes"},
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


def run_ours(args):
    import numpy as np
    import torch
    rank, world, local = _dist()
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    from cuvegas_gb300 import _build, _lib as L, replicas, runtime, integrands as I
    from cuvegas_gb300 import analytic as A
    _build.build()
    stream = torch.cuda.Stream(device=local)
    ctx = runtime.Context(local, stream=C_stream(stream))
    f = ctx.integrand(I.GAUSS, DIM)
    exact = A.gauss_normalised(DIM)
    steps, warm = args.steps, args.warmup
    skip = 5

    def barrier():
        torch.cuda.synchronize()
        if world > 1:
            torch.distributed.barrier()

    def measure(prec, n_it):
        p = runtime.make_params(DIM, n_it * (warm + steps), warm + steps, skip=min(skip, warm + steps - 1),
                                n_intervals=NBINS, seed=SEED + rank, precision=prec,
                                flags=L.FLAG_TIME_FILL, instance=replicas.instance_id(rank))
        with runtime.Run(f, p) as r:
            r.iterate(warm)
            r.sync()
            r.fill_times()
            barrier()
            with ClockSampler(local) as clk:
                t0 = time.perf_counter()
                it_ms = timed_iterations(r, steps, stream, torch)
                wall = time.perf_counter() - t0
            fills = r.fill_times()
            st = r.get(L.BUF_STATS)
            info = r.info
        evals = float(st[2, warm:warm + steps].sum())
        ms = float(sum(it_ms))
        return dict(evals=evals, ms=ms, wall=wall, fills=fills, clk=clk.summary(), info=info,
                    samples=st[2, warm:warm + steps])

    def convergence(prec, n_it, iters=ITERS):
        p = runtime.make_params(DIM, n_it * iters, iters, skip=skip, n_intervals=NBINS,
                                seed=SEED + rank, precision=prec, instance=rank)
        with runtime.Run(f, p) as r:
            it_ms = timed_iterations(r, iters, stream, torch)
            res, it_res, it_sig = r.result()
        t, nit, Ival, err = time_to_rel(it_res, it_sig, it_ms, skip, exact=exact)
        return dict(time_to_1e4_s=t, iterations=nit, result=res.result, error=res.error,
                    chi2_dof=res.chi2_dof, exact=exact, pull=(res.result - exact) / res.error,
                    total_s=sum(it_ms) / 1e3)

    # warm the JIT cache for both forms
    for prec in (L.PREC_FP32, L.PREC_FP64):
        with runtime.Run(f, runtime.make_params(DIM, 4 * 100000, 4, n_intervals=NBINS,
                                                precision=prec)) as r:
            r.iterate(4)
            r.sync()

    chosen = measure(L.PREC_FP32, N_IT)
    # slowest rank's timed region, all ranks' evaluations
    ms_all, ev_all = replicas.reduce_timing(chosen["ms"], chosen["evals"], device="cuda")
    value = ev_all / (ms_all / 1e3)

    extra = {}
    if rank == 0 and not args.quick:
        plain = measure(L.PREC_FP64, N_IT)
        extra["plain"] = {"value": plain["evals"] / (plain["ms"] / 1e3), "unit": "evals/s",
                          "ms_per_step": plain["ms"] / steps, "dtype": "f64",
                          "fill_ms_mean": float(np.mean(plain["fills"])) if len(plain["fills"]) else None}
        conv32 = convergence(L.PREC_FP32, N_IT)
        conv64 = convergence(L.PREC_FP64, N_IT)
        extra["time_to_1e-4"] = {"chosen_s": conv32["time_to_1e4_s"], "plain_s": conv64["time_to_1e4_s"],
                                 "chosen": conv32, "plain": conv64}
        extra["speedup_chosen_vs_plain"] = {
            "evals_per_s": value / extra["plain"]["value"],
            "time_to_1e-4": (conv64["time_to_1e4_s"] / conv32["time_to_1e4_s"]
                             if conv32["time_to_1e4_s"] and conv64["time_to_1e4_s"] else None)}

    # roofline of the fill kernel (chosen form)
    fills = chosen["fills"]
    roof = None
    if rank == 0 and len(fills):
        mean_ms = float(np.mean(fills))
        evals_per_launch = float(np.mean(chosen["samples"]))
        roof = fill_roofline(ctx, evals_per_launch, mean_ms, FLOPS_PER_EVAL, SFU_PER_EVAL,
                             PHILOX_PER_EVAL)
        roof["kernel"] = "cvg_fill_entry (FP32, d=8, 1024 bins)"
        roof["fill_share_of_step"] = mean_ms / (chosen["ms"] / steps)
        tr = _ncu_traffic()
        if tr:
            roof["traffic"] = tr * evals_per_launch   # ncu DRAM bytes per evaluation x evaluations
            roof["traffic_note"] = ("ncu dram__bytes_read+write of the fill at 3e7 evals, per "
                                    "evaluation, scaled to this launch; HBM share %.1f%% of %.0f GB/s"
                                    % (100 * roof["traffic"] / (mean_ms * 1e-3) / 1e9 / HBM_GBS,
                                       HBM_GBS))

    # end to end through the C ABI: host params in, host result out
    e2e = None
    if rank == 0 and not args.quick:
        p = runtime.make_params(DIM, N_IT * ITERS, ITERS, skip=skip, n_intervals=NBINS,
                                seed=SEED, precision=L.PREC_FP32, flags=L.FLAG_GRAPH)
        runtime.integrate_once(f, p)              # allocator / JIT warm
        t0 = time.perf_counter()
        res, _, _ = runtime.integrate_once(f, p)
        dt = time.perf_counter() - t0
        h2d = 8 * DIM * (NBINS + 1)                # initial grid
        d2h = 8 * 3 * ITERS + 64 + 4               # per-iteration stats, sums, status
        e2e = {"value": res.tot_nevals / dt, "unit": "evals/s",
               "h2d_bytes_per_step": h2d / ITERS, "d2h_bytes_per_step": d2h / ITERS,
               "call": "cvg_integrate", "wall_s": dt, "result": res.result, "error": res.error}

    cpu = None
    if rank == 0 and not args.quick and not args.no_cpu:
        n_cpu = N_IT          # the workload's own size per iteration, 3 iterations
        rate, tot, dt = cpu_oracle_rate(n_cpu, 3)
        cpu = {"value": rate, "unit": "evals/s", "cores": os.cpu_count(), "kind": "port",
               "sample": "3 VEGAS+ iterations of the same d=8 Gaussian workload at %d "
                         "evals/iteration, FP64 CPU oracle on all host cores, %d evals in %.1f s"
                         % (n_cpu, tot, dt)}

    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": "evals/s", "n_gpus": world,
                "steps": steps, "warmup": warm, "ms_per_step": ms_all / steps,
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
                "dtype": "f32", "data": "synthetic",
                "config": {"workload": WORKLOAD, "dim": DIM, "evals_per_iteration": N_IT,
                           "nbins": NBINS, "alpha": 0.5, "beta": 0.75, "seed": SEED,
                           "n_strat": chosen["info"].n_strat, "n_cubes": chosen["info"].n_cubes,
                           "parallelism": "replicas" if world > 1 else "single",
                           "l2": "per-hypercube state %.0f MB > L2 (129 MB), streamed every "
                                 "iteration" % (chosen["info"].n_cubes * 36 / 1e6)},
                "gpu_launches": LAUNCHES_PER_IT * steps,
                "clocks": chosen["clk"], "roofline": roof, "cpu_baseline": cpu, "e2e": e2e}
        line.update(extra)
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


def run_workload(args):
    """Lines for the other benchmark configurations (one JSON line each)."""
    import numpy as np
    import torch
    from cuvegas_gb300 import _build, _lib as L, replicas, runtime, integrands as I
    from cuvegas_gb300 import analytic as A
    _build.build()
    torch.cuda.set_device(0)
    stream = torch.cuda.Stream(device=0)
    ctx = runtime.Context(0, stream=C_stream(stream))
    out = {"workload": args.workload, "n_gpus": 1, "data": "synthetic"}

    def run_timed(f, dim, n_it, iters, prec, theta=None, skip=5):
        # iterations timed as CUDA-graph replays; fill launch times from an
        # eager run of the same workload (events around each fill)
        p = runtime.make_params(dim, n_it * iters, iters, skip=skip, n_intervals=1024, seed=0,
                                precision=prec, flags=L.FLAG_TIME_FILL)
        with runtime.Run(f, p, theta) as r:
            r.iterate(iters)
            fills = r.fill_times()[1:]
        p = runtime.make_params(dim, n_it * iters, iters, skip=skip, n_intervals=1024, seed=0,
                                precision=prec, flags=L.FLAG_GRAPH)
        with runtime.Run(f, p, theta) as r:
            r.iterate(1)          # warm (graph capture, first adaptation): not timed
            r.sync()
            with ClockSampler(0) as clk:
                it_ms = timed_iterations(r, iters - 1, stream, torch)
            res, it_res, it_sig = r.result()
            st = r.get(L.BUF_STATS)
            info = r.info
        ev = float(st[2, 1:iters].sum())
        return dict(res=res, it_res=it_res, it_sig=it_sig, it_ms=it_ms, fills=fills, evals=ev,
                    ms=float(sum(it_ms)), clk=clk.summary(), info=info, samples=st[2])

    if args.workload in ("c1", "c5"):
        if args.workload == "c1":
            dim, n_it, iters, src, th, P = 4, args.evals or 1_000_000, 10, I.GAUSS, None, 0
            exact = A.gauss_normalised(4)
            forms = [("plain", L.PREC_FP64), ("chosen", L.PREC_FP32)]
        else:
            dim, n_it, iters, src = 16, args.evals or 1_000_000_000, 20, I.CORNER
            th, P = I.corner_theta(0, 16), 16
            exact = A.corner_peak(th)
            forms = [("chosen", L.PREC_FP32), ("plain", L.PREC_FP64)]
        f = ctx.integrand(src, dim, n_params=P)
        for name, prec in forms:
            if name == "plain" and args.workload == "c5" and args.quick:
                continue
            m = run_timed(f, dim, n_it, iters, prec, th)
            t, nit, _, _ = time_to_rel(m["it_res"], m["it_sig"], [0.0] + m["it_ms"], 5,
                                       exact=exact)
            fill_ms = float(np.mean(m["fills"]))
            step_ms = m["ms"] / (iters - 1)
            d = {"value": m["evals"] / (m["ms"] / 1e3), "unit": "evals/s", "ms_per_step": step_ms,
                 "fill_ms_mean": fill_ms, "realloc_refine_ms": step_ms - fill_ms,
                 "result": m["res"].result, "error": m["res"].error, "exact": exact,
                 "pull": (m["res"].result - exact) / m["res"].error, "chi2_dof": m["res"].chi2_dof,
                 "time_to_1e-4_s": t, "clocks": m["clk"], "n_cubes": m["info"].n_cubes,
                 "dtype": "f32" if prec == L.PREC_FP32 else "f64"}
            # reallocation traffic: ~72 algorithmic bytes per hypercube and iteration
            d["realloc_algorithmic_gbs"] = 72.0 * m["info"].n_cubes / ((step_ms - fill_ms) * 1e-3) / 1e9
            out[name] = d
        if args.workload == "c1" and not args.no_cpu:
            rate_t = time.perf_counter()
            from oracle import pyoracle as Po
            u, _ = Po.uniforms(Po.U_PHILOX_F64, seed=0)
            o = Po.integrate(Po.F_GAUSS, 4, n_it * iters, iters, theta=np.array([0.5, 0.1]),
                             skip=5, u=u)
            dt = time.perf_counter() - rate_t
            out["cpu_baseline"] = {"value": o["tot_nevals"] / dt, "unit": "evals/s",
                                   "cores": os.cpu_count(), "kind": "port",
                                   "sample": "the whole C1 run (10 x 1e6), FP64 oracle",
                                   "result": o["result"], "error": o["error"]}
        if "plain" in out:
            out["speedup_chosen_vs_plain"] = out["chosen"]["value"] / out["plain"]["value"]
    elif args.workload == "c3":
        from cuvegas_gb300 import autograd as AG
        th = I.mixture_theta(0, 6)
        f = ctx.integrand(I.MIXTURE, 6, n_params=16, has_grad=True)
        for name, prec in (("chosen", L.PREC_FP32), ("plain", L.PREC_FP64)):
            p = runtime.make_params(6, 10_000_000 * 15, 15, skip=5, n_intervals=1024, seed=0,
                                    precision=prec)
            # warm-up at the timed iteration size: the same fill variants
            # (tile shape included) are compiled before the timed call
            AG.forward_with_grad(f, runtime.make_params(6, 10_000_000 * 2, 2, skip=1,
                                                        n_intervals=1024, precision=prec), th)
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            Ival, err, G, g_it, _, res = AG.forward_with_grad(f, p, th)
            dt = time.perf_counter() - t0
            gex = A.mixture_grad(th, 6)
            sg = g_it.std(axis=0, ddof=1) / np.sqrt(len(g_it))
            out[name] = {"forward_backward_s": dt, "result": Ival, "error": err,
                         "exact": A.mixture(th, 6), "chi2_dof": res.chi2_dof,
                         "grad_max_err_vs_analytic_rel_to_max": float(
                             np.max(np.abs(G - gex)) / np.max(np.abs(gex))),
                         "grad_max_pull_vs_analytic": float(np.max(np.abs(G - gex) / sg)),
                         "evals": int(res.tot_nevals)}
        # same-seed finite differences of the frozen-state estimator, FP32
        p = runtime.make_params(6, 1_000_000 * 6, 6, skip=3, n_intervals=1024, seed=1,
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
    elif args.workload == "c4":
        from cuvegas_gb300 import autotune, batch as B
        insts = I.batch_instances(0, 512)
        ppd = [2 * d for d in range(17)]
        block, spt = autotune.tune_batch(ctx, I.PRODPEAK, insts, ppd, L.PREC_FP32)
        with B.Batch(ctx, I.PRODPEAK, insts, ppd, max_it=10, skip=5, seed=0,
                     precision=L.PREC_FP32, graph=True, block=block, spt=spt) as b:
            b.iterate(1)
            torch.cuda.synchronize()
            evs = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
            with ClockSampler(0) as clk:
                evs[0].record(stream)
                b.iterate(9)
                evs[1].record(stream)
                stream.synchronize()
            ms = evs[0].elapsed_time(evs[1])
            res, it_res, it_sig = b.results()
        ev = sum(r.tot_nevals for r in res)
        ev_timed = ev * 0.9          # iterations 2..10 (all instances have ~constant counts)
        pulls = []
        for r, inst in zip(res, insts):
            ex = A.product_peak(inst["c"], inst["u"])
            pulls.append((r.result - ex) / r.error)
        pulls = np.abs(np.array(pulls))
        out["chosen"] = {"value": ev_timed / (ms / 1e3), "unit": "evals/s", "ms_per_step": ms / 9,
                         "block": block, "spt": spt, "graph": True, "instances": len(insts),
                         "evals_per_iteration": ev / 10, "clocks": clk.summary(),
                         "frac_within_4sigma": float(np.mean(pulls < 4)),
                         "max_pull": float(pulls.max())}
        # plain form: FP64, one integral per call (the reference's interface shape)
        # compile every dimension's fill first, in both tile shapes (a run
        # picks warp tiles when its iterations are large), so no JIT is timed
        saved = os.environ.get("CVG_FILL_WARP_TILES")
        for wt in ("0", "1"):
            os.environ["CVG_FILL_WARP_TILES"] = wt
            for d in range(2, 13):
                fi = ctx.integrand(I.PRODPEAK, d, n_params=2 * d)
                runtime.integrate_once(fi, runtime.make_params(d, 4 * 4000, 4, skip=1,
                                                               n_intervals=1024,
                                                               precision=L.PREC_FP64),
                                       np.ones(2 * d))
        if saved is None:
            del os.environ["CVG_FILL_WARP_TILES"]
        else:
            os.environ["CVG_FILL_WARP_TILES"] = saved
        t0 = time.perf_counter()
        ev_p = 0
        n_plain = 64
        for i, inst in enumerate(insts[:n_plain]):
            d = inst["dim"]
            fi = ctx.integrand(I.PRODPEAK, d, n_params=2 * d)
            p = runtime.make_params(d, inst["n_eval_it"] * 10, 10, skip=5, n_intervals=1024,
                                    seed=0, precision=L.PREC_FP64, instance=i)
            r, _, _ = runtime.integrate_once(fi, p, inst["theta"])
            ev_p += r.tot_nevals
        dt = time.perf_counter() - t0
        out["plain"] = {"value": ev_p / dt, "unit": "evals/s", "instances_timed": n_plain,
                        "note": "FP64, cvg_integrate per instance (JIT cached after first use)"}
        out["speedup_chosen_vs_plain"] = out["chosen"]["value"] / out["plain"]["value"]
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
    ap.add_argument("--quick", action="store_true", help="headline number only")
    ap.add_argument("--no-cpu", action="store_true")
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
