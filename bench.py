#!/usr/bin/env python
"""Headline benchmark of the GB300 Monte Carlo engine.

Workload (the Bates strip of the baseline configurations): Bates model =
Heston(kappa 2, theta 0.05, sigma 0.9 [Feller violated], rho -0.6, v0 0.05) +
Merton jumps (lambda 0.5, mu -0.1, delta 0.15); SchemeNCI; European calls with
64 strikes uniform on [60, 140] x 8 maturities {0.25, 0.5, 1, 1.5, 2, 2.5, 3, 4};
200 steps per year; 2^22 paths; GreekMode::Full (CRN delta, gamma, vega, theta,
rho, vanna, charm: 7 scenarios per path, of which the two rho scenarios of these
European options are derived from the base path); S0 100, r 0.02, q 0, seed 42.
One step = pricing the whole strip = 8 pricing requests (one per maturity, as
the reference prices one maturity per MonteCarloPricer::calculate call).

Metric: paths*steps/s = path-steps of the workload (paths x time steps, each with
its 7 Full-Greek scenarios) per second.
  value -- device time of the 8 requests (CUDA events on the launching stream,
           inputs resident, L2 flushed between steps)
  e2e   -- the same through the C ABI (myql_mc_price) with pinned host strike
           and result buffers, host<->device copies inside the timed region
The reference arm (--impl reference) times the reference's Monte Carlo
algorithm on the host cores: the FP64 C restatement of the reference (the
reference's own headers need Boost and cannot be built on the GPU machine) at the
reference's release flags, on a bounded sample of the same workload.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

MATURITIES = [0.25, 0.5, 1.0, 1.5, 2.0, 2.5, 3.0, 4.0]
STRIKES = list(60.0 + 80.0 * np.arange(64) / 63.0)
PATHS = 1 << 22
STEPS_PER_YEAR = 200
SEED = 42
N_SCENARIOS = 7      # base, v0 up/down, T up/down, r up/down
N_SIMULATED = 5      # the r-bumped scenarios of a European are the base path shifted by (r' - r) T
# algorithmic work per simulated path-step of this workload (Bates, NCI):
# inverse normal 42 ALU + 1 XU, Poisson inversion 58 ALU + 3 XU, NCI Hermite
# lookup with its uniform 46 ALU, log-S update 7 ALU + 1 XU; one 16-byte table
# gather
ALU_PER_STEP, XU_PER_STEP, GATHER_BYTES = 153, 5, 16


def workload_jobs(m, stream_offset: int = 0, paths: int = PATHS):
    model = m.BatesModel(m.HestonParams(2.0, 0.05, 0.9, -0.6, 0.05), m.MertonParams(0.5, -0.1, 0.15))
    jobs = []
    for T in MATURITIES:
        cfg = m.MonteCarloConfig(num_paths=paths, time_steps=int(round(STEPS_PER_YEAR * T)), seed=SEED,
                                 stream_offset=stream_offset)
        jobs.append(m.make_job(model, m.BatesStepper(m.SchemeNCI), m.EuropeanOption(STRIKES, T),
                               m.GreekMode.FULL, cfg, 100.0, 0.02, 0.0))
    return jobs


def path_steps(paths: int = PATHS) -> tuple[int, int]:
    """(simulated scenario path-steps, workload path-steps) of one pass over the strip."""
    base = sum(paths * int(round(STEPS_PER_YEAR * T)) for T in MATURITIES)
    return base * N_SIMULATED, base


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.lines: list[str] = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.device}", f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self) -> dict:
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx.append(float(parts[2]))
            except ValueError:
                continue
            for name, val in zip(names, parts[5:9]):
                if val.lower().startswith("active"):
                    reasons.add(name)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


def read_peaks() -> dict:
    p = ROOT / "MEASURED_PEAKS.json"
    return json.loads(p.read_text()) if p.exists() else {}


def read_traffic() -> float | None:
    """DRAM bytes (read + write) of one full-size simulate_lockstep_kernel launch (T = 1, 2^22
    paths), from the ncu summary committed under profiles/ (a `dram_bytes_per_launch: N` line)."""
    p = ROOT / "profiles" / "simulate_lockstep_bates_nci_traffic.md"
    if p.exists():
        for line in p.read_text().splitlines():
            if line.startswith("dram_bytes_per_launch:"):  # the T = 1 request (2^22 paths)
                return float(line.split(":", 1)[1])
    return None


def read_issued() -> float | None:
    """Lane-operations the lockstep kernel issues per simulated scenario path-step, from the ncu
    summary committed under profiles/ (warp instructions x active lanes / 32)."""
    p = ROOT / "profiles" / "simulate_lockstep_bates_nci_small.md"
    if p.exists():
        for line in p.read_text().splitlines():
            if line.startswith("issued_lane_ops_per_scenario_path_step:"):
                return float(line.split(":", 1)[1])
    return None


def cpu_strip_pass(paths: int, cores: int) -> float:
    """Wall seconds of one pass of the reference's algorithm over the whole strip workload
    (8 maturities x 64 strikes, Full Greeks) at `paths` paths on `cores` OpenMP threads: the
    FP64 restatement at the reference's release flags (-O3 -ffast-math)."""
    from oracle import oracle
    import myquantlib_gb300 as m
    jobs = workload_jobs(m, paths=paths)
    t0 = time.perf_counter()
    for j in jobs:
        oracle.mc_price(j, oracle.LAYOUT_REFERENCE, cores, fast=True)
    return time.perf_counter() - t0


def cpu_reference(args) -> dict:
    """The reference's algorithm on the host cores, measured on one pass over the whole
    workload at args.cpu_paths paths (no extrapolation).  Each of its 8 calls builds its
    SchemeNCI tables (one per distinct step size: the base and the two T-bumped ones), as
    the reference's calculate does; that fixed cost is measured on its own at 256 paths and
    reported beside the rate."""
    from oracle import oracle
    oracle.build(ref=False)
    cores = os.cpu_count() or 1
    cpu_strip_pass(256, cores)  # thread start-up, page-in
    t = cpu_strip_pass(args.cpu_paths, cores)
    fixed = cpu_strip_pass(256, cores)
    _, base = path_steps(args.cpu_paths)
    return {"value": base / t, "unit": "paths*steps/s", "cores": cores, "kind": "port",
            "sample": (f"one pass over the whole workload (8 maturities x 64 strikes, Full Greeks, the two "
                       f"rho scenarios re-simulated as the reference does) at {args.cpu_paths} paths: "
                       f"{t:.1f} s on {cores} threads, measured"),
            "seconds": t, "fixed_cost_s": fixed,
            "fixed_cost": "the same pass at 256 paths: the per-call NCI table builds and OpenMP start-up",
            "value_without_fixed_cost": base / max(t - fixed, 1e-9)}


def run_reference(args) -> dict:
    """The reference arm: every timed step is one measured pass of the reference's algorithm
    over the whole strip at args.cpu_paths paths on all host threads (warm-up steps run the
    T = 0.25 maturity at 1024 paths).  value = the path-steps of the timed passes / their
    wall time; ms_per_step = the wall time actually spent per pass."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return {}
    from oracle import oracle
    import myquantlib_gb300 as m
    oracle.build(ref=False)
    cores = os.cpu_count() or 1
    for _ in range(args.warmup):
        oracle.mc_price(workload_jobs(m, paths=1024)[0], oracle.LAYOUT_REFERENCE, cores, fast=True)
    times = [cpu_strip_pass(args.cpu_paths, cores) for _ in range(args.steps)]
    fixed = cpu_strip_pass(256, cores)
    _, base = path_steps(args.cpu_paths)
    v = base * len(times) / sum(times)
    cpu = {"value": v, "unit": "paths*steps/s", "cores": cores, "kind": "port",
           "sample": (f"{args.steps} passes over the whole workload (8 maturities x 64 strikes, Full Greeks, "
                      f"rho scenarios re-simulated as the reference does) at {args.cpu_paths} paths each, on "
                      f"{cores} threads, measured (median pass {statistics.median(times):.1f} s)"),
           "fixed_cost_s": fixed,
           "fixed_cost": "one pass at 256 paths: the per-call NCI table builds and OpenMP start-up",
           "value_without_fixed_cost": base / max(statistics.median(times) - fixed, 1e-9)}
    cfg = workload_config(args)
    cfg["paths"] = args.cpu_paths
    cfg["sample_of"] = f"the {PATHS}-path workload, at {args.cpu_paths} paths per step"
    return {"metric": "paths*steps/s", "value": v, "unit": "paths*steps/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": sum(times) / len(times) * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic", "impl": "reference", "cpu_baseline": cpu,
            "e2e": {"value": v, "unit": "paths*steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "config": cfg}


def workload_config(args) -> dict:
    sim, base = path_steps()
    return {"workload": "Bates SchemeNCI European call strip, Full CRN Greeks (configuration 2)",
            "strikes": 64, "maturities": MATURITIES, "paths": PATHS, "steps_per_year": STEPS_PER_YEAR,
            "scenarios_per_path": N_SCENARIOS, "simulated_scenarios_per_path": N_SIMULATED,
            "simulated_path_steps_per_step": sim,
            "base_path_steps_per_step": base, "l2": "flushed between steps (256 MiB write)",
            "parallelism": f"replicas x{args.gpus} (disjoint xoshiro stream ranges)"}


def run_engine(args) -> dict:
    import torch
    import myquantlib_gb300 as m

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    eng = m.Engine(local)
    from myquantlib_gb300.replicas import default_streams
    streams_per_rank = default_streams(PATHS)  # disjoint stream ranges per replica
    jobs = workload_jobs(m, stream_offset=rank * streams_per_rank)
    nk = len(STRIKES)
    stream = torch.cuda.Stream(device=local)
    outs = [torch.empty(2 * 10 * nk, dtype=torch.float64, device=f"cuda:{local}") for _ in jobs]
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=f"cuda:{local}")

    def step_device():
        for j, o in zip(jobs, outs):
            m._abi.check(eng.lib.myql_mc_price_async(eng.handle, m.pricers.C.byref(j.c), o.data_ptr(),
                                                     stream.cuda_stream))

    # warm-up (also builds the NCI table and the stream table once)
    launches_per_step = 0
    for w in range(max(args.warmup, 1)):
        tot = 0
        for j in jobs:
            _, st = eng.price(j)
            tot += st.kernel_launches
        launches_per_step = tot
    with torch.cuda.stream(stream):
        step_device()
    torch.cuda.synchronize()

    # ---- device-timed region
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    with ClockSampler(local) as clk:
        for k in range(args.steps):
            with torch.cuda.stream(stream):
                flush.zero_()
                ev[k][0].record(stream)
                step_device()
                ev[k][1].record(stream)
        torch.cuda.synchronize()
    if dist:
        dist.barrier()
    dev_ms = sum(a.elapsed_time(b) for a, b in ev)

    # ---- end-to-end through the C ABI: pinned host strikes in, pinned results out
    pin_k = [torch.tensor(STRIKES, dtype=torch.float64).pin_memory() for _ in jobs]
    pin_o = [torch.empty(2 * 10 * nk, dtype=torch.float64).pin_memory() for _ in jobs]
    for j, pk in zip(jobs, pin_k):
        j.c.instrument.strikes = m.pricers.C.cast(pk.data_ptr(), m.pricers.C.POINTER(m.pricers.C.c_double))
    stats = []
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        for j, po in zip(jobs, pin_o):
            st = m._abi.McStatsC()
            m._abi.check(eng.lib.myql_mc_price(eng.handle, m.pricers.C.byref(j.c),
                                               m.pricers.C.cast(po.data_ptr(), m.pricers.C.POINTER(m.pricers.C.c_double)),
                                               m.pricers.C.byref(st)))
            stats.append((st.simulate_ms, st.payoff_ms, st.device_ms, st.kernel_launches, st.table_fallbacks))
    torch.cuda.synchronize()
    e2e_s = time.perf_counter() - t0

    sim, base = path_steps()
    t_dev = dev_ms / 1e3
    if dist:
        import torch as _t
        buf = _t.tensor([t_dev, e2e_s], device=f"cuda:{local}", dtype=_t.float64)
        dist.all_reduce(buf, op=dist.ReduceOp.MAX)
        t_dev, e2e_s = float(buf[0]), float(buf[1])
    value = world * base * args.steps / t_dev
    e2e = world * base * args.steps / e2e_s
    pooled = None
    if dist:
        # the replicas' estimates pooled into the whole job's (one FP64 all-reduce per maturity,
        # outside the timed regions): W x 2^22 paths on disjoint stream ranges
        from myquantlib_gb300.replicas import allreduce_price
        worst, atm = 0.0, None
        for t, (j, pk) in enumerate(zip(jobs, pin_o)):
            mine = pk.numpy().reshape(20, nk)   # this rank's last e2e result of the maturity
            pr = allreduce_price(mine, PATHS)
            worst = max(worst, float(np.max(pr[1] / np.maximum(np.abs(pr[0]), 1e-300))))
            if MATURITIES[t] == 1.0:
                k = int(np.argmin(np.abs(np.asarray(STRIKES) - 100.0)))
                atm = {"K": STRIKES[k], "price": float(pr[0, k]), "se": float(pr[1, k]),
                       "rank0_se": float(mine[1, k])}
        pooled = {"paths": world * PATHS, "T1_atm": atm, "max_rel_se_price": worst,
                  "how": "replicas.allreduce_price: FP64 moment sums over all ranks"}
    if rank != 0:
        return {}

    # ---- roofline of the dominant kernel (simulate), from its own CUDA events
    sim_ms = sum(s[0] for s in stats) / args.steps
    pay_ms = sum(s[1] for s in stats) / args.steps
    alu_peak = eng.peak(0)
    xu_peak = eng.peak(1)
    alu_ach = ALU_PER_STEP * sim / (sim_ms / 1e3)
    xu_ach = XU_PER_STEP * sim / (sim_ms / 1e3)
    alu_frac, xu_frac = alu_ach / alu_peak, xu_ach / xu_peak
    bound = "alu" if alu_frac >= xu_frac else "xu"
    roof = {"bound": bound, "kernel": "simulate_lockstep_kernel<1,NCI,-,5 scenarios,merged variance paths>",
            "note": ("achieved counts the algorithmic ops of every simulated scenario path-step (153 ALU, "
                     "5 XU); the lockstep kernel shares the draws of a step across scenarios and, once a "
                     "v0-bumped variance path has merged into the base's, its Poisson inversion and table "
                     "cell, so it issues fewer (about 100 lane-ops per scenario path-step under ncu)"),
            "achieved": (alu_ach if bound == "alu" else xu_ach) / 1e9,
            "peak": (alu_peak if bound == "alu" else xu_peak) / 1e9, "unit": "Gop/s",
            "frac": max(alu_frac, xu_frac),
            "peak_source": "measured by myql_probe_peak (FP32-FMA / MUFU microbenchmark on this GPU)",
            "alu": {"achieved": alu_ach / 1e9, "peak": alu_peak / 1e9, "frac": alu_frac, "ops_per_path_step": ALU_PER_STEP},
            "xu": {"achieved": xu_ach / 1e9, "peak": xu_peak / 1e9, "frac": xu_frac, "ops_per_path_step": XU_PER_STEP},
            "simulate_ms_per_step": sim_ms, "payoff_ms_per_step": pay_ms,
            "traffic": read_traffic(),
            "issued": None if read_issued() is None else {
                "lane_ops_per_scenario_path_step": read_issued(),
                "frac": alu_frac * read_issued() / ALU_PER_STEP,
                "note": ("the lane-operations the kernel issues (ncu: warp instructions x active lanes), "
                         "per second, against the same FP32 lane rate: what the hardware executes, where "
                         "frac counts the contracted work")},
            "l2_gather": {"achieved": GATHER_BYTES * sim / (sim_ms / 1e3) / 1e9, "unit": "GB/s",
                          "note": ("16 B of NCI table per simulated scenario path-step, gathered from L2 (the "
                                   "18.5 MB table stays resident); an algorithmic rate, not DRAM traffic"),
                          "hbm_peak_gbs": read_peaks().get("hbm_gbs")}}
    line = {"metric": "paths*steps/s", "value": value, "unit": "paths*steps/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": dev_ms / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic", "config": workload_config(args),
            "e2e": {"value": e2e, "unit": "paths*steps/s", "h2d_bytes_per_step": 8 * nk * len(jobs),
                    "d2h_bytes_per_step": 8 * 2 * 10 * nk * len(jobs)},
            "gpu_launches": launches_per_step * args.steps, "roofline": roof, "clocks": clk.summary(),
            "nci_table_fallbacks_per_step": sum(s[4] for s in stats) / args.steps}
    if pooled:
        line["pooled_estimate"] = pooled
    if world == 1:
        line.update(strip_reports(eng, m, jobs, local, args))
    return line


def fourier_z(eng, m, jobs) -> tuple[dict, np.ndarray]:
    """Every price and Greek of the strip against the FP64 Gil-Pelaez oracle: signed
    z = (MC - Fourier) / SE, shape (maturities, quantities, strikes); NaN where SE = 0."""
    nq = len(m._abi.Q_NAMES)
    z = np.full((len(jobs), nq, len(STRIKES)), np.nan)
    for t, j in enumerate(jobs):
        raw, _ = eng.price(j)
        four = eng.fourier(j, m.GreekMode.FULL)
        for qi in range(nq):
            se = raw[2 * qi + 1]
            ok = se > 0
            z[t, qi, ok] = (raw[2 * qi][ok] - four[2 * qi][ok]) / se[ok]
    return z


def fourier_summary(m, z: np.ndarray) -> dict:
    a = np.abs(z[np.isfinite(z)])
    zmax = {name: float(np.nanmax(np.abs(z[:, qi]))) for qi, name in enumerate(m._abi.Q_NAMES)
            if np.isfinite(z[:, qi]).any()}
    # a correct estimator leaves about 0.27 % of |z| above 3; the strikes and maturities share
    # paths, so the z are correlated and the fractions are noisier than for independent tests
    return {"max_abs_z": zmax, "comparisons": int(a.size), "frac_abs_z_above_3": float(np.mean(a > 3.0)),
            "frac_abs_z_above_2": float(np.mean(a > 2.0))}


def fourier_seeds(eng, m, seeds, nci_slopes: int, precise_theta: bool = False) -> dict:
    """The strip on several seeds against the Fourier oracle.  Per (maturity, quantity) the
    strike-averaged signed z is averaged over the seeds; with independent seeds its spread
    gives a standard error, so a residual bias shows as a mean that stays away from 0 by
    several of those standard errors (one seed cannot tell correlation from bias)."""
    eng.set_nci_slopes(nci_slopes)
    eng.set_precise_theta(precise_theta)
    try:
        zs = []
        for sd in seeds:
            js = workload_jobs(m)
            for j in js:
                j.c.config.seed = sd
            zs.append(fourier_z(eng, m, js))
    finally:
        eng.set_nci_slopes(0)
        eng.set_precise_theta(False)
    Z = np.stack(zs)                                     # (seed, maturity, quantity, strike)
    # quantities without a Fourier value (the second factor's) are all NaN: left out
    has = np.isfinite(Z).any(axis=3)                     # (seed, maturity, quantity)
    per = np.full(Z.shape[:3], np.nan)
    per[has] = np.nanmean(Z[has], axis=-1)               # strike-averaged signed z per seed
    mean = np.full(Z.shape[1:3], np.nan)
    sem = np.zeros(Z.shape[1:3])
    cols = has.all(axis=0)                               # (maturity, quantity) on every seed
    mean[cols] = per[:, cols].mean(axis=0)
    if len(seeds) > 1:  # one seed has no spread: t stays 0
        sem[cols] = per[:, cols].std(axis=0, ddof=1) / np.sqrt(len(seeds))
    t = np.where(sem > 0, mean / np.where(sem > 0, sem, 1.0), 0.0)
    names = m._abi.Q_NAMES
    cells = {}
    for ti, T in enumerate(MATURITIES):
        for qi, name in enumerate(names):
            if np.isfinite(mean[ti, qi]):
                cells[f"T{T}/{name}"] = {"mean_z": round(float(mean[ti, qi]), 3), "t": round(float(t[ti, qi]), 2)}
    a = np.abs(Z[np.isfinite(Z)])
    worst = max(cells.items(), key=lambda kv: abs(kv[1]["t"]))
    return {"seeds": list(seeds), "nci_cells": "exact slopes, mean-preserving first cell" if nci_slopes
            else "the reference's", "precise_theta": precise_theta, "comparisons": int(a.size),
            "pooled_frac_abs_z_above_3": float(np.mean(a > 3.0)),
            "pooled_frac_abs_z_above_2": float(np.mean(a > 2.0)),
            "max_abs_mean_z": float(np.nanmax(np.abs(mean))), "max_abs_t": float(np.nanmax(np.abs(t))),
            "worst_cell": {worst[0]: worst[1]},
            "cells_abs_t_above_3": sorted(k for k, v in cells.items() if abs(v["t"]) > 3.0),
            "per_cell": cells,
            "note": ("per (maturity, quantity): mean over seeds of the strike-averaged signed z, and t = that "
                     "mean / its standard error from the seed spread")}


def cold_e2e(m, local: int) -> dict:
    """The strip through myql_mc_price on a fresh context: no NCI tables, no stream tables and
    no buffers cached, host strike and result buffers; wall time of the first pass."""
    import torch
    eng2 = m.Engine(local)
    try:
        jobs = workload_jobs(m)
        outs = [np.zeros(2 * 10 * len(STRIKES)) for _ in jobs]
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for j, o in zip(jobs, outs):
            st = m._abi.McStatsC()
            m._abi.check(eng2.lib.myql_mc_price(eng2.handle, m.pricers.C.byref(j.c),
                                                o.ctypes.data_as(m.pricers.C.POINTER(m.pricers.C.c_double)),
                                                m.pricers.C.byref(st)))
        t = time.perf_counter() - t0
    finally:
        eng2.close()
    _, base = path_steps()
    return {"value": base / t, "unit": "paths*steps/s", "seconds": t,
            "includes": "context creation excluded; NCI table builds, stream seeding, buffer allocation, "
                        "first launches and host<->device copies included"}


def strip_reports(eng, m, jobs, local: int, args) -> dict:
    """The reports of a 1-GPU run beside the headline rate: the Fourier checks, the cold first
    pass, the metric's time-to-relative-SE block and the CPU baseline."""
    out = {}
    try:
        out["fourier_check"] = dict(fourier_summary(m, fourier_z(eng, m, jobs)), options=len(jobs) * len(STRIKES),
                                    oracle="FP64 Gil-Pelaez on the GPU (myql_fourier_price)",
                                    nci_cells="the reference's", seed=SEED)
        seeds = tuple(range(SEED, SEED + args.fourier_seeds))
        out["fourier_seeds_exact_nci"] = fourier_seeds(eng, m, seeds, 1)
        out["fourier_seeds"] = fourier_seeds(eng, m, seeds, 0)
        # theta and charm with the T-bumped constants carried beyond FP32 (opt-in mode)
        out["fourier_seeds_exact_nci_precise_theta"] = fourier_seeds(eng, m, seeds, 1, precise_theta=True)
    except Exception as exc:  # the oracle is a report, not the measurement
        out["fourier_check"] = {"error": repr(exc)}
    out["e2e_cold"] = cold_e2e(m, local)
    if not args.no_cv:
        out["time_to_se"] = cv_report(eng, m)
    if not args.no_cpu:
        out["cpu_baseline"] = cpu_reference(args)
    return out


def run_c1(args) -> dict:
    """Configuration 1: Heston SchemeNV European call (kappa 1.5, theta .04, sigma .3, rho -.7,
    v0 .04; S0 = K = 100, T 1, r .02, q 0), 2^20 paths x 100 steps, seed 42, GreekMode::None.
    value: path-steps / device time of R = 16 back-to-back requests per step (CUDA events on
    the launching stream, L2 flushed between steps); e2e: the same through myql_mc_price with
    a pinned host result buffer; cpu_baseline: the CPU port on the whole request."""
    import torch
    import myquantlib_gb300 as m

    if int(os.environ.get("RANK", "0")) != 0:
        return {}
    R, paths, steps = 16, 1 << 20, 100
    eng = m.Engine(0)
    job = m.make_job(m.HestonModel(m.HestonParams(1.5, 0.04, 0.3, -0.7, 0.04)), m.HestonStepper(m.SchemeNV),
                     m.EuropeanOption(100.0, 1.0), m.GreekMode.NONE,
                     m.MonteCarloConfig(num_paths=paths, time_steps=steps, seed=SEED), 100.0, 0.02, 0.0)
    stream = torch.cuda.Stream(device=0)
    out = torch.empty(2 * 10, dtype=torch.float64, device="cuda:0")
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda:0")
    launches = 0
    for _ in range(max(args.warmup, 1)):
        _, st = eng.price(job)
        launches = st.kernel_launches
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    sims = []
    torch.cuda.synchronize()
    with ClockSampler(0) as clk:
        for k in range(args.steps):
            with torch.cuda.stream(stream):
                flush.zero_()
                ev[k][0].record(stream)
                for _ in range(R):
                    m._abi.check(eng.lib.myql_mc_price_async(eng.handle, m.pricers.C.byref(job.c), out.data_ptr(),
                                                             stream.cuda_stream))
                ev[k][1].record(stream)
        torch.cuda.synchronize()
        dev_ms = sum(a.elapsed_time(b) for a, b in ev)
        pin = torch.empty(2 * 10, dtype=torch.float64).pin_memory()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(args.steps * R):
            st = m._abi.McStatsC()
            m._abi.check(eng.lib.myql_mc_price(eng.handle, m.pricers.C.byref(job.c),
                                               m.pricers.C.cast(pin.data_ptr(), m.pricers.C.POINTER(m.pricers.C.c_double)),
                                               m.pricers.C.byref(st)))
            sims.append(st.simulate_ms)
        e2e_s = time.perf_counter() - t0
    work = paths * steps * R
    value = work * args.steps / (dev_ms / 1e3)
    sim_ms = statistics.median(sims)
    alu_peak = eng.peak(0)
    alu_ach = 97 * paths * steps / (sim_ms / 1e3)
    line = {"metric": "paths*steps/s", "value": value, "unit": "paths*steps/s", "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": dev_ms / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": "Heston SchemeNV European call, 2^20 paths x 100 steps, GreekMode None "
                                   "(configuration 1)", "requests_per_step": R, "path_steps_per_step": work,
                       "l2": "flushed between steps (256 MiB write)", "price": float(pin[0])},
            "e2e": {"value": work * args.steps / e2e_s, "unit": "paths*steps/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 8 * 20 * R},
            "gpu_launches": launches * R * args.steps,
            "roofline": {"bound": "alu", "kernel": "simulate_kernel<1,NV,-,false>", "achieved": alu_ach / 1e9,
                         "peak": alu_peak / 1e9, "unit": "Gop/s", "frac": alu_ach / alu_peak,
                         "ops_per_path_step": 97, "simulate_ms_per_request": sim_ms,
                         "peak_source": "measured by myql_probe_peak (FP32-FMA microbenchmark on this GPU)"},
            "clocks": clk.summary()}
    if not args.no_cpu:
        from oracle import oracle
        oracle.build(ref=False)
        cores = os.cpu_count() or 1
        t0 = time.perf_counter()
        oracle.mc_price(job, oracle.LAYOUT_REFERENCE, cores, fast=True)
        t = time.perf_counter() - t0
        line["cpu_baseline"] = {"value": paths * steps / t, "unit": "paths*steps/s", "cores": cores, "kind": "port",
                                "sample": f"the whole request, 2^20 paths x 100 steps ({t:.2f} s)"}
    return line


def run_ncu_c1_case() -> None:
    """Profiling case of configuration 1: two pricing requests of the full 2^20 paths x 100
    steps, no timing."""
    import myquantlib_gb300 as m
    eng = m.Engine(0)
    job = m.make_job(m.HestonModel(m.HestonParams(1.5, 0.04, 0.3, -0.7, 0.04)), m.HestonStepper(m.SchemeNV),
                     m.EuropeanOption(100.0, 1.0), m.GreekMode.NONE,
                     m.MonteCarloConfig(num_paths=1 << 20, time_steps=100, seed=SEED), 100.0, 0.02, 0.0)
    for _ in range(2):
        eng.price(job)


def run_ncu_mlmc_case() -> None:
    """Profiling case of the MLMC workload: two evaluations of level 6 (64 fine steps) of the
    Heston down-and-out put with 2^20 coupled paths, no timing."""
    import ctypes as C
    import myquantlib_gb300 as m
    from myquantlib_gb300 import _abi
    eng = m.Engine(0)
    model = m.HestonModel(m.HestonParams(2.0, 0.04, 0.5, -0.7, 0.04))
    job = m.make_job(model, m.HestonStepper(m.SchemeNV, m.TrackerBarrier), m.DownAndOutPut(100.0, 80.0, 1.0),
                     m.GreekMode.NONE, m.MonteCarloConfig(), 100.0, 0.02, 0.0)
    c = _abi.MlmcConfigC()
    c.epsilon, c.L_min, c.L_max, c.N0, c.base_steps = 1e-3, 2, 10, 10000, 1
    c.alpha, c.beta, c.adaptive_rates, c.seed, c.fd_bump, c.n_streams = 2.0, 1.0, 1, SEED, 1e-4, 0
    out = np.zeros(4)
    for _ in range(2):
        _abi.check(eng.lib.myql_mlmc_level(eng.handle, C.byref(job.c), C.byref(c), 6, 1 << 20,
                                           out.ctypes.data_as(C.POINTER(C.c_double))))


def run_batch(args) -> dict:
    """Batched uneven requests (4096 jobs, myquantlib_gb300.workloads.uneven_requests) in one
    persistent launch per step.  value: path-steps / device time of the batch graph (descriptor
    upload, persistent kernel, finalize, result download); e2e: the same over the wall-clock of
    the whole myql_mc_price_batch call (host planning included)."""
    import torch
    import myquantlib_gb300 as m
    from myquantlib_gb300 import workloads

    if int(os.environ.get("RANK", "0")) != 0:
        return {}
    eng = m.Engine(0)
    nci = args.batch_scheme == "nci"
    if nci:  # one table per distinct d, each capped at batch_nci_rows rows (resident together)
        eng.set_nci_rows(args.batch_nci_rows)
    rq = workloads.uneven_requests(args.batch_jobs, scheme=m.SchemeNCI if nci else m.SchemeExact)
    jobs = [m.make_job(r.model, m.stepper_for(r.model, r.instrument, r.scheme), r.instrument, r.mode, r.cfg,
                       r.S0, r.r, r.q) for r in rq]
    total = workloads.path_steps(rq)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda:0")
    launches = 0
    t_first = time.perf_counter()
    for w in range(max(args.warmup, 1)):
        _, st = eng.price_batch(jobs)
        launches = st.kernel_launches
        if w == 0:
            t_first = time.perf_counter() - t_first  # the first batch: tables, tuning, graph
    dev_ms, wall, fallbacks = [], [], []
    with ClockSampler(0) as clk:
        for _ in range(args.steps):
            flush.zero_()
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            _, st = eng.price_batch(jobs)
            wall.append(time.perf_counter() - t0)
            dev_ms.append(st.device_ms)
            fallbacks.append(int(st.table_fallbacks))
    value = total * args.steps / (sum(dev_ms) / 1e3)
    e2e = total * args.steps / sum(wall)
    line = {"metric": "paths*steps/s", "value": value, "unit": "paths*steps/s", "n_gpus": 1,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": sum(dev_ms) / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic",
            "config": {"workload": f"{len(jobs)} uneven requests (Heston / Bates-Kou / Double Heston, "
                                   f"arithmetic Asian or up-and-out call, {'SchemeNCI' if nci else 'SchemeExact'}) "
                                   "in one persistent launch",
                       "jobs": len(jobs), "path_steps_per_step": total, "l2": "flushed between steps"},
            "first_batch_s": t_first,
            "e2e": {"value": e2e, "unit": "paths*steps/s", "h2d_bytes_per_step": None,
                    "d2h_bytes_per_step": 8 * 20 * len(jobs)},
            "gpu_launches": launches * args.steps, "clocks": clk.summary(),
            # per kernel class: the launch shape the batch autotuner picked and its timings
            "tuner": [{k: (round(v, 4) if isinstance(v, float) else v) for k, v in p.items()}
                      for p in eng.batch_plan()]}
    if nci:
        line["config"]["nci_rows_cap"] = args.batch_nci_rows
        line["nci_table_fallbacks_per_step"] = statistics.median(fallbacks)
    if not args.no_cpu:
        from oracle import oracle
        oracle.build(ref=False)
        cores = os.cpu_count() or 1
        n_s = 8 if nci else 32  # the port builds each NCI job's FP64 table, as the reference does
        t0 = time.perf_counter()
        for j in jobs[:n_s]:
            oracle.mc_price(j, oracle.LAYOUT_REFERENCE, cores, fast=True)
        t = time.perf_counter() - t0
        line["cpu_baseline"] = {"value": workloads.path_steps(rq[:n_s]) / t, "unit": "paths*steps/s",
                                "cores": cores, "kind": "port",
                                "sample": f"the first {n_s} requests at full size, one after another ({t:.1f} s)"}
    return line


# ---------------------------------------------------------------- neural control variate
def cv_jobs(m, kind: str, paths: int, seed: int = 42):
    """The control-variate workloads: the Double Bates arithmetic Asian call (factors
    (v0 .03, kappa 2, theta .03, sigma .4, rho -.7) and (.02, .5, .02, .3, -.3), Merton
    (.3, -.05, .1), K 100, T 2, 256 steps, SchemeNCI) and the Heston European call
    (kappa 1.5, theta .04, sigma .3, rho -.7, v0 .04, K 100, T 1, 100 steps, SchemeNV)."""
    if kind == "asian":
        model = m.DoubleBatesModel(m.HestonParams(2.0, 0.03, 0.4, -0.7, 0.03),
                                   m.HestonParams(0.5, 0.02, 0.3, -0.3, 0.02), m.MertonParams(0.3, -0.05, 0.1))
        instr = m.AsianOption(m.TrackerArithAsian, m.PayoffVanilla(), True, 100.0, 2.0)
        stepper = m.DoubleBatesStepper(m.SchemeNCI, m.SchemeNCI, m.TrackerArithAsian)
        steps = 256
    else:
        model = m.HestonModel(m.HestonParams(1.5, 0.04, 0.3, -0.7, 0.04))
        instr = m.EuropeanOption(100.0, 1.0)
        stepper = m.HestonStepper(m.SchemeNV)
        steps = 100
    cfg = m.MonteCarloConfig(num_paths=paths, time_steps=steps, seed=seed)
    return m.make_job(model, stepper, instr, m.GreekMode.NONE, cfg, 100.0, 0.02, 0.0), steps


def cv_config(m, kind: str, pilot: int = 1 << 19, iterations: int = 120, plain_seconds: float | None = None):
    """The control variate's settings: the training budget and hedging interval sized by
    ControlVariateConfig.for_plain_time from the plain estimator's time, or (for warm-up and
    profiling) the given budget, hedging every 8 (Asian) or 5 (European) steps."""
    he = 8 if kind == "asian" else 5
    if plain_seconds is not None:
        steps = 256 if kind == "asian" else 100
        return m.pricers.ControlVariateConfig.for_plain_time(plain_seconds, time_steps=steps, learning_rate=5e-3,
                                                             seed=7).c()
    return m.pricers.ControlVariateConfig(hedge_every=he, iterations=iterations, pilot_paths=pilot,
                                          batch_paths=4096, learning_rate=5e-3, seed=7).c()


def _pool(parts):
    """Pools independent (price, standard error, paths) estimates from their FP64 moments."""
    n = sum(p for _, _, p in parts)
    s1 = sum(p * v for v, _, p in parts)
    s2 = sum(p * (se * se * p + v * v) for v, se, p in parts)
    mean = s1 / n
    return mean, float(np.sqrt(max(s2 / n - mean * mean, 0.0) / n)), n


def time_to_se(eng, m, kind: str, target: float, probe_paths: int = 1 << 22, top_ups: int = 4) -> dict:
    """Wall time until the relative standard error reaches `target`: plain GPU Monte Carlo
    against the neural control variate, each through the public API.  Untimed probes fix each
    estimator's variance (the plain engine at probe_paths; the control variate trained, untimed,
    on the very pilot paths its timed arm trains on again, which gives the same network bit for
    bit).  In the timed region each arm prices the path count its probe gives
    for the target and, while its estimated relative error is still above the target, prices
    more paths on fresh seeds and pools them (at most `top_ups` times).  The control
    variate's timed region includes its own pilot simulation and training.  A third arm runs
    the same control variate on randomized QMC paths (myql_cv_qmc_price, 16 digital shifts),
    sized by _qmc_size from its own untimed probe."""
    import torch
    job, steps = cv_jobs(m, kind, probe_paths)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    raw, _ = eng.price(job)
    t_probe = time.perf_counter() - t0
    price, se = raw[0, 0], raw[1, 0]
    n_plain = int(probe_paths * (se / (target * price)) ** 2) + 1
    # the training budget follows the plain estimator's expected time to the target
    cfg = cv_config(m, kind, plain_seconds=t_probe * n_plain / probe_paths)
    eng.cv_train(cv_jobs(m, kind, 1 << 16, seed=45)[0], cfg)  # the CV arm's network
    probe = eng.cv_price(cv_jobs(m, kind, probe_paths, seed=43)[0], cfg)
    n_cv = max(int(probe_paths * (probe.price_std_err / (target * probe.price)) ** 2) + 1, 128)

    def run_arm(first_n, price_fn, seed0):
        parts, n, rounds = [], first_n, 0
        while True:
            v, e, p = price_fn(n, seed0 + rounds)
            parts.append((v, e, p))
            mean, err, tot = _pool(parts)
            rounds += 1
            if err <= target * mean or rounds > top_ups:
                return mean, err, tot, rounds
            n = max(int(tot * ((err / (target * mean)) ** 2 - 1.0)) + 1, 128)

    def plain_fn(n, sd):
        r, _ = eng.price(cv_jobs(m, kind, n, seed=sd)[0])
        return float(r[0, 0]), float(r[1, 0]), n

    cv_last = {"sim_ms": 0.0, "mlp_ms": 0.0, "price_ms": 0.0}

    def cv_fn(n, sd):
        r = eng.cv_price(cv_jobs(m, kind, n, seed=sd)[0], cfg)
        cv_last["vr"] = r.variance_ratio
        cv_last["sim_ms"] += r.simulate_ms
        cv_last["mlp_ms"] += r.mlp_ms
        cv_last["price_ms"] += r.total_ms
        return r.price, r.price_std_err, n

    # the same network on randomized QMC paths: sized like qmc_time_to_se from its own probe
    R, quantum = 16, 16 * 2048
    eng.cv_train(cv_jobs(m, kind, 1 << 16, seed=46)[0], cfg)  # the QMC arm's network
    def cvq_probe(n, i):
        r = eng.cv_qmc_price(cv_jobs(m, kind, n, seed=44 + 1000 * i)[0], cfg, R)
        return r.price, r.price_std_err

    n_cvq, cvq_decay = _qmc_size(cvq_probe, target, quantum)
    cvq_last = {"sim_ms": 0.0, "mlp_ms": 0.0, "price_ms": 0.0}

    def run_cvq():
        parts, n, runs = [], n_cvq, 0
        while True:
            r = eng.cv_qmc_price(cv_jobs(m, kind, n, seed=3000 + runs)[0], cfg, R)
            cvq_last["vr"] = r.variance_ratio
            cvq_last["sim_ms"] += r.simulate_ms
            cvq_last["mlp_ms"] += r.mlp_ms
            cvq_last["price_ms"] += r.total_ms
            parts.append((r.price, r.price_std_err, n))
            runs += 1
            mean, err, tot = _pool_qmc(parts)
            if err <= target * mean or runs > top_ups:
                return mean, err, tot, runs
            n = max(-(-int(tot * ((err / (target * mean)) ** 2 - 1.0)) // quantum) * quantum, quantum)

    torch.cuda.synchronize()
    t0 = time.perf_counter()
    p_mean, p_err, p_n, p_rounds = run_arm(n_plain, plain_fn, 1000)
    t_plain = time.perf_counter() - t0
    t0 = time.perf_counter()
    tr = eng.cv_train(cv_jobs(m, kind, 1 << 16, seed=45)[0], cfg)
    c_mean, c_err, c_n, c_rounds = run_arm(n_cv, cv_fn, 2000)
    t_cv = time.perf_counter() - t0
    t0 = time.perf_counter()
    trq = eng.cv_train(cv_jobs(m, kind, 1 << 16, seed=46)[0], cfg)
    q_mean, q_err, q_n, q_runs = run_cvq()
    t_cvq = time.perf_counter() - t0
    t_plain_path = t_plain / p_n
    t_cv_path = (t_cv - tr.total_ms / 1e3) / c_n
    return {"instrument": "Double Bates arithmetic Asian call" if kind == "asian" else "Heston European call",
            "target_rel_se": target, "speedup": t_plain / t_cv,
            "plain_s": t_plain, "plain_paths": p_n, "plain_runs": p_rounds, "plain_rel_se": p_err / p_mean,
            "plain_path_steps_per_s": p_n * steps / t_plain,
            "cv_s": t_cv, "cv_paths": c_n, "cv_runs": c_rounds, "cv_rel_se": c_err / c_mean,
            "cv_pilot_and_training_s": tr.total_ms / 1e3, "cv_train_s": tr.train_ms / 1e3,
            "cv_pilot_paths": int(tr.paths), "cv_iterations": int(cfg.iterations),
            "cv_batch_paths": int(cfg.batch_paths), "cv_hedge_every": int(cfg.hedge_every),
            "variance_ratio": cv_last.get("vr"), "pricing_only_speedup": cv_last.get("vr", 0.0) * t_plain_path / t_cv_path,
            # where the control variate's time goes (its own timers): pilot simulation and set-up,
            # the Adam steps, then the pricing run's path simulation, MLP rows and the rest
            "cv_breakdown_s": {"pilot_and_setup": (tr.total_ms - tr.train_ms) / 1e3, "adam_steps": tr.train_ms / 1e3,
                               "price_simulate": cv_last["sim_ms"] / 1e3, "price_mlp": cv_last["mlp_ms"] / 1e3,
                               "price_other": (cv_last["price_ms"] - cv_last["sim_ms"] - cv_last["mlp_ms"]) / 1e3,
                               "host": t_cv - (tr.total_ms + cv_last["price_ms"]) / 1e3},
            "price_cv": c_mean, "price_plain": p_mean,
            # the control variate on randomized QMC paths (R = 16 digital shifts), pilot and
            # training inside its timed region as above
            "cv_qmc": {"s": t_cvq, "speedup": t_plain / t_cvq, "points": q_n, "runs": q_runs,
                       "probe_decay_exponent": cvq_decay,
                       "rel_se": q_err / q_mean, "price": q_mean, "replicate_variance_ratio": cvq_last.get("vr"),
                       "breakdown_s": {"pilot_and_training": trq.total_ms / 1e3,
                                       "price_simulate": cvq_last["sim_ms"] / 1e3,
                                       "price_mlp": cvq_last["mlp_ms"] / 1e3,
                                       "price_other": (cvq_last["price_ms"] - cvq_last["sim_ms"]
                                                       - cvq_last["mlp_ms"]) / 1e3}}}


def cv_report(eng, m) -> dict:
    """The time-to-relative-SE block: the Double Bates arithmetic Asian at 1e-3 and 1e-4 and the
    Heston European at 1e-4, neural control variate against plain GPU Monte Carlo, plus the same
    workloads by randomized QMC; clocks sampled over the whole block."""
    for kind in ("asian", "european"):  # warm-up: tables, stream tables, first launches
        eng.price(cv_jobs(m, kind, 1 << 16)[0])
        eng.cv_train(cv_jobs(m, kind, 1 << 16)[0], cv_config(m, kind, pilot=1 << 16, iterations=10))
    eng.qmc_price(cv_jobs(m, "european", 1 << 19)[0], 16)
    eng.qmc_price(cv_jobs(m, "asian", 1 << 19)[0], 16)
    with ClockSampler(eng.device) as clk:
        res = {"asian_1e-3": time_to_se(eng, m, "asian", 1e-3),
               "asian_1e-4": time_to_se(eng, m, "asian", 1e-4),
               "european_1e-4": time_to_se(eng, m, "european", 1e-4),
               "european_qmc_1e-4": qmc_time_to_se(eng, m, "european", 1e-4),
               "asian_qmc_1e-3": qmc_time_to_se(eng, m, "asian", 1e-3),
               "asian_qmc_1e-4": qmc_time_to_se(eng, m, "asian", 1e-4)}
    res["clocks"] = clk.summary()
    res["method"] = ("wall time through the public API, synchronised; each arm sized by an untimed probe "
                     "and topped up on fresh seeds until its estimated relative SE meets the target; the "
                     "control variate's pilot simulation and training are inside its timed region")
    return res


def _pool_qmc(parts):
    """Pools independent randomized-QMC estimates (price, standard error, points), weighted by
    their point counts: at the c / sqrt(n) rate that weighting matches one run of all the points."""
    n = sum(p for _, _, p in parts)
    mean = sum(p * v for v, _, p in parts) / n
    return mean, float(np.sqrt(sum((p * se) ** 2 for _, se, p in parts))) / n, n


def _qmc_size(run, target: float, quantum: int, n1: int = 1 << 19, n2: int = 1 << 21, shifts: int = 4):
    """Points for a randomized-QMC run to reach the relative standard error `target`, from an
    untimed probe: the error at two sizes, each from `shifts` shift sets of replicates
    (run(n, i) -> (price, standard error)), its decay n^-a with a fitted from the two and clamped
    to [0.5, 0.75] (1/sqrt(n) is plain Monte Carlo's rate; QMC decays faster), and a 0.85 margin
    on the run's own noisy error estimate; in whole quanta.  Returns (points, a)."""
    def err(n):
        rs = [run(n, i) for i in range(shifts)]
        return float(np.mean([p for p, _ in rs])), float(np.sqrt(np.mean([e * e for _, e in rs])))
    _, e1 = err(n1)
    p2, e2 = err(n2)
    a = float(min(max(np.log(e1 / e2) / np.log(n2 / n1), 0.5), 0.75))
    need = n2 * (e2 / (0.85 * target * p2)) ** (1.0 / a)
    return max(-(-int(need) // quantum) * quantum, quantum), a


def qmc_time_to_se(eng, m, kind: str = "european", target: float = 1e-4, R: int = 16,
                   top_ups: int = 4) -> dict:
    """A control-variate workload (the Heston European call, SchemeNV, 100 steps, or the Double
    Bates arithmetic Asian, SchemeNCI factors and Merton jumps, 256 steps) priced by randomized
    quasi-Monte Carlo (Sobol + Brownian bridge for the normals, Sobol uniforms for the NCI and jump
    draws, R digital shifts): wall time to the relative standard error target against plain GPU
    Monte Carlo.  An untimed probe (_qmc_size: the error at 2^19 and 2^21 points, 4 shift sets of
    R replicates each, and its fitted decay) sizes the timed run for 0.85 x the target, in whole
    2048-point blocks per replicate; while the pooled error is still above the target it prices
    the shortfall on fresh seeds and pools the runs (at most `top_ups` times), every run inside
    the timed region."""
    import torch
    quantum = R * 2048

    def size(n):  # whole 2048-point blocks per replicate
        return max(-(-int(n) // quantum) * quantum, quantum)

    def probe(n, i):
        q, _ = eng.qmc_price(cv_jobs(m, kind, n, seed=700 + i)[0], R)
        return q[0, 0], q[1, 0]

    n_q, decay = _qmc_size(probe, target, quantum)
    pj, _ = cv_jobs(m, kind, 1 << 22)
    raw, _ = eng.price(pj)
    n_plain = int((1 << 22) * (raw[1, 0] / (target * raw[0, 0])) ** 2) + 1
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    parts, n, runs = [], n_q, 0
    while True:
        r, _ = eng.qmc_price(cv_jobs(m, kind, n, seed=48 + runs)[0], R)
        parts.append((float(r[0, 0]), float(r[1, 0]), n))
        runs += 1
        mean, err, tot = _pool_qmc(parts)
        if err <= target * mean or runs > top_ups:
            break
        n = size(tot * ((err / (target * mean)) ** 2 - 1.0))
    t_q = time.perf_counter() - t0
    t0 = time.perf_counter()
    raw, _ = eng.price(cv_jobs(m, kind, n_plain, seed=49)[0])
    t_plain = time.perf_counter() - t0
    return {"instrument": ("Heston European call (SchemeNV, 100 steps)" if kind == "european" else
                           "Double Bates arithmetic Asian call (SchemeNCI factors, Merton jumps, 256 steps)"),
            "target_rel_se": target, "replicates": R, "qmc_paths": tot, "qmc_runs": runs, "qmc_s": t_q,
            "probe_decay_exponent": decay,
            "qmc_rel_se": err / mean, "plain_paths": n_plain,
            "plain_s": t_plain, "plain_rel_se": raw[1, 0] / raw[0, 0], "speedup": t_plain / t_q,
            "price_qmc": mean, "price_plain": raw[0, 0]}


def run_cv(args) -> dict:
    """Headline metric part 1 on its own: time-to-relative-SE of the neural control variate
    against plain GPU Monte Carlo (seconds, lower is better); value = the Asian at 1e-3."""
    import myquantlib_gb300 as m
    if int(os.environ.get("RANK", "0")) != 0:
        return {}
    eng = m.Engine(0)
    res = cv_report(eng, m)
    a = res["asian_1e-3"]
    return {"metric": "time-to-relative-SE (s) neural-CV vs plain MC", "value": a["cv_s"], "unit": "s",
            "n_gpus": 1, "steps": 1, "warmup": 1, "ms_per_step": a["cv_s"] * 1e3, "higher_is_better": False,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32 paths, bf16 MLP (fp32 accumulation)",
            "data": "synthetic", "config": {"workload": "neural martingale control variate, Double Bates Asian "
                                                        "(and Heston European)", "l2": "inputs larger than L2"},
            "time_to_se": res, "clocks": res["clocks"]}


def run_mlmc(args) -> dict:
    """MLMC down-and-out put (Heston kappa 2, theta .04, sigma .5, rho -.7, v0 .04, SchemeNV,
    K 100, B 80, T 1; levels 2..10, dt = T / 2^l; target RMSE 1e-3 x price): plain MLMC
    against MLMC with the neural control variate (training included; each level keeps the
    control only where its variance ratio pays for the MLP rows), both through the public
    API, wall-clock, and at equal standard error (time x SE^2)."""
    import myquantlib_gb300 as m
    from myquantlib_gb300 import _abi
    if int(os.environ.get("RANK", "0")) != 0:
        return {}
    eng = m.Engine(0)
    model = m.HestonModel(m.HestonParams(2.0, 0.04, 0.5, -0.7, 0.04))
    job = m.make_job(model, m.HestonStepper(m.SchemeNV, m.TrackerBarrier), m.DownAndOutPut(100.0, 80.0, 1.0),
                     m.GreekMode.NONE, m.MonteCarloConfig(num_paths=1 << 20, time_steps=1024), 100.0, 0.02, 0.0)
    raw, _ = eng.price(job)
    price = float(raw[0, 0])

    def cfg(eps):
        c = _abi.MlmcConfigC()
        c.epsilon, c.L_min, c.L_max, c.N0, c.base_steps = eps, 2, 10, 10000, 1
        c.alpha, c.beta, c.adaptive_rates, c.seed, c.fd_bump, c.n_streams = 2.0, 1.0, 1, 42, 1e-4, 0
        return c

    eps = 1e-3 * price
    # warm-up (tables, streams, first launches)
    eng.mlmc_cv_price(job, cfg(20 * eps), m.pricers.ControlVariateConfig(
        hedge_every=1, iterations=10, pilot_paths=1 << 15, batch_paths=2048, learning_rate=3e-3, seed=7).c())
    # Each arm on three controller seeds: one run's allocation rests on pilot variance estimates
    # of rare barrier events, and a single noisy estimate on the finest level can triple its
    # path count, so one seed per arm compares allocations rather than estimators.
    seeds = (42, 43, 44)
    runs_plain, runs_cv = [], []
    with ClockSampler(0) as clk:
        for sd in seeds:
            c = cfg(eps)
            c.seed = sd
            res_plain = _abi.MlmcResultC()
            t0 = time.perf_counter()
            _abi.check(eng.lib.myql_mlmc_price(eng.handle, m.pricers.C.byref(job.c), m.pricers.C.byref(c),
                                               m.pricers.C.byref(res_plain)))
            runs_plain.append((time.perf_counter() - t0, res_plain, None))
        # the training budget follows plain MLMC's median time (the networks train on 32 steps)
        cvc = m.pricers.ControlVariateConfig.for_plain_time(statistics.median(t for t, _, _ in runs_plain),
                                                            time_steps=32, learning_rate=3e-3, seed=7).c()
        for sd in seeds:
            c = cfg(eps)
            c.seed = sd
            t0 = time.perf_counter()
            res_cv, plain_var = eng.mlmc_cv_price(job, c, cvc)
            runs_cv.append((time.perf_counter() - t0, res_cv, plain_var))

    def arm(runs, with_ratio):
        out = []
        for t, r, pv in runs:
            nl = int(r.n_levels)
            d = {"s": t, "price": r.price, "se": r.price_std_err, "levels": nl,
                 "paths_per_level": [int(r.paths_per_level[l]) for l in range(nl)], "path_steps": int(r.total_steps)}
            if with_ratio:
                d["variance_ratio_per_level"] = [float(pv[l] / max(r.var_diffs[l], 1e-300)) for l in range(nl)]
                d["cv_levels"] = [l for l in range(nl) if abs(pv[l] / max(r.var_diffs[l], 1e-300) - 1.0) > 1e-9]
            out.append(d)
        return out

    t_plain = statistics.median(t for t, _, _ in runs_plain)
    t_cv = statistics.median(t for t, _, _ in runs_cv)
    cost_plain = sum(t * r.price_std_err ** 2 for t, r, _ in runs_plain)
    cost_cv = sum(t * r.price_std_err ** 2 for t, r, _ in runs_cv)
    return {"metric": "time-to-RMSE (s) MLMC + neural CV vs plain MLMC", "value": t_cv, "unit": "s", "n_gpus": 1,
            "steps": len(seeds), "warmup": 1, "ms_per_step": t_cv * 1e3, "higher_is_better": False,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32 paths, fp64 level sums, bf16 MLP",
            "data": "synthetic",
            "config": {"workload": "MLMC Heston down-and-out put, SchemeNV, levels 2..10", "epsilon": eps,
                       "price": price, "controller_seeds": list(seeds),
                       "cv_training": {"pilot_paths": int(cvc.pilot_paths), "iterations": int(cvc.iterations),
                                       "batch_paths": int(cvc.batch_paths), "hedge_every": int(cvc.hedge_every)},
                       "value": "median over the seeds of the MLMC + CV wall time"},
            "plain": {"median_s": t_plain, "runs": arm(runs_plain, False)},
            "cv": {"median_s": t_cv, "runs": arm(runs_cv, True)},
            "speedup": t_plain / t_cv,
            # cost at equal standard error (the controllers stop at different SEs): sum of time x SE^2
            "efficiency_ratio": cost_plain / cost_cv,
            "clocks": clk.summary()}


def run_ncu_cv_case() -> None:
    """A small control-variate case for ncu: 2^16 pilot paths, 40 Adam steps, 2^18 priced paths."""
    import myquantlib_gb300 as m
    eng = m.Engine(0)
    cfg = cv_config(m, "asian", pilot=1 << 16, iterations=40)
    eng.cv_train(cv_jobs(m, "asian", 1 << 16)[0], cfg)
    eng.cv_price(cv_jobs(m, "asian", 1 << 18)[0], cfg)


def run_ncu_batch_case(scheme: str = "nci") -> None:
    """A small batched case for ncu: the first 256 uneven requests at up to 2^16 paths, priced twice,
    on the default launch shape (the one the autotuner keeps on the full batch), so that the first
    batch_kernel launch is a class kernel of the batch graph rather than a tuning candidate.  The
    scheme is the batch bench's (SchemeNCI with 64-row tables, or SchemeExact)."""
    import myquantlib_gb300 as m
    from myquantlib_gb300 import workloads
    eng = m.Engine(0)
    eng.set_batch_shape(128, 1, 0)
    if scheme == "nci":
        eng.set_nci_rows(64)
    rq = workloads.uneven_requests(256, max_log2_paths=16.0, scheme=m.SchemeNCI if scheme == "nci" else m.SchemeExact)
    jobs = [m.make_job(r.model, m.stepper_for(r.model, r.instrument, r.scheme), r.instrument, r.mode, r.cfg,
                       r.S0, r.r, r.q) for r in rq]
    for _ in range(2):
        eng.price_batch(jobs)


def run_ncu_qmc_case() -> None:
    """A small randomized-QMC case for ncu: the Double Bates Asian of the control-variate
    comparison (SchemeNCI factors, Merton jumps, 256 steps) on 2^19 Sobol points in 16 replicates
    (about 600 MB of records and tables on the device), priced twice."""
    import myquantlib_gb300 as m
    eng = m.Engine(0)
    for _ in range(2):
        eng.qmc_price(cv_jobs(m, "asian", 1 << 19)[0], 16)


def run_ncu_case(full: bool = False) -> None:
    """One maturity (T = 1) of the workload, priced twice, for an ncu capture: 2^18 paths (a few
    hundred MB on the device), or the full 2^22 paths for one-pass metrics."""
    import myquantlib_gb300 as m
    eng = m.Engine(0)
    job = workload_jobs(m, paths=PATHS if full else 1 << 18)[MATURITIES.index(1.0)]
    for _ in range(2):
        eng.price(job)


def main():
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["engine", "reference"], default="engine")
    ap.add_argument("--cpu-paths", type=int, default=1 << 16,
                    help="paths of one CPU pass over the strip (the reference arm's step and the cpu_baseline sample)")
    ap.add_argument("--no-cpu", action="store_true", help="skip the cpu_baseline leg")
    ap.add_argument("--no-cv", action="store_true", help="skip the time-to-relative-SE block of the strip line")
    ap.add_argument("--fourier-seeds", type=int, default=8, help="seeds of the multi-seed Fourier check")
    ap.add_argument("--workload", choices=["strip", "batch", "cv", "mlmc", "c1", "qmc"], default="strip",
                    help="strip: the Bates Full-Greeks strip (headline); batch: uneven requests in one launch; "
                         "cv: time-to-relative-SE of the neural control variate against plain MC; mlmc: MLMC "
                         "with and without the control variate; c1: plain Heston NV European (configuration 1); "
                         "qmc: randomized QMC (profiling case only, with --ncu-case)")
    ap.add_argument("--batch-jobs", type=int, default=4096)
    ap.add_argument("--batch-scheme", choices=["nci", "exact"], default="nci",
                    help="CIR scheme of the batched requests: nci, the dispatcher's default scheme, with "
                         "capped tables (the default), or exact")
    ap.add_argument("--batch-nci-rows", type=int, default=64,
                    help="row cap of each SchemeNCI table under --batch-scheme nci (Poisson counts beyond "
                         "it take the Wilson-Hilferty quantile, dof >= 2 x cap)")
    ap.add_argument("--ncu-case", action="store_true",
                    help="profiling case: one maturity (T=1), 2^18 paths, two requests, no timing")
    ap.add_argument("--ncu-full", action="store_true",
                    help="profiling case at the full 2^22 paths: for one-pass metrics (DRAM bytes, duration) "
                         "captured on one kernel (-k) and one launch (-c 1) only")
    args = ap.parse_args()
    if args.ncu_case or args.ncu_full:
        if args.workload == "cv":
            run_ncu_cv_case()
        elif args.workload == "batch":
            run_ncu_batch_case(args.batch_scheme)
        elif args.workload == "c1":
            run_ncu_c1_case()
        elif args.workload == "mlmc":
            run_ncu_mlmc_case()
        elif args.workload == "qmc":
            run_ncu_qmc_case()
        else:
            run_ncu_case(full=args.ncu_full)
        return
    if args.workload == "qmc":
        ap.error("--workload qmc is a profiling case: use it with --ncu-case")
    if args.impl == "reference":
        line = run_reference(args)
    else:
        line = {"batch": run_batch, "cv": run_cv, "mlmc": run_mlmc, "c1": run_c1}.get(args.workload, run_engine)(args)
    if line:
        print(json.dumps(line), flush=True)


if __name__ == "__main__":
    main()
