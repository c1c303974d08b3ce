"""Times the FP64 C restatement (oracle/_build/liboracle_fast.so) against the
reference's own headers compiled here (oracle/_ref/libmyql_ref_fast.so), both
at the reference's release flags, on samples of the Bates SchemeNCI strip
workload (Heston kappa 2, theta .05, sigma .9, rho -.6, v0 .05 + Merton
.5/-.1/.15; 200 steps per year; S0 100, r .02, q 0, seed 42).

TEST INFRASTRUCTURE: it shows that the restatement, which stands in for the
reference on machines where the reference's sources are absent, is as fast as
the reference itself.  Run where the reference sources exist:

    python oracle/time_port_vs_ref.py [--threads N] [--paths P] [--reps R]

Two samples, because the reference's GreekMode::Full on a strike strip writes
into empty vectors (undefined behaviour):
  * the 64-strike strip at each maturity in GreekMode::Essential;
  * GreekMode::Full for one strike (K 100.6349) at each maturity.
Each library prices the same jobs on the same thread count; the best of R
repetitions is kept.  Prints one JSON line.
"""
from __future__ import annotations

import argparse
import json
import os
import sys
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent.parent
sys.path[0] = str(ROOT)  # the repository root, not oracle/ (its oracle.py would shadow the package)

MATURITIES = [0.25, 0.5, 1.0, 1.5, 2.0, 2.5, 3.0, 4.0]
STRIKES = list(60.0 + 80.0 * np.arange(64) / 63.0)


def jobs(m, paths: int, full_scalar: bool):
    model = m.BatesModel(m.HestonParams(2.0, 0.05, 0.9, -0.6, 0.05), m.MertonParams(0.5, -0.1, 0.15))
    out = []
    for T in MATURITIES:
        cfg = m.MonteCarloConfig(num_paths=paths, time_steps=int(round(200 * T)), seed=42)
        if full_scalar:
            ins, mode = m.EuropeanOption(STRIKES[26], T), m.GreekMode.FULL
        else:
            ins, mode = m.EuropeanOption(STRIKES, T), m.GreekMode.ESSENTIAL
        out.append(m.make_job(model, m.BatesStepper(m.SchemeNCI), ins, mode, cfg, 100.0, 0.02, 0.0))
    return out


def best_time(fn, reps: int) -> float:
    best = float("inf")
    for _ in range(reps):
        t0 = time.perf_counter()
        fn()
        best = min(best, time.perf_counter() - t0)
    return best


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--threads", type=int, default=os.cpu_count() or 1)
    ap.add_argument("--paths", type=int, default=1 << 14)
    ap.add_argument("--reps", type=int, default=3)
    args = ap.parse_args()
    import myquantlib_gb300 as m
    from oracle import oracle
    oracle.build(ref=True)
    res = {"threads": args.threads, "paths": args.paths, "reps": args.reps}
    for name, full in (("strip_essential", False), ("scalar_full", True)):
        js = jobs(m, args.paths, full)
        port = best_time(lambda: [oracle.mc_price(j, oracle.LAYOUT_REFERENCE, args.threads, fast=True)
                                  for j in js], args.reps)
        ref = best_time(lambda: [oracle.ref_mc_price(j, args.threads, fast=True) for j in js], args.reps)
        res[name] = {"port_s": port, "reference_s": ref, "port_over_reference_speed": ref / port}
    print(json.dumps(res))


if __name__ == "__main__":
    main()
