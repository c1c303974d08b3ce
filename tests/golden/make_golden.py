"""Generates tests/golden/*.json from the reference itself.

Run here, where the reference sources are present:
    python tests/golden/make_golden.py
It builds oracle/_ref (the reference's unmodified headers compiled against the
Boost-API shim in oracle/compat) and records, for every job spec below:
  reference_mc.json      -- MonteCarloPricer::calculate outputs (1 and 3 threads)
  reference_fourier.json -- FourierPricer<..., GreekMode::Full> values (tol 1e-10)
The tests compare the oracle's C restatement against these numbers and the
GPU engine against the restatement and the Fourier values.  The reference's
OpenMP reductions merge in a run-dependent order, so regenerated values can
move in the last digits (about 1e-14 relative for the Fourier prices and on the
3-thread MC outputs); the 1-thread MC outputs are reproducible bit for bit.
"""
from __future__ import annotations

import json
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(HERE.parent))

import numpy as np  # noqa: E402

from oracle import oracle  # noqa: E402
import jobspec  # noqa: E402

H1 = [1.5, 0.04, 0.3, -0.7, 0.04]            # configuration 1 Heston
HB = [2.0, 0.05, 0.9, -0.6, 0.05]            # configuration 2 Heston part (Feller violated)
HK = [2.0, 0.04, 0.4, -0.7, 0.04]            # mc_full_greek_verifier.cpp:137 h1
HK2 = [3.0, 0.02, 0.2, -0.3, 0.02]           # mc_full_greek_verifier.cpp:138 h2
H5 = [2.0, 0.04, 0.5, -0.7, 0.04]            # configuration 5 Heston
MERTON2 = {"kind": "merton", "lambda": 0.5, "mu": -0.1, "delta": 0.15}
KOU3 = {"kind": "kou", "lambda": 0.5, "p_up": 0.4, "eta1": 10.0, "eta2": 5.0}
KOUV = {"kind": "kou", "lambda": 3.0, "p_up": 0.3, "eta1": 25.0, "eta2": 15.0}


def eur(K=100.0, T=1.0, **kw):
    return {"kind": "european", "K": K, "T": T, **kw}


MC_SPECS = [
    {"name": "c1_heston_nv_call", "model": {"heston": [H1]}, "schemes": ["NV"], "instrument": eur(),
     "mode": "none", "config": {"paths": 20000, "steps": 100}},
    {"name": "heston_nv_call_essential", "model": {"heston": [H1]}, "schemes": ["NV"], "instrument": eur(),
     "mode": "essential", "config": {"paths": 20000, "steps": 100}},
    {"name": "heston_nv_put_full", "model": {"heston": [H1]}, "schemes": ["NV"],
     "instrument": eur(95.0, 0.5, type="put"), "mode": "full", "config": {"paths": 4000, "steps": 50}},
    {"name": "heston_exact_call", "model": {"heston": [H1]}, "schemes": ["Exact"], "instrument": eur(),
     "mode": "none", "config": {"paths": 8000, "steps": 25}},
    {"name": "heston_nci_call", "model": {"heston": [H1]}, "schemes": ["NCI"], "instrument": eur(),
     "mode": "essential", "config": {"paths": 8000, "steps": 25}},
    {"name": "c2_bates_nci_full_k100_t1", "model": {"heston": [HB], "jump": MERTON2}, "schemes": ["NCI"],
     "instrument": eur(100.63492063492063, 1.0), "mode": "full", "config": {"paths": 2000, "steps": 200}},
    {"name": "c2_bates_nci_strip_essential", "model": {"heston": [HB], "jump": MERTON2}, "schemes": ["NCI"],
     "instrument": eur([60.0, 80.0, 100.0, 120.0, 140.0], 0.5), "mode": "essential",
     "config": {"paths": 2000, "steps": 100}},
    {"name": "c3_bateskou_nci_asian", "model": {"heston": [H5], "jump": KOU3}, "schemes": ["NCI"],
     "instrument": {"kind": "asian_arith", "K": 95.0, "T": 1.0}, "mode": "none",
     "config": {"paths": 2000, "steps": 64}},
    {"name": "c3_bateskou_nci_upout", "model": {"heston": [H5], "jump": KOU3}, "schemes": ["NCI"],
     "instrument": {"kind": "barrier", "dir": "up", "action": "out", "K": 105.0, "B": 130.0, "T": 1.0},
     "mode": "essential", "config": {"paths": 2000, "steps": 64}},
    {"name": "c3_dheston_nci_asian", "model": {"heston": [HK, HK2]}, "schemes": ["NCI", "NCI"],
     "instrument": {"kind": "asian_arith", "K": 100.0, "T": 1.0}, "mode": "none",
     "config": {"paths": 2000, "steps": 32}},
    {"name": "c4_dbates_nv_nci_asian", "model": {"heston": [[2.0, 0.03, 0.4, -0.7, 0.03], [0.5, 0.02, 0.3, -0.3, 0.02]],
                                               "jump": {"kind": "merton", "lambda": 0.3, "mu": -0.05, "delta": 0.1}},
     "schemes": ["NV", "NCI"], "instrument": {"kind": "asian_arith", "K": 100.0, "T": 2.0}, "mode": "none",
     "config": {"paths": 2000, "steps": 256}},
    {"name": "c5_heston_nv_downout_put", "model": {"heston": [H5]}, "schemes": ["NV"],
     "instrument": {"kind": "barrier", "dir": "down", "action": "out", "K": 100.0, "B": 80.0, "T": 1.0,
                    "type": "put"}, "mode": "full", "config": {"paths": 2000, "steps": 64}},
    {"name": "heston_lookback_float_call", "model": {"heston": [H1]}, "schemes": ["NV"],
     "instrument": {"kind": "lookback", "K": 100.0, "T": 1.0, "fixed": False}, "mode": "essential",
     "config": {"paths": 4000, "steps": 64}},
    {"name": "heston_lookback_inflight", "model": {"heston": [H1]}, "schemes": ["NV"],
     "instrument": {"kind": "lookback", "K": 100.0, "T": 0.5, "fixed": False, "hist_min_S": 92.0,
                    "hist_max_S": 108.0}, "mode": "none", "config": {"paths": 4000, "steps": 32}},
    {"name": "bs_geo_asian_inflight", "model": {"vol": 0.2}, "schemes": [],
     "instrument": {"kind": "asian_geo", "K": 100.0, "T": 0.75, "past_avg_log": 4.58, "t_elapsed": 0.25},
     "mode": "essential", "config": {"paths": 4000, "steps": 50}},
    {"name": "heston_arith_asian_inflight", "model": {"heston": [H1]}, "schemes": ["NV"],
     "instrument": {"kind": "asian_arith", "K": 100.0, "T": 0.5, "past_avg_S": 101.5, "past_avg_log": 4.62,
                    "t_elapsed": 0.5}, "mode": "essential", "config": {"paths": 4000, "steps": 50}},
    {"name": "heston_cash_digital_essential", "model": {"heston": [H1]}, "schemes": ["NV"],
     "instrument": eur(105.0, 1.0, payoff="cash"), "mode": "essential", "config": {"paths": 8000, "steps": 50}},
    {"name": "heston_asset_digital_put_full", "model": {"heston": [H1]}, "schemes": ["NV"],
     "instrument": eur(95.0, 1.0, payoff="asset", type="put"), "mode": "full",
     "config": {"paths": 4000, "steps": 50}},
    {"name": "dbateskou_nv_full", "model": {"heston": [HK, HK2], "jump": KOUV}, "schemes": ["NV", "NV"],
     "instrument": eur(), "mode": "full", "config": {"paths": 2000, "steps": 50}},
    {"name": "bs_call_oneshot", "model": {"vol": 0.25}, "schemes": [], "instrument": eur(110.0, 2.0),
     "mode": "essential", "config": {"paths": 20000, "steps": 100}},
    {"name": "bs_downout_put_day0_breach", "model": {"vol": 0.25}, "schemes": [],
     "instrument": {"kind": "barrier", "dir": "down", "action": "out", "K": 100.0, "B": 100.5, "T": 1.0,
                    "type": "put"}, "mode": "essential", "config": {"paths": 2000, "steps": 20}},
] + [
    # every remaining instrument branch: floating-strike Asians and Asian puts
    # (Asian.hpp:31-37), fixed-strike lookbacks and lookback puts (Lookback.hpp:22-33,
    # 70-74), knock-in barriers and the AtHit / AtMaturity rebates (Barrier.hpp:29-45)
    {"name": name, "model": model, "schemes": ["NV"] if "heston" in model else [], "instrument": ins,
     "mode": mode, "config": {"paths": paths, "steps": steps}}
    for name, model, ins, mode, paths, steps in [
        ("heston_asian_arith_float_call", {"heston": [H1]},
         {"kind": "asian_arith", "K": 100.0, "T": 1.0, "fixed": False}, "essential", 4000, 64),
        ("heston_asian_arith_fixed_put", {"heston": [H1]},
         {"kind": "asian_arith", "K": 100.0, "T": 1.0, "type": "put"}, "essential", 4000, 64),
        ("heston_asian_geo_float_put_full", {"heston": [H1]},
         {"kind": "asian_geo", "K": 100.0, "T": 1.0, "fixed": False, "type": "put"}, "full", 2000, 50),
        ("heston_asian_geo_fixed_put_inflight", {"heston": [H1]},
         {"kind": "asian_geo", "K": 100.0, "T": 0.6, "type": "put", "past_avg_log": 4.63, "t_elapsed": 0.4},
         "essential", 4000, 40),
        ("bs_asian_arith_float_put_inflight", {"vol": 0.25},
         {"kind": "asian_arith", "K": 100.0, "T": 0.7, "fixed": False, "type": "put", "past_avg_S": 98.0,
          "past_avg_log": 4.58, "t_elapsed": 0.3}, "essential", 4000, 35),
        ("heston_lookback_fixed_call", {"heston": [H1]},
         {"kind": "lookback", "K": 105.0, "T": 1.0, "fixed": True}, "essential", 4000, 64),
        ("heston_lookback_fixed_put_inflight", {"heston": [H1]},
         {"kind": "lookback", "K": 98.0, "T": 0.5, "fixed": True, "type": "put", "hist_min_S": 95.0,
          "hist_max_S": 104.0}, "none", 4000, 32),
        ("heston_lookback_float_put_full", {"heston": [H1]},
         {"kind": "lookback", "K": 100.0, "T": 1.0, "fixed": False, "type": "put"}, "full", 2000, 50),
        ("bs_lookback_fixed_put", {"vol": 0.3},
         {"kind": "lookback", "K": 95.0, "T": 1.0, "fixed": True, "type": "put"}, "essential", 4000, 50),
        ("heston_upin_call", {"heston": [H1]},
         {"kind": "barrier", "dir": "up", "action": "in", "K": 100.0, "B": 120.0, "T": 1.0},
         "essential", 4000, 64),
        ("heston_downin_put_full", {"heston": [H1]},
         {"kind": "barrier", "dir": "down", "action": "in", "K": 100.0, "B": 85.0, "T": 1.0, "type": "put"},
         "full", 2000, 50),
        ("heston_upout_call_rebate_at_hit", {"heston": [H1]},
         {"kind": "barrier", "dir": "up", "action": "out", "K": 100.0, "B": 125.0, "T": 1.0, "rebate": 3.0,
          "r": 0.02, "rebate_timing": "at_hit"}, "essential", 4000, 64),
        ("heston_downout_call_rebate_at_maturity", {"heston": [H1]},
         {"kind": "barrier", "dir": "down", "action": "out", "K": 95.0, "B": 85.0, "T": 1.0, "rebate": 2.0,
          "r": 0.02, "rebate_timing": "at_maturity"}, "essential", 4000, 64),
        ("heston_upin_put_rebate_at_maturity", {"heston": [H1]},
         {"kind": "barrier", "dir": "up", "action": "in", "K": 105.0, "B": 115.0, "T": 1.0, "type": "put",
          "rebate": 1.5, "r": 0.02, "rebate_timing": "at_maturity"}, "none", 4000, 64),
        ("heston_downin_call_rebate_at_hit", {"heston": [H1]},
         {"kind": "barrier", "dir": "down", "action": "in", "K": 100.0, "B": 90.0, "T": 1.0, "rebate": 2.5,
          "r": 0.03, "rebate_timing": "at_hit"}, "essential", 4000, 64),
        ("heston_upout_put_rebate_at_hit_full", {"heston": [H1]},
         {"kind": "barrier", "dir": "up", "action": "out", "K": 100.0, "B": 120.0, "T": 1.0, "type": "put",
          "rebate": 4.0, "r": 0.02, "rebate_timing": "at_hit"}, "full", 2000, 50),
        ("bs_downout_call_rebate_at_hit", {"vol": 0.3},
         {"kind": "barrier", "dir": "down", "action": "out", "K": 100.0, "B": 90.0, "T": 1.0, "rebate": 5.0,
          "r": 0.05, "rebate_timing": "at_hit"}, "essential", 4000, 50),
    ]
]

FOURIER_SPECS = [
    {"name": "c1_heston_call", "model": {"heston": [H1]}, "instrument": eur()},
    {"name": "heston_put_k95_t05", "model": {"heston": [H1]}, "instrument": eur(95.0, 0.5, type="put")},
    {"name": "heston_cash_k105", "model": {"heston": [H1]}, "instrument": eur(105.0, 1.0, payoff="cash")},
    {"name": "heston_asset_put_k95", "model": {"heston": [H1]}, "instrument": eur(95.0, 1.0, payoff="asset", type="put")},
    {"name": "heston_vg_call", "model": {"heston": [HK]}, "instrument": eur(), "r": 0.05, "q": 0.02},
    {"name": "dheston_vg_call", "model": {"heston": [HK, HK2]}, "instrument": eur(), "r": 0.05, "q": 0.02},
    {"name": "bateskou_vg_call", "model": {"heston": [HK], "jump": KOUV}, "instrument": eur(), "r": 0.05, "q": 0.02},
    {"name": "dbateskou_vg_call", "model": {"heston": [HK, HK2], "jump": KOUV}, "instrument": eur(), "r": 0.05,
     "q": 0.02},
    {"name": "bs_call_k110_t2", "model": {"vol": 0.25}, "instrument": eur(110.0, 2.0)},
    {"name": "merton_call", "model": {"vol": 0.2, "jump": MERTON2}, "instrument": eur()},
    {"name": "kou_call", "model": {"vol": 0.2, "jump": KOU3}, "instrument": eur()},
    {"name": "heston_nci_call_k100", "model": {"heston": [H5]}, "instrument": eur()},
] + [
    {"name": f"c2_bates_call_k{K:.4f}_t{T}", "model": {"heston": [HB], "jump": MERTON2},
     "instrument": eur(K, T)}
    for T in (0.25, 1.0, 4.0) for K in (60.0, 100.63492063492063, 140.0)
]


def main() -> None:
    oracle.build(ref=True)
    mc = []
    for spec in MC_SPECS:
        job = jobspec.make_job(spec)
        rec = dict(spec)
        rec["outputs"] = {}
        for nt in (1, 3):
            out = oracle.ref_mc_price(job, nt)
            if out is None:
                raise RuntimeError(f"{spec['name']}: not instantiated in oracle/ref_shim.cpp")
            rec["outputs"][str(nt)] = out.tolist()
        mc.append(rec)
        print("mc", spec["name"], rec["outputs"]["1"][0])
    four = []
    for spec in FOURIER_SPECS:
        s = dict(spec)
        s.setdefault("schemes", ["NV"] * len(spec["model"].get("heston", [])))
        s.setdefault("config", {"paths": 1, "steps": 1})
        job = jobspec.make_job(s)
        vals = oracle.ref_fourier(job, 1e-10)
        rec = dict(spec)
        rec["fourier"] = vals.tolist()
        four.append(rec)
        print("fourier", spec["name"], vals[0])
    (HERE / "reference_mc.json").write_text(json.dumps(mc, indent=1))
    (HERE / "reference_fourier.json").write_text(json.dumps(four, indent=1))


if __name__ == "__main__":
    main()
