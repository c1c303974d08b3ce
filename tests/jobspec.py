"""Job specifications as plain dicts (the format of tests/golden/*.json).

A spec names the model, stepper schemes, instrument, Greek mode, Monte Carlo
configuration and market data; make_job() lowers it through the package's
reference-style API to the C ABI job.
"""
from __future__ import annotations

import copy

import myquantlib_gb300 as m

SCHEMES = {"NV": m.SchemeNV, "Exact": m.SchemeExact, "NCI": m.SchemeNCI}


def model_of(spec: dict):
    md = spec["model"]
    jump = md.get("jump")
    if jump is None:
        jp = m.NoJumpParams()
    elif jump["kind"] == "merton":
        jp = m.MertonParams(jump["lambda"], jump["mu"], jump["delta"])
    else:
        jp = m.KouParams(jump["lambda"], jump["p_up"], jump["eta1"], jump["eta2"])
    hs = [m.HestonParams(*h) for h in md.get("heston", [])]
    if len(hs) == 0:
        return m.ZeroFactorModel(md["vol"], jp)
    if len(hs) == 1:
        return m.SingleFactorModel(hs[0], jp)
    return m.DoubleFactorModel(hs[0], hs[1], jp)


def payoff_of(d: dict):
    ot = m.OptionType.Call if d.get("type", "call") == "call" else m.OptionType.Put
    kind = d.get("payoff", "vanilla")
    if kind == "vanilla":
        return m.PayoffVanilla(ot)
    if kind == "cash":
        return m.PayoffCashOrNothing(ot, d.get("eps", -1.0))
    return m.PayoffAssetOrNothing(ot, d.get("eps", -1.0))


def instrument_of(spec: dict):
    d = spec["instrument"]
    K = d["K"]
    T = d["T"]
    pay = payoff_of(d)
    kind = d["kind"]
    if kind == "european":
        return m.EuropeanOption(K, T, pay)
    if kind in ("asian_arith", "asian_geo"):
        trk = m.TrackerArithAsian if kind == "asian_arith" else m.TrackerGeoAsian
        return m.AsianOption(trk, pay, d.get("fixed", True), K, T, past_avg_S=d.get("past_avg_S", 0.0),
                             past_avg_log=d.get("past_avg_log", 0.0), t_elapsed=d.get("t_elapsed", 0.0))
    if kind == "lookback":
        return m.LookbackOption(pay, d.get("fixed", False), K, T, d.get("hist_min_S", 0.0),
                                d.get("hist_max_S", 0.0))
    if kind == "barrier":
        direction = m.BarrierDirection.Up if d["dir"] == "up" else m.BarrierDirection.Down
        action = m.BarrierAction.Out if d["action"] == "out" else m.BarrierAction.In
        timing = {"none": m.RebateTiming.NONE, "at_hit": m.RebateTiming.AtHit,
                  "at_maturity": m.RebateTiming.AtMaturity}[d.get("rebate_timing", "none")]
        return m.BarrierOption(pay, direction, action, timing, K, d["B"], T, d.get("r", 0.0),
                               d.get("rebate", 0.0))
    raise ValueError(kind)


def stepper_of(spec: dict, model, instr):
    sch = [SCHEMES[s] for s in spec.get("schemes", [])]
    nf = model.num_variance_factors
    v1 = sch[0] if nf >= 1 else m.NullVolScheme
    v2 = sch[1] if nf == 2 else m.NullVolScheme
    jp = {m.NoJumpParams: m.NoJumps, m.MertonParams: m.MertonJump, m.KouParams: m.KouJump}[type(model.jump)]
    return m.ASVJStepper(v1, v2, jp, instr.Tracker)


def config_of(spec: dict) -> m.MonteCarloConfig:
    c = spec.get("config", {})
    return m.MonteCarloConfig(num_paths=c.get("paths", 10000), time_steps=c.get("steps", 100),
                              seed=c.get("seed", 42), fd_bump=c.get("fd_bump", 1e-4),
                              vol_bump=c.get("vol_bump", 1e-4), t_bump=c.get("t_bump", 1e-4),
                              r_bump=c.get("r_bump", 1e-4), n_streams=c.get("streams", 0))


MODES = {"none": m.GreekMode.NONE, "essential": m.GreekMode.ESSENTIAL, "full": m.GreekMode.FULL}


def make_job(spec: dict):
    model = model_of(spec)
    instr = instrument_of(spec)
    return m.make_job(model, stepper_of(spec, model, instr), instr, MODES[spec.get("mode", "none")],
                      config_of(spec), spec.get("S0", 100.0), spec.get("r", 0.02), spec.get("q", 0.0))


def with_config(spec: dict, **kw) -> dict:
    s = copy.deepcopy(spec)
    s.setdefault("config", {}).update(kw)
    return s
