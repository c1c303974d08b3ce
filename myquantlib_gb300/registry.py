"""Runtime registries and a record front-end for the dispatcher.

- **Registries.** `build_model`, `build_european` and `build_instrument` mirror
  dispatcher/ModelRegistry.hpp:35-72 and dispatcher/InstrumentRegistry.hpp:142-257. They build a
  model or instrument from its type name and a flat parameter struct (`RuntimeModelParams`,
  `RuntimeInstrumentParams`). An unknown name raises ValueError, the reference's
  std::invalid_argument, with the reference's message.
- **Fourier.** `price_fourier` is dispatcher::price_fourier (PricingDispatch.hpp:128-155) on the
  engine's FP64 Gil-Pelaez kernel; `price_mc` lives in dispatch.py.
- **Records.** `request_from_record`, `load_requests` and `price_records` read pricing requests
  from JSON objects or CSV rows; the reference's demo decodes them by hand
  (benchmarks/runtime_dispatch_demo.cpp:12-45). Every request that the batched launch accepts
  (a scalar instrument with GreekMode None or Essential) is priced in one persistent launch; the
  others go through price_mc one by one. Results come back in input order.

A record is a dict:

    {"model": "Bates", "heston1": [kappa, theta, sigma, rho, v0], "merton": [lambda, mu, delta],
     "instrument": "Vanilla", "option_type": "Call", "strikes": [90, 100, 110], "maturity": 1.0,
     "S0": 100, "r": 0.02, "q": 0.0, "paths": 100000, "steps": 50, "seed": 42,
     "mode": "Essential", "scheme": "NCI"}

with optional "heston2", "vol", "kou" ([lambda, p_up, eta1, eta2]), "barrier", "rebate",
"rate" (rebate discounting; defaults to r), "fd_bump", "vol_bump", "t_bump", "r_bump",
"streams" and "stream_offset". "mode" defaults to None and "scheme" to NCI, the defaults of
dispatcher::price_mc. A CSV row carries the same fields flat: kappa, theta, sigma, rho, v0
(factor 1), kappa2 … v02 (factor 2), jump_lambda, merton_mu, merton_delta, kou_p_up, kou_eta1,
kou_eta2, and strikes separated by ';'.
"""
from __future__ import annotations

import csv
import io
import json
import time
from dataclasses import dataclass, field
from pathlib import Path

from . import dispatch as _d
from . import pricers as _p

MODEL_TYPES = ("BlackScholes", "Merton", "Kou", "Heston", "Bates", "BatesKou", "DoubleHeston",
               "DoubleBates", "DoubleBatesKou")
EUROPEAN_TYPES = ("Vanilla", "CashOrNothing", "AssetOrNothing")
INSTRUMENT_TYPES = EUROPEAN_TYPES + ("GeoAsian", "GeoAsianFloating", "ArithAsian", "ArithAsianFloating",
                                     "LookbackFixed", "LookbackFloating", "UpAndOut", "UpAndIn",
                                     "DownAndOut", "DownAndIn")
_ZERO_HESTON = _p.HestonParams(0.0, 0.0, 0.0, 0.0, 0.0)


@dataclass
class RuntimeModelParams:  # ModelRegistry.hpp:22-30
    heston1: _p.HestonParams = _ZERO_HESTON
    heston2: _p.HestonParams = _ZERO_HESTON
    vol: float = 0.0
    merton: _p.MertonParams = field(default_factory=lambda: _p.MertonParams(0.0, 0.0, 0.0))
    kou: _p.KouParams = field(default_factory=lambda: _p.KouParams(0.0, 0.0, 0.0, 0.0))


def build_model(model_type: str, params: RuntimeModelParams):  # ModelRegistry.hpp:35-72
    p = params
    makers = {
        "BlackScholes": lambda: _p.BlackScholesModel(p.vol),
        "Merton": lambda: _p.MertonModel(p.vol, p.merton),
        "Kou": lambda: _p.KouModel(p.vol, p.kou),
        "Heston": lambda: _p.HestonModel(p.heston1),
        "Bates": lambda: _p.BatesModel(p.heston1, p.merton),
        "BatesKou": lambda: _p.BatesKouModel(p.heston1, p.kou),
        "DoubleHeston": lambda: _p.DoubleHestonModel(p.heston1, p.heston2),
        "DoubleBates": lambda: _p.DoubleBatesModel(p.heston1, p.heston2, p.merton),
        "DoubleBatesKou": lambda: _p.DoubleBatesKouModel(p.heston1, p.heston2, p.kou),
    }
    if model_type not in makers:
        raise ValueError("Unknown model type: " + model_type)
    return makers[model_type]()


@dataclass
class RuntimeInstrumentParams:  # InstrumentRegistry.hpp:127-137
    strikes: list = field(default_factory=list)
    maturity: float = 0.0
    barrier_level: float = 0.0
    rebate: float = 0.0
    rate: float = 0.0  # AtHit rebate discounting


def _option_type(option_type: str):
    return {"Call": _p.OptionType.Call, "Put": _p.OptionType.Put}.get(option_type)


def build_european(type_: str, option_type: str, params: RuntimeInstrumentParams):
    """InstrumentRegistry.hpp:142-171: the European instruments (strips), for price_mc and
    price_fourier alike."""
    ot = _option_type(option_type)
    payoff = {"Vanilla": _p.PayoffVanilla, "CashOrNothing": _p.PayoffCashOrNothing,
              "AssetOrNothing": _p.PayoffAssetOrNothing}.get(type_)
    if ot is None or payoff is None:
        raise ValueError("Unknown European instrument: " + type_ + " " + option_type)
    return _p.EuropeanOption(list(params.strikes), params.maturity, payoff(ot))


def build_instrument(type_: str, option_type: str, params: RuntimeInstrumentParams):
    """InstrumentRegistry.hpp:176-257: every MC instrument.  Europeans are strips; fixed-strike
    exotics take the first strike (0 if none); floating-strike ones take none; barriers carry
    RebateTiming::None."""
    if type_ in EUROPEAN_TYPES:
        try:
            return build_european(type_, option_type, params)
        except ValueError:
            raise ValueError("Unknown instrument: " + type_ + " " + option_type) from None
    ot = _option_type(option_type)
    if ot is None or type_ not in INSTRUMENT_TYPES:
        raise ValueError("Unknown instrument: " + type_ + " " + option_type)
    K0 = float(params.strikes[0]) if len(params.strikes) else 0.0
    T = params.maturity
    pay = _p.PayoffVanilla(ot)
    if type_ in ("GeoAsian", "GeoAsianFloating", "ArithAsian", "ArithAsianFloating"):
        tracker = _p.TrackerGeoAsian if type_.startswith("Geo") else _p.TrackerArithAsian
        fixed = not type_.endswith("Floating")
        return _p.AsianOption(tracker, pay, fixed, K0 if fixed else 0.0, T)
    if type_ in ("LookbackFixed", "LookbackFloating"):
        fixed = type_ == "LookbackFixed"
        return _p.LookbackOption(pay, fixed, K0 if fixed else 0.0, T)
    direction = _p.BarrierDirection.Up if type_.startswith("Up") else _p.BarrierDirection.Down
    action = _p.BarrierAction.Out if type_.endswith("Out") else _p.BarrierAction.In
    return _p.BarrierOption(pay, direction, action, _p.RebateTiming.NONE, K0, params.barrier_level, T,
                            params.rate, params.rebate)


# --------------------------------------------------------------------------- Fourier dispatch
def price_fourier(model, instrument, S0: float, r: float, q: float,
                  mode: _p.GreekMode = _p.GreekMode.NONE,
                  engine: _p.Engine | None = None) -> _d.DispatchResult:
    """dispatcher::price_fourier (PricingDispatch.hpp:128-155): FP64 Gil-Pelaez prices and Greeks
    of a European instrument.  The standard-error fields stay empty, as for the reference's
    FourierResult."""
    if instrument.kind != _p._abi.INSTR_EUROPEAN:
        raise TypeError("price_fourier takes European instruments (AnyEuropeanInstrument)")
    eng = engine or _p.default_engine()
    mode = _p.GreekMode(mode)
    job = _p.make_job(model, _p.stepper_for(model, instrument, _p.SchemeNCI), instrument, mode,
                      _p.MonteCarloConfig(num_paths=1, time_steps=1), S0, r, q)
    t0 = time.perf_counter()
    raw = eng.fourier(job, mode)
    out = _d._format(raw, mode, (time.perf_counter() - t0) * 1e3)
    for name in ("prices_std_err", "deltas_std_err", "gammas_std_err", "vegas_std_err",
                 "thetas_std_err", "rhos_std_err"):
        setattr(out, name, [])
    return out


# --------------------------------------------------------------------------- records
_MODES = {"None": _p.GreekMode.NONE, "Essential": _p.GreekMode.ESSENTIAL, "Full": _p.GreekMode.FULL}
_SCHEMES = {"NCI": _p.SchemeNCI, "NV": _p.SchemeNV, "Exact": _p.SchemeExact}
_CSV_HESTON = (("kappa", "theta", "sigma", "rho", "v0"), ("kappa2", "theta2", "sigma2", "rho2", "v02"))


def _heston(v) -> _p.HestonParams:
    if isinstance(v, dict):
        return _p.HestonParams(*(float(v[k]) for k in ("kappa", "theta", "sigma", "rho", "v0")))
    if len(v) != 5:
        raise ValueError("Heston parameters are [kappa, theta, sigma, rho, v0]")
    return _p.HestonParams(*(float(x) for x in v))


def record_from_csv_row(row: dict) -> dict:
    """A flat CSV row -> the record form (empty cells are absent fields)."""
    row = {k.strip(): v.strip() for k, v in row.items() if k is not None and v is not None and v.strip() != ""}
    rec = {k: row[k] for k in ("model", "instrument", "option_type", "mode", "scheme") if k in row}
    for i, keys in enumerate(_CSV_HESTON):
        if all(k in row for k in keys):
            rec["heston%d" % (i + 1)] = [float(row[k]) for k in keys]
    if "jump_lambda" in row:
        if "merton_mu" in row:
            rec["merton"] = [float(row["jump_lambda"]), float(row["merton_mu"]), float(row["merton_delta"])]
        if "kou_p_up" in row:
            rec["kou"] = [float(row["jump_lambda"]), float(row["kou_p_up"]), float(row["kou_eta1"]),
                          float(row["kou_eta2"])]
    if "strikes" in row:
        rec["strikes"] = [float(x) for x in row["strikes"].split(";") if x.strip()]
    for k in ("vol", "maturity", "barrier", "rebate", "rate", "S0", "r", "q", "fd_bump", "vol_bump",
              "t_bump", "r_bump"):
        if k in row:
            rec[k] = float(row[k])
    for k in ("paths", "steps", "seed", "streams", "stream_offset"):
        if k in row:
            rec[k] = int(row[k])
    return rec


def request_from_record(rec: dict) -> _d.Request:
    """One record -> a dispatcher Request (the arguments of one price_mc call)."""
    mp = RuntimeModelParams()
    if "heston1" in rec:
        mp.heston1 = _heston(rec["heston1"])
    if "heston2" in rec:
        mp.heston2 = _heston(rec["heston2"])
    mp.vol = float(rec.get("vol", 0.0))
    if "merton" in rec:
        mp.merton = _p.MertonParams(*(float(x) for x in rec["merton"]))
    if "kou" in rec:
        mp.kou = _p.KouParams(*(float(x) for x in rec["kou"]))
    model = build_model(rec["model"], mp)
    strikes = rec.get("strikes", rec.get("strike", []))
    strikes = [float(strikes)] if isinstance(strikes, (int, float)) else [float(k) for k in strikes]
    r = float(rec.get("r", 0.0))
    ip = RuntimeInstrumentParams(strikes=strikes, maturity=float(rec["maturity"]),
                                 barrier_level=float(rec.get("barrier", 0.0)),
                                 rebate=float(rec.get("rebate", 0.0)), rate=float(rec.get("rate", r)))
    instrument = build_instrument(rec["instrument"], rec.get("option_type", "Call"), ip)
    mode = rec.get("mode", "None")
    if mode not in _MODES:
        raise ValueError("Unknown GreekMode: " + str(mode))
    scheme = rec.get("scheme", "NCI")
    if scheme not in _SCHEMES:
        raise ValueError("Unknown vol scheme: " + str(scheme))
    cfg = _p.MonteCarloConfig(num_paths=int(rec.get("paths", 100000)), time_steps=int(rec.get("steps", 100)),
                              seed=int(rec.get("seed", 42)), n_streams=int(rec.get("streams", 0)),
                              stream_offset=int(rec.get("stream_offset", 0)))
    for k in ("fd_bump", "vol_bump", "t_bump", "r_bump"):
        if k in rec:
            setattr(cfg, k, float(rec[k]))
    return _d.Request(model, instrument, cfg, float(rec.get("S0", 100.0)), r, float(rec.get("q", 0.0)),
                      _MODES[mode], _SCHEMES[scheme])


def load_records(source) -> list[dict]:
    """Records from a .json / .csv path, JSON or CSV text, or a list of dicts."""
    if isinstance(source, list):
        return [dict(r) for r in source]
    text = source
    is_csv = False
    if isinstance(source, Path) or (isinstance(source, str) and "\n" not in source and
                                    source.endswith((".json", ".csv"))):
        path = Path(source)
        text = path.read_text()
        is_csv = path.suffix == ".csv"
    else:
        is_csv = not text.lstrip().startswith(("[", "{"))
    if is_csv:
        return [record_from_csv_row(row) for row in csv.DictReader(io.StringIO(text))]
    data = json.loads(text)
    return [data] if isinstance(data, dict) else list(data)


def load_requests(source) -> list[_d.Request]:
    return [request_from_record(r) for r in load_records(source)]


def batchable(rq: _d.Request) -> bool:
    """Whether myql_mc_price_batch takes the request: a scalar instrument, GreekMode None or
    Essential."""
    return (not rq.instrument.is_strip) and _p.GreekMode(rq.mode) != _p.GreekMode.FULL


def price_requests(requests: list[_d.Request], engine: _p.Engine | None = None) -> list[_d.DispatchResult]:
    """Prices every request: the batchable ones in one persistent launch, the others one by one."""
    eng = engine or _p.default_engine()
    out: list = [None] * len(requests)
    idx = [i for i, rq in enumerate(requests) if batchable(rq)]
    if idx:
        for i, res in zip(idx, _d.price_mc_batch([requests[i] for i in idx], eng)):
            out[i] = res
    for i, rq in enumerate(requests):
        if out[i] is None:
            out[i] = _d.price_mc(rq.model, rq.instrument, rq.cfg, rq.S0, rq.r, rq.q, rq.mode, rq.scheme, eng)
    return out


def price_records(source, engine: _p.Engine | None = None) -> list[_d.DispatchResult]:
    return price_requests(load_requests(source), engine)
