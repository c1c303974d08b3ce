"""Runtime dispatcher mirror (myql/dispatcher/PricingDispatch.hpp).

`price_mc(model, instrument, cfg, S0, r, q, mode, scheme)` is
dispatcher::price_mc<Mode, ExplicitVolScheme> (PricingDispatch.hpp:93-126):
the stepper follows dispatcher::StepperFor (StepperTraits.hpp:67-81) and the
result is a DispatchResult (PricingDispatch.hpp:18-38).

`price_mc_batch(requests)` has no single counterpart in the reference, whose
callers loop over price_mc (benchmarks/runtime_dispatch_demo.cpp:52): here
the whole list is one persistent GPU launch (myql_mc_price_batch).  Batched
requests take scalar instruments (one strike) with GreekMode NONE or
ESSENTIAL, and each returns what the same request priced alone returns up
to FP32 summation order.
"""
from __future__ import annotations

import time
from dataclasses import dataclass, field

import numpy as np

from . import pricers as _p


@dataclass
class DispatchResult:  # PricingDispatch.hpp:18-38
    prices: list = field(default_factory=list)
    deltas: list = field(default_factory=list)
    gammas: list = field(default_factory=list)
    vegas: list = field(default_factory=list)
    thetas: list = field(default_factory=list)
    rhos: list = field(default_factory=list)
    prices_std_err: list = field(default_factory=list)
    deltas_std_err: list = field(default_factory=list)
    gammas_std_err: list = field(default_factory=list)
    vegas_std_err: list = field(default_factory=list)
    thetas_std_err: list = field(default_factory=list)
    rhos_std_err: list = field(default_factory=list)
    time_ms: float = 0.0


def _format(raw: np.ndarray, mode: _p.GreekMode, time_ms: float) -> DispatchResult:
    """format_dispatch_result (PricingDispatch.hpp:42-86) from the raw [2Q][strike] rows."""
    row = lambda q, se=0: [float(x) for x in raw[2 * q + se]]  # noqa: E731
    out = DispatchResult(prices=row(0), prices_std_err=row(0, 1), time_ms=time_ms)
    if mode >= _p.GreekMode.ESSENTIAL:
        out.deltas, out.gammas = row(1), row(2)
        out.deltas_std_err, out.gammas_std_err = row(1, 1), row(2, 1)
    if mode == _p.GreekMode.FULL:
        out.vegas, out.vegas_std_err = [row(3), row(4)], [row(3, 1), row(4, 1)]
        out.thetas, out.thetas_std_err = row(5), row(5, 1)
        out.rhos, out.rhos_std_err = row(6), row(6, 1)
    return out


def price_mc(model, instrument, cfg: _p.MonteCarloConfig, S0: float, r: float, q: float,
             mode: _p.GreekMode = _p.GreekMode.NONE, scheme=_p.SchemeNCI,
             engine: _p.Engine | None = None) -> DispatchResult:
    eng = engine or _p.default_engine()
    job = _p.make_job(model, _p.stepper_for(model, instrument, scheme), instrument, _p.GreekMode(mode),
                      cfg, S0, r, q)
    t0 = time.perf_counter()
    raw, _ = eng.price(job)
    return _format(raw, _p.GreekMode(mode), (time.perf_counter() - t0) * 1e3)


@dataclass
class Request:
    """One entry of a batch: the arguments of one price_mc call."""
    model: object
    instrument: object
    cfg: _p.MonteCarloConfig
    S0: float
    r: float
    q: float
    mode: _p.GreekMode = _p.GreekMode.NONE
    scheme: object = _p.SchemeNCI
    stepper: object = None  # overrides `scheme` (per-factor schemes)


def price_mc_batch(requests: list[Request], engine: _p.Engine | None = None) -> list[DispatchResult]:
    eng = engine or _p.default_engine()
    jobs = [_p.make_job(rq.model, rq.stepper or _p.stepper_for(rq.model, rq.instrument, rq.scheme),
                        rq.instrument, _p.GreekMode(rq.mode), rq.cfg, rq.S0, rq.r, rq.q) for rq in requests]
    t0 = time.perf_counter()
    raws, _ = eng.price_batch(jobs)
    ms = (time.perf_counter() - t0) * 1e3
    return [_format(raw, _p.GreekMode(rq.mode), ms) for raw, rq in zip(raws, requests)]
