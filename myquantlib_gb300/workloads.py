"""Seeded synthetic request sets (no market data ships with the engine).

`uneven_requests` is the batched workload of many uneven pricing requests:
model uniform over {Heston, Bates-Kou, Double Heston}; per factor
v0, theta ~ U[0.01, 0.1], kappa ~ U[0.5, 4], sigma ~ U[0.1, 1],
rho ~ U[-0.9, 0]; Kou lambda ~ U[0, 1], p = 0.4, eta1 = 10, eta2 = 5;
paths = round(2^U[14, 20]), steps = round(2^U[4, 9]); instrument an
arithmetic-Asian call or an up-and-out call with B = 1.3 S0 (50/50),
K ~ U[80, 120], T = 1, S0 = 100, r = 0.02, q = 0, seed 42 for every request
(MonteCarloConfig's default, MonteCarloPricer.hpp:16-26).

Variance scheme: SchemeExact for every factor.  The dispatcher's default
(SchemeNCI, StepperTraits.hpp:68) builds a chi-squared quantile table per
parameter set (VolSchemes.hpp:240-300, up to 1024 x 10000 FP64 quantiles), so
with thousands of distinct parameter sets the table builds, not the paths,
would be the workload; SchemeExact samples the same CIR transition law with
no table and is the reference's price_mc<Mode, SchemeExact>.
"""
from __future__ import annotations

import numpy as np

from . import dispatch as _d
from . import pricers as _p

UNEVEN_SEED = 20261203


def _heston(rng) -> _p.HestonParams:
    v0, theta = rng.uniform(0.01, 0.1, 2)
    kappa = rng.uniform(0.5, 4.0)
    sigma = rng.uniform(0.1, 1.0)
    rho = rng.uniform(-0.9, 0.0)
    return _p.HestonParams(v0=v0, kappa=kappa, theta=theta, sigma=sigma, rho=rho)


def uneven_requests(n_jobs: int = 4096, seed: int = UNEVEN_SEED, max_log2_paths: float = 20.0,
                    max_log2_steps: float = 9.0, mode: _p.GreekMode = _p.GreekMode.NONE,
                    scheme=_p.SchemeExact) -> list[_d.Request]:
    rng = np.random.default_rng(seed)
    out = []
    for j in range(n_jobs):
        kind = int(rng.integers(0, 3))
        if kind == 0:
            model = _p.HestonModel(_heston(rng))
        elif kind == 1:
            model = _p.BatesKouModel(_heston(rng), _p.KouParams(rng.uniform(0.0, 1.0), 0.4, 10.0, 5.0))
        else:
            model = _p.DoubleHestonModel(_heston(rng), _heston(rng))
        paths = int(round(2.0 ** rng.uniform(14.0, max_log2_paths)))
        steps = int(round(2.0 ** rng.uniform(4.0, max_log2_steps)))
        K = float(rng.uniform(80.0, 120.0))
        if rng.uniform() < 0.5:
            instr = _p.AsianOption(_p.TrackerArithAsian, _p.PayoffVanilla(_p.OptionType.Call), True, K, 1.0)
        else:
            instr = _p.UpAndOutCall(K, 130.0, 1.0)
        cfg = _p.MonteCarloConfig(num_paths=paths, time_steps=steps)  # seed 42, the reference default
        out.append(_d.Request(model, instr, cfg, 100.0, 0.02, 0.0, mode=mode, scheme=scheme))
    return out


def path_steps(requests) -> int:
    return sum(int(r.cfg.num_paths) * int(r.cfg.time_steps) for r in requests)
