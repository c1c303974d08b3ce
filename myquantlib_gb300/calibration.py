"""Calibration of the ASVJ models to option prices.

The reference lists a calibration module as future work (README.md:333).  This is a
Levenberg-Marquardt fit of a model's parameters to quoted prices:

- **Parameters.** Each model type (the names of dispatcher/ModelRegistry.hpp:35-72) has a
  parameter vector (Heston kappa, theta, sigma, rho, v0, then the second factor's, then the
  jump parameters).  Bounds are enforced by a logistic map of an unconstrained vector.
- **Pricing.** The quotes are grouped into one strip per maturity, so every evaluation of the
  residuals is one batch of strips.  The pricer is the engine's FP64 Gil-Pelaez kernel
  (`myql_fourier_price`, European instruments) or the Monte Carlo engine on common random
  numbers (fixed seed and streams, so the residuals are smooth in the parameters and the
  finite-difference Jacobian is usable).
- **Solver.** Residuals r_i = (model_i - quote_i) / weight_i; Jacobian by forward differences
  in the unconstrained coordinates; the damped Gauss-Newton step with Marquardt's diagonal
  scaling, the damping raised on a rejected step and lowered on an accepted one.
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

from . import pricers as _p
from . import registry as _reg

# parameter names per model type and their default bounds
_HESTON = [("kappa", 0.05, 10.0), ("theta", 1e-4, 1.0), ("sigma", 0.01, 2.5), ("rho", -0.99, 0.99), ("v0", 1e-4, 1.0)]
_MERTON = [("lambda", 0.0, 5.0), ("mu", -1.0, 1.0), ("delta", 1e-3, 1.0)]
_KOU = [("lambda", 0.0, 5.0), ("p_up", 0.01, 0.99), ("eta1", 1.05, 50.0), ("eta2", 0.05, 50.0)]
PARAMETERS = {
    "Heston": _HESTON,
    "Bates": _HESTON + _MERTON,
    "BatesKou": _HESTON + _KOU,
    "DoubleHeston": _HESTON + [(n + "2", lo, hi) for n, lo, hi in _HESTON],
    "DoubleBates": _HESTON + [(n + "2", lo, hi) for n, lo, hi in _HESTON] + _MERTON,
}


def model_from_vector(model_type: str, x) -> object:
    """The model of `model_type` with parameter vector x (the order of PARAMETERS)."""
    x = [float(v) for v in x]
    p = _reg.RuntimeModelParams(heston1=_p.HestonParams(*x[0:5]))
    k = 5
    if model_type.startswith("Double"):
        p.heston2 = _p.HestonParams(*x[5:10])
        k = 10
    if model_type in ("Bates", "DoubleBates"):
        p.merton = _p.MertonParams(*x[k:k + 3])
    elif model_type == "BatesKou":
        p.kou = _p.KouParams(*x[k:k + 4])
    return _reg.build_model(model_type, p)


@dataclass
class Quote:
    strike: float
    maturity: float
    price: float
    option_type: str = "Call"
    weight: float = 1.0


@dataclass
class CalibrationResult:
    params: np.ndarray
    names: list
    rmse: float
    iterations: int
    evaluations: int
    converged: bool
    residuals: np.ndarray = field(default_factory=lambda: np.zeros(0))


class _Pricer:
    """Model prices of the quotes, one strip per (maturity, option type)."""

    def __init__(self, quotes: list[Quote], S0: float, r: float, q: float, method: str,
                 engine: _p.Engine, mc_paths: int, mc_steps_per_year: int, seed: int, mc_scheme):
        self.quotes, self.S0, self.r, self.q = quotes, S0, r, q
        self.method, self.engine, self.mc_scheme = method, engine, mc_scheme
        self.mc_paths, self.mc_spy, self.seed = mc_paths, mc_steps_per_year, seed
        self.groups: dict = {}
        for i, qt in enumerate(quotes):
            self.groups.setdefault((qt.maturity, qt.option_type), []).append(i)

    def __call__(self, model_type: str, x) -> np.ndarray:
        model = model_from_vector(model_type, x)
        out = np.empty(len(self.quotes))
        for (T, ot), idx in self.groups.items():
            strikes = [self.quotes[i].strike for i in idx]
            instr = _reg.build_european("Vanilla", ot, _reg.RuntimeInstrumentParams(strikes=strikes, maturity=T))
            if self.method == "fourier":
                job = _p.make_job(model, _p.stepper_for(model, instr, _p.SchemeNCI), instr, _p.GreekMode.NONE,
                                  _p.MonteCarloConfig(num_paths=1, time_steps=1), self.S0, self.r, self.q)
                raw = self.engine.fourier(job, _p.GreekMode.NONE)
            else:
                cfg = _p.MonteCarloConfig(num_paths=self.mc_paths, seed=self.seed,
                                          time_steps=max(1, int(round(self.mc_spy * T))))
                job = _p.make_job(model, _p.stepper_for(model, instr, self.mc_scheme), instr, _p.GreekMode.NONE,
                                  cfg, self.S0, self.r, self.q)
                raw, _ = self.engine.price(job)
            out[idx] = raw[0]
        return out


def levenberg_marquardt(resid, z0, max_iter: int = 50, fd_step: float = 1e-5, tol: float = 1e-10,
                        lam0: float = 1e-3):
    """Minimises |resid(z)|^2 over unconstrained z -> (z, r, iterations, evaluations, converged)."""
    z = np.asarray(z0, dtype=np.float64).copy()
    r = resid(z)
    evals = 1
    lam = lam0
    cost = float(r @ r)
    converged = False
    it = 0
    for it in range(1, max_iter + 1):
        J = np.empty((r.size, z.size))
        for j in range(z.size):
            h = fd_step * max(1.0, abs(z[j]))
            zh = z.copy()
            zh[j] += h
            J[:, j] = (resid(zh) - r) / h
            evals += 1
        A = J.T @ J
        g = J.T @ r
        diag = np.maximum(np.diag(A), 1e-12)
        accepted = False
        for _ in range(30):
            try:
                dz = -np.linalg.solve(A + lam * np.diag(diag), g)
            except np.linalg.LinAlgError:
                lam *= 10.0
                continue
            r_new = resid(z + dz)
            evals += 1
            cost_new = float(r_new @ r_new)
            if np.isfinite(cost_new) and cost_new < cost:
                rel = (cost - cost_new) / max(cost, 1e-300)
                z, r, cost = z + dz, r_new, cost_new
                lam = max(lam / 3.0, 1e-12)
                accepted = True
                if rel < tol or cost < 1e-28:
                    converged = True
                break
            lam *= 4.0
        if not accepted:
            converged = True  # no descent left at this damping: a (local) minimum
        if converged:
            break
    return z, r, it, evals, converged


def calibrate(model_type: str, quotes: list[Quote], S0: float, r: float, q: float, x0,
              bounds=None, method: str = "fourier", engine: _p.Engine | None = None,
              mc_paths: int = 1 << 18, mc_steps_per_year: int = 100, seed: int = 42,
              max_iter: int = 50, mc_scheme=_p.SchemeNV) -> CalibrationResult:
    """Fits `model_type`'s parameters (PARAMETERS[model_type], starting at x0) to the quotes'
    prices.  bounds: [(lo, hi)] per parameter (the defaults of PARAMETERS when None).
    method "mc" prices with mc_paths paths on a fixed seed; its scheme should draw a fixed
    number of normals per step (SchemeNV, the default) so that the prices stay smooth in
    the parameters."""
    if model_type not in PARAMETERS:
        raise ValueError("Unknown model type: " + model_type)
    spec = PARAMETERS[model_type]
    names = [n for n, _, _ in spec]
    lo = np.array([b[0] for b in (bounds or [(lo_, hi_) for _, lo_, hi_ in spec])], dtype=np.float64)
    hi = np.array([b[1] for b in (bounds or [(lo_, hi_) for _, lo_, hi_ in spec])], dtype=np.float64)
    x0 = np.clip(np.asarray(x0, dtype=np.float64), lo + 1e-9 * (hi - lo), hi - 1e-9 * (hi - lo))
    if method not in ("fourier", "mc"):
        raise ValueError("method is 'fourier' or 'mc'")
    pricer = _Pricer(quotes, S0, r, q, method, engine or _p.default_engine(), mc_paths, mc_steps_per_year, seed,
                     mc_scheme)
    target = np.array([qt.price for qt in quotes])
    w = np.array([qt.weight for qt in quotes])

    def to_x(z):
        return lo + (hi - lo) / (1.0 + np.exp(-z))

    def to_z(x):
        u = (x - lo) / (hi - lo)
        return np.log(u / (1.0 - u))

    def resid(z):
        try:
            return (pricer(model_type, to_x(z)) - target) / w
        except _p._abi.MyqlError:  # e.g. the NV condition of an MC pricer: reject the point
            return np.full(target.size, 1e6)

    z, res, it, evals, conv = levenberg_marquardt(resid, to_z(x0), max_iter=max_iter)
    return CalibrationResult(params=to_x(z), names=names, rmse=float(np.sqrt(np.mean((res * w) ** 2))),
                             iterations=it, evaluations=evals, converged=conv, residuals=res * w)
