"""GPU tests of the multilevel Monte Carlo path (MultiLevelMonteCarloPricer /
CoupledASVJStepper of the reference), through the C ABI.

 * per level: one evaluate_level call on the GPU and in the FP64 oracle on the
   same xoshiro streams -- the level mean of P_l - P_(l-1) must agree far
   inside its standard error and the second moment to FP32 accuracy;
 * whole pricer: the GPU's adaptive MLMC against the reference's estimator
   (oracle restatement, OpenMP thread layout) within 4 combined standard
   errors, and against the FP64 Fourier price within 4 SE plus the RMSE target.
"""
import ctypes as C
import json
from pathlib import Path

import numpy as np
import pytest

import myquantlib_gb300 as m
from myquantlib_gb300 import _abi

pytestmark = pytest.mark.gpu
FOURIER = {s["name"]: s for s in json.loads(
    (Path(__file__).resolve().parent / "golden" / "reference_fourier.json").read_text())}


def mlmc_cfg(eps, L_min=2, L_max=6, N0=4000, base=1, seed=42, streams=0):
    c = _abi.MlmcConfigC()
    c.epsilon, c.L_min, c.L_max, c.N0, c.base_steps = eps, L_min, L_max, N0, base
    c.alpha, c.beta, c.adaptive_rates, c.seed, c.fd_bump, c.n_streams = 2.0, 1.0, 1, seed, 1e-4, streams
    return c


H5 = m.HestonModel(m.HestonParams(2.0, 0.04, 0.5, -0.7, 0.04))
H1 = m.HestonModel(m.HestonParams(1.5, 0.04, 0.3, -0.7, 0.04))


def job(model, stepper, instr):
    return m.make_job(model, stepper, instr, m.GreekMode.NONE, m.MonteCarloConfig(), 100.0, 0.02, 0.0)


CASES = {
    "c5_do_put": lambda: job(H5, m.HestonStepper(m.SchemeNV), m.DownAndOutPut(100.0, 80.0, 1.0)),
    "heston_eur": lambda: job(H1, m.HestonStepper(m.SchemeNV), m.EuropeanOption(100.0, 1.0)),
    "bates_nci_eur": lambda: job(m.BatesModel(m.HestonParams(2.0, 0.05, 0.9, -0.6, 0.05),
                                              m.MertonParams(0.5, -0.1, 0.15)),
                                 m.BatesStepper(m.SchemeNCI), m.EuropeanOption(100.0, 1.0)),
    "bs_asian": lambda: job(m.BlackScholesModel(0.2), m.BlackScholesStepper(),
                            m.AsianOption(m.TrackerArithAsian, m.PayoffVanilla(), True, 100.0, 1.0)),
    "dbk_lookback": lambda: job(m.DoubleBatesKouModel(m.HestonParams(2.0, 0.04, 0.3, -0.7, 0.04),
                                                      m.HestonParams(3.0, 0.02, 0.2, -0.3, 0.02),
                                                      m.KouParams(1.0, 0.4, 10.0, 5.0)),
                                m.DoubleBatesKouStepper(m.SchemeNV, m.SchemeExact),
                                m.LookbackOption(m.PayoffVanilla(), False, 100.0, 1.0)),
    "bs_merton_uo": lambda: job(m.MertonModel(0.2, m.MertonParams(1.0, -0.05, 0.1)), m.MertonJDStepper(),
                                m.UpAndOutCall(100.0, 130.0, 1.0)),
}
LEVELS = [("c5_do_put", 0), ("c5_do_put", 1), ("c5_do_put", 4), ("heston_eur", 3), ("bates_nci_eur", 0),
          ("bates_nci_eur", 2), ("bs_asian", 3), ("dbk_lookback", 2), ("bs_merton_uo", 2)]


@pytest.mark.parametrize("name,level", LEVELS, ids=[f"{n}-L{l}" for n, l in LEVELS])
def test_level_replay_against_oracle(engine, oracle_lib, name, level):
    j = CASES[name]()
    cfg = mlmc_cfg(0.01, L_max=8, streams=1024)
    dN = 8192
    got = np.zeros(2)
    _abi.check(engine.lib.myql_mlmc_level(engine.handle, C.byref(j.c), C.byref(cfg), level, dN,
                                          got.ctypes.data_as(C.POINTER(C.c_double))))
    want = oracle_lib.mlmc_level(j, cfg, level, dN, oracle_lib.LAYOUT_STREAMS, 8)
    mean_g, mean_w = got[0] / dN, want[0] / dN
    var_w = max(want[1] / dN - mean_w ** 2, 1e-30)
    se = np.sqrt(var_w / dN)
    assert abs(mean_g - mean_w) <= 0.2 * se + 1e-7 * abs(mean_w), (mean_g, mean_w, se)
    assert abs(got[1] - want[1]) <= 5e-3 * abs(want[1]) + 1e-12, (got[1], want[1])


def run_mlmc(engine, j, cfg):
    res = _abi.MlmcResultC()
    _abi.check(engine.lib.myql_mlmc_price(engine.handle, C.byref(j.c), C.byref(cfg), C.byref(res)))
    return res


@pytest.mark.parametrize("name,eps,L_max", [("c5_do_put", 0.01, 8), ("bs_asian", 0.005, 7),
                                            ("bates_nci_eur", 0.05, 5)])
def test_mlmc_against_reference_estimator(engine, oracle_lib, name, eps, L_max):
    j = CASES[name]()
    cfg = mlmc_cfg(eps, L_max=L_max)
    g = run_mlmc(engine, j, cfg)
    r = oracle_lib.mlmc_price(j, cfg, oracle_lib.LAYOUT_REFERENCE, 8)
    se = np.hypot(g.price_std_err, r.price_std_err)
    assert abs(g.price - r.price) < 4 * se, (g.price, r.price, se)
    assert g.n_levels >= 3 and all(g.paths_per_level[l] >= 20 for l in range(g.n_levels))
    assert g.total_steps > 0


def test_mlmc_european_against_fourier(engine):
    j = CASES["heston_eur"]()
    cfg = mlmc_cfg(0.01, L_max=8)
    g = run_mlmc(engine, j, cfg)
    four = FOURIER["c1_heston_call"]["fourier"][0]
    assert abs(g.price - four) < 4 * g.price_std_err + cfg.epsilon / np.sqrt(2.0), (g.price, four)
    # the level differences decay (weak order estimate positive)
    assert g.alpha_estimated > 0.3


# ---------------------------------------------------------------- multilevel Richardson-Romberg
def ml2r_weights(L, alpha):
    """W_l = sum_{r >= l} w_r, w the Richardson weights (sum_l w_l x_l^k = [k == 0], x_l = 2^(-alpha l))."""
    x = 2.0 ** (-alpha * np.arange(L + 1))
    w = np.linalg.solve(np.vander(x, increasing=True).T, np.eye(L + 1)[0])
    return np.cumsum(w[::-1])[::-1]


def fixed_order_cfg(eps, alpha, L_min=1, L_max=8):
    c = mlmc_cfg(eps, L_min=L_min, L_max=L_max)
    c.alpha, c.adaptive_rates = alpha, 0
    return c


def test_ml2r_european_against_fourier(engine):
    """Heston call (SchemeNV, weak order 1): the ML2R price is the W-weighted sum of the
    level means, agrees with the reference's FP64 Fourier value, and needs no more levels
    than MLMC at the same tolerance."""
    j = CASES["heston_eur"]()
    cfg = fixed_order_cfg(0.01, 1.0)
    g = engine.ml2r_price(j, cfg)
    four = FOURIER["c1_heston_call"]["fourier"][0]
    assert abs(g.price - four) < 4 * g.price_std_err + cfg.epsilon / np.sqrt(2.0), (g.price, four)
    W = ml2r_weights(g.n_levels - 1, 1.0)
    assert abs(W[0] - 1.0) < 1e-12
    assert abs(g.price - sum(W[l] * g.mean_diffs[l] for l in range(g.n_levels))) < 1e-9 * abs(g.price)
    mc = engine.mlmc_price(j, fixed_order_cfg(0.01, 1.0))
    assert g.n_levels <= mc.n_levels, (g.n_levels, mc.n_levels)


def test_ml2r_asian_against_mlmc(engine):
    """Black-Scholes arithmetic Asian (weak order 1): ML2R and MLMC agree within their
    standard errors and tolerances, ML2R with no more levels.  (A discretely monitored
    barrier has no regular expansion of its error in powers of h, so ML2R is not applied
    to barriers.)"""
    j = CASES["bs_asian"]()
    g = engine.ml2r_price(j, fixed_order_cfg(0.005, 1.0))
    mc = engine.mlmc_price(j, fixed_order_cfg(0.005, 1.0))
    assert g.n_levels >= 2 and g.total_steps > 0 and g.n_levels <= mc.n_levels
    tol = 4 * np.hypot(g.price_std_err, mc.price_std_err) + 0.005 * np.sqrt(2.0)
    assert abs(g.price - mc.price) < tol, (g.price, mc.price, tol)


# ---------------------------------------------------------------- MLMC with the neural control variate
def cv_cfg_c(iterations=200, pilot=1 << 16):
    return m.pricers.ControlVariateConfig(hedge_every=1, iterations=iterations, pilot_paths=pilot,
                                          batch_paths=4096, learning_rate=3e-3, seed=7).c()


@pytest.mark.parametrize("name", ["c5_do_put", "heston_eur"])
def test_mlmc_cv_levels_unbiased_and_reduced(engine, name):
    j = CASES[name]()
    cfg = mlmc_cfg(0.01, L_max=8, streams=4096)
    train = CASES[name]()
    train.c.config.time_steps = 32
    engine.cv_train(train, cv_cfg_c())
    dN = 1 << 16
    ratios = []
    for level in (0, 2, 4):
        s = engine.mlmc_cv_level(j, cfg, level, dN)
        my, mz = s[0] / dN, s[2] / dN
        vy, vz = max(s[1] / dN - my * my, 0.0), max(s[3] / dN - mz * mz, 0.0)
        # E[C] = 0: the corrected and plain level means differ by mean(C), whose SE is
        # at most (sd(Y) + sd(Y - C)) / sqrt(dN)
        bound = 4.0 * (np.sqrt(vy) + np.sqrt(vz)) / np.sqrt(dN)
        assert abs(mz - my) < bound + 1e-9, (level, my, mz, bound)
        ratios.append(vy / max(vz, 1e-30))
    if name == "heston_eur":
        assert ratios[0] > 3.0, ratios  # the plain level (one step here) gains most
    else:
        # the knock-out put's level differences are driven by discrete monitoring, which the
        # asset hedge does not span: the control must at least not add variance
        assert min(ratios) > 0.9, ratios


@pytest.mark.parametrize("name,eps", [("c5_do_put", 0.01), ("heston_eur", 0.01)])
def test_mlmc_cv_price_against_plain_mlmc(engine, oracle_lib, name, eps):
    """MLMC with the control variate agrees with plain MLMC and the reference's estimator.
    A level keeps the control only where its variance ratio beats the cost of the MLP rows
    (about 25 coupled path-steps a row): on the one-step and few-step low levels a CV path
    costs 9 to 26 plain ones, so there the level runs the plain estimator and its variance
    is the plain one."""
    j = CASES[name]()
    cfg = mlmc_cfg(eps, L_max=8)
    plain = run_mlmc(engine, j, cfg)
    res, plain_var = engine.mlmc_cv_price(j, cfg, cv_cfg_c())
    se = np.hypot(res.price_std_err, plain.price_std_err)
    assert abs(res.price - plain.price) < 4 * se + cfg.epsilon, (res.price, plain.price, se)
    r = oracle_lib.mlmc_price(j, cfg, oracle_lib.LAYOUT_REFERENCE, 8)
    assert abs(res.price - r.price) < 4 * np.hypot(res.price_std_err, r.price_std_err) + cfg.epsilon
    v_cv = np.array([res.var_diffs[l] for l in range(res.n_levels)])
    for level in range(3):
        assert abs(v_cv[level] - plain_var[level]) <= 1e-9 * plain_var[level] + 1e-18, (level, v_cv, plain_var)
