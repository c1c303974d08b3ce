"""GPU test of myql_ctx_set_precise_theta: theta and charm difference the scenarios at
maturity T +- t_bump, whose FP32 per-step constants carry their small difference with a
systematic relative error; the precise one-factor NCI lockstep kernel adds each constant's
FP32 rounding error back for those two scenarios.  On the Bates strip's T = 4 request at
800 steps a year the default mode's theta and charm sit about 2.8 and 1.8 standard errors
below the FP64 Fourier values over 24 seeds; the precise mode moves them most of the way
back, and leaves every quantity that does not use the T-bumped scenarios bit for bit
unchanged."""
import numpy as np
import pytest

import myquantlib_gb300 as m
from myquantlib_gb300 import _abi

pytestmark = pytest.mark.gpu
MODEL = m.BatesModel(m.HestonParams(2.0, 0.05, 0.9, -0.6, 0.05), m.MertonParams(0.5, -0.1, 0.15))
STRIKES = [float(k) for k in 60.0 + 80.0 * np.arange(16) / 15.0]
Q = {n: i for i, n in enumerate(_abi.Q_NAMES)}


def test_precise_theta_moves_theta_and_charm_toward_fourier(engine):
    T, steps = 4.0, 3200
    dz = {"theta": [], "charm": []}
    engine.set_nci_slopes(1)
    try:
        four = None
        for seed in range(42, 50):
            cfg = m.MonteCarloConfig(num_paths=1 << 22, time_steps=steps, seed=seed)
            job = m.make_job(MODEL, m.BatesStepper(m.SchemeNCI), m.EuropeanOption(STRIKES, T),
                             m.GreekMode.FULL, cfg, 100.0, 0.02, 0.0)
            if four is None:
                four = engine.fourier(job, m.GreekMode.FULL)
            out = {}
            for precise in (False, True):
                engine.set_precise_theta(precise)
                out[precise], _ = engine.price(job)
            # the base and v0-bumped scenarios are the same kernels' arithmetic in both modes
            for q in ("price", "delta", "gamma", "vega0", "rho", "vanna0"):
                np.testing.assert_array_equal(out[True][2 * Q[q]], out[False][2 * Q[q]], err_msg=q)
            for q in dz:
                z = [(out[p][2 * Q[q]] - four[2 * Q[q]]) / out[p][2 * Q[q] + 1] for p in (False, True)]
                dz[q].append(float(np.mean(z[1]) - np.mean(z[0])))
    finally:
        engine.set_precise_theta(False)
        engine.set_nci_slopes(0)
    # paired over the same paths: the correction is systematic, the seed spread small
    assert np.mean(dz["theta"]) > 1.0 and min(dz["theta"]) > 0.5, dz["theta"]
    assert np.mean(dz["charm"]) > 0.6 and min(dz["charm"]) > 0.3, dz["charm"]


def test_precise_theta_refuses_other_values(engine):
    assert engine.lib.myql_ctx_set_precise_theta(engine.handle, 2) == _abi.ERR_INVALID_ARG
    assert engine.lib.myql_ctx_set_precise_theta(None, 1) == _abi.ERR_INVALID_ARG
