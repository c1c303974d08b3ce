"""GPU tests of the calibration loop: Heston and Bates recovered from their own FP64 Fourier
prices (noise-free quotes), and a Monte Carlo calibration on common random numbers that
lands near the truth."""
import numpy as np
import pytest

import myquantlib_gb300 as m
from myquantlib_gb300 import calibration as cal
from myquantlib_gb300 import registry as reg

pytestmark = pytest.mark.gpu
STRIKES = [80.0, 90.0, 100.0, 110.0, 120.0]
MATURITIES = [0.25, 0.5, 1.0, 2.0]


def fourier_quotes(engine, model_type, x, strikes=STRIKES, maturities=MATURITIES):
    model = cal.model_from_vector(model_type, x)
    quotes = []
    for T in maturities:
        ins = reg.build_european("Vanilla", "Call", reg.RuntimeInstrumentParams(strikes=strikes, maturity=T))
        res = reg.price_fourier(model, ins, 100.0, 0.02, 0.0, m.GreekMode.NONE, engine)
        quotes += [cal.Quote(K, T, p) for K, p in zip(strikes, res.prices)]
    return quotes


def test_heston_recovered_from_fourier_quotes(engine):
    truth = [1.5, 0.04, 0.3, -0.7, 0.04]
    quotes = fourier_quotes(engine, "Heston", truth)
    res = cal.calibrate("Heston", quotes, 100.0, 0.02, 0.0, [2.5, 0.06, 0.5, -0.4, 0.06], engine=engine)
    assert res.rmse < 1e-6, res.rmse
    assert np.allclose(res.params, truth, rtol=2e-3, atol=2e-4), res.params
    assert res.names == ["kappa", "theta", "sigma", "rho", "v0"]


def test_bates_fit_to_fourier_quotes(engine):
    truth = [2.0, 0.05, 0.9, -0.6, 0.05, 0.5, -0.1, 0.15]
    quotes = fourier_quotes(engine, "Bates", truth)
    res = cal.calibrate("Bates", quotes, 100.0, 0.02, 0.0, [1.5, 0.04, 0.6, -0.5, 0.04, 0.3, -0.05, 0.1],
                        engine=engine, max_iter=100)
    assert res.rmse < 1e-4, (res.rmse, res.params)


def test_heston_monte_carlo_calibration(engine):
    truth = [1.5, 0.04, 0.3, -0.7, 0.04]
    quotes = fourier_quotes(engine, "Heston", truth, strikes=[90.0, 100.0, 110.0], maturities=[0.5, 1.0])
    res = cal.calibrate("Heston", quotes, 100.0, 0.02, 0.0, [2.0, 0.05, 0.4, -0.5, 0.05], engine=engine,
                        method="mc", mc_paths=1 << 17, mc_steps_per_year=64, max_iter=30)
    # Monte Carlo error (~1e-2 at 2^17 paths) and NV discretisation keep it off the exact fit
    assert res.rmse < 0.05, (res.rmse, res.params)
    assert abs(res.params[4] - truth[4]) < 0.01 and abs(res.params[3] - truth[3]) < 0.25, res.params
