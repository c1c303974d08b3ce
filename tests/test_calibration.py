"""CPU tests of the calibration module's host logic: the Levenberg-Marquardt solver, the
parameter vectors of every model type and the bounds map."""
import numpy as np
import pytest

import myquantlib_gb300 as m
from myquantlib_gb300 import calibration as cal


def test_levenberg_marquardt_recovers_a_nonlinear_fit():
    t = np.linspace(0.0, 4.0, 40)
    a, b, c = 2.0, 1.3, 0.4
    y = a * np.exp(-b * t) + c

    def resid(z):
        return z[0] * np.exp(-z[1] * t) + z[2] - y

    z, r, it, evals, conv = cal.levenberg_marquardt(resid, np.array([1.0, 0.5, 0.0]))
    assert conv and np.allclose(z, [a, b, c], atol=1e-6) and float(r @ r) < 1e-16
    assert evals > it


def test_model_from_vector_every_type():
    h = [2.0, 0.05, 0.9, -0.6, 0.05]
    h2 = [0.5, 0.03, 0.2, -0.3, 0.03]
    assert cal.model_from_vector("Heston", h) == m.HestonModel(m.HestonParams(*h))
    assert cal.model_from_vector("Bates", h + [0.5, -0.1, 0.15]) == m.BatesModel(m.HestonParams(*h), m.MertonParams(0.5, -0.1, 0.15))
    assert cal.model_from_vector("BatesKou", h + [0.8, 0.4, 10.0, 5.0]) == m.BatesKouModel(m.HestonParams(*h), m.KouParams(0.8, 0.4, 10.0, 5.0))
    assert cal.model_from_vector("DoubleHeston", h + h2) == m.DoubleHestonModel(m.HestonParams(*h), m.HestonParams(*h2))
    assert cal.model_from_vector("DoubleBates", h + h2 + [0.3, -0.05, 0.1]) == \
        m.DoubleBatesModel(m.HestonParams(*h), m.HestonParams(*h2), m.MertonParams(0.3, -0.05, 0.1))
    for name, spec in cal.PARAMETERS.items():
        x = [0.5 * (lo + hi) for _, lo, hi in spec]
        cal.model_from_vector(name, x)  # every vector length matches its model


def test_unknown_model_and_method():
    with pytest.raises(ValueError, match="Unknown model type"):
        cal.calibrate("SABR", [], 100.0, 0.0, 0.0, [])
    with pytest.raises(ValueError, match="method"):
        cal.calibrate("Heston", [cal.Quote(100.0, 1.0, 8.0)], 100.0, 0.0, 0.0, [1.5, 0.04, 0.3, -0.7, 0.04],
                      method="pde")
