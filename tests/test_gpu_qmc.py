"""GPU tests of randomized quasi-Monte Carlo (myql_qmc_price): unbiased against the plain
engine at the same time grid, against the reference's Fourier value, and with a variance
gain at equal path counts; unsupported configurations are refused with their status."""
import numpy as np
import pytest

import myquantlib_gb300 as m
from myquantlib_gb300 import _abi

pytestmark = pytest.mark.gpu
H1 = m.HestonParams(1.5, 0.04, 0.3, -0.7, 0.04)
H2 = m.HestonParams(0.5, 0.03, 0.2, -0.3, 0.03)


def job(model, stepper, instr, paths, steps, seed=7):
    return m.make_job(model, stepper, instr, m.GreekMode.NONE,
                      m.MonteCarloConfig(num_paths=paths, time_steps=steps, seed=seed), 100.0, 0.02, 0.0)


CASES = {
    "heston_call": (m.HestonModel(H1), m.HestonStepper(m.SchemeNV), lambda: m.EuropeanOption([90.0, 100.0, 110.0], 1.0), 64),
    "bs_arith_asian": (m.BlackScholesModel(0.2), m.BlackScholesStepper(m.TrackerArithAsian),
                       lambda: m.AsianOption(m.TrackerArithAsian, m.PayoffVanilla(), True, 100.0, 1.0), 64),
    "dheston_call": (m.DoubleHestonModel(H1, H2), m.DoubleHestonStepper(m.SchemeNV, m.SchemeNV),
                     lambda: m.EuropeanOption(100.0, 1.0), 32),
    "heston_uo_call": (m.HestonModel(H1), m.HestonStepper(m.SchemeNV, m.TrackerBarrier),
                       lambda: m.UpAndOutCall(100.0, 130.0, 1.0), 64),
}
# least variance ratio (plain variance / QMC variance, equal paths) each case must show
GAIN = {"heston_call": 5.0, "bs_arith_asian": 20.0, "dheston_call": 5.0, "heston_uo_call": 1.0}


@pytest.mark.parametrize("name", list(CASES))
def test_qmc_unbiased_with_variance_gain(engine, name):
    model, stepper, instr, steps = CASES[name]
    R, paths = 16, 1 << 18
    q, st = engine.qmc_price(job(model, stepper, instr(), paths, steps), R)
    p, _ = engine.price(job(model, stepper, instr(), 1 << 22, steps, seed=11))
    se_q, se_p = q[1], p[1]
    assert np.all(np.abs(q[0] - p[0]) < 4.0 * np.hypot(se_q, se_p)), (q[0], p[0], se_q, se_p)
    # the plain estimator's variance at the QMC path count, against the QMC variance
    var_plain = se_p ** 2 * (1 << 22) / paths
    ratio = var_plain / np.maximum(se_q ** 2, 1e-300)
    assert np.all(ratio > GAIN[name]), ratio
    assert st.kernel_launches == 2 and st.paths == paths


def test_qmc_heston_call_against_fourier(engine):
    # 256 steps make the NV discretisation bias small next to the QMC standard error
    model, stepper, _, _ = CASES["heston_call"]
    q, _ = engine.qmc_price(job(model, stepper, m.EuropeanOption(100.0, 1.0), 1 << 20, 256), 32)
    assert abs(q[0, 0] - 8.628108103110) < 4 * q[1, 0] + 2e-3, (q[0, 0], q[1, 0])


def test_qmc_refuses_unsupported_configurations(engine):
    bates = m.BatesModel(H1, m.MertonParams(0.5, -0.1, 0.15))
    with pytest.raises(_abi.MyqlError) as e:
        engine.qmc_price(job(bates, m.BatesStepper(m.SchemeNV), m.EuropeanOption(100.0, 1.0), 1 << 16, 16), 8)
    assert e.value.status == _abi.ERR_UNSUPPORTED
    with pytest.raises(_abi.MyqlError) as e:
        engine.qmc_price(job(m.HestonModel(H1), m.HestonStepper(m.SchemeNCI), m.EuropeanOption(100.0, 1.0),
                             1 << 16, 16), 8)
    assert e.value.status == _abi.ERR_UNSUPPORTED
    with pytest.raises(_abi.MyqlError) as e:
        engine.qmc_price(job(m.HestonModel(H1), m.HestonStepper(m.SchemeNV), m.EuropeanOption(100.0, 1.0),
                             3 * 2048, 16), 2)
    assert e.value.status == _abi.ERR_INVALID_ARG
