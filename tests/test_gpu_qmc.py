"""GPU tests of randomized quasi-Monte Carlo (myql_qmc_price): unbiased against the plain
engine at the same time grid (SchemeNV and SchemeNCI factors, Merton jumps), against the
reference's Fourier values, and with a variance gain at equal path counts; unsupported
configurations (SchemeExact, Kou jumps) are refused with their status."""
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


HB = m.HestonParams(2.0, 0.05, 0.9, -0.6, 0.05)        # Feller violated: SchemeNCI only
C4_F1 = m.HestonParams(2.0, 0.03, 0.4, -0.7, 0.03)     # the Double Bates Asian's factors
C4_F2 = m.HestonParams(0.5, 0.02, 0.3, -0.3, 0.02)
C4_JUMP = m.MertonParams(0.3, -0.05, 0.1)

CASES = {
    "heston_call": (m.HestonModel(H1), m.HestonStepper(m.SchemeNV), lambda: m.EuropeanOption([90.0, 100.0, 110.0], 1.0), 64),
    "bs_arith_asian": (m.BlackScholesModel(0.2), m.BlackScholesStepper(m.TrackerArithAsian),
                       lambda: m.AsianOption(m.TrackerArithAsian, m.PayoffVanilla(), True, 100.0, 1.0), 64),
    "dheston_call": (m.DoubleHestonModel(H1, H2), m.DoubleHestonStepper(m.SchemeNV, m.SchemeNV),
                     lambda: m.EuropeanOption(100.0, 1.0), 32),
    "heston_uo_call": (m.HestonModel(H1), m.HestonStepper(m.SchemeNV, m.TrackerBarrier),
                       lambda: m.UpAndOutCall(100.0, 130.0, 1.0), 64),
    # SchemeNCI factors (Poisson and chi-squared uniforms from Sobol coordinates) and Merton jumps
    "heston_nci_call": (m.HestonModel(HB), m.HestonStepper(m.SchemeNCI), lambda: m.EuropeanOption([90.0, 100.0, 110.0], 1.0), 64),
    "bates_nci_asian": (m.BatesModel(HB, m.MertonParams(0.5, -0.1, 0.15)),
                        m.BatesStepper(m.SchemeNCI, m.TrackerArithAsian),
                        lambda: m.AsianOption(m.TrackerArithAsian, m.PayoffVanilla(), True, 100.0, 1.0), 64),
    "dbates_nci_nci_asian": (m.DoubleBatesModel(C4_F1, C4_F2, C4_JUMP),
                             m.DoubleBatesStepper(m.SchemeNCI, m.SchemeNCI, m.TrackerArithAsian),
                             lambda: m.AsianOption(m.TrackerArithAsian, m.PayoffVanilla(), True, 100.0, 2.0), 64),
    "dbates_nv_nci_call": (m.DoubleBatesModel(C4_F1, C4_F2, C4_JUMP), m.DoubleBatesStepper(m.SchemeNV, m.SchemeNCI),
                           lambda: m.EuropeanOption(100.0, 1.0), 32),
}
# least variance ratio (plain variance / QMC variance, equal paths) each case must show
GAIN = {"heston_call": 5.0, "bs_arith_asian": 20.0, "dheston_call": 5.0, "heston_uo_call": 1.0,
        "heston_nci_call": 1.0, "bates_nci_asian": 1.0, "dbates_nci_nci_asian": 1.0, "dbates_nv_nci_call": 1.0}


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
    assert st.paths == paths
    # a second call reuses the tables (Sobol directions, bridge, NCI): the shift, simulation and
    # payoff launches only, and the same replicate estimates bit for bit
    q2, st2 = engine.qmc_price(job(model, stepper, instr(), paths, steps), R)
    assert st2.kernel_launches == 3
    np.testing.assert_array_equal(q2, q)


def test_qmc_heston_call_against_fourier(engine):
    # 256 steps make the NV discretisation bias small next to the QMC standard error
    model, stepper, _, _ = CASES["heston_call"]
    q, _ = engine.qmc_price(job(model, stepper, m.EuropeanOption(100.0, 1.0), 1 << 20, 256), 32)
    assert abs(q[0, 0] - 8.628108103110) < 4 * q[1, 0] + 2e-3, (q[0, 0], q[1, 0])


def test_qmc_refuses_unsupported_configurations(engine):
    # Kou jumps (one exponential per jump) and SchemeExact (a rejection loop) have no fixed draw count
    kou = m.BatesKouModel(H1, m.KouParams(0.5, 0.4, 10.0, 5.0))
    with pytest.raises(_abi.MyqlError) as e:
        engine.qmc_price(job(kou, m.BatesKouStepper(m.SchemeNV), m.EuropeanOption(100.0, 1.0), 1 << 16, 16), 8)
    assert e.value.status == _abi.ERR_UNSUPPORTED
    with pytest.raises(_abi.MyqlError) as e:
        engine.qmc_price(job(m.HestonModel(H1), m.HestonStepper(m.SchemeExact), m.EuropeanOption(100.0, 1.0),
                             1 << 16, 16), 8)
    assert e.value.status == _abi.ERR_UNSUPPORTED
    with pytest.raises(_abi.MyqlError) as e:
        engine.qmc_price(job(m.HestonModel(H1), m.HestonStepper(m.SchemeNV), m.EuropeanOption(100.0, 1.0),
                             3 * 2048, 16), 2)
    assert e.value.status == _abi.ERR_INVALID_ARG


def test_qmc_bates_nci_call_against_fourier(engine):
    """SchemeNCI with Merton jumps: the Bates call of the headline strip (T = 1, 200 steps) against
    the reference's FP64 Fourier value (9.675798595347402, K 100.6349), on the NCI tables whose
    cells keep the chi-squared mean (the reference's cells bias long paths slightly)."""
    model = m.BatesModel(HB, m.MertonParams(0.5, -0.1, 0.15))
    engine.set_nci_slopes(1)
    try:
        q, _ = engine.qmc_price(job(model, m.BatesStepper(m.SchemeNCI),
                                    m.EuropeanOption(100.63492063492063, 1.0), 1 << 20, 200), 32)
    finally:
        engine.set_nci_slopes(0)
    assert abs(q[0, 0] - 9.675798595347402) < 4 * q[1, 0] + 2e-3, (q[0, 0], q[1, 0])


@pytest.mark.parametrize("steps", [1, 33, 512])
def test_qmc_segment_edges_unbiased(engine, steps):
    """The segmented bridge at its edges: one step (a single one-step segment), 33 steps (a last
    segment of one step) and the 512-step maximum (16 full segments), against the plain engine."""
    model, stepper = m.HestonModel(H1), m.HestonStepper(m.SchemeNV, m.TrackerArithAsian)
    instr = lambda: m.AsianOption(m.TrackerArithAsian, m.PayoffVanilla(), True, 100.0, 1.0)  # noqa: E731
    q, _ = engine.qmc_price(job(model, stepper, instr(), 1 << 18, steps), 16)
    p, _ = engine.price(job(model, stepper, instr(), 1 << 21, steps, seed=11))
    assert abs(q[0, 0] - p[0, 0]) < 4.0 * np.hypot(q[1, 0], p[1, 0]), (steps, q[0, 0], p[0, 0], q[1, 0], p[1, 0])
    assert q[1, 0] < p[1, 0] * np.sqrt((1 << 21) / (1 << 18)), (q[1, 0], p[1, 0])  # no worse than plain MC


def test_qmc_refuses_more_than_512_steps(engine):
    with pytest.raises(_abi.MyqlError) as e:
        engine.qmc_price(job(m.HestonModel(H1), m.HestonStepper(m.SchemeNV), m.EuropeanOption(100.0, 1.0),
                             1 << 15, 513), 16)
    assert e.value.status == _abi.ERR_UNSUPPORTED


def test_qmc_direction_seed_selects_the_point_set(engine):
    """Another direction seed gives another randomly initialised Sobol point set: a different
    but still unbiased estimate; going back to a seed reproduces its estimate bit for bit."""
    model, stepper, instr, steps = CASES["heston_call"]
    j = lambda: job(model, stepper, instr(), 1 << 18, steps)  # noqa: E731
    p, _ = engine.price(job(model, stepper, instr(), 1 << 22, steps, seed=11))
    try:
        engine.set_qmc_direction_seed(1)
        a, _ = engine.qmc_price(j(), 16)
        engine.set_qmc_direction_seed(2)
        b, _ = engine.qmc_price(j(), 16)
        engine.set_qmc_direction_seed(1)
        c, _ = engine.qmc_price(j(), 16)
    finally:
        engine.set_qmc_direction_seed(_abi.QMC_DEFAULT_DIRECTION_SEED)
    np.testing.assert_array_equal(a, c)
    assert not np.array_equal(a[0], b[0])
    for q in (a, b):
        assert np.all(np.abs(q[0] - p[0]) < 4.0 * np.hypot(q[1], p[1])), (q[0], p[0])
