"""GPU tests of the engine's building blocks and edge cases (through the C ABI):
bit-exact jump-ahead streams, the device samplers against the oracle, the FP64
chi-squared tables against scipy, size edge cases, determinism, chunking and
host-side fault injection (loop caps), which faults no GPU."""
import dataclasses
import json
from pathlib import Path

import numpy as np
import pytest
from scipy import stats

import jobspec
import myquantlib_gb300 as m
import pyrng
from myquantlib_gb300 import _abi

pytestmark = pytest.mark.gpu
GOLDEN = Path(__file__).resolve().parent / "golden"
KAT = json.loads((GOLDEN / "rng_kat.json").read_text())
MC_SPECS = {s["name"]: s for s in json.loads((GOLDEN / "reference_mc.json").read_text())}


def test_stream_states_bit_exact(engine):
    got = engine.stream_states(42, 0, 4)
    assert [[int(x) for x in row] for row in got] == KAT["seed42_stream_states_0_3"]
    for seed, first, n in [(7, 0, 300), (2**63 + 11, 129, 3), (123456789, 1000, 2)]:
        got = engine.stream_states(seed, first, n)
        for k in ([0, 1, n - 1] if n > 3 else range(n)):
            assert [int(x) for x in got[k]] == pyrng.stream_state(seed, first + k), (seed, first, k)


def test_stream_draws_bit_exact(engine):
    got = engine.draws(42, 0, 2, 3)
    assert [int(x) for x in got[0]] == KAT["seed42_first3"]
    s = pyrng.stream_state(42, 1)
    want = []
    for _ in range(3):
        o, s = pyrng.next_out(s)
        want.append(o)
    assert [int(x) for x in got[1]] == want


def test_device_inverse_normal(engine, oracle_lib):
    lib = oracle_lib.restatement()
    rng = np.random.default_rng(3)
    x = rng.integers(0, 2**64, 20000, dtype=np.uint64)
    x = np.concatenate([x, np.array([1, 2**10, 2**40, 2**63, 2**64 - 2**11, 2**63 + 1], dtype=np.uint64)])
    got = engine.sampler(0, x).astype(np.float64)
    want = np.array([lib.myql_oracle_normcdfinv(lib.myql_oracle_uniform_of(int(v))) for v in x])
    assert np.max(np.abs(got - want) / np.maximum(1.0, np.abs(want))) < 2e-6


def test_device_inverse_poisson(engine, oracle_lib):
    lib = oracle_lib.restatement()
    rng = np.random.default_rng(5)
    n = 40000
    lam = np.concatenate([rng.uniform(0, 4, n // 4), rng.uniform(4, 30, n // 4),
                          rng.uniform(30, 800, n // 4), rng.lognormal(0, 2, n // 4)])
    x = rng.integers(0, 2**64, n, dtype=np.uint64)
    got = engine.sampler(1, x, lam).astype(np.float64)
    want = np.array([lib.myql_oracle_poissinvcdf(l, lib.myql_oracle_uniform_of(int(v))) for l, v in zip(lam, x)])
    mism = got != want
    assert np.mean(mism) < 2e-4, np.mean(mism)
    assert np.all(np.abs(got - want) <= 1)



def test_device_inverse_poisson_at_cdf_steps(engine):
    """U placed 1e-5 on either side of every step F(n) of the CDF, for means on both
    sides of the summation / asymptotic-estimate boundary: the inversion must be the
    exact quantile there, where a wrong floor of the estimate would show."""
    lams, xs, want = [], [], []
    for lam in np.linspace(0.05, 30.0, 600):
        n = np.arange(0, int(lam + 8.0 * np.sqrt(lam) + 10))
        F = stats.poisson.cdf(n, lam)
        for d in (-1e-5, 1e-5):
            U = F + d
            # keep points at least 2e-6 from every step: nearer ones are within FP32
            # rounding of the summed CDF
            gap = np.min(np.abs(U[:, None] - F[None, :]), axis=1)
            U = U[(U > 1e-7) & (U < 1.0 - 1e-7) & (gap > 2e-6)]
            lams.append(np.full(U.size, lam))
            xs.append(np.floor(U * 2.0**64).astype(np.uint64))
            want.append(stats.poisson.ppf(U, lam))
    lam, x, want = np.concatenate(lams), np.concatenate(xs), np.concatenate(want)
    got = engine.sampler(1, x, lam).astype(np.float64)
    bad = got != want
    assert not bad.any(), (int(bad.sum()), lam[bad][:5], x[bad][:5] / 2.0**64, got[bad][:5], want[bad][:5])


def test_device_chi2_quantile(engine):
    rng = np.random.default_rng(9)
    dof = np.concatenate([[0.494] * 6, rng.uniform(0.05, 2500, 200)])
    p = np.concatenate([[1e-4, 0.001, 0.5, 0.9, 0.999, 1 - 1e-12], rng.uniform(0, 0.999, 200)])
    got = engine.chi2_quantile(dof, p)
    want = stats.chi2.ppf(p, dof)
    assert np.max(np.abs(got - want) / want) < 1e-9


@pytest.mark.parametrize("d,rows", [(0.494, 110), (3.7, 40), (0.05, 1024)])
def test_device_nci_nodes(engine, d, rows):
    """Every FP64 node of the SchemeNCI table (main grid p = i 0.999/9999 and the upper tail
    q = e^-w) against scipy's chi-squared quantiles, to 1e-11 relative.  The nodes of a row
    are built from the previous node's quantile by a Taylor step plus Newton, so a row's
    values depend on each other: the test covers whole rows, up to the 1024-row maximum."""
    main, tail = engine.nci_nodes(d, rows)
    nu = d + 2.0 * np.arange(rows)[:, None]
    p = np.arange(10000) * (0.999 / 9999)
    want = stats.chi2.ppf(p[None, :], nu)
    assert np.all(main[:, 0] == 0.0)
    rel = np.abs(main[:, 1:] - want[:, 1:]) / want[:, 1:]
    assert rel.max() < 1e-11, (rel.max(), np.unravel_index(rel.argmax(), rel.shape))
    assert np.all(np.diff(main, axis=1) > 0)
    w0 = -np.log1p(-0.999)
    w = w0 + np.arange(512) * ((44.5 - w0) / 511)
    want_t = stats.chi2.isf(np.exp(-w)[None, :], nu)
    rel_t = np.abs(tail - want_t) / want_t
    assert rel_t.max() < 1e-11, (rel_t.max(), np.unravel_index(rel_t.argmax(), rel_t.shape))


def test_jump_count_tail_draws_end_without_the_cap(engine):
    """A Merton jump count drawn by sequential inversion from a uniform within about 1e-7 of 1
    runs to the loop cap in FP32 (the remainder stays above every later term) unless the
    inversion stops in the deep tail.  The Bates strip's T = 1.5 request on seed 43 (2^22 paths,
    5 simulated scenarios) holds such draws: it must price without a cap hit."""
    model = m.BatesModel(m.HestonParams(2.0, 0.05, 0.9, -0.6, 0.05), m.MertonParams(0.5, -0.1, 0.15))
    cfg = m.MonteCarloConfig(num_paths=1 << 22, time_steps=300, seed=43)
    job = m.make_job(model, m.BatesStepper(m.SchemeNCI), m.EuropeanOption([80.0, 100.0, 120.0], 1.5),
                     m.GreekMode.FULL, cfg, 100.0, 0.02, 0.0)
    raw, st = engine.price(job)
    assert st.loop_cap_hits == 0
    assert np.all(np.isfinite(raw))


def test_nci_exact_slopes_remove_the_table_mean_bias(engine):
    """The reference's NCI cells bias the chi-squared draw's mean low (mostly in the first cell,
    a cubic from the node y(0) = 0), and the log-spot step turns that into a price bias of sign
    -rho that grows with the step count.  Heston (rho = 0.6, sigma^2 > 4 kappa theta), T = 2 at
    800 steps a year, 2^22 paths: with the reference's cells the strikes' mean z against the
    FP64 Fourier price is far below zero (about -7.5 on seeds 42-44); with mode 1 (exact slopes,
    mean-preserving first cell) it is within the noise of a few correlated SEs."""
    model = m.HestonModel(m.HestonParams(2.0, 0.05, 0.9, 0.6, 0.05))
    cfg = m.MonteCarloConfig(num_paths=1 << 22, time_steps=1600, seed=42)
    job = m.make_job(model, m.HestonStepper(m.SchemeNCI), m.EuropeanOption([80.0, 90.0, 100.0, 110.0, 120.0], 2.0),
                     m.GreekMode.NONE, cfg, 100.0, 0.02, 0.0)
    four = engine.fourier(job, m.GreekMode.NONE)[0]
    zs = []
    for mode in (0, 1):
        engine.set_nci_slopes(mode)
        try:
            raw, _ = engine.price(job)
        finally:
            engine.set_nci_slopes(0)
        zs.append(float(np.mean((raw[0] - four) / raw[1])))
    assert zs[0] < -4.0, zs
    assert abs(zs[1]) < 3.0, zs


def test_nci_rows_beyond_the_table(oracle_lib):
    """Poisson counts at or beyond the table's rows: with the rows capped at 24 for a Heston
    SchemeNCI call whose counts sit near 44 at v = theta (C0 v, dt = 1/50), about 63 % of the
    variance draws (under the stationary law of v) leave the table and take the Wilson-Hilferty
    quantile of d + 2N degrees of freedom; the estimate
    stays within 4 combined SE of the reference's estimator, whose own table covers these rows
    (n_max 179 here; exact quantile past it, VolSchemes.hpp:368-369), and every such draw is
    counted."""
    eng = m.Engine(0)
    try:
        eng.set_nci_rows(24)
        spec = jobspec.with_config(MC_SPECS["heston_nci_call"], paths=1 << 20, steps=50)
        raw, st = eng.price(jobspec.make_job(spec))
    finally:
        eng.close()
    assert st.table_fallbacks > 0.5 * (1 << 20) * 50, st.table_fallbacks
    ref, _ = oracle_lib.mc_price(jobspec.make_job(jobspec.with_config(spec, paths=1 << 16)),
                                 oracle_lib.LAYOUT_REFERENCE, 8)
    se = np.sqrt(raw[1::2] ** 2 + ref[1::2] ** 2)
    z = np.abs(raw[0::2] - ref[0::2])[:3] / se[:3]   # price, delta, gamma (Essential)
    assert np.max(z) < 4.0, z


def base_spec():
    return jobspec.with_config(MC_SPECS["c1_heston_nv_call"], paths=50000, steps=50, streams=1024)


def test_deterministic_and_chunking_invariant(engine):
    job = jobspec.make_job(base_spec())
    a, _ = engine.price(job)
    b, _ = engine.price(job)
    assert np.array_equal(a, b)
    engine.set_records_limit(1 << 14)  # forces many chunks of whole stream rounds
    try:
        c, st = engine.price(job)
    finally:
        engine.set_records_limit(0)
    assert np.allclose(a, c, rtol=1e-12, atol=0)
    assert st.kernel_launches > 4


@pytest.mark.parametrize("paths,streams", [(1, 0), (3, 0), (1000, 4096), (131073, 0), (5000, 7)])
def test_path_count_edges(engine, oracle_lib, paths, streams):
    spec = jobspec.with_config(MC_SPECS["heston_nv_put_full"], paths=paths, streams=streams, steps=20)
    job = jobspec.make_job(spec)
    raw, st = engine.price(job)
    want, _ = oracle_lib.mc_price(job, oracle_lib.LAYOUT_STREAMS, 8)
    assert st.paths == paths
    assert np.all(np.isfinite(raw))
    np.testing.assert_allclose(raw[0], want[0], rtol=2e-4, atol=1e-5)


def test_large_strip(engine, oracle_lib):
    spec = jobspec.with_config(MC_SPECS["c2_bates_nci_strip_essential"], paths=4096, streams=512)
    spec["instrument"]["K"] = list(np.linspace(50.0, 150.0, 1000))
    job = jobspec.make_job(spec)
    raw, _ = engine.price(job)
    want, _ = oracle_lib.mc_price(job, oracle_lib.LAYOUT_STREAMS, 8)
    se = np.maximum(raw[1::2], want[1::2])
    floor = 1e-7 * float(np.max(np.abs(want[0])))
    assert np.all(np.abs(raw[0::2] - want[0::2]) <= 0.35 * se + floor)


def test_day0_barrier_breach_prices_zero(engine):
    raw, _ = engine.price(jobspec.make_job(MC_SPECS["bs_downout_put_day0_breach"]))
    assert raw[0, 0] == 0.0 and raw[1, 0] == 0.0


def test_loop_cap_fault_injection_keeps_context_usable(engine):
    """A capped device loop reports MYQL_ERR_LOOP_CAP (no trap, no hang) and the
    context keeps working: the next call returns the normal result."""
    spec = jobspec.with_config(MC_SPECS["heston_exact_call"], paths=20000)
    job = jobspec.make_job(spec)
    good, _ = engine.price(job)
    engine.set_loop_cap(1)
    try:
        with pytest.raises(_abi.MyqlError) as e:
            engine.price(job)
        assert e.value.status == _abi.ERR_LOOP_CAP
    finally:
        engine.set_loop_cap(0)
    again, _ = engine.price(job)
    assert np.array_equal(good, again)


def test_nv_condition_status_through_engine(engine):
    model = m.HestonModel(m.HestonParams(1.0, 0.01, 0.5, -0.7, 0.04))
    pr = m.MonteCarloPricer(model, m.HestonStepper(m.SchemeNV), m.GreekMode.NONE,
                            m.MonteCarloConfig(num_paths=1000), engine=engine)
    with pytest.raises(_abi.MyqlError) as e:
        pr.calculate(100.0, 0.02, 0.0, m.EuropeanOption(100.0, 1.0))
    assert e.value.status == _abi.ERR_NV_CONDITION


def test_barrier_in_plus_out_equals_european(engine):
    """barrier_test.cpp:97-98: with common random numbers, in + out = vanilla exactly."""
    h = m.HestonModel(m.HestonParams(1.5, 0.04, 0.3, -0.7, 0.04))
    cfg = m.MonteCarloConfig(num_paths=1 << 16, time_steps=252, seed=7)
    st = m.HestonStepper(m.SchemeNV)
    vin = m.MonteCarloPricer(h, st, m.GreekMode.NONE, cfg, engine).calculate(100.0, 0.02, 0.0, m.UpAndInCall(100.0, 120.0, 1.0))
    vout = m.MonteCarloPricer(h, st, m.GreekMode.NONE, cfg, engine).calculate(100.0, 0.02, 0.0, m.UpAndOutCall(100.0, 120.0, 1.0))
    # the European leg must use the same stream consumption: a path-dependent tracker
    # that never knocks (barrier far away) reproduces the vanilla payoff path by path
    veur = m.MonteCarloPricer(h, st, m.GreekMode.NONE, cfg, engine).calculate(100.0, 0.02, 0.0, m.UpAndOutCall(100.0, 1e9, 1.0))
    # per-batch FP32 sums: in + out and the vanilla agree to FP32 summation rounding
    assert abs((vin.price + vout.price) - veur.price) < 2e-6 * veur.price


def test_arith_asian_one_step_equals_half_european(engine):
    """asian_test.cpp:75-77: a one-step arithmetic Asian (trapezoid of S0 and S_T)
    equals 1/2 of a European call struck at 2K - S0."""
    h = m.HestonModel(m.HestonParams(1.5, 0.04, 0.3, -0.7, 0.04))
    cfg = m.MonteCarloConfig(num_paths=1 << 18, time_steps=1, seed=11)
    a = m.MonteCarloPricer(h, m.HestonStepper(m.SchemeNV), m.GreekMode.NONE, cfg, engine).calculate(
        100.0, 0.02, 0.0, m.AsianOption(m.TrackerArithAsian, m.PayoffVanilla(), True, 100.0, 1.0))
    e = m.MonteCarloPricer(h, m.HestonStepper(m.SchemeNV), m.GreekMode.NONE, cfg, engine).calculate(
        100.0, 0.02, 0.0, m.EuropeanOption(100.0, 1.0))
    # same path: avg = (S0 + S_T)/2, payoff = max(S_T - (2K - S0), 0)/2 = max(S_T - K,0)/2 at K=S0
    assert abs(a.price - 0.5 * e.price) < 1e-4 * e.price


_H_NCI = m.HestonParams(2.0, 0.05, 0.9, -0.6, 0.05)   # sigma^2 > 4 kappa theta: NCI only
_H_NV = m.HestonParams(1.5, 0.04, 0.3, -0.7, 0.04)
_H_NV2 = m.HestonParams(0.5, 0.04, 0.2, -0.3, 0.03)
_MJ = m.MertonParams(0.5, -0.1, 0.15)
_KJ = m.KouParams(0.8, 0.4, 10.0, 5.0)
LOCKSTEP = {
    "bates_nci": (m.BatesModel(_H_NCI, _MJ), m.BatesStepper(m.SchemeNCI)),
    "heston_nv": (m.HestonModel(_H_NV), m.HestonStepper(m.SchemeNV)),
    "bateskou_nci": (m.BatesKouModel(_H_NV, _KJ), m.BatesKouStepper(m.SchemeNCI)),
    "dbates_nci_nv": (m.DoubleBatesModel(_H_NCI, _H_NV2, _MJ), m.DoubleBatesStepper(m.SchemeNCI, m.SchemeNV)),
    "dheston_nv_nci": (m.DoubleHestonModel(_H_NV, _H_NCI), m.DoubleHestonStepper(m.SchemeNV, m.SchemeNCI)),
    # both factors on NCI: the v0-bumped variance paths merge into the base's
    "dbates_nci_nci": (m.DoubleBatesModel(_H_NCI, m.HestonParams(1.0, 0.03, 0.6, -0.4, 0.03), _MJ),
                       m.DoubleBatesStepper(m.SchemeNCI, m.SchemeNCI)),
}


LOCKSTEP_CASES = [(n, 40) for n in LOCKSTEP] + [(n, 200) for n in ("bates_nci", "dbates_nci_nci")]


@pytest.mark.parametrize("T", [0.25, 1.0, 4.0])
def test_t_bumped_counts_shared_at_scale(engine, T):
    """The lockstep kernel's records at the headline strip's scale: the Bates SchemeNCI model
    and step size (200 a year), 2^20 paths of 50 to 800 steps.  The base and the T-bumped
    scenarios, evolved together on shared draws (with the merged v0-bumped variance paths),
    must equal requests that price T and T +- t_bump alone, bit for bit."""
    model, stepper = m.BatesModel(_H_NCI, _MJ), m.BatesStepper(m.SchemeNCI)
    steps = int(round(200 * T))
    cfg = m.MonteCarloConfig(num_paths=1 << 20, time_steps=steps, seed=11, n_streams=1 << 20)
    full = m.make_job(model, stepper, m.EuropeanOption([100.0], T), m.GreekMode.FULL, cfg, 100.0, 0.02, 0.0)
    g = engine.paths(full)

    def single(t):
        return engine.paths(m.make_job(model, stepper, m.EuropeanOption([100.0], t), m.GreekMode.NONE, cfg,
                                       100.0, 0.02, 0.0))[0]

    np.testing.assert_array_equal(g[3], single(T + cfg.t_bump))
    np.testing.assert_array_equal(g[4], single(T - cfg.t_bump))
    np.testing.assert_array_equal(g[0], single(T))


@pytest.mark.parametrize("name,steps", LOCKSTEP_CASES, ids=[f"{n}-{k}" for n, k in LOCKSTEP_CASES])
def test_full_greek_scenarios_equal_single_scenario_runs(engine, name, steps):
    """Full Greeks of a European advance every bumped scenario of a path in lockstep
    on shared draws.  Each scenario's records must be bit-identical to a request
    that prices that bumped scenario alone (MonteCarloPricer.hpp:302-410 replays
    the path from rng_start for each bump).  The v0-bumped variance paths of NCI factors
    merge into the base's; the 200-step cases run most steps merged."""
    model, stepper = LOCKSTEP[name]
    # one path per stream: a stream continues from the base scenario's end state, and a
    # bumped scenario priced alone continues from its own, which differs once its jump
    # count (and so its draw count) differs from the base's
    cfg = m.MonteCarloConfig(num_paths=6000, time_steps=steps, seed=7, n_streams=6000)
    T, S0, r, q = 0.75, 100.0, 0.02, 0.01
    full = m.make_job(model, stepper, m.EuropeanOption([90.0, 100.0, 110.0], T), m.GreekMode.FULL,
                      cfg, S0, r, q)
    g = engine.paths(full)
    nf = model.num_variance_factors
    assert g.shape[0] == (9 if nf == 2 else 7)

    def single(mod, t):
        j = m.make_job(mod, stepper, m.EuropeanOption([100.0], t), m.GreekMode.NONE, cfg, S0, r, q)
        return engine.paths(j)[0]

    def bump_v0(f, s):
        if nf == 1:
            return dataclasses.replace(model, heston=dataclasses.replace(model.heston, v0=model.heston.v0 + s * cfg.vol_bump))
        key = "heston1" if f == 0 else "heston2"
        h = getattr(model, key)
        return dataclasses.replace(model, **{key: dataclasses.replace(h, v0=h.v0 + s * cfg.vol_bump)})

    np.testing.assert_array_equal(g[0], single(model, T))
    np.testing.assert_array_equal(g[1], single(bump_v0(0, +1), T))
    np.testing.assert_array_equal(g[2], single(bump_v0(0, -1), T))
    np.testing.assert_array_equal(g[3], single(model, T + cfg.t_bump))
    np.testing.assert_array_equal(g[4], single(model, T - cfg.t_bump))
    if nf == 2:
        np.testing.assert_array_equal(g[7], single(bump_v0(1, +1), T))
        np.testing.assert_array_equal(g[8], single(bump_v0(1, -1), T))
    # rate bumps: the base path shifted by (r' - r) T
    np.testing.assert_allclose(g[5], g[0] + np.float32(cfg.r_bump * T), rtol=0, atol=2e-6)
    np.testing.assert_allclose(g[6], g[0] - np.float32(cfg.r_bump * T), rtol=0, atol=2e-6)
