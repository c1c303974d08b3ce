"""GPU tests of the batched persistent engine (myql_mc_price_batch): many
uneven requests in one launch must return what each request returns when it
is priced alone, and what the oracle returns on the same streams."""
import numpy as np
import pytest

import myquantlib_gb300 as m
from myquantlib_gb300 import dispatch, workloads

pytestmark = pytest.mark.gpu

H = m.HestonParams(kappa=1.5, theta=0.04, sigma=0.3, rho=-0.7, v0=0.04)
H2 = m.HestonParams(kappa=2.0, theta=0.05, sigma=0.9, rho=-0.6, v0=0.05)
H3 = m.HestonParams(kappa=3.0, theta=0.02, sigma=0.2, rho=-0.3, v0=0.02)


def mixed_requests():
    """One request per kernel class, path-dependent and European, both Greek modes."""
    E = lambda K=100.0: m.EuropeanOption(K, 1.0)  # noqa: E731
    A = lambda K=100.0: m.AsianOption(m.TrackerArithAsian, m.PayoffVanilla(), True, K, 1.0)  # noqa: E731
    rq = []
    add = lambda model, instr, sch, paths, steps, mode=m.GreekMode.NONE, seed=7, streams=0: rq.append(  # noqa: E731
        dispatch.Request(model, instr, m.MonteCarloConfig(num_paths=paths, time_steps=steps, seed=seed,
                                                          n_streams=streams),
                         100.0, 0.02, 0.0, mode=mode, stepper=sch))
    bs, mj = m.BlackScholesModel(0.2), m.MertonModel(0.2, m.MertonParams(1.0, -0.05, 0.1))
    add(bs, E(), m.BlackScholesStepper(), 20000, 16, m.GreekMode.ESSENTIAL)
    add(mj, m.UpAndOutCall(100.0, 130.0, 1.0), m.MertonJDStepper(m.TrackerBarrier), 30000, 50)
    add(m.HestonModel(H), E(95.0), m.HestonStepper(m.SchemeNV), 50000, 100, m.GreekMode.ESSENTIAL)
    add(m.HestonModel(H), A(), m.HestonStepper(m.SchemeExact, m.TrackerArithAsian), 40000, 64)
    add(m.BatesModel(H2, m.MertonParams(0.5, -0.1, 0.15)), E(), m.BatesStepper(m.SchemeNCI), 65536, 200,
        m.GreekMode.ESSENTIAL, seed=11)
    add(m.BatesKouModel(H2, m.KouParams(0.7, 0.4, 10.0, 5.0)), m.UpAndOutCall(100.0, 130.0, 1.0),
        m.BatesKouStepper(m.SchemeExact, m.TrackerBarrier), 20000, 100, seed=12)
    add(m.DoubleHestonModel(H, H3), A(105.0), m.DoubleHestonStepper(m.SchemeNV, m.SchemeNV, m.TrackerArithAsian),
        16384, 32)
    add(m.DoubleHestonModel(H2, H3), E(), m.DoubleHestonStepper(m.SchemeExact, m.SchemeNCI), 12345, 40,
        m.GreekMode.ESSENTIAL, streams=1000)
    add(m.DoubleHestonModel(H2, H), m.LookbackOption(m.PayoffVanilla(), True, 100.0, 1.0),
        m.DoubleHestonStepper(m.SchemeNCI, m.SchemeExact, m.TrackerLookback), 9000, 24)
    add(m.DoubleBatesKouModel(H3, H2, m.KouParams(1.0, 0.4, 10.0, 5.0)), E(110.0),
        m.DoubleBatesKouStepper(m.SchemeNV, m.SchemeExact), 25000, 30)
    add(m.DoubleHestonModel(H2, H2), E(), m.DoubleHestonStepper(m.SchemeExact, m.SchemeExact), 3000, 12)
    add(m.DoubleHestonModel(H3, H2), E(), m.DoubleHestonStepper(m.SchemeNV, m.SchemeNCI), 5000, 20)
    add(m.DoubleHestonModel(H2, H3), E(), m.DoubleHestonStepper(m.SchemeNCI, m.SchemeNV), 5000, 20)
    add(m.DoubleHestonModel(H2, H3), E(), m.DoubleHestonStepper(m.SchemeNCI, m.SchemeNCI), 5000, 20)
    add(m.DoubleHestonModel(H3, H3), E(), m.DoubleHestonStepper(m.SchemeNV, m.SchemeExact), 5000, 20)
    add(m.DoubleHestonModel(H2, H3), E(), m.DoubleHestonStepper(m.SchemeExact, m.SchemeNV), 5000, 20)
    add(m.HestonModel(H3), E(), m.HestonStepper(m.SchemeNV), 1, 5)  # a one-path job
    add(m.HestonModel(H3), m.DownAndOutPut(100.0, 80.0, 1.0), m.HestonStepper(m.SchemeNV, m.TrackerBarrier),
        7777, 33, seed=2**63 + 5, streams=300)
    return rq


def jobs_of(rq):
    return [m.make_job(r.model, r.stepper or m.stepper_for(r.model, r.instrument, r.scheme), r.instrument,
                       m.GreekMode(r.mode), r.cfg, r.S0, r.r, r.q) for r in rq]


def nq(mode):
    return 3 if mode == m.GreekMode.ESSENTIAL else 1


def test_batch_equals_single_requests(engine):
    rq = mixed_requests()
    jobs = jobs_of(rq)
    outs, st = engine.price_batch(jobs)
    assert st.paths == sum(r.cfg.num_paths for r in rq)
    for r, j, got in zip(rq, jobs, outs):
        want, _ = engine.price(j)
        for q in range(nq(r.mode)):
            v, se = want[2 * q, 0], want[2 * q + 1, 0]
            # same streams, same FP32 path arithmetic: only the summation order differs
            assert abs(got[2 * q, 0] - v) <= 2e-6 * abs(v) + 1e-3 * se + 1e-12, (q, got[2 * q, 0], v, se)
            assert abs(got[2 * q + 1, 0] - se) <= 1e-4 * se + 1e-12, (q, got[2 * q + 1, 0], se)
        assert np.all(got[2 * nq(r.mode):] == 0.0)


def test_batch_replays_oracle_streams(engine, oracle_lib):
    rq = mixed_requests()[:8]
    jobs = jobs_of(rq)
    outs, _ = engine.price_batch(jobs)
    for r, j, got in zip(rq, jobs, outs):
        want, _ = oracle_lib.mc_price(j, oracle_lib.LAYOUT_STREAMS, 8)
        for q in range(nq(r.mode)):
            se = want[2 * q + 1, 0]
            assert abs(got[2 * q, 0] - want[2 * q, 0]) <= 0.3 * se + 1e-5 * abs(want[2 * q, 0]) + 1e-10, \
                (q, got[2 * q, 0], want[2 * q, 0], se)


def test_batch_deterministic_and_graph_replay(engine):
    rq = workloads.uneven_requests(64, max_log2_paths=15.0, max_log2_steps=6.0)
    jobs = jobs_of(rq)
    a, _ = engine.price_batch(jobs)
    b, _ = engine.price_batch(jobs)          # graph replay of the same shape
    for x, y in zip(a, b):
        assert np.array_equal(x, y)
    # a different request list of the same shape re-uses the graph with new descriptors
    rq2 = workloads.uneven_requests(64, seed=5, max_log2_paths=15.0, max_log2_steps=6.0)
    c, _ = engine.price_batch(jobs_of(rq2))
    d = [engine.price(j)[0] for j in jobs_of(rq2)]
    for x, y in zip(c, d):
        assert abs(x[0, 0] - y[0, 0]) <= 2e-6 * abs(y[0, 0]) + 1e-3 * y[1, 0] + 1e-12


def test_uneven_workload_against_oracle(engine, oracle_lib):
    rq = workloads.uneven_requests(24, seed=9, max_log2_paths=14.5, max_log2_steps=7.0)
    res = dispatch.price_mc_batch(rq, engine=engine)
    for r, got, j in zip(rq, res, jobs_of(rq)):
        want, _ = oracle_lib.mc_price(j, oracle_lib.LAYOUT_STREAMS, 8)
        se = want[1, 0]
        assert abs(got.prices[0] - want[0, 0]) <= 0.3 * se + 1e-5 * abs(want[0, 0]) + 1e-10
        assert got.prices_std_err[0] == pytest.approx(se, rel=1e-3)


def test_batch_rejects_strips_and_full(engine):
    j = m.make_job(m.HestonModel(H), m.HestonStepper(m.SchemeNV), m.EuropeanOption([90.0, 100.0], 1.0),
                   m.GreekMode.NONE, m.MonteCarloConfig(num_paths=1000, time_steps=10), 100.0, 0.02, 0.0)
    with pytest.raises(m._abi.MyqlError):
        engine.price_batch([j])
    j = m.make_job(m.HestonModel(H), m.HestonStepper(m.SchemeNV), m.EuropeanOption(100.0, 1.0),
                   m.GreekMode.FULL, m.MonteCarloConfig(num_paths=1000, time_steps=10), 100.0, 0.02, 0.0)
    with pytest.raises(m._abi.MyqlError):
        engine.price_batch([j])


SHAPES = [(128, 1, 0), (64, 2, 0), (256, 1, 0), (128, 2, 0), (256, 2, 0), (128, 1, 2), (64, 4, 0)]


def test_every_launch_shape_gives_the_same_prices(engine):
    """Threads per block, streams per thread and unroll depth change only the FP64 grouping of
    the per-item sums: every shape returns the default shape's prices to 1e-12."""
    jobs = jobs_of(mixed_requests())
    base = None
    try:
        for sh in SHAPES:
            engine.set_batch_shape(*sh)
            outs, _ = engine.price_batch(jobs)
            plan = engine.batch_plan()
            assert {(p["block"], p["streams_per_thread"], p["unroll"]) for p in plan} == {sh}
            assert all(p["tuned"] == -1 for p in plan)
            if base is None:
                base = outs
                continue
            for x, y in zip(outs, base):
                np.testing.assert_allclose(x, y, rtol=1e-12, atol=1e-15)
    finally:
        engine.set_batch_shape(0)


def test_autotuner_picks_a_shape_per_class(engine):
    """A class with enough items is tuned over the launch shapes and grids on its leading items;
    the choice is reported per class and is never slower there than the default shape."""
    eng = m.Engine(0)
    try:
        rq = []
        for k in range(12):   # 12 jobs x 2^17 streams: 12288 items of one class (Heston NV Asian)
            rq.append(dispatch.Request(m.HestonModel(H), m.AsianOption(m.TrackerArithAsian, m.PayoffVanilla(), True,
                                                                       95.0 + k, 1.0),
                                       m.MonteCarloConfig(num_paths=1 << 17, time_steps=16, seed=k),
                                       100.0, 0.02, 0.0, stepper=m.HestonStepper(m.SchemeNV, m.TrackerArithAsian)))
        rq += mixed_requests()[:4]
        jobs = jobs_of(rq)
        outs, _ = eng.price_batch(jobs)
        plan = eng.batch_plan()
        big = [p for p in plan if p["factors"] == 1 and p["scheme1"] == 1 and p["path_dependent"] == 1]
        assert len(big) == 1 and big[0]["tuned"] == 1 and big[0]["items"] == 12 * 1024
        p = big[0]
        assert (p["block"], p["streams_per_thread"], p["unroll"]) in SHAPES
        assert 0 < p["tuned_ms"] <= p["default_ms"] * 1.0001 and p["grid"] > 0
        assert all(q["tuned"] == 0 for q in plan if q is not p)   # too few items to tune
        # the tuned shape prices what each request priced alone prices
        for r, j, got in zip(rq, jobs, outs):
            want, _ = eng.price(j)
            assert abs(got[0, 0] - want[0, 0]) <= 2e-6 * abs(want[0, 0]) + 1e-3 * want[1, 0] + 1e-12
        again, _ = eng.price_batch(jobs)       # cached choice, same graph: identical
        for x, y in zip(outs, again):
            assert np.array_equal(x, y)
    finally:
        eng.close()
