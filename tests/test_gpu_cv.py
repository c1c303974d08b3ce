"""GPU tests of the neural control variate: the tcgen05 operand layouts, the
MLP forward/backward kernels against an FP64 CPU MLP, and the control-variate
estimator against plain Monte Carlo."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def bf16(x):
    """Round to BF16 (nearest even), returned as float64."""
    a = np.ascontiguousarray(x, dtype=np.float32).view(np.uint32).astype(np.uint64)
    a = ((a + 0x7FFF + ((a >> 16) & 1)) >> 16) << 16
    return a.astype(np.uint32).view(np.float32).astype(np.float64)


@pytest.mark.parametrize("mode,K,N", [(0, 16, 128), (1, 128, 128), (2, 128, 16), (3, 128, 128)])
def test_mma_operand_layouts(engine, mode, K, N):
    rng = np.random.default_rng(mode)
    A = rng.standard_normal((128, K)).astype(np.float32)
    B = rng.standard_normal((N, K)).astype(np.float32)
    D = np.zeros((128, N), dtype=np.float32)
    fp = lambda a: a.ctypes.data_as(C.POINTER(C.c_float))  # noqa: E731
    from myquantlib_gb300 import _abi
    _abi.check(engine.lib.myql_probe_mma(engine.handle, mode, fp(A), fp(B), fp(D)))
    want = bf16(A) @ bf16(B).T
    err = np.abs(D - want).max()
    assert err < 1e-3 * np.abs(want).max(), (err, D[:2, :4], want[:2, :4])


# ---------------------------------------------------------------- MLP kernels vs the FP64 CPU MLP
import myquantlib_gb300 as m  # noqa: E402
from oracle import mlp_oracle as mo  # noqa: E402


def mlp_problem(seed, n_paths, n_hedge):
    rng = np.random.default_rng(seed)
    rows = n_paths * n_hedge
    t = np.tile(np.arange(n_hedge) / n_hedge, n_paths)
    feats = np.stack([t, rng.normal(0, 0.7, rows), rng.gamma(2.0, 0.5, rows), rng.gamma(2.0, 0.5, rows),
                      rng.uniform(0, 1, rows) * t, np.ones(rows)], axis=1)
    dM = rng.normal(0.0, 2.0, rows)
    Y = np.maximum(rng.normal(2.0, 8.0, n_paths), 0.0) + 0.5 * (dM.reshape(n_paths, n_hedge).sum(1))
    return feats, dM, Y


def network(engine, seed=3):
    engine.cv_init(seed)
    p = engine.cv_params().astype(np.float64)
    o, s = mo.LAYOUT["w4"]
    p[o:o + 128] *= 30.0          # a non-trivial output layer
    p[mo.LAYOUT["b4"][0]] = 0.05
    engine.cv_set_params(p.astype(np.float32))
    return engine.cv_params().astype(np.float64)


# the first two run tile-major (minibatch sizes); 160037 paths (1251 ragged path blocks,
# above 8 per SM) run path-major, whole path blocks per tile group
@pytest.mark.parametrize("n_paths,n_hedge", [(300, 7), (1024, 32), (160037, 1)])
def test_cv_forward_matches_cpu_mlp(engine, n_paths, n_hedge):
    params = network(engine)
    feats, dM, _ = mlp_problem(1, n_paths, n_hedge)
    cv, g = engine.cv_forward(feats, dM, n_paths, n_hedge)
    g_ref, _ = mo.forward(params, mo.bf16(feats.astype(np.float32)))
    cv_ref = (g_ref * dM.astype(np.float32)).reshape(n_paths, n_hedge).sum(1)
    assert np.linalg.norm(g - g_ref) <= 1e-2 * np.linalg.norm(g_ref), np.abs(g - g_ref).max()
    assert np.abs(g - g_ref).max() <= 3e-2 * np.abs(g_ref).max()
    assert np.linalg.norm(cv - cv_ref) <= 1e-2 * np.linalg.norm(cv_ref)


def test_cv_gradient_is_deterministic(engine):
    """The backward blocks write per-block gradient slices that one kernel sums in block
    order: the same data gives the same gradient bit for bit."""
    network(engine)
    feats, dM, Y = mlp_problem(3, 4096, 16)
    l1, g1 = engine.cv_gradient(feats, dM, Y, 4096, 16)
    l2, g2 = engine.cv_gradient(feats, dM, Y, 4096, 16)
    assert np.array_equal(g1, g2) and l1 == l2


@pytest.mark.parametrize("n_paths,n_hedge", [(300, 8), (2048, 16)])
def test_cv_gradient_matches_cpu_mlp(engine, n_paths, n_hedge):
    params = network(engine)
    feats, dM, Y = mlp_problem(2, n_paths, n_hedge)
    loss, grad = engine.cv_gradient(feats, dM, Y, n_paths, n_hedge)
    L_ref, g_ref = mo.loss_and_grad(params, feats.astype(np.float32).astype(np.float64),
                                    dM.astype(np.float32).astype(np.float64),
                                    Y.astype(np.float32).astype(np.float64), n_paths, n_hedge)
    assert loss == pytest.approx(L_ref, rel=5e-3)
    for name, (o, s) in mo.LAYOUT.items():
        k = int(np.prod(s))
        a, b = grad[o:o + k].astype(np.float64), g_ref[o:o + k]
        if name == "W1":  # only the 6 used input slots carry gradient
            a, b = a.reshape(128, 16)[:, :6].ravel(), b.reshape(128, 16)[:, :6].ravel()
            assert np.all(grad[o:o + k].reshape(128, 16)[:, 6:] == 0.0)
        rel = np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-30)
        cos = float(a @ b / max(np.linalg.norm(a) * np.linalg.norm(b), 1e-30))
        assert rel < 3e-2 and cos > 0.999, (name, rel, cos)


# ---------------------------------------------------------------- the control variate on engine paths
FOURIER_C1 = 8.628108103110  # FP64 Gil-Pelaez price of the Heston call below (reference FourierPricer)


def heston_call_job(paths, steps=100):
    model = m.HestonModel(m.HestonParams(kappa=1.5, theta=0.04, sigma=0.3, rho=-0.7, v0=0.04))
    return m.make_job(model, m.HestonStepper(m.SchemeNV), m.EuropeanOption(100.0, 1.0), m.GreekMode.NONE,
                      m.MonteCarloConfig(num_paths=paths, time_steps=steps, seed=42), 100.0, 0.02, 0.0)


def double_bates_asian_job(paths, seed=42):
    model = m.DoubleBatesModel(m.HestonParams(kappa=2.0, theta=0.03, sigma=0.4, rho=-0.7, v0=0.03),
                               m.HestonParams(kappa=0.5, theta=0.02, sigma=0.3, rho=-0.3, v0=0.02),
                               m.MertonParams(0.3, -0.05, 0.1))
    instr = m.AsianOption(m.TrackerArithAsian, m.PayoffVanilla(), True, 100.0, 2.0)
    return m.make_job(model, m.DoubleBatesStepper(m.SchemeNCI, m.SchemeNCI, m.TrackerArithAsian), instr,
                      m.GreekMode.NONE, m.MonteCarloConfig(num_paths=paths, time_steps=256, seed=seed),
                      100.0, 0.02, 0.0)


def cv_cfg(hedge_every, iterations=250, pilot=1 << 16, batch=4096):
    return m.pricers.ControlVariateConfig(hedge_every=hedge_every, iterations=iterations, pilot_paths=pilot,
                                          batch_paths=batch, learning_rate=2e-3, seed=7).c()


def test_cv_heston_european_unbiased_and_gains(engine):
    cfg = cv_cfg(5)
    tr = engine.cv_train(heston_call_job(1 << 16), cfg)
    assert tr.final_loss < tr.initial_loss
    res = engine.cv_price(heston_call_job(1 << 18), cfg)
    assert abs(res.plain_price - FOURIER_C1) < 4 * res.plain_std_err
    assert abs(res.price - FOURIER_C1) < 4 * res.price_std_err + 1e-3, (res.price, res.price_std_err)
    assert res.variance_ratio > 10.0, res.variance_ratio


def test_cv_double_bates_asian_against_plain_engine(engine):
    cfg = cv_cfg(8)
    engine.cv_train(double_bates_asian_job(1 << 16, seed=5), cfg)
    res = engine.cv_price(double_bates_asian_job(1 << 18), cfg)
    raw, _ = engine.price(double_bates_asian_job(1 << 20, seed=77))
    ref, ref_se = raw[0, 0], raw[1, 0]
    assert abs(res.price - ref) < 4 * np.hypot(res.price_std_err, ref_se), (res.price, ref, res.price_std_err, ref_se)
    assert abs(res.plain_price - ref) < 4 * np.hypot(res.plain_std_err, ref_se)
    assert res.variance_ratio > 8.0, res.variance_ratio


def test_cv_untrained_network_is_still_unbiased(engine):
    """Any network keeps the estimator unbiased: a random one only fails to reduce variance."""
    cfg = cv_cfg(4)
    network(engine, seed=11)
    res = engine.cv_price(heston_call_job(1 << 18), cfg)
    assert abs(res.price - FOURIER_C1) < 4 * res.price_std_err + 1e-3, (res.price, res.price_std_err)


def test_cv_training_and_pricing_are_reproducible(engine):
    """Every reduction of the control variate (gradient slices, residuals, hedge ratio,
    price sums) runs on a fixed grid in a fixed order: training twice from the same seed
    gives the same network bit for bit, and pricing twice gives the same estimate."""
    cfg = cv_cfg(8, iterations=30, pilot=1 << 14)
    job = double_bates_asian_job(1 << 14)
    r1 = engine.cv_train(job, cfg)
    p1 = engine.cv_params()
    r2 = engine.cv_train(job, cfg)
    p2 = engine.cv_params()
    assert np.array_equal(p1, p2)
    assert r1.final_loss == r2.final_loss and r1.variance_ratio == r2.variance_ratio
    pj = double_bates_asian_job(1 << 17, seed=9)
    a, b = engine.cv_price(pj, cfg), engine.cv_price(pj, cfg)
    assert a.price == b.price and a.price_std_err == b.price_std_err


# ---------------------------------------------------------------- the control variate on QMC paths
def test_cv_qmc_simulates_the_qmc_pricer_paths(engine):
    """myql_cv_qmc_price steps the points of myql_qmc_price: its plain replicate means give the
    QMC price of the same job (FP32 payoffs summed in another order: equal to ~1e-6)."""
    cfg = cv_cfg(8, iterations=20, pilot=1 << 14)
    engine.cv_train(double_bates_asian_job(1 << 14, seed=5), cfg)
    job = double_bates_asian_job(1 << 17, seed=21)
    q, _ = engine.qmc_price(double_bates_asian_job(1 << 17, seed=21), 16)
    res = engine.cv_qmc_price(job, cfg, 16)
    assert abs(res.plain_price - q[0, 0]) < 1e-5 * q[0, 0], (res.plain_price, q[0, 0])
    assert abs(res.plain_std_err - q[1, 0]) < 1e-3 * q[1, 0], (res.plain_std_err, q[1, 0])


def test_cv_qmc_heston_european_unbiased_and_gains(engine):
    cfg = cv_cfg(5)
    engine.cv_train(heston_call_job(1 << 16), cfg)
    res = engine.cv_qmc_price(heston_call_job(1 << 18), cfg, 16)
    assert abs(res.price - FOURIER_C1) < 4 * res.price_std_err + 1e-3, (res.price, res.price_std_err)
    # against the control variate on pseudo-random paths of the same count: at least twice less
    # variance (a 16-replicate standard error carries about 18 % noise)
    ps = engine.cv_price(heston_call_job(1 << 18), cfg)
    assert res.price_std_err < 0.7 * ps.price_std_err, (res.price_std_err, ps.price_std_err)


def test_cv_qmc_double_bates_asian_against_plain_engine(engine):
    cfg = cv_cfg(8)
    engine.cv_train(double_bates_asian_job(1 << 16, seed=5), cfg)
    res = engine.cv_qmc_price(double_bates_asian_job(1 << 18), cfg, 16)
    raw, _ = engine.price(double_bates_asian_job(1 << 20, seed=77))
    ref, ref_se = raw[0, 0], raw[1, 0]
    assert abs(res.price - ref) < 4 * np.hypot(res.price_std_err, ref_se), (res.price, ref, res.price_std_err, ref_se)
    ps = engine.cv_price(double_bates_asian_job(1 << 18), cfg)
    assert res.price_std_err < ps.price_std_err, (res.price_std_err, ps.price_std_err)


def test_cv_qmc_refuses_what_qmc_refuses(engine):
    from myquantlib_gb300 import _abi
    cfg = cv_cfg(5, iterations=5, pilot=1 << 12)
    engine.cv_train(heston_call_job(1 << 12), cfg)
    with pytest.raises(_abi.MyqlError) as e:
        engine.cv_qmc_price(heston_call_job(3 * 2048), cfg, 2)
    assert e.value.status == _abi.ERR_INVALID_ARG
    exact = m.make_job(m.HestonModel(m.HestonParams(1.5, 0.04, 0.3, -0.7, 0.04)), m.HestonStepper(m.SchemeExact),
                       m.EuropeanOption(100.0, 1.0), m.GreekMode.NONE,
                       m.MonteCarloConfig(num_paths=1 << 15, time_steps=16, seed=1), 100.0, 0.02, 0.0)
    with pytest.raises(_abi.MyqlError) as e:
        engine.cv_qmc_price(exact, cfg, 16)
    assert e.value.status == _abi.ERR_UNSUPPORTED
