"""CPU checks of the FP64 MLP oracle that the tensor-core kernels are compared
with: its back-propagated gradient against central finite differences."""
import numpy as np

from oracle import mlp_oracle as mo


def small_problem(seed=0, n_paths=12, n_hedge=5):
    rng = np.random.default_rng(seed)
    params = np.zeros(mo.NPARAM)
    for k, (o, s) in mo.LAYOUT.items():
        scale = 1.0 / np.sqrt(s[-1]) if len(s) == 2 else 0.3
        params[o:o + int(np.prod(s))] = rng.uniform(-scale, scale, int(np.prod(s)))
    feats = rng.uniform(-1, 1, (n_paths * n_hedge, 6))
    dM = rng.standard_normal(n_paths * n_hedge)
    Y = rng.standard_normal(n_paths) * 3 + 1
    return params, feats, dM, Y, n_paths, n_hedge


def test_backprop_matches_finite_differences():
    params, feats, dM, Y, n, h = small_problem()
    _, grad = mo.loss_and_grad(params, feats, dM, Y, n, h, bf16_storage=False)
    rng = np.random.default_rng(1)
    # every parameter group, a few coordinates each (padding inputs of W1 included)
    idx = []
    for k, (o, s) in mo.LAYOUT.items():
        size = int(np.prod(s))
        idx += list(o + rng.choice(size, min(size, 6), replace=False))
    idx += [mo.LAYOUT["W1"][0] + 7]  # weight of a zero input: gradient exactly 0
    eps = 1e-6
    for i in idx:
        p1, p2 = params.copy(), params.copy()
        p1[i] += eps
        p2[i] -= eps
        fd = (mo.loss(p1, feats, dM, Y, n, h) - mo.loss(p2, feats, dM, Y, n, h)) / (2 * eps)
        assert abs(fd - grad[i]) <= 1e-6 * max(1.0, abs(fd)), (i, fd, grad[i])


def test_bf16_rounding():
    x = np.array([1.0, 1.0 + 2 ** -8, 1.0 + 3 * 2 ** -8, -3.1415926, 0.0])
    assert list(mo.bf16(x)) == [1.0, 1.0, 1.0 + 2 ** -6, -3.140625, 0.0]


def test_cv_training_budget_follows_the_plain_time():
    """The control variate's training budget grows with the plain estimator's time to the
    target, and explicit settings (hedging interval, seed) pass through."""
    from myquantlib_gb300.pricers import ControlVariateConfig
    light = ControlVariateConfig.for_plain_time(0.02, hedge_every=8, seed=7)
    mid = ControlVariateConfig.for_plain_time(0.1)
    full = ControlVariateConfig.for_plain_time(2.0, iterations=150)
    assert light.pilot_paths < mid.pilot_paths < full.pilot_paths
    assert light.iterations < mid.iterations < full.iterations
    assert (light.hedge_every, light.seed, full.iterations) == (8, 7, 150)
    c = light.c()
    assert (c.pilot_paths, c.iterations, c.batch_paths) == (1 << 15, 15, 2048)
    # hedge times per path: 8 for short jobs, 10 mid-size, 32 long
    assert ControlVariateConfig.for_plain_time(0.02, time_steps=256).hedge_every == 32
    assert ControlVariateConfig.for_plain_time(0.1, time_steps=100).hedge_every == 10
    assert ControlVariateConfig.for_plain_time(2.0, time_steps=256).hedge_every == 8
    assert ControlVariateConfig.for_plain_time(2.0, time_steps=16).hedge_every == 1
    assert ControlVariateConfig.for_plain_time(0.02, time_steps=256, hedge_every=4).hedge_every == 4
