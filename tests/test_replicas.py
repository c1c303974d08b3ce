"""Replicas on CPU ranks (gloo, world size 2): each rank prices its shard of a
request with the oracle on its own stream range, the ranks pool the FP64
moments with one all-reduce, and the pooled result equals the single request
over all the streams."""
import os
import socket

import numpy as np
import pytest
import torch.distributed as dist
import torch.multiprocessing as mp

import jobspec
import myquantlib_gb300 as m
from myquantlib_gb300 import replicas

SPEC = {"name": "bates_nci_strip", "config": {"paths": 4096, "steps": 20}, "mode": "essential",
        "instrument": {"K": [90.0, 100.0, 110.0], "T": 1.0, "kind": "european"},
        "model": {"heston": [[2.0, 0.05, 0.9, -0.6, 0.05]], "jump": {"kind": "merton", "lambda": 0.5, "mu": -0.1,
                                                                   "delta": 0.15}},
        "schemes": ["NCI"]}


def _job(paths, streams):
    spec = dict(SPEC, config={"paths": paths, "steps": 20})
    j = jobspec.make_job(spec)
    j.c.config.n_streams = streams
    return j


def _rank(rank, world, port, out_q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        from oracle import oracle
        shard = replicas.shard_job(_job(4096, 512 * world), rank, world)
        raw, _ = oracle.mc_price(shard, oracle.LAYOUT_STREAMS, 1)
        pooled = replicas.allreduce_price(raw, int(shard.c.config.num_paths))
        out_q.put((rank, int(shard.c.config.stream_offset), pooled))
    finally:
        dist.destroy_process_group()


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_two_rank_pool_equals_single_request(oracle_lib):
    world = 2
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    got = [q.get(timeout=120) for _ in range(world)]
    for p in procs:
        p.join(60)
        assert p.exitcode == 0
    got.sort(key=lambda t: t[0])
    assert [g[1] for g in got] == [0, 512]
    want, _ = oracle_lib.mc_price(_job(4096, 512 * world), oracle_lib.LAYOUT_STREAMS, 1)
    for _, _, pooled in got:
        np.testing.assert_allclose(pooled[:6], want[:6], rtol=1e-11, atol=1e-13)


def test_shard_job_layout():
    j = _job(1 << 20, 0)
    s = replicas.shard_job(j, 3, 4)
    assert int(s.c.config.num_paths) == 1 << 18
    assert int(s.c.config.n_streams) == 32768 and int(s.c.config.stream_offset) == 3 * 32768
    with pytest.raises(ValueError):
        replicas.shard_job(_job(1001, 0), 0, 2)


def test_combine_is_compute_stats():
    """Pooling per-replica (mean, standard error) rows reproduces the statistics of all samples."""
    rng = np.random.default_rng(0)
    x = rng.standard_normal((3, 1000)) * 2 + 1
    mom = 0
    for part in (x[:, :400], x[:, 400:]):
        rows = np.empty((6, 1))
        rows[0::2, 0] = part.mean(1)
        rows[1::2, 0] = np.sqrt(part.var(1) / part.shape[1])
        mom = mom + replicas.moments(rows, part.shape[1])
    pooled = replicas.combine(mom, 1000)
    np.testing.assert_allclose(pooled[0::2, 0], x.mean(1), rtol=1e-12)
    np.testing.assert_allclose(pooled[1::2, 0], np.sqrt(x.var(1) / 1000), rtol=1e-10)


def test_pool_estimates():
    """Fixed-weight pooling of independent estimates: equal weights by default, the planned
    budgets when given; SE = sqrt(sum w^2 se^2) / sum w.  A zero standard error is accepted
    only when every replica agrees on it."""
    p, se = replicas.pool_estimates([3.0, 5.0, 7.0, 9.0], [0.4] * 4)
    assert abs(p - 6.0) < 1e-14 and abs(se - 0.2) < 1e-15
    p, se = replicas.pool_estimates([1.0, 2.0], [0.1, 0.2], weights=[3.0, 1.0])
    assert abs(p - 1.25) < 1e-15 and abs(se - np.sqrt(9 * 0.01 + 0.04) / 4) < 1e-15
    # unequal sample SEs do not move the weights (1/se^2 weights would bias the pool low)
    p, _ = replicas.pool_estimates([1.0, 2.0], [0.1, 0.2])
    assert abs(p - 1.5) < 1e-15
    assert replicas.pool_estimates([2.5, 2.5], [0.0, 0.0]) == (2.5, 0.0)
    for bad in (([], []), ([1.0], [0.1, 0.2]), ([1.0], [-0.1]), ([np.nan], [0.1]), ([4.0, 2.5], [0.3, 0.0]),
                ([1.0, 1.0], [0.0, 0.0], [1.0, -1.0])):
        with pytest.raises(ValueError):
            replicas.pool_estimates(*bad)


def _mlmc_cfg(seed):
    from myquantlib_gb300 import _abi
    c = _abi.MlmcConfigC()
    c.epsilon, c.L_min, c.L_max, c.N0, c.base_steps = 0.05, 2, 5, 2000, 1
    c.alpha, c.beta, c.adaptive_rates, c.seed, c.fd_bump, c.n_streams = 2.0, 1.0, 1, seed, 1e-4, 0
    return c


def _mlmc_job():
    return m.make_job(m.HestonModel(m.HestonParams(1.5, 0.04, 0.3, -0.7, 0.04)), m.HestonStepper(m.SchemeNV),
                      m.EuropeanOption(100.0, 1.0), m.GreekMode.NONE, m.MonteCarloConfig(), 100.0, 0.02, 0.0)


def _mlmc_rank(rank, world, port, out_q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        from oracle import oracle
        r = oracle.mlmc_price(_mlmc_job(), _mlmc_cfg(42 + rank), oracle.LAYOUT_REFERENCE, 1)
        out_q.put((rank, replicas.allreduce_estimate(r.price, r.price_std_err, float(r.total_steps))))
    finally:
        dist.destroy_process_group()


def test_two_rank_mlmc_estimates_pool(oracle_lib):
    """Two CPU ranks each run an independent MLMC estimate (own controller seed) and pool them,
    weighted by their path-step budgets, through one all-gather; every rank gets the pooled
    estimate of both."""
    world = 2
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_mlmc_rank, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    got = [q.get(timeout=120) for _ in range(world)]
    for p in procs:
        p.join(60)
        assert p.exitcode == 0
    runs = [oracle_lib.mlmc_price(_mlmc_job(), _mlmc_cfg(42 + r), oracle_lib.LAYOUT_REFERENCE, 1) for r in range(world)]
    want = replicas.pool_estimates([r.price for r in runs], [r.price_std_err for r in runs],
                                   [float(r.total_steps) for r in runs])
    for _, (p, se) in got:
        assert abs(p - want[0]) < 1e-12 * abs(want[0]) and abs(se - want[1]) < 1e-12 * want[1]
    assert want[1] < min(r.price_std_err for r in runs)
