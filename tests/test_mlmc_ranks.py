"""Multi-rank MLMC on CPU ranks (gloo, world size 2): the controller all-reduces
each level batch's FP64 sums and rank 0 broadcasts the next batch size and the
level count.  The two-rank run must equal one process that evaluates both ranks'
shares of every batch (the union of the streams) -- same schedule, same sums,
same price -- and the estimate must be a correct MLMC estimate of the Heston
call (the reference's Fourier value)."""
import math
import os
import socket

import pytest
import torch.distributed as dist
import torch.multiprocessing as mp

import myquantlib_gb300 as m
from myquantlib_gb300 import _abi, mlmc_ranks

STREAMS = 64          # streams per rank share (small: the oracle jumps its streams one by one)
FOURIER_C1 = 8.628108103110   # the reference's FP64 Fourier price of this call


def _cfg():
    c = _abi.MlmcConfigC()
    c.epsilon, c.L_min, c.L_max, c.N0, c.base_steps = 0.04, 2, 6, 4000, 1
    c.alpha, c.beta, c.adaptive_rates, c.seed, c.fd_bump, c.n_streams = 2.0, 1.0, 1, 42, 1e-4, STREAMS
    return c


def _job():
    return m.make_job(m.HestonModel(m.HestonParams(1.5, 0.04, 0.3, -0.7, 0.04)), m.HestonStepper(m.SchemeNV),
                      m.EuropeanOption(100.0, 1.0), m.GreekMode.NONE, m.MonteCarloConfig(), 100.0, 0.02, 0.0)


def _summary(res):
    n = int(res.n_levels)
    return (res.price, res.price_std_err, n, [int(res.paths_per_level[l]) for l in range(n)],
            [res.mean_diffs[l] for l in range(n)], int(res.total_steps))


def _rank(rank, world, port, out_q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        from oracle import oracle
        cfg = _cfg()
        ev = mlmc_ranks.oracle_level_evaluator(oracle, _job(), cfg)
        res = mlmc_ranks.mlmc_price(mlmc_ranks.rank_evaluator(ev, rank, world, STREAMS), cfg, 1.0, 0.02,
                                    mlmc_ranks.Exchange())
        out_q.put((rank, _summary(res)))
    finally:
        dist.destroy_process_group()


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_two_rank_controller_equals_union_of_streams(oracle_lib):
    world = 2
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    got = [q.get(timeout=300) for _ in range(world)]
    for p in procs:
        p.join(60)
        assert p.exitcode == 0
    got.sort(key=lambda t: t[0])
    cfg = _cfg()
    ev = mlmc_ranks.oracle_level_evaluator(oracle_lib, _job(), cfg)
    want = _summary(mlmc_ranks.mlmc_price(mlmc_ranks.union_evaluator(ev, world, STREAMS), cfg, 1.0, 0.02))
    for _, s in got:
        assert s == want  # two summands: the all-reduce and the in-process sum round alike
    price, se, n_levels, paths, _, _ = want
    assert n_levels >= 3 and paths[0] > paths[-1]
    assert abs(price - FOURIER_C1) < 4 * se + cfg.epsilon


def test_share_and_stream_blocks_are_disjoint():
    world, S = 3, 8
    for dN in (1, 2, 3, 7, 100):
        assert sum(mlmc_ranks.share(dN, r, world) for r in range(world)) == dN
    blocks = {mlmc_ranks.stream_offset(5, b, r, world, S) for b in range(4) for r in range(world)}
    assert len(blocks) == 12 and all((o - 5) % S == 0 for o in blocks)


def test_single_rank_controller_schedule_follows_the_reference_rules(oracle_lib):
    """One rank: pilot batches of max(20, N0 / 2^l) on the first pass, levels added by the
    bias test, and the optimal allocation met at the end."""
    cfg = _cfg()
    ev = mlmc_ranks.oracle_level_evaluator(oracle_lib, _job(), cfg)
    calls = []

    def rec(level, dN, batch):
        calls.append((level, dN, batch))
        return mlmc_ranks.rank_evaluator(ev, 0, 1, STREAMS)(level, dN, batch)

    res = mlmc_ranks.mlmc_price(rec, cfg, 1.0, 0.02)
    assert [c[:2] for c in calls[:3]] == [(0, 4000), (1, 2000), (2, 1000)]
    assert [c[2] for c in calls] == list(range(len(calls)))
    n = int(res.n_levels)
    V = [res.var_diffs[l] / math.exp(-0.04) for l in range(n)]
    cost = [float(1 << l) for l in range(n)]
    svc = sum(math.sqrt(V[l] * cost[l]) for l in range(n))
    for l in range(n):
        # the final allocation meets the optimal N_l of the pooled variances (up to one path of rounding)
        assert res.paths_per_level[l] + 1 >= 2.0 * cfg.epsilon ** -2 * math.sqrt(V[l] / cost[l]) * svc
    assert abs(res.price - FOURIER_C1) < 4 * res.price_std_err + cfg.epsilon


@pytest.mark.gpu
def test_gpu_multi_rank_controller_single_rank(engine):
    """The controller on the GPU level evaluator (one rank): a correct MLMC estimate."""
    cfg = _cfg()
    cfg.n_streams = 0
    cfg.epsilon = 0.01
    ev = mlmc_ranks.engine_level_evaluator(engine, _job(), cfg)
    res = mlmc_ranks.mlmc_price(mlmc_ranks.rank_evaluator(ev, 0, 1, mlmc_ranks.streams_of(cfg)), cfg, 1.0, 0.02)
    assert abs(res.price - FOURIER_C1) < 4 * res.price_std_err + cfg.epsilon
