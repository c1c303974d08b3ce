"""Multilevel Monte Carlo over several ranks, with one exchange per level batch.

The controller is Giles' adaptive loop as the reference runs it
(pricers/mlmc/MultiLevelMonteCarloPricer.hpp:64-211): pilot paths N0 / 2^l per
level, the optimal allocation N_l = ceil(2 eps^-2 sqrt(V_l / C_l) sum_k sqrt(V_k C_k)),
the three-level log regression of the weak and strong orders (capped at 2), and
the bias test max(|Y_L|, |Y_{L-1}| / 2) / (2^alpha - 1) <= eps / sqrt(2) that adds
levels.  Spread over W ranks it runs the same schedule everywhere:

  * every level batch of dN coupled paths is split over the ranks: rank r takes
    dN // W paths, plus one when r < dN % W;
  * each rank's share runs on its own block of S xoshiro streams, stream offset
    base + (batch * W + r) * S (batch = the controller's running batch count),
    so the blocks are disjoint across ranks and batches and every batch draws
    fresh random numbers;
  * after the batch, the ranks all-reduce the level's FP64 sums (sum, sum of
    squares) -- the exchange step;
  * rank 0 alone decides the next batch size, the level count L and
    convergence from the pooled sums, and broadcasts them.

With W = 1 it is a single controller whose batches take fresh stream blocks.
`union_evaluator` runs the W ranks' shares of every batch inside one process,
in rank order: a W-rank run and that single-process run see the same sums.

The level evaluator is any callable (level, paths, stream_offset) -> (sum, sum
of squares) of the undiscounted level differences P_l - P_{l-1} (P_0 at level
0): `engine_level_evaluator` runs myql_mlmc_level on the GPU,
`oracle_level_evaluator` the CPU restatement (tests).
"""
from __future__ import annotations

import ctypes as C
import math
from typing import Callable

import numpy as np

from . import _abi

Evaluator = Callable[[int, int, int], "tuple[float, float]"]
DEFAULT_STREAMS = 131072  # streams per level evaluation when the configuration names none


class Exchange:
    """The collectives of the controller over a torch.distributed group (identity when the
    process group is not initialised, i.e. one rank)."""

    def __init__(self, group=None):
        self.group = group
        self.dist = None
        self.rank, self.world, self.device = 0, 1, "cpu"
        try:
            import torch.distributed as dist
            if dist.is_available() and dist.is_initialized():
                self.dist = dist
                self.rank = dist.get_rank(group)
                self.world = dist.get_world_size(group)
                self.device = "cuda" if dist.get_backend(group) == "nccl" else "cpu"
                self.src = dist.get_global_rank(group, 0) if group is not None else 0
        except ImportError:
            pass

    def sum(self, vals: list[float]) -> list[float]:
        if not self.dist:
            return list(vals)
        import torch
        t = torch.tensor(vals, dtype=torch.float64, device=self.device)
        self.dist.all_reduce(t, op=self.dist.ReduceOp.SUM, group=self.group)
        return t.cpu().tolist()

    def bcast(self, vals: list[int]) -> list[int]:
        if not self.dist:
            return list(vals)
        import torch
        t = torch.tensor(vals, dtype=torch.int64, device=self.device)
        self.dist.broadcast(t, src=self.src, group=self.group)
        return [int(x) for x in t.cpu().tolist()]


def share(dN: int, rank: int, world: int) -> int:
    """Paths of a dN-path batch that rank `rank` of `world` evaluates."""
    return dN // world + (1 if rank < dN % world else 0)


def stream_offset(base: int, batch: int, rank: int, world: int, streams: int) -> int:
    """First stream of rank `rank`'s share of batch `batch`: disjoint blocks of `streams`."""
    return base + (batch * world + rank) * streams


def union_evaluator(evaluate: Evaluator, world: int, streams: int, base: int = 0):
    """The W ranks' shares of each batch evaluated in one process, summed in rank order: the
    controller run with this evaluator on one rank sees the sums of a W-rank run."""
    def ev(level: int, dN: int, batch: int) -> tuple[float, float]:
        a = b = 0.0
        for r in range(world):
            n = share(dN, r, world)
            if n:
                x, y = evaluate(level, n, stream_offset(base, batch, r, world, streams))
                a += x
                b += y
        return a, b
    return ev


def rank_evaluator(evaluate: Evaluator, rank: int, world: int, streams: int, base: int = 0):
    """This rank's share of each batch (0 paths -> zero sums)."""
    def ev(level: int, dN: int, batch: int) -> tuple[float, float]:
        n = share(dN, rank, world)
        if n == 0:
            return 0.0, 0.0
        return evaluate(level, n, stream_offset(base, batch, rank, world, streams))
    return ev


def _order(values: list[float], L: int) -> float:
    """Decay rate of values[L-2..L] from a log-linear fit (MultiLevelMonteCarloPricer.hpp:140-165);
    -1 when fewer than two values are usable."""
    xs, ys = [], []
    for l in range(L - 2, L + 1):
        if values[l] > 1e-16:
            xs.append(float(l - (L - 2)))
            ys.append(math.log(values[l]))
    n = len(xs)
    if n < 2:
        return -1.0
    sx, sy = sum(xs), sum(ys)
    sxy = sum(x * y for x, y in zip(xs, ys))
    sxx = sum(x * x for x in xs)
    slope = (n * sxy - sx * sy) / (n * sxx - sx * sx)
    return -slope / math.log(2.0)


def mlmc_price(evaluate_batch, cfg: "_abi.MlmcConfigC", maturity: float, rate: float,
               exchange: Exchange | None = None) -> "_abi.MlmcResultC":
    """Giles' controller over the ranks of `exchange`.  evaluate_batch(level, dN, batch) returns
    THIS rank's undiscounted (sum, sum of squares) of its share of a dN-path batch (see
    rank_evaluator); the sums are all-reduced after every batch.  Returns the pooled result on
    every rank (price and standard error discounted by exp(-rate * maturity))."""
    ex = exchange or Exchange()
    L_max = int(cfg.L_max)
    if not (cfg.epsilon > 0.0) or int(cfg.L_min) > L_max or L_max + 1 > _abi.MLMC_MAX_LEVELS:
        raise ValueError("MLMC needs epsilon > 0 and L_min <= L_max < the level limit")
    base_steps = int(cfg.base_steps)
    df = math.exp(-rate * maturity)
    L = int(cfg.L_min)
    N = [0] * (L_max + 1)
    s1 = [0.0] * (L_max + 1)
    s2 = [0.0] * (L_max + 1)
    V = [0.0] * (L_max + 1)
    cost = [float(base_steps << l) for l in range(L_max + 1)]
    alpha, beta = float(cfg.alpha), float(cfg.beta)
    eps_m2 = float(cfg.epsilon) ** -2.0
    batch = 0
    for _ in range(10000):
        for l in range(L + 1):
            dN = 0
            if ex.rank == 0:
                pilot_sum = sum(math.sqrt(V[k] * cost[k]) for k in range(L + 1))
                opt = math.ceil(2.0 * eps_m2 * math.sqrt(V[l] / cost[l]) * pilot_sum) if V[l] > 1e-18 else 0
                target = max(max(20, int(cfg.N0) >> l), opt)
                dN = target - N[l] if N[l] < target else 0
            dN = ex.bcast([dN])[0]
            if dN == 0:
                continue
            a, b = evaluate_batch(l, dN, batch)
            a, b = ex.sum([a, b])  # the exchange: pooled level sums
            batch += 1
            s1[l] += a
            s2[l] += b
            N[l] += dN
            if N[l] > 1:
                mean = s1[l] / N[l]
                V[l] = max(1e-18, s2[l] / N[l] - mean * mean)
        if cfg.adaptive_rates and L >= 2:
            ea = _order([abs(s1[l] / N[l]) for l in range(L + 1)], L)
            eb = _order(V[:L + 1], L)
            if ea > 0.3:
                alpha = min(2.0, ea)
            if eb > 0.3:
                beta = min(2.0, eb)
        decision = [L, 0]
        if ex.rank == 0:
            sum_vc = sum(math.sqrt(V[l] * cost[l]) for l in range(L + 1))
            more = any(math.ceil(2.0 * eps_m2 * math.sqrt(V[l] / cost[l]) * sum_vc) > N[l] for l in range(L + 1))
            if not more:
                eff = abs(s1[L] / N[L])
                if L > 0:
                    eff = max(eff, 0.5 * abs(s1[L - 1] / N[L - 1]))
                if eff / (2.0 ** alpha - 1.0) > float(cfg.epsilon) / math.sqrt(2.0) and L < L_max:
                    decision = [L + 1, 0]
                else:
                    decision = [L, 1]
        L, done = ex.bcast(decision)
        if done:
            break
    else:
        raise RuntimeError("MLMC controller did not converge")
    res = _abi.MlmcResultC()
    res.alpha_estimated, res.beta_estimated = alpha, beta
    res.n_levels = L + 1
    var = 0.0
    for l in range(L + 1):
        res.paths_per_level[l] = N[l]
        res.total_steps += N[l] * (base_steps if l == 0 else base_steps * (1 << l) * 3 // 2)
        mean = s1[l] / N[l]
        res.mean_diffs[l] = mean * df
        res.var_diffs[l] = V[l] * df * df
        res.price += mean * df
        var += V[l] / N[l]
    res.price_std_err = math.sqrt(var) * df
    return res


def _with_offset(job, offset: int):
    c = _abi.McJobC()
    C.memmove(C.addressof(c), C.addressof(job.c), C.sizeof(c))
    c.config.stream_offset = offset
    return c


def engine_level_evaluator(engine, job, cfg: "_abi.MlmcConfigC") -> Evaluator:
    """myql_mlmc_level on the GPU: (level, paths, stream offset) -> undiscounted (sum, sum sq)."""
    def ev(level: int, n: int, offset: int) -> tuple[float, float]:
        c = _with_offset(job, offset)
        out = np.zeros(4)
        _abi.check(engine.lib.myql_mlmc_level(engine.handle, C.byref(c), C.byref(cfg), level, n,
                                              out.ctypes.data_as(C.POINTER(C.c_double))))
        return float(out[0]), float(out[1])
    return ev


def oracle_level_evaluator(oracle_mod, job, cfg: "_abi.MlmcConfigC", n_threads: int = 1) -> Evaluator:
    """The CPU restatement's evaluate_level (streams layout); test infrastructure."""
    from . import pricers as _p

    def ev(level: int, n: int, offset: int) -> tuple[float, float]:
        j = _p._Job(_with_offset(job, offset), job.strikes)
        s = oracle_mod.mlmc_level(j, cfg, level, n, oracle_mod.LAYOUT_STREAMS, n_threads)
        return float(s[0]), float(s[1])
    return ev


def streams_of(cfg: "_abi.MlmcConfigC") -> int:
    return int(cfg.n_streams) or DEFAULT_STREAMS
