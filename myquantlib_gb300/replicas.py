"""Replicas: one pricing request split over processes or GPUs.

Paths are independent, so a request of M paths runs as W replicas of M / W
paths on disjoint xoshiro stream ranges (replica r takes streams
[r S / W, (r + 1) S / W) of the request's S streams) and the results are pooled
from the FP64 moments (n * mean, n * E[x^2]) of each replica -- the reduction
the reference does with its OpenMP critical merge (MonteCarloPricer.hpp:413-440).
When M is a multiple of S every stream runs the same paths as in the single
request, so the pooled result equals the single request's up to FP64
summation order.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _abi
from . import pricers as _p


def default_streams(M: int) -> int:
    """The engine's stream count for a request of M paths when none is given."""
    return min(M, max(131072, min(524288, M // 8)))


def shard_job(job: "_p._Job", rank: int, world: int) -> "_p._Job":
    """The replica of `job` that rank `rank` of `world` prices: M / W paths on the
    stream range [r S / W, (r + 1) S / W) of the request's S streams."""
    M = int(job.c.config.num_paths)
    S = int(job.c.config.n_streams) or default_streams(M)
    if M % world or S % world:
        raise ValueError(f"num_paths {M} and the {S} streams must divide into {world} replicas")
    c = _abi.McJobC()                    # byte copy; the strikes array stays shared
    C.memmove(C.addressof(c), C.addressof(job.c), C.sizeof(c))
    c.config.num_paths = M // world
    c.config.n_streams = S // world
    c.config.stream_offset = int(job.c.config.stream_offset) + rank * (S // world)
    return _p._Job(c, job.strikes)


def moments(raw: np.ndarray, n_paths: int) -> np.ndarray:
    """(2Q, n) result rows of one replica -> FP64 moment sums [n mean; n E[x^2]] (discounted units)."""
    v, se = raw[0::2], raw[1::2]
    return np.concatenate([n_paths * v, n_paths * (se * se * n_paths + v * v)], axis=0)


def combine(mom: np.ndarray, n_total: int) -> np.ndarray:
    """Pooled moment sums -> (2Q, n) result rows (compute_stats, MonteCarloPricer.hpp:448-457)."""
    q = mom.shape[0] // 2
    mean = mom[:q] / n_total
    var = np.maximum(mom[q:] / n_total - mean * mean, 0.0)
    out = np.empty((2 * q, mom.shape[1]))
    out[0::2] = mean
    out[1::2] = np.sqrt(var / n_total)
    return out


def allreduce_price(raw: np.ndarray, n_local: int, group=None) -> np.ndarray:
    """Pools one replica's result with every rank's through torch.distributed (one FP64 sum)."""
    import torch
    import torch.distributed as dist
    world = dist.get_world_size(group)
    mom = torch.from_numpy(moments(np.asarray(raw, dtype=np.float64), n_local))
    if dist.get_backend(group) == "nccl":
        mom = mom.cuda()
    dist.all_reduce(mom, op=dist.ReduceOp.SUM, group=group)
    return combine(mom.cpu().numpy(), n_local * world)


def pool_estimates(prices, std_errs, weights=None) -> tuple[float, float]:
    """Pools independent unbiased estimates (for example one MLMC run per replica on disjoint
    stream ranges) with FIXED weights: the replicas' planned budgets (path counts or cost) when
    given, equal weights otherwise.  Fixed weights keep the pooled estimate unbiased.  Weights
    taken from each replica's own sample standard error would not: for option payoffs the
    sample standard error grows with the sample mean, so 1/se^2 weights favour the low
    estimates.  Pooled standard error: sqrt(sum w_i^2 se_i^2) / sum w_i.  A zero standard
    error is accepted only when every replica reports it with the same price (a
    deterministic payoff); otherwise it is an error, not an exact estimate."""
    p = np.asarray(prices, dtype=np.float64)
    se = np.asarray(std_errs, dtype=np.float64)
    if p.shape != se.shape or p.size == 0:
        raise ValueError("one standard error per estimate, at least one estimate")
    if np.any(se < 0.0) or not np.all(np.isfinite(se)) or not np.all(np.isfinite(p)):
        raise ValueError("finite estimates and non-negative standard errors")
    w = np.ones_like(p) if weights is None else np.asarray(weights, dtype=np.float64)
    if w.shape != p.shape or np.any(w <= 0.0) or not np.all(np.isfinite(w)):
        raise ValueError("one positive weight per estimate")
    if np.any(se == 0.0):
        if np.all(se == 0.0) and np.all(p == p[0]):
            return float(p[0]), 0.0
        raise ValueError("a replica reported a zero standard error that the others do not share")
    return float(np.sum(w * p) / np.sum(w)), float(np.sqrt(np.sum(w * w * se * se)) / np.sum(w))


def allreduce_estimate(price: float, std_err: float, weight: float = 1.0, group=None) -> tuple[float, float]:
    """pool_estimates over every rank's (price, standard error, planned budget) through
    torch.distributed (one all-gather).  For MLMC, mlmc_ranks runs one controller over all ranks
    instead; this pools runs that were planned independently."""
    import torch
    import torch.distributed as dist
    world = dist.get_world_size(group)
    mine = torch.tensor([price, std_err, weight], dtype=torch.float64)
    if dist.get_backend(group) == "nccl":
        mine = mine.cuda()
    allv = [torch.zeros_like(mine) for _ in range(world)]
    dist.all_gather(allv, mine, group=group)
    allv = torch.stack(allv).cpu().numpy()
    return pool_estimates(allv[:, 0], allv[:, 1], allv[:, 2])


assert _abi.Q_COUNT == 10
