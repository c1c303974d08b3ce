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


def pool_estimates(prices, std_errs) -> tuple[float, float]:
    """Inverse-variance pooling of independent unbiased estimates (for example one MLMC run per
    replica on disjoint stream ranges): sum(p_i / se_i^2) / sum(1 / se_i^2), with standard error
    1 / sqrt(sum(1 / se_i^2)).  An estimate with zero standard error is exact and returned as is."""
    p = np.asarray(prices, dtype=np.float64)
    se = np.asarray(std_errs, dtype=np.float64)
    if p.shape != se.shape or p.size == 0:
        raise ValueError("one standard error per estimate, at least one estimate")
    if np.any(se < 0.0) or not np.all(np.isfinite(se)) or not np.all(np.isfinite(p)):
        raise ValueError("finite estimates and non-negative standard errors")
    exact = se == 0.0
    if exact.any():
        return float(p[exact][0]), 0.0
    w = 1.0 / (se * se)
    return float(np.sum(w * p) / np.sum(w)), float(1.0 / np.sqrt(np.sum(w)))


def allreduce_estimate(price: float, std_err: float, group=None) -> tuple[float, float]:
    """pool_estimates over every rank's (price, standard error) through torch.distributed."""
    import torch
    import torch.distributed as dist
    world = dist.get_world_size(group)
    mine = torch.tensor([price, std_err], dtype=torch.float64)
    if dist.get_backend(group) == "nccl":
        mine = mine.cuda()
    allv = [torch.zeros_like(mine) for _ in range(world)]
    dist.all_gather(allv, mine, group=group)
    allv = torch.stack(allv).cpu().numpy()
    return pool_estimates(allv[:, 0], allv[:, 1])


assert _abi.Q_COUNT == 10
