"""Families sharded over ranks (one GPU each).

The likelihood of a vector of CCDs is a sum over independent families minus
N·condition (src/core.jl:58-64), so a model's families can be split across
processes: each rank evaluates its shard (conditioned by its own family
count) and one all-reduce of ``[Σ log L, ∇...]`` gives the whole.  The
reference parallelises the same sum over threads (src/core.jl:49-54).
"""
from __future__ import annotations

from typing import Callable, List, Optional, Sequence, Tuple

import numpy as np


def family_work(ccd) -> float:
    """Work estimate of one family (clades + split triples)."""
    return float(ccd.n_clades + ccd.n_triples)


def shard_families(weights: Sequence[float], world: int) -> List[List[int]]:
    """Greedy longest-processing-time split of families over ``world`` ranks:
    heaviest first onto the least-loaded rank (ties by rank).  Deterministic."""
    order = sorted(range(len(weights)), key=lambda i: (-weights[i], i))
    load = [0.0] * world
    shards: List[List[int]] = [[] for _ in range(world)]
    for i in order:
        r = min(range(world), key=lambda k: (load[k], k))
        shards[r].append(i)
        load[r] += weights[i]
    return [sorted(s) for s in shards]


def distributed_logpdf_gradient(wm, ccds: Sequence, group=None,
                                evaluate: Optional[Callable] = None) -> Tuple[float, np.ndarray]:
    """Σ log L - N·condition and its flat gradient ([λ; μ; q; η] as
    ``core.gradient``) over the families of all ranks of ``group``.  Every rank
    passes the full family list; each evaluates its shard with ``evaluate``
    (default: the GPU path) and the partial results are summed by one
    all-reduce."""
    import torch
    import torch.distributed as dist

    world = dist.get_world_size(group) if dist.is_initialized() else 1
    rank = dist.get_rank(group) if dist.is_initialized() else 0
    shard = shard_families([family_work(c) for c in ccds], world)[rank]
    if evaluate is None:
        from .core import logpdf_gradient
        from .model import ConstantDLWGD

        def evaluate(model, xs):
            tot, g = logpdf_gradient(model, xs)
            if isinstance(model.rates, ConstantDLWGD):
                return tot, np.concatenate([[g["λ"], g["μ"]], g["q"], [g["η"]]])
            return tot, np.concatenate([g["λ"], g["μ"], g["q"], [g["η"]]])

    mine = [ccds[i] for i in shard]
    if mine:
        tot, g = evaluate(wm, mine)
    else:
        tot, g = 0.0, None
    P = _n_params(wm)
    buf = np.zeros(1 + P)
    buf[0] = tot
    if g is not None:
        buf[1:] = g
    t = torch.from_numpy(buf)
    if dist.is_initialized() and world > 1:
        dist.all_reduce(t, op=dist.ReduceOp.SUM, group=group)
    out = t.numpy()
    total = float(out[0]) if np.isfinite(out[0]) else float("-inf")
    return total, out[1:].copy()


def _n_params(wm) -> int:
    r = wm.rates
    lam = np.atleast_1d(r.λ)
    return lam.size + np.atleast_1d(r.μ).size + r.q.size + 1
