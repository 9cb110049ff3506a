"""Shots and independent problems across GPUs: one process per GPU, a static
share of the work units each, and one sum of the gradient fields at the end.

The reference runs the shots of a gradient one after another in the same
buffers and adds each shot's kernel into one accumulator (solver.rs:1386-1498);
shots of one problem and independent problems share nothing during their
forward and reverse sweeps.  So the units are split without any exchange on
the data path, and the only collective is the final sum of the per-rank
gradient fields.  That sum is taken in rank order (all-gather, then a
left-to-right sum in FP64), so every rank holds the same bits whatever the
collective's internal reduction order.
"""
from __future__ import annotations

from typing import Dict, List, Sequence

import numpy as np


def assign(costs: Sequence[float], world: int) -> List[List[int]]:
    """Longest-processing-time assignment of units (cost e.g. cells x nt) to
    `world` ranks: units in decreasing cost (ties: lower index first), each to
    the rank with the smallest load so far (ties: lower rank).  Deterministic;
    each rank's list is in increasing unit index."""
    if world < 1:
        raise ValueError("world must be >= 1")
    order = sorted(range(len(costs)), key=lambda u: (-float(costs[u]), u))
    loads = [0.0] * world
    out: List[List[int]] = [[] for _ in range(world)]
    for u in order:
        r = min(range(world), key=lambda q: (loads[q], q))
        loads[r] += float(costs[u])
        out[r].append(u)
    for lst in out:
        lst.sort()
    return out


def my_units(costs: Sequence[float], rank: int, world: int) -> List[int]:
    """The units of one rank under `assign`."""
    if not 0 <= rank < world:
        raise ValueError("rank out of range")
    return assign(costs, world)[rank]


def imbalance(costs: Sequence[float], world: int) -> float:
    """Largest rank load over the mean load (1.0 = perfect balance)."""
    parts = assign(costs, world)
    loads = [sum(float(costs[u]) for u in p) for p in parts]
    mean = sum(loads) / world
    return max(loads) / mean if mean > 0 else 1.0


def reduce_gradients(fields: Dict[str, np.ndarray], group=None) -> Dict[str, np.ndarray]:
    """Sum each rank's gradient fields over all ranks, in rank order.

    `fields` maps a parameter name to this rank's partial sum (same names and
    shapes on every rank).  Uses torch.distributed (gloo on host tensors);
    returns FP32 arrays equal on every rank.  With one process (no process
    group) the fields are returned unchanged."""
    import torch
    import torch.distributed as dist

    if not (dist.is_available() and dist.is_initialized()):
        return {k: np.asarray(v, np.float32) for k, v in fields.items()}
    world = dist.get_world_size(group)
    out = {}
    for name in sorted(fields):
        local = torch.from_numpy(np.ascontiguousarray(fields[name], np.float32))
        parts = [torch.empty_like(local) for _ in range(world)]
        dist.all_gather(parts, local, group=group)
        acc = np.zeros(local.shape, np.float64)
        for p in parts:
            acc += p.numpy().astype(np.float64)
        out[name] = acc.astype(np.float32)
    return out
