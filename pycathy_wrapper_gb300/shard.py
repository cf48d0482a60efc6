"""Ensemble sharding across GPUs (one process per GPU).

The members of a data-assimilation ensemble are independent forward runs
(pyCATHY runs them through a process pool, DA/cathy_DA.py:1389, one
``./cathy`` per member).  Across several GPUs the ensemble is split into one
shard per rank with no collective on the data path: each rank runs its own
members as one batched solve.  Members differ in size (30..80-cell DEMs,
10..20 layers), so the split balances the matrix slots (nnz), which set the
cost of every kernel of the batched Picard iteration: greedy
longest-processing-time assignment (largest member first, to the rank with
the least nnz so far; ties to the lower rank).  The result is deterministic
and the same on every rank, so no rank has to send its shard to another.
"""
from __future__ import annotations

from typing import List, Sequence

import numpy as np


def member_nnz(cases) -> List[int]:
    """Matrix slots of each member's full CSR pattern (host-side mesh
    construction, no device needed)."""
    from .api import build_mesh
    return [int(len(build_mesh(c)["cols"])) for c in cases]


def member_nodes(cases) -> List[int]:
    """Nodes of each member's 3-D mesh, from its DEM alone: the vertices of
    the active cells (TRIANGOLI keeps the cells whose elevation is not 0)
    times NSTR+1 layers.  Proportional to nnz for these extruded meshes
    (about 14 slots per node) and cheap enough for thousands of members."""
    out = []
    for c in cases:
        act = np.asarray(c.dem.dem) != 0.0
        v = np.zeros((act.shape[0] + 1, act.shape[1] + 1), bool)
        v[:-1, :-1] |= act
        v[1:, :-1] |= act
        v[:-1, 1:] |= act
        v[1:, 1:] |= act
        out.append(int(v.sum()) * (c.dem.nstr + 1))
    return out


def shard_members(costs: Sequence[float], nranks: int) -> List[List[int]]:
    """Split members 0..len(costs)-1 into ``nranks`` shards, greedy by cost.

    Returns one ascending list of member indices per rank.  Every member is
    in exactly one shard, and the largest shard exceeds the smallest by at
    most the largest single cost."""
    if nranks < 1:
        raise ValueError("nranks must be >= 1")
    costs = np.asarray(costs, dtype=np.float64)
    order = sorted(range(len(costs)), key=lambda m: (-costs[m], m))
    load = np.zeros(nranks)
    shards: List[List[int]] = [[] for _ in range(nranks)]
    for m in order:
        r = int(np.argmin(load))  # first minimum: ties go to the lower rank
        shards[r].append(m)
        load[r] += costs[m]
    return [sorted(s) for s in shards]


def shard_of(costs: Sequence[float], rank: int, nranks: int) -> List[int]:
    """The members of ``rank``'s shard."""
    return shard_members(costs, nranks)[rank]
