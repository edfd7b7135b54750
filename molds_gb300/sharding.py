"""Assignment of independent molecules to ranks (one GPU each) by predicted cost.

A molecule's SCF costs about N^3 per iteration (the FP64 tridiagonalisation
and back-transformation dominate; the Fock build and DIIS grow as N^2), and
the iteration count is not known before the solve, so the prediction is
N^3 times a constant.  Molecules are placed longest first on the rank with
the smallest load so far (LPT scheduling: the most loaded rank ends within
4/3 of the optimum).  The result depends only on the list of basis sizes and
the rank count, so every rank computes the same assignment without
communication; there is no data-path collective.
"""
from __future__ import annotations

import numpy as np


def predicted_cost(n_ao) -> np.ndarray:
    """Relative cost of one SCF per molecule: N^3 (N = basis functions)."""
    n = np.asarray(n_ao, dtype=np.float64)
    return n * n * n


def shard_by_cost(costs, world: int) -> list[list[int]]:
    """Molecule indices per rank: longest first onto the least-loaded rank
    (ties: the lower rank; equal costs keep input order)."""
    if world < 1:
        raise ValueError("world must be >= 1")
    costs = np.asarray(costs, dtype=np.float64)
    order = np.argsort(-costs, kind="stable")
    load = np.zeros(world)
    shards: list[list[int]] = [[] for _ in range(world)]
    for i in order:
        r = int(np.argmin(load))
        shards[r].append(int(i))
        load[r] += costs[i]
    return [sorted(s) for s in shards]


def shard_loads(costs, shards) -> np.ndarray:
    costs = np.asarray(costs, dtype=np.float64)
    return np.array([costs[s].sum() if len(s) else 0.0 for s in shards])
