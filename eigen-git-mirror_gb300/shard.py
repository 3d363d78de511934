"""Partition of independent SPD systems over ranks (one process per GPU) for the batched solver.

A batch of LLT solves (a loop of `LLT<MatrixXd> llt(A_s); x_s = llt.solve(b_s);`,
Eigen/src/Cholesky/LLT.h:430-498, over independent systems) has no data exchange between systems,
so a multi-GPU run shards the systems and never communicates on the data path: each rank builds a
plan (gbllt_batch_plan_create) for its own systems and solves them with one graph-replayed launch.
The host needs only a barrier for timing and, if it wants the results in one place, a gather.

The split is longest-processing-time first: systems sorted by cost (n^3/3 + 2 n^2 flops, the
factor-plus-solve work) in decreasing order, each assigned to the currently least-loaded rank
(ties to the lowest rank), a 4/3-approximation of the best makespan (Graham 1969).  It is
deterministic, so every rank computes the same partition without communicating.
"""
from __future__ import annotations

import numpy as np


def system_cost(n: np.ndarray) -> np.ndarray:
    """Flops of one factor + solve of order n (n^3/3 + 2 n^2)."""
    n = np.asarray(n, dtype=np.float64)
    return n ** 3 / 3.0 + 2.0 * n * n


def partition(sizes, world_size: int) -> list[np.ndarray]:
    """Indices of the systems of each rank (each array ascending); every system in exactly one."""
    if world_size < 1:
        raise ValueError("world_size must be >= 1")
    sizes = np.asarray(sizes, dtype=np.int64)
    cost = system_cost(sizes)
    order = np.argsort(-cost, kind="stable")
    load = np.zeros(world_size)
    owner = np.empty(len(sizes), dtype=np.int64)
    for i in order:
        r = int(np.argmin(load))  # first minimum: the lowest rank among the least loaded
        owner[i] = r
        load[r] += cost[i]
    return [np.flatnonzero(owner == r) for r in range(world_size)]


def loads(sizes, parts: list[np.ndarray]) -> np.ndarray:
    """Total cost per rank of a partition."""
    cost = system_cost(np.asarray(sizes))
    return np.array([cost[p].sum() for p in parts])


def pack(sizes, idx: np.ndarray, a_packed: np.ndarray, b_packed: np.ndarray):
    """The packed A / b arrays of the systems idx (in that order) cut from the packed arrays of the
    whole batch (A_s n_s x n_s column-major at sum_{t<s} n_t^2, b_s at sum_{t<s} n_t)."""
    sizes = np.asarray(sizes, dtype=np.int64)
    aoff = np.concatenate([[0], np.cumsum(sizes * sizes)])
    boff = np.concatenate([[0], np.cumsum(sizes)])
    a = np.concatenate([a_packed[aoff[i]:aoff[i + 1]] for i in idx]) if len(idx) else a_packed[:0].copy()
    b = np.concatenate([b_packed[boff[i]:boff[i + 1]] for i in idx]) if len(idx) else b_packed[:0].copy()
    return a, b


def unpack_into(sizes, idx: np.ndarray, a_part: np.ndarray, b_part: np.ndarray, a_packed: np.ndarray,
                b_packed: np.ndarray) -> None:
    """Writes a rank's results (packed in idx order) back to the batch-wide packed arrays."""
    sizes = np.asarray(sizes, dtype=np.int64)
    aoff = np.concatenate([[0], np.cumsum(sizes * sizes)])
    boff = np.concatenate([[0], np.cumsum(sizes)])
    pa = pb = 0
    for i in idx:
        na, nb = int(sizes[i] * sizes[i]), int(sizes[i])
        a_packed[aoff[i]:aoff[i] + na] = a_part[pa:pa + na]
        b_packed[boff[i]:boff[i] + nb] = b_part[pb:pb + nb]
        pa += na
        pb += nb
