"""Serial FP64 personalized PageRank: the oracle of the batched PPR kernels.

TEST INFRASTRUCTURE ONLY (imported by tests/ and bench.py's CPU legs).

The reference has no personalized PageRank.  This is its PageRank iteration
(edge pull, source/phase_edge_pull_pr.asm:45-171; vertex phase,
source/phase_vertex_pr.asm:75-134) with the teleport term and the dangling mass sent
to the seed instead of spread over all vertices:

    prop[u]  = rank[u] / deg'(u)           deg' = outdegree, or V when 0 (phase_vertex_pr.asm:75-134)
    accum[v] = sum over in-edges (u, v) of prop[u]
    S        = sum over v of accum[v]
    rank'[v] = d * accum[v] + [v == seed] * (d * (1 - S) + (1 - d))

from rank = one-hot(seed).  Averaged over all V seeds it is the reference's PageRank
exactly (linearity): the CPU test pins this oracle to the reference through that
identity, since the reference pins nothing about PPR itself.
"""
from __future__ import annotations

import numpy as np


def ppr(V: int, pull_pairs: np.ndarray, seed: int, iterations: int, damping: float) -> np.ndarray:
    """Ranks after `iterations` iterations (float64[V])."""
    p = np.asarray(pull_pairs, dtype=np.int64).reshape(-1, 2)
    src, dst = p[:, 0], p[:, 1]
    outdeg = np.bincount(src, minlength=V).astype(np.float64)
    degp = np.where(outdeg == 0, float(V), outdeg)
    rank = np.zeros(V)
    rank[seed] = 1.0
    for _ in range(iterations):
        prop = rank / degp
        acc = np.bincount(dst, weights=prop[src], minlength=V)
        S = acc.sum()
        rank = damping * acc
        rank[seed] += damping * (1.0 - S) + (1.0 - damping)
    return rank


def pagerank_mean_of_ppr(V: int, pull_pairs: np.ndarray, iterations: int, damping: float) -> np.ndarray:
    """Mean over all V seeds of ppr(): equals the reference's PageRank ranks."""
    p = np.asarray(pull_pairs, dtype=np.int64).reshape(-1, 2)
    src, dst = p[:, 0], p[:, 1]
    outdeg = np.bincount(src, minlength=V).astype(np.float64)
    degp = np.where(outdeg == 0, float(V), outdeg)
    R = np.eye(V)  # column s = instance with seed s
    for _ in range(iterations):
        P = R / degp[:, None]
        A = np.zeros((V, V))
        np.add.at(A, dst, P[src])
        S = A.sum(axis=0)
        R = damping * A
        R[np.arange(V), np.arange(V)] += damping * (1.0 - S) + (1.0 - damping)
    return R.mean(axis=1)
