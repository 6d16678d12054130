"""The personalized-PageRank oracle (oracle/ppr.py) pinned to the reference's PageRank.

The reference has no PPR.  On a graph without dangling vertices every instance keeps all its
mass on the edges (S = 1), so the mean of PPR over all V seeds is exactly the reference's
PageRank (teleport (1-d)/V to every vertex).  The reference's own 16-iteration output for such
a golden graph (star_chain1001, rank = prop * deg') pins the oracle; with dangling vertices the
two differ by the dangling term, which PPR sends to the seed.
"""
import numpy as np
import pytest

from conftest import load_golden
from oracle import oracle as O
from oracle import ppr as P


def test_mean_of_ppr_is_reference_pagerank():
    rec, g = load_golden("star_chain1001")
    V = g.num_vertices
    pull = g.pull_order().pairs()
    L = O.layout(V, pull, g.push_order().pairs())
    assert (L.outdeg > 0).all()
    ref_rank = rec["pr_n1"][:V] * L.outdeg  # the reference's props after 16 iterations, d = 0.875
    mean = P.pagerank_mean_of_ppr(V, pull, 16, 0.875)
    assert np.abs(mean - ref_rank).sum() / np.abs(ref_rank).sum() < 1e-12
    for iters in (1, 5):
        pr = O.pr_pull(L, iters, 0.875)[:V] * L.outdeg
        mean = P.pagerank_mean_of_ppr(V, pull, iters, 0.875)
        assert np.abs(mean - pr).sum() / np.abs(pr).sum() < 1e-12


def test_dangling_mass_goes_to_the_seed():
    """With dangling vertices the PPR mass a dangling vertex holds returns to the seed: ranks
    still sum to 1, and the mean over seeds differs from PageRank only by that redistribution."""
    rec, g = load_golden("tiny13")
    V = g.num_vertices
    pull = g.pull_order().pairs()
    for s in range(V):
        r = P.ppr(V, pull, s, 7, 0.875)
        assert abs(r.sum() - 1.0) < 1e-13


def test_ppr_properties():
    from grazelle import graphgen as gg
    g = gg.rmat(9, seed=3)
    pull = g.pull_order().pairs()
    V = g.num_vertices
    r = P.ppr(V, pull, 5, 20, 0.85)
    assert abs(r.sum() - 1.0) < 1e-12
    assert (r >= 0).all()
    # the column of the dense formulation equals the sparse one
    mean = P.pagerank_mean_of_ppr(V, pull, 3, 0.85)
    cols = np.mean([P.ppr(V, pull, s, 3, 0.85) for s in range(V)], axis=0)
    assert np.abs(mean - cols).max() < 1e-14


def test_multi_seed_ppr_matches_the_serial_oracle():
    """The C multi-seed PPR (the bench's check of all 32 batch graphs) equals oracle/ppr.py seed
    by seed within 1e-13 relative L1 (only the order of the S sum differs); a seed >= V leaves
    its column zero."""
    from grazelle import graphgen as gg
    for g in (gg.rmat(11, seed=5), gg.erdos_renyi(1500, 6, seed=2)):
        V, pull = g.num_vertices, g.pull_order().pairs()
        seeds = [0, 7, V - 1, 0xffffffff, 123]
        R = O.ppr_multi(V, pull, seeds, 20, 0.85, threads=4)
        for k, s in enumerate(seeds):
            if s >= V:
                assert not R[:, k].any()
                continue
            ref = P.ppr(V, pull, s, 20, 0.85)
            assert O.relative_l1(R[:, k], ref) < 1e-13


def test_multi_root_bfs_levels_match_single_root():
    from grazelle import graphgen as gg
    g = gg.rmat(12, seed=9)
    V, push = g.num_vertices, g.push_order().pairs()
    roots = [0, 3, 77, V - 1]
    L = O.bfs_levels_multi(push, V, roots, threads=3)
    for k, r in enumerate(roots):
        np.testing.assert_array_equal(L[k], O.bfs_levels(push, V, r))
