"""Batched personalized PageRank and multi-source BFS (csrc/grz_batch.cu) against the CPU oracles.

Graphs of uneven size (R-MAT, Erdos-Renyi, a golden graph) are merged into one batch.  Every
PPR instance must match the serial FP64 oracle (oracle/ppr.py) within 1e-12 relative L1; every
BFS instance's levels must equal the reference-pinned oracle's levels exactly.
"""
import numpy as np
import pytest

from conftest import load_golden
from oracle import oracle as O
from oracle import ppr as P

pytestmark = pytest.mark.gpu

NONE = 0xFFFFFFFF


def batch_graphs():
    from grazelle import graphgen as gg
    gs = [gg.rmat(10, seed=1), gg.rmat(12, seed=2, symmetric=True), gg.erdos_renyi(1 << 11, 4, seed=3),
          gg.rmat(14, seed=4), load_golden("star_chain1001")[1], gg.erdos_renyi(300, 16, seed=5)]
    return gs


def pick(g, n, seed):
    deg = g.out_degrees()
    cand = np.nonzero(deg)[0]
    rng = np.random.default_rng(seed)
    return [int(x) for x in rng.choice(cand, size=min(n, cand.shape[0]), replace=False)]


@pytest.fixture(scope="module")
def batch():
    from grazelle.batch import Batch
    gs = batch_graphs()
    B = Batch(0)
    for g in gs:
        B.add_graph(g.num_vertices, g.pull_order().pairs())
    B.build()
    yield B, gs
    B.close()


def test_info(batch):
    B, gs = batch
    info = B.info()
    assert info["graphs"] == len(gs)
    assert info["vertices"] == sum(g.num_vertices for g in gs)
    assert info["edges"] == sum(g.num_edges for g in gs)


@pytest.mark.parametrize("k", [8, 3])
def test_ppr_matches_oracle(batch, k):
    B, gs = batch
    seeds = [pick(g, k, 10 + i) for i, g in enumerate(gs)]
    seeds[1] = seeds[1][:2]  # uneven instance counts
    ranks, st = B.ppr(seeds, iterations=20, damping=0.85)
    assert st.iterations == 20
    for g, gr, sd in zip(gs, ranks, seeds):
        pull = g.pull_order().pairs()
        for i in range(gr.shape[1]):
            if i >= len(sd):
                assert not gr[:, i].any()
                continue
            ref = P.ppr(g.num_vertices, pull, sd[i], 20, 0.85)
            err = np.abs(gr[:, i] - ref).sum() / np.abs(ref).sum()
            assert err < 1e-12, err
            assert abs(gr[:, i].sum() - 1.0) < 1e-12


def test_ppr_replay_and_iteration_change(batch):
    B, gs = batch
    seeds = [pick(g, 8, 20 + i) for i, g in enumerate(gs)]
    a, _ = B.ppr(seeds, iterations=7, damping=0.85)
    b, _ = B.ppr(seeds, iterations=7, damping=0.85)
    c, _ = B.ppr(seeds, iterations=3, damping=0.5)
    for x, y in zip(a, b):
        np.testing.assert_array_equal(x, y)
    g = gs[0]
    ref = P.ppr(g.num_vertices, g.pull_order().pairs(), seeds[0][1], 3, 0.5)
    assert np.abs(c[0][:, 1] - ref).sum() / np.abs(ref).sum() < 1e-12


def test_ppr_gathered_prop_forms_agree(batch):
    """The gather reads 16-byte fixed-point props or the doubles they convert from exactly: the
    ranks are the same bit for bit, and the tuning switches between them on the next run."""
    B, gs = batch
    seeds = [pick(g, 8, 30 + i) for i, g in enumerate(gs)]
    runs = {}
    for props in (1, 2, 1, 0):
        B.tune(ppr_props=props)
        assert B.tuning()["ppr_props"] == props
        runs.setdefault(props, []).append(B.ppr(seeds, iterations=9, damping=0.85)[0])
    for x, y, z in zip(runs[1][0], runs[2][0], runs[1][1]):
        np.testing.assert_array_equal(x, y)
        np.testing.assert_array_equal(x, z)
    for x, y in zip(runs[1][0], runs[0][0]):
        np.testing.assert_array_equal(x, y)
    g = gs[3]
    ref = P.ppr(g.num_vertices, g.pull_order().pairs(), seeds[3][0], 9, 0.85)
    assert np.abs(runs[2][0][3][:, 0] - ref).sum() / np.abs(ref).sum() < 1e-12
    with pytest.raises(Exception):
        B.tune(ppr_props=3)


@pytest.mark.parametrize("k", [8, 5])
def test_msbfs_levels_match_oracle(batch, k):
    B, gs = batch
    roots = [pick(g, k, 30 + i) for i, g in enumerate(gs)]
    roots[2] = roots[2][:1]
    levels, st = B.msbfs(roots)
    for g, lv, rt in zip(gs, levels, roots):
        push = g.push_order().pairs()
        for i in range(lv.shape[1]):
            if i >= len(rt):
                assert (lv[:, i] == -1).all()
                continue
            ref = O.bfs_levels(push, g.num_vertices, rt[i])
            np.testing.assert_array_equal(lv[:, i].astype(np.int64), ref)
    depth = max(int(l.max()) for l in levels)
    assert st.iterations == depth + 1


def test_shared_roots_and_repeat(batch):
    B, gs = batch
    roots = [[0, 0, 1, 1] for _ in gs]  # instances may share a root
    a, _ = B.msbfs(roots)
    b, _ = B.msbfs(roots)
    for g, x, y in zip(gs, a, b):
        np.testing.assert_array_equal(x, y)
        np.testing.assert_array_equal(x[:, 0], x[:, 1])
        np.testing.assert_array_equal(x[:, 0].astype(np.int64), O.bfs_levels(g.push_order().pairs(), g.num_vertices, 0))


def test_bad_inputs():
    from grazelle import graphgen as gg, native
    from grazelle.batch import Batch
    g = gg.rmat(8, seed=1)
    with Batch(0) as B:
        with pytest.raises(native.GrzError):
            B.add_graph(16, np.array([0, 1, 1, 2], dtype=np.uint64))  # fewer than 32 vertices
        bad = g.pull_order().pairs().copy().reshape(-1, 2)[::-1].reshape(-1)
        with pytest.raises(native.GrzError):
            B.add_graph(g.num_vertices, bad)  # not (dst, src) sorted
        B.add_graph(g.num_vertices, g.pull_order().pairs()).build()
        with pytest.raises(native.GrzError):
            B.ppr([[g.num_vertices + 5]])  # seed outside its graph


@pytest.mark.parametrize("props", [0, 2])
def test_ppr_and_bfs_in_one_launch_match_the_separate_runs(batch, props):
    """grz_batch_run: PPR and multi-source BFS as two branches of one CUDA graph launch give
    exactly the results of the separate calls (the same kernels), with different seeds and roots
    and uneven instance counts, twice in a row (the graph is replayed from its initial state)."""
    B, gs = batch
    B.tune(ppr_props=props)
    seeds = [pick(g, 8, 40 + i) for i, g in enumerate(gs)]
    roots = [pick(g, 5, 80 + i) for i, g in enumerate(gs)]
    seeds[2] = seeds[2][:3]
    r_sep, _ = B.ppr(seeds, iterations=12, damping=0.85)
    l_sep, st_b = B.msbfs(roots)
    for _ in range(2):
        ranks, levels, sp, sb, tot = B.run(seeds, roots, iterations=12, damping=0.85)
        for a, b in zip(ranks, r_sep):
            np.testing.assert_array_equal(a, b)
        for a, b in zip(levels, l_sep):
            np.testing.assert_array_equal(a, b)
        assert sp.iterations == 12 and sb.iterations == st_b.iterations
        assert 0 < sp.ms <= tot * 1.01 and 0 < sb.ms <= tot * 1.01
    for g, lv, rt in zip(gs, levels, roots):
        for i, r in enumerate(rt):
            np.testing.assert_array_equal(lv[:, i].astype(np.int64), O.bfs_levels(g.push_order().pairs(), g.num_vertices, r))
    B.tune(ppr_props=0)
