"""The autotuner (grazelle/autotune.py) picks kernel shapes by timing them; results never
depend on the shape it picks."""
import numpy as np
import pytest

from conftest import load_golden
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def test_tune_cc_and_pr_keep_results():
    from grazelle import autotune, graphgen as gg
    from grazelle.engine import Graph
    g = gg.rmat(16, seed=9, symmetric=True)
    with Graph(0) as G:
        G.load_pairs(g.num_vertices, g.pull_order().pairs(), g.push_order().pairs())
        lab0 = G.connected_components()
        pr0 = G.pagerank(5)
        rep = autotune.tune_cc(G, trials=2, threads=(256, 512), grids_per_sm=(0, 1), forms=(4, 1, 0))
        assert rep["candidates"] == 10 and rep["default_ms"] is not None
        assert rep["best_ms"] <= rep["default_ms"]
        t = G.tuning()
        assert all(t[k] == v for k, v in rep["best"].items())
        rep2 = autotune.tune_pr(G, trials=2, grids_per_sm=(0, 2))
        assert rep2["candidates"] == 4 and rep2["best_ms"] <= rep2["default_ms"]
        t = G.tuning()
        assert all(t[k] == v for k, v in rep2["best"].items())
        np.testing.assert_array_equal(G.connected_components(), lab0)
        np.testing.assert_array_equal(G.pagerank(5), pr0)


def test_tune_batch_keeps_results():
    from grazelle import autotune, graphgen as gg
    from grazelle.batch import Batch
    gs = [gg.rmat(11, seed=1), gg.erdos_renyi(1 << 10, 8, seed=2)]
    seeds = [[1, 2, 3], [4, 5]]
    with Batch(0) as B:
        for g in gs:
            B.add_graph(g.num_vertices, g.pull_order().pairs())
        B.build()
        r0, _ = B.ppr(seeds, 6, 0.85)
        l0, _ = B.msbfs(seeds)
        rep = autotune.tune_batch(B, seeds, iterations=3, trials=1, blocks=(2, 8))
        assert B.tuning() == {"ppr_blocks": rep["ppr_blocks"]["best"], "bfs_blocks": rep["bfs_blocks"]["best"], "ppr_props": 0}
        r1, _ = B.ppr(seeds, 6, 0.85)
        l1, _ = B.msbfs(seeds)
        for a, b in zip(r0, r1):
            np.testing.assert_array_equal(a, b)  # exact sums: bit-identical under any grid
        for a, b, g, s in zip(l0, l1, gs, seeds):
            np.testing.assert_array_equal(a, b)
            for i, r in enumerate(s):
                np.testing.assert_array_equal(a[:, i].astype(np.int64), O.bfs_levels(g.push_order().pairs(), g.num_vertices, r))


def test_bad_tuning_values():
    from grazelle import native
    from grazelle.batch import Batch
    from grazelle.engine import Graph
    with Graph(0) as G:
        with pytest.raises(native.GrzError):
            G.tune(cc_threads=300)
        with pytest.raises(native.GrzError):
            G.tune(hubs=1 << 20)
    with Batch(0) as B:
        with pytest.raises(native.GrzError):
            B.tune(ppr_blocks=0)
