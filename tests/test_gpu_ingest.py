"""Ingest: the -push list derived on the device from the -pull pairs (GRZ_LOAD_DERIVE_PUSH) must be
bit-identical to the one built from the -push pairs themselves, including duplicate edges and
self-loops; loads from pinned host memory, pageable host memory and device memory agree."""
import numpy as np
import pytest

from conftest import golden_names, load_golden

pytestmark = pytest.mark.gpu


def _lists(G):
    from grazelle import native
    return (G.list_vectors(native.LIST_PULL), G.list_vectors(native.LIST_PUSH), G.vertex_index(native.LIST_PUSH),
            G.outdegrees())


def _check_derived(V, pull, push, chunks=0):
    import torch
    from grazelle.engine import Graph
    with Graph(0) as A, Graph(0) as B:
        A.load_pairs(V, pull, push)
        B.tune(ingest_chunks=chunks)
        if chunks:   # chunks read in place from device memory
            dp = torch.from_numpy(pull.view(np.int64)).cuda()
            B.load_pull_derive_push(V, pull.shape[0] // 2, dp.data_ptr())
            for a, b in zip(_lists(A), _lists(B)):
                np.testing.assert_array_equal(a, b)
        hp = torch.from_numpy(pull.view(np.int64)).pin_memory()   # chunks copied through staging slots
        B.load_pull_derive_push(V, pull.shape[0] // 2, hp.data_ptr())
        for a, b in zip(_lists(A), _lists(B)):
            np.testing.assert_array_equal(a, b)
        np.testing.assert_array_equal(A.connected_components(), B.connected_components())
        pa, la = A.bfs(0)
        pb, lb = B.bfs(0)
        np.testing.assert_array_equal(pa, pb)
        np.testing.assert_array_equal(la, lb)


@pytest.mark.parametrize("name", golden_names())
def test_derived_push_list_equals_built(name):
    rec, g = load_golden(name)
    _check_derived(g.num_vertices, g.pull_order().pairs(), g.push_order().pairs())


@pytest.mark.parametrize("scale", [12, 17])
def test_derived_push_list_multigraph(scale):
    """Duplicate edges and self-loops kept, several sort passes (V > 2^16 at scale 17)."""
    from grazelle import graphgen as gg
    g = gg.rmat(scale, seed=scale)
    src = np.concatenate([g.src, g.src[:1000], np.arange(50, dtype=g.src.dtype)])
    dst = np.concatenate([g.dst, g.dst[:1000], np.arange(50, dtype=g.dst.dtype)])
    V = g.num_vertices
    o = np.lexsort((src, dst))
    pull = np.empty(2 * src.shape[0], dtype=np.uint64)
    pull[0::2], pull[1::2] = src[o], dst[o]
    o = np.lexsort((dst, src))
    push = np.empty_like(pull)
    push[0::2], push[1::2] = src[o], dst[o]
    _check_derived(V, pull, push)


def _pairs(src, dst):
    o = np.lexsort((src, dst))
    pull = np.empty(2 * len(o), dtype=np.uint64)
    pull[0::2], pull[1::2] = src[o], dst[o]
    o = np.lexsort((dst, src))
    push = np.empty(2 * len(o), dtype=np.uint64)
    push[0::2], push[1::2] = src[o], dst[o]
    return pull, push


@pytest.mark.parametrize("chunks", [2, 3, 7, 64])
def test_pull_only_ingest_in_chunks(chunks):
    """The ingest cuts the pairs into chunks that are sorted while later chunks cross the link;
    an edge's rank in its source's run adds up over chunks.  Hubs whose edges fall in every chunk,
    destinations whose runs cross chunk edges, duplicates and a last chunk shorter than the rest
    must give the lists of one sort."""
    from grazelle import graphgen as gg
    g = gg.rmat(14, seed=chunks)
    V = g.num_vertices
    rng = np.random.default_rng(chunks)
    hub_dst = rng.integers(0, V, size=3000).astype(np.uint64)          # source 7: edges everywhere
    long_src = rng.integers(0, V, size=5000).astype(np.uint64)         # destination 9: a run over chunks
    src = np.concatenate([g.src, np.full(3000, 7, dtype=np.uint64), long_src, g.src[:777]])
    dst = np.concatenate([g.dst, hub_dst, np.full(5000, 9, dtype=np.uint64), g.dst[:777]])
    pull, push = _pairs(src, dst)
    _check_derived(V, pull, push, chunks=chunks)


def test_chunked_ingest_input_errors_leave_the_graph_usable():
    """Unsorted pairs and out-of-range IDs are reported after the chunks were already being
    sorted; the graph loads the next valid list."""
    import torch
    from grazelle import graphgen as gg, native
    from grazelle.engine import Graph
    g = gg.rmat(13, seed=5)
    V = g.num_vertices
    pull, push = _pairs(g.src, g.dst)
    unsorted = pull.copy()
    unsorted[1::2][[10, len(unsorted) // 2 - 10]] = unsorted[1::2][[len(unsorted) // 2 - 10, 10]]
    out_of_range = pull.copy()
    out_of_range[2 * 1000] = V + 5
    with Graph(0) as A, Graph(0) as B:
        A.load_pairs(V, pull, push)
        B.tune(ingest_chunks=5)
        for bad, code in ((unsorted, -4), (out_of_range, -5)):
            hb = torch.from_numpy(bad.view(np.int64)).pin_memory()
            with pytest.raises(native.GrzError) as ei:
                B.load_pull_derive_push(V, len(bad) // 2, hb.data_ptr())
            assert ei.value.code == code
        hp = torch.from_numpy(pull.view(np.int64)).pin_memory()
        B.load_pull_derive_push(V, len(pull) // 2, hp.data_ptr())
        for a, b in zip(_lists(A), _lists(B)):
            np.testing.assert_array_equal(a, b)


def test_device_and_host_sources_agree():
    import torch
    from grazelle import graphgen as gg
    from grazelle.engine import Graph
    g = gg.rmat(15, seed=3, symmetric=True)
    V, E = g.num_vertices, g.num_edges
    pull, push = g.pull_order().pairs(), g.push_order().pairs()
    dp = torch.from_numpy(pull.view(np.int64)).cuda()
    dq = torch.from_numpy(push.view(np.int64)).cuda()
    with Graph(0) as A, Graph(0) as B, Graph(0) as C:
        A.load_pairs(V, pull, push)                               # pageable host
        B.load_device_pairs(V, E, dp.data_ptr(), dq.data_ptr())   # device
        C.load_pull_derive_push(V, E, dp.data_ptr())              # device, derived push
        for G in (B, C):
            for a, b in zip(_lists(A), _lists(G)):
                np.testing.assert_array_equal(a, b)
        for _ in range(2):                                        # reloads reuse pooled memory
            C.load_pull_derive_push(V, E, dp.data_ptr())
            np.testing.assert_array_equal(A.connected_components(), C.connected_components())


def test_derive_rejects_both_lists():
    from grazelle import graphgen as gg, native
    from grazelle.engine import Graph
    g = gg.rmat(8, seed=1)
    pull, push = g.pull_order().pairs(), g.push_order().pairs()
    with Graph(0) as G:
        rc = G.lib.grz_graph_load_pairs_ex(G.h, g.num_vertices, pull.shape[0] // 2, pull.ctypes.data, push.ctypes.data,
                                           native.LOAD_DERIVE_PUSH)
        assert rc == -1  # GRZ_ERR_ARG


def test_streamed_file_load(tmp_path):
    """`<base>-pull` / `<base>-push` streamed through the pinned staging buffers (several 64 MB
    chunks here) give the lists of an in-memory load; with derive_push only the -pull file is
    read."""
    import os
    from grazelle import graphgen as gg
    from grazelle.engine import Graph
    g = gg.rmat(19, seed=41)  # ~8M edges: 128 MB per file
    base = str(tmp_path / "g")
    gg.write_grazelle(g, base)
    with Graph(0) as A, Graph(0) as B, Graph(0) as C:
        A.load_pairs(g.num_vertices, g.pull_order().pairs(), g.push_order().pairs())
        B.load_files(base)
        os.rename(base + "-push", base + "-push.hidden")
        C.load_files(base, derive_push=True)
        la, lb, lc = _lists(A), _lists(B), _lists(C)
        for a, b, c in zip(la, lb, lc):
            np.testing.assert_array_equal(a, b)
            np.testing.assert_array_equal(a, c)
        np.testing.assert_array_equal(B.connected_components(), A.connected_components())


def test_file_load_errors(tmp_path):
    from grazelle import native
    from grazelle.engine import Graph
    base = str(tmp_path / "bad")
    np.array([10, 5, 1, 2], dtype=np.uint64).tofile(base + "-pull")  # header promises 5 edges
    with Graph(0) as G:
        with pytest.raises(native.GrzError):
            G.load_files(base)
        np.array([10, 1, 3, 2], dtype=np.uint64).tofile(base + "-pull")
        np.array([11, 1, 3, 2], dtype=np.uint64).tofile(base + "-push")  # V differs
        with pytest.raises(native.GrzError):
            G.load_files(base)
        np.array([10, 2, 3, 2, 1, 1], dtype=np.uint64).tofile(base + "-pull")  # not grouped by dst
        with pytest.raises(native.GrzError):
            G.load_files(base, derive_push=True)


def test_vector_model_and_iteration_stats():
    """MODEL_LONG_VECTORS: vectors at 4, 8 and 16 lanes are sums of ceil(run / lanes) over the
    shared vertices.  ITERATION_STATS: a pull iteration processes every pull vector and all E
    edges; a push iteration the frontier's out-vectors (the first CC push: all of them)."""
    from grazelle import graphgen as gg
    from grazelle import native
    g = gg.rmat(14, seed=51)
    pull, push = g.pull_order().pairs(), g.push_order().pairs()
    V, E = g.num_vertices, g.num_edges
    indeg = np.bincount(pull[1::2].astype(np.int64), minlength=V)
    outdeg = np.bincount(push[0::2].astype(np.int64), minlength=V)
    with _graph(V, pull, push) as G:
        info = G.info()
        assert G.vector_model(native.LIST_PULL, 4) == info.pull_vectors
        assert G.vector_model(native.LIST_PUSH, 4) == info.push_vectors
        for lanes in (8, 16):
            assert G.vector_model(native.LIST_PULL, lanes) == int(np.sum((indeg + lanes - 1) // lanes))
            assert G.vector_model(native.LIST_PUSH, lanes) == int(np.sum((outdeg + lanes - 1) // lanes))
        G.stats_enable(True)
        for app in (native.APP_CONNECTED_COMPONENTS, native.APP_BREADTH_FIRST_SEARCH):
            G.frontier_begin(app, 0, native.FORCE_PUSH if app == native.APP_CONNECTED_COMPONENTS else 0)
            first = True
            for _ in range(200):
                running, used, _ = G.frontier_next()
                v, e = G.stats_take()
                if used == 1:  # pull
                    if app == native.APP_CONNECTED_COMPONENTS:
                        assert (v, e) == (info.pull_vectors, E)
                    else:
                        assert v <= info.pull_vectors and v <= e <= 4 * v
                else:
                    if first and app == native.APP_CONNECTED_COMPONENTS:
                        assert (v, e) == (info.push_vectors, E)  # every vertex starts in the frontier
                    assert v <= info.push_vectors and v <= e <= 4 * v
                first = False
                if not running:
                    break
        G.stats_enable(False)


def _graph(V, pull, push):
    from grazelle.engine import Graph
    G = Graph(0)
    G.load_pairs(V, pull, push)
    return G


@pytest.mark.parametrize("V, edges", [
    (1, [(0, 0)]),                                   # one vertex, one self-loop
    (2, [(1, 0)]),                                   # one edge
    (3, [(2, 0), (2, 0), (0, 1), (1, 1), (2, 1)]),   # duplicates and a self-loop
    (200, "random"),                                 # one radix pass (V <= 256)
    (257, "random"),                                 # two passes
    (5000, "sparse"),                                # mostly isolated vertices
])
def test_pull_only_ingest_small_and_ragged(V, edges):
    import torch
    from grazelle.engine import Graph
    rng = np.random.default_rng(V)
    if edges == "random":
        e = rng.integers(0, V, size=(4 * V, 2))
    elif edges == "sparse":
        e = rng.integers(0, V, size=(40, 2))
    else:
        e = np.array(edges)
    src, dst = e[:, 0].astype(np.uint64), e[:, 1].astype(np.uint64)
    o = np.lexsort((src, dst))
    pull = np.empty(2 * len(o), dtype=np.uint64)
    pull[0::2], pull[1::2] = src[o], dst[o]
    o = np.lexsort((dst, src))
    push = np.empty(2 * len(o), dtype=np.uint64)
    push[0::2], push[1::2] = src[o], dst[o]
    with Graph(0) as A, Graph(0) as B:
        A.load_pairs(V, pull, push)
        hp = torch.from_numpy(pull.view(np.int64)).pin_memory()
        B.load_pull_derive_push(V, len(o), hp.data_ptr())
        for a, b in zip(_lists(A), _lists(B)):
            np.testing.assert_array_equal(a, b)
        np.testing.assert_array_equal(A.connected_components(), B.connected_components())


def test_reload_with_same_vertex_count_keeps_buffers_and_results():
    """A reload with the same V keeps the CC/BFS and PageRank buffers (no cudaFree/cudaMalloc);
    what depends on the lists (non-empty bitmaps, push tiles, straddle bits, the captured run) is
    rebuilt.  Every reload must give a fresh graph's results, also after a larger list and after
    a reload with another V."""
    import torch
    from grazelle import graphgen as gg
    from grazelle.engine import Graph
    graphs = [gg.rmat(13, 8, seed=1, symmetric=True), gg.rmat(13, 16, seed=2, symmetric=True),
              gg.rmat(13, 4, seed=3), gg.rmat(12, 16, seed=4, symmetric=True), gg.rmat(13, 16, seed=5)]
    with Graph(0) as R:
        for i, g in enumerate(graphs):
            V = g.num_vertices
            pull, push = g.pull_order().pairs(), g.push_order().pairs()
            if i % 2:
                R.load_pairs(V, pull, push)
            else:
                hp = torch.from_numpy(pull.view(np.int64)).pin_memory()
                R.load_pull_derive_push(V, g.num_edges, hp.data_ptr())
            with Graph(0) as F:
                F.load_pairs(V, pull, push)
                np.testing.assert_array_equal(R.connected_components(), F.connected_components())
                for root in (0, 5):
                    pr_, lr = R.bfs(root)
                    pf, lf = F.bfs(root)
                    np.testing.assert_array_equal(pr_, pf)
                    np.testing.assert_array_equal(lr, lf)
                np.testing.assert_array_equal(R.pagerank(8), F.pagerank(8))


def test_ingest_chunks_tuning_bounds():
    from grazelle import native
    from grazelle.engine import Graph
    with Graph(0) as G:
        G.tune(ingest_chunks=64)
        assert G.tuning()["ingest_chunks"] == 64
        with pytest.raises(native.GrzError) as ei:
            G.tune(ingest_chunks=65)
        assert ei.value.code == -5
        assert G.tuning()["ingest_chunks"] == 64


def test_calls_out_of_order_after_a_reload_are_rejected():
    """A reload with the same V keeps the CC/BFS and PageRank buffers, but their contents belong
    to the graph loaded before.  Until grz_frontier_begin / grz_pr_init runs for the new lists,
    every call that would read or advance that state returns GRZ_ERR_STATE, also when the new
    -push list has more vectors than the push tiles were sized for, and launches nothing."""
    import ctypes as C
    from grazelle import graphgen as gg, native
    from grazelle.engine import Graph
    small, big = gg.rmat(13, 4, seed=3, symmetric=True), gg.rmat(13, 32, seed=4, symmetric=True)
    assert small.num_vertices == big.num_vertices
    with Graph(0) as R:
        R.load_pairs(small.num_vertices, small.pull_order().pairs(), small.push_order().pairs())
        R.connected_components()
        R.pagerank(2)
        R.load_pairs(big.num_vertices, big.pull_order().pairs(), big.push_order().pairs())
        lib, h = R.lib, R.h
        V = big.num_vertices
        before = R.launch_count()
        eng, vote = C.c_int(), C.c_uint64()
        assert lib.grz_frontier_next(h, -1, C.byref(eng), C.byref(vote)) == native.GRZ_ERR_STATE
        lv = np.zeros(V, dtype=np.int64)
        assert lib.grz_read_levels(h, lv.ctypes.data_as(C.c_void_p), V) == native.GRZ_ERR_STATE
        dg = (C.c_uint64 * 3)()
        assert lib.grz_result_digest(h, dg) == native.GRZ_ERR_STATE
        assert lib.grz_frontier_snapshot(h) == native.GRZ_ERR_STATE
        assert lib.grz_pr_iterate(h, 1) == native.GRZ_ERR_STATE
        ms = C.c_float()
        assert lib.grz_pr_time_iterations(h, 1, C.byref(ms)) == native.GRZ_ERR_STATE
        props = np.zeros(V, dtype=np.float64)
        assert lib.grz_read_props(h, props.ctypes.data_as(C.c_void_p), V) == native.GRZ_ERR_STATE
        assert R.launch_count() == before
        # after the initialisations the graph gives a fresh graph's results
        with Graph(0) as F:
            F.load_pairs(V, big.pull_order().pairs(), big.push_order().pairs())
            np.testing.assert_array_equal(R.connected_components(), F.connected_components())
            np.testing.assert_array_equal(R.pagerank(3), F.pagerank(3))
