"""GPU layout builder and PageRank against the reference's golden outputs and the CPU oracle.

Tolerance: PageRank props must be within 1e-12 relative L1 of the reference
(FP64; the reference itself differs by up to ~1e-14 between thread counts).
Layout arrays must be bit-identical.
"""
import hashlib

import numpy as np
import pytest

from conftest import golden_names, load_golden
from oracle import oracle as O

pytestmark = pytest.mark.gpu
PR_TOL = 1e-12


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def gpu_graph(g):
    from grazelle.engine import Graph
    G = Graph(0)
    G.load_pairs(g.num_vertices, g.pull_order().pairs(), g.push_order().pairs())
    return G


@pytest.mark.parametrize("name", golden_names())
def test_device_layout_bit_identical(name):
    rec, g = load_golden(name)
    with gpu_graph(g) as G:
        from grazelle import native
        pl = G.list_vectors(native.LIST_PULL)
        sl = G.list_vectors(native.LIST_PUSH)
        assert sha(pl) == str(rec["pull_list_sha"])
        assert sha(sl) == str(rec["push_list_sha"])
        assert sha(G.vertex_index(native.LIST_PULL)) == str(rec["pull_index_sha"])
        assert sha(G.vertex_index(native.LIST_PUSH)) == str(rec["push_index_sha"])
        np.testing.assert_array_equal(G.outdegrees(), rec["outdeg"])
        info = G.info()
        assert info.pull_vectors == int(rec["pull_nvec"])
        assert info.push_vectors == int(rec["push_nvec"])


@pytest.mark.parametrize("name", golden_names())
def test_pagerank_matches_reference(name):
    rec, g = load_golden(name)
    with gpu_graph(g) as G:
        p = G.pagerank(16, damping=0.875)
    assert O.relative_l1(p, rec["pr_n1"]) < PR_TOL
    assert O.relative_l1(p, rec["pr_n4"]) < PR_TOL


def test_pagerank_damping_085_against_oracle():
    from grazelle import graphgen as gg
    g = gg.rmat(14, seed=3)
    L = O.layout(g.num_vertices, g.pull_order().pairs(), g.push_order().pairs())
    ref = O.pr_pull(L, 16, damping=0.85)
    with gpu_graph(g) as G:
        p = G.pagerank(16, damping=0.85)
    assert O.relative_l1(p, ref) < PR_TOL


@pytest.mark.parametrize("scale", [16, 18])
def test_pagerank_rmat_against_oracle(scale):
    from grazelle import graphgen as gg
    g = gg.rmat(scale, seed=scale)
    L = O.layout(g.num_vertices, g.pull_order().pairs(), g.push_order().pairs())
    ref = O.pr_pull(L, 16, damping=0.875, units=256)
    with gpu_graph(g) as G:
        np.testing.assert_array_equal(G.outdegrees(), L.outdeg)
        p = G.pagerank(16)
        p2 = G.pagerank(16)
    assert O.relative_l1(p, ref) < PR_TOL
    # exact fixed-point accumulation: repeated runs are bit-identical
    np.testing.assert_array_equal(p.view(np.uint64), p2.view(np.uint64))


def test_pagerank_phase_api_equals_fused():
    """The reference-named phase entry points compose to exactly the fused iteration."""
    import ctypes as C
    from grazelle import graphgen as gg, native
    g = gg.rmat(15, seed=9)
    with gpu_graph(g) as G:
        fused = G.pagerank(8)
        lib = G.lib
        G.pr_init(0.875)
        native.check(lib.grz_phases_bind(G.h, native.APP_PAGERANK))
        info = G.info()
        rb = np.zeros(8, dtype=np.uint64)
        mb = np.zeros(32 * 4, dtype=np.uint64)
        mb[0::4] = np.uint64(0xFFFFFFFFFFFFFFFF)  # unused merge-buffer entries (graphdata.c:1060-1065)
        acc_host = np.zeros(g.num_vertices + 8)
        for _ in range(8):
            lib.phase_op_reset_global_accum()
            lib.perform_edge_pull_phase_pr(C.c_void_p(info.pull_list_device), info.pull_vectors)
            lib.edge_pull_op_merge_with_merge_buffer(C.c_void_p(mb.ctypes.data), 32, C.c_void_p(acc_host.ctypes.data))
            lib.phase_op_write_global_accum_to_buf(C.c_void_p(rb.ctypes.data))
            lib.perform_vertex_phase_pr(0, g.num_vertices, C.c_void_p(rb.ctypes.data))
        assert lib.grz_phases_last_status() == 0
        phased = G.props()
    np.testing.assert_array_equal(phased.view(np.uint64), fused.view(np.uint64))


def test_pagerank_push_equals_pull():
    import ctypes as C
    from grazelle import graphgen as gg, native
    g = gg.rmat(14, seed=4)
    with gpu_graph(g) as G:
        pull = G.pagerank(6)
        lib = G.lib
        G.pr_init(0.875)
        native.check(lib.grz_phases_bind(G.h, native.APP_PAGERANK))
        info = G.info()
        rb = np.zeros(8, dtype=np.uint64)
        for _ in range(6):
            lib.phase_op_reset_global_accum()
            lib.perform_edge_push_phase_pr(C.c_void_p(info.push_list_device), info.push_vectors)
            lib.phase_op_write_global_accum_to_buf(C.c_void_p(rb.ctypes.data))
            lib.perform_vertex_phase_pr(0, g.num_vertices, C.c_void_p(rb.ctypes.data))
        assert lib.grz_phases_last_status() == 0
        push = G.props()
    np.testing.assert_array_equal(push.view(np.uint64), pull.view(np.uint64))


def test_pagerank_scale20_properties():
    """Full benchmark size (R-MAT scale 20): rank mass and agreement with the oracle."""
    from grazelle import graphgen as gg
    g = gg.rmat(20, seed=1)
    L = O.layout(g.num_vertices, g.pull_order().pairs(), g.push_order().pairs())
    ref = O.pr_pull(L, 16, damping=0.875, units=256, threads=0, multithreaded=True)
    with gpu_graph(g) as G:
        p = G.pagerank(16)
    assert O.relative_l1(p, ref) < PR_TOL
    od = np.where(L.outdeg == 0, float(g.num_vertices), L.outdeg)
    assert abs((p * od).sum() - 1.0) < 1e-9


def test_bad_inputs_rejected():
    from grazelle import graphgen as gg, native
    from grazelle.engine import Graph
    g = gg.rmat(10, seed=1)
    pull = g.pull_order().pairs()
    with Graph(0) as G:
        with pytest.raises(native.GrzError) as ei:
            G.load_pairs(g.num_vertices, g.push_order().pairs())  # src-sorted passed as pull
        assert ei.value.code == -4
        bad = pull.copy()
        bad[1] = np.uint64(g.num_vertices + 5)
        with pytest.raises(native.GrzError) as ei:
            G.load_pairs(g.num_vertices, bad)
        assert ei.value.code in (-4, -5)
        with pytest.raises(native.GrzError) as ei:
            G.pr_iterate(1)
        assert ei.value.code == -6


def test_empty_graph():
    from grazelle.engine import Graph
    with Graph(0) as G:
        G.load_pairs(100, np.zeros(0, dtype=np.uint64), np.zeros(0, dtype=np.uint64))
        assert G.info().pull_vectors == 1
        p = G.pagerank(4)
    # every vertex is dangling: prop = rank / V with rank = 1/V in every iteration
    np.testing.assert_allclose(p, np.full(100, 1.0 / 100 / 100), rtol=1e-12)


@pytest.mark.parametrize("scale, seed", [(12, 31), (17, 32)])
def test_gathered_prop_form_does_not_change_results(scale, seed):
    """The gather can read 8-byte doubles instead of 16-byte fixed-point props (GRZ_TUNE_PR_PROPS):
    the apply's fixed-point prop is the exact conversion of the same double, so every sum and
    every reported prop is bit-identical."""
    from grazelle import graphgen as gg
    g = gg.rmat(scale, seed=seed)
    with gpu_graph(g) as G:
        G.tune(pr_props=1)
        fixed = G.pagerank(16)
        G.tune(pr_props=2)
        dbl = G.pagerank(16)
        G.tune(pr_props=0)
        auto = G.pagerank(16)
    np.testing.assert_array_equal(dbl.view(np.uint64), fixed.view(np.uint64))
    np.testing.assert_array_equal(auto.view(np.uint64), fixed.view(np.uint64))


def test_phase_api_continues_fused_double_gather_iterations():
    """Fused iterations that gather doubles, then phase-API iterations on the fixed-point form:
    the same props as fused iterations throughout."""
    import ctypes as C
    from grazelle import graphgen as gg, native
    g = gg.rmat(14, seed=33)
    with gpu_graph(g) as G:
        G.tune(pr_props=1)
        ref = G.pagerank(8)
        G.tune(pr_props=2)
        G.pr_init(0.875).pr_iterate(4)
        lib = G.lib
        native.check(lib.grz_phases_bind(G.h, native.APP_PAGERANK))
        info = G.info()
        rb = np.zeros(8, dtype=np.uint64)
        mb = np.zeros(32 * 4, dtype=np.uint64)
        mb[0::4] = np.uint64(0xFFFFFFFFFFFFFFFF)
        acc_host = np.zeros(g.num_vertices + 8)
        for _ in range(4):
            lib.phase_op_reset_global_accum()
            lib.perform_edge_pull_phase_pr(C.c_void_p(info.pull_list_device), info.pull_vectors)
            lib.edge_pull_op_merge_with_merge_buffer(C.c_void_p(mb.ctypes.data), 32, C.c_void_p(acc_host.ctypes.data))
            lib.phase_op_write_global_accum_to_buf(C.c_void_p(rb.ctypes.data))
            lib.perform_vertex_phase_pr(0, g.num_vertices, C.c_void_p(rb.ctypes.data))
        assert lib.grz_phases_last_status() == 0
        mixed = G.props()
    np.testing.assert_array_equal(mixed.view(np.uint64), ref.view(np.uint64))


@pytest.mark.parametrize("props", [1, 2])
def test_persistent_iterations_bit_identical_to_two_kernels(props):
    """All iterations in one cooperative launch (gather and apply separated by a grid barrier)
    give exactly the props of the two-kernel iterations, for fixed-point and double gathers, on
    graphs whose destinations straddle tiles and with hub encoding, also when a call continues
    from the state an earlier call left (odd counts switch the ping-pong buffers)."""
    from grazelle import graphgen as gg
    from grazelle.engine import Graph
    for g, hubs in ((gg.rmat(16, seed=21), 0), (gg.rmat(14, 8, seed=22, symmetric=True), 512), (gg.erdos_renyi(3000, 5, seed=4), 0)):
        V = g.num_vertices
        pull, push = g.pull_order().pairs(), g.push_order().pairs()
        out = {}
        for mode in (1, 2):
            with Graph(0) as G:
                G.tune(pr_persistent=mode, pr_props=props, hubs=hubs)
                G.load_pairs(V, pull, push)
                G.pr_init(0.85).pr_iterate(3).pr_iterate(10)
                out[mode] = G.props()
        np.testing.assert_array_equal(out[1], out[2])
        L = O.layout(V, pull, push)
        assert O.relative_l1(out[2], O.pr_pull(L, 13, damping=0.85)) < PR_TOL


def test_persistent_barrier_wait_runs_out_and_the_graph_recovers():
    """A block that never arrives at the first grid barrier (injected on the host side) makes the
    other blocks' bounded waits run out: grz_pr_iterate returns GRZ_ERR_TIMEOUT, PageRank is
    left uninitialised (GRZ_ERR_STATE), and after grz_pr_init the same graph gives the oracle's
    props.  Nothing faults or hangs: every wait has a time and an iteration bound."""
    from grazelle import graphgen as gg, native
    from grazelle.engine import Graph
    g = gg.rmat(14, seed=23)
    V = g.num_vertices
    pull, push = g.pull_order().pairs(), g.push_order().pairs()
    with Graph(0) as G:
        G.load_pairs(V, pull, push)
        G.tune(pr_persistent=2, pr_wait_limit_us=20000, pr_withhold=1)
        G.pr_init(0.875)
        assert G.lib.grz_pr_iterate(G.h, 4) == native.GRZ_ERR_TIMEOUT
        assert b"barrier 1" in G.lib.grz_graph_last_error(G.h)
        assert G.lib.grz_pr_iterate(G.h, 1) == native.GRZ_ERR_STATE
        G.tune(pr_withhold=0)
        p = G.pagerank(16, damping=0.875)
    L = O.layout(V, pull, push)
    assert O.relative_l1(p, O.pr_pull(L, 16, damping=0.875)) < PR_TOL


def test_persistent_phase_times_reach_the_profiler():
    from grazelle import graphgen as gg
    from grazelle.engine import Graph
    g = gg.rmat(15, seed=24)
    with Graph(0) as G:
        G.load_pairs(g.num_vertices, g.pull_order().pairs(), g.push_order().pairs())
        G.tune(pr_persistent=2)
        G.pr_init(0.875)
        G.profile(True)
        G.pr_iterate(5)
        recs = G.profile_read()
        G.profile(False)
    kinds = [k for k, _ in recs]
    assert kinds == ["pr_gather", "pr_apply"] * 5
    assert all(ms > 0 for _, ms in recs)


@pytest.mark.parametrize("bits", [8, 10, 12])
def test_source_segmented_gather_is_bit_identical(bits):
    """PageRank over source-segmented pull lists (each iteration gathers segment by segment and
    adds into the exact accumulators) gives exactly the props of the unsegmented gather of the
    same (double) props, on directed and symmetric R-MAT and Erdos-Renyi graphs with 2^bits
    sources per segment (up to 64 segments), across a reload with the same V."""
    from grazelle import graphgen as gg
    from grazelle.engine import Graph
    graphs = [gg.rmat(14, seed=51), gg.rmat(13, 16, seed=52, symmetric=True), gg.erdos_renyi(5000, 7, seed=53)]
    for g in graphs:
        V = g.num_vertices
        pull, push = g.pull_order().pairs(), g.push_order().pairs()
        with Graph(0) as A, Graph(0) as B:
            A.tune(pr_props=2, pr_segment_bits=1)
            A.load_pairs(V, pull, push)
            B.tune(pr_segment_bits=bits)
            B.load_pairs(V, pull, push)
            for it in (1, 5, 16):
                np.testing.assert_array_equal(A.pagerank(it, damping=0.85), B.pagerank(it, damping=0.85))
            B.load_pairs(V, pull, push)
            np.testing.assert_array_equal(A.pagerank(7), B.pagerank(7))
        L = O.layout(V, pull, push)
        with Graph(0) as B:
            B.tune(pr_segment_bits=bits)
            B.load_pairs(V, pull, push)
            assert O.relative_l1(B.pagerank(16), O.pr_pull(L, 16)) < PR_TOL


@pytest.mark.parametrize("props,seg", [(1, 1), (2, 1), (2, 10)])
def test_props_do_not_depend_on_the_gather_grid(props, seg):
    """The gather's persistent grid (how many blocks, hence which tiles each block walks and how
    many blocks are resident per SM) changes nothing: fixed-point and double props, with and
    without source segments, and the persistent forms."""
    from grazelle import graphgen as gg
    from grazelle.engine import Graph
    g = gg.rmat(15, seed=61)
    V = g.num_vertices
    pull, push = g.pull_order().pairs(), g.push_order().pairs()
    with Graph(0) as G:
        G.tune(pr_props=props, pr_segment_bits=seg)
        G.load_pairs(V, pull, push)
        a = G.pagerank(9)
        for grid in (37, 152, 456, 1216, 3000):
            G.tune(pr_grid=grid)
            np.testing.assert_array_equal(G.pagerank(9), a, err_msg="grid %d" % grid)
        G.tune(pr_grid=0)
        for form in (2, 3):
            G.tune(pr_persistent=form)
            np.testing.assert_array_equal(G.pagerank(9), a, err_msg="form %d" % form)
        G.tune(pr_persistent=0)
        np.testing.assert_array_equal(G.pagerank(9), a)
