"""GPU Connected Components and BFS against the reference's golden outputs and the CPU oracle.

CC labels must be bit-exact whichever engine runs.  BFS levels must be
bit-exact, and the parents must form a legal BFS tree.  The GPU's BFS parent
rules are deterministic and its vote counts each visited vertex once.  So it
also reproduces the single-thread reference's parents, engine sequence and
iteration counts exactly.  The tests check that too.
"""
import ctypes as C

import numpy as np
import pytest

from conftest import golden_names, load_golden
from oracle import oracle as O

pytestmark = pytest.mark.gpu

CC_VARIANTS = [("cc", 0), ("cc_twc", O.WITHOUT_COUNT), ("cc_pull", O.FORCE_PULL), ("cc_push", O.FORCE_PUSH)]
BFS_VARIANTS = [("bfs", 0), ("bfs_twc", O.WITHOUT_COUNT), ("bfs_pull", O.FORCE_PULL), ("bfs_push", O.FORCE_PUSH)]


def gpu_graph(g):
    from grazelle.engine import Graph
    G = Graph(0)
    G.load_pairs(g.num_vertices, g.pull_order().pairs(), g.push_order().pairs())
    return G


@pytest.mark.parametrize("name", golden_names())
def test_cc_labels_match_reference(name):
    rec, g = load_golden(name)
    with gpu_graph(g) as G:
        for variant, flags in CC_VARIANTS:
            lab, st = G.connected_components(flags, stats=True)
            np.testing.assert_array_equal(lab, rec[variant + "_labels"], err_msg=variant)
            assert st.iterations == st.pull_iterations + st.push_iterations
            if flags == O.FORCE_PULL:
                assert st.push_iterations == 0
            if flags == O.FORCE_PUSH:
                assert st.pull_iterations == 0


@pytest.mark.parametrize("name", golden_names())
def test_bfs_matches_single_thread_reference(name):
    rec, g = load_golden(name)
    push = g.push_order().pairs()
    ref_lv = O.bfs_levels(push, g.num_vertices, 0)
    with gpu_graph(g) as G:
        for variant, flags in BFS_VARIANTS:
            par, lv, st = G.bfs(0, flags, stats=True)
            np.testing.assert_array_equal(lv, ref_lv, err_msg=variant)
            assert O.bfs_check_tree(push, g.num_vertices, 0, lv, par.astype(np.int64)) == 0, variant
            np.testing.assert_array_equal(par, rec[variant + "_parents"], err_msg=variant)
            np.testing.assert_array_equal([st.iterations, st.pull_iterations, st.push_iterations],
                                          rec[variant + "_iters"], err_msg=variant)


@pytest.mark.parametrize("scale", [16, 18])
def test_cc_bfs_rmat_against_oracle(scale):
    from grazelle import graphgen as gg
    g = gg.rmat(scale, seed=100 + scale)
    pull, push = g.pull_order().pairs(), g.push_order().pairs()
    L = O.layout(g.num_vertices, pull, push)
    with gpu_graph(g) as G:
        lab = G.connected_components()
        np.testing.assert_array_equal(lab, O.cc(L)[0])
        ref_par, ref_it, _ = O.bfs(L)
        par, lv, st = G.bfs(0, stats=True)
        np.testing.assert_array_equal(lv, O.bfs_levels(push, g.num_vertices, 0))
        np.testing.assert_array_equal(par, ref_par)
        assert st.iterations == ref_it[0]


def test_cc_symmetric_graph_components():
    """On a symmetrised graph the labels are the minimum vertex ID of each weak component."""
    from grazelle import graphgen as gg
    g = gg.symmetrize(gg.rmat(15, seed=42))
    with gpu_graph(g) as G:
        lab = G.connected_components()
    # union-find reference
    parent = np.arange(g.num_vertices)

    def find(x):
        while parent[x] != x:
            parent[x] = parent[parent[x]]
            x = parent[x]
        return x
    for s, d in zip(g.src.tolist(), g.dst.tolist()):
        a, b = find(s), find(d)
        if a != b:
            parent[max(a, b)] = min(a, b)
    comp_min = np.array([find(v) for v in range(g.num_vertices)], dtype=np.float64)
    np.testing.assert_array_equal(lab, comp_min)


def test_bfs_other_roots_equal_relabelled_reference():
    """A root other than 0 gives the same levels as the reference run on the root<->0 relabelled graph."""
    from grazelle import graphgen as gg
    g = gg.rmat(14, seed=5)
    deg = g.out_degrees()
    roots = [int(r) for r in np.nonzero(deg)[0][:4]]
    with gpu_graph(g) as G:
        for r in roots:
            par, lv = G.bfs(r)
            np.testing.assert_array_equal(lv, O.bfs_levels(g.push_order().pairs(), g.num_vertices, r))
            assert O.bfs_check_tree(g.push_order().pairs(), g.num_vertices, r, lv, par.astype(np.int64)) == 0
            # same levels as the relabelled graph seen from vertex 0, mapped back
            h = gg.relabel_swap(g, r)
            lv0 = O.bfs_levels(h.push_order().pairs(), h.num_vertices, 0)
            perm = np.arange(g.num_vertices)
            perm[[0, r]] = perm[[r, 0]]
            np.testing.assert_array_equal(lv, lv0[perm])


def test_phase_api_cc_and_bfs_drivers():
    """The reference's CC/BFS driver loops (execution_cc.c:94-268, execution_bfs.c:120-276) over the phases.h calls."""
    from grazelle import graphgen as gg, native
    g = gg.rmat(13, seed=8)
    L = O.layout(g.num_vertices, g.pull_order().pairs(), g.push_order().pairs())
    with gpu_graph(g) as G:
        lib = G.lib
        info = G.info()
        rb = np.zeros(8, dtype=np.uint64)
        rbp = C.c_void_p(rb.ctypes.data)
        for app, ref in ((native.APP_CONNECTED_COMPONENTS, O.cc(L)[0]), (native.APP_BREADTH_FIRST_SEARCH, O.bfs(L)[0])):
            native.check(lib.grz_phases_bind(G.h, app))
            native.check(lib.grz_frontier_begin(G.h, app, 0, 0))
            vote, _ = G.frontier_vote()
            E = info.num_edges
            pull_phase = lib.perform_edge_pull_phase_cc if app == 1 else lib.perform_edge_pull_phase_bfs
            push_phase = lib.perform_edge_push_phase_cc if app == 1 else lib.perform_edge_push_phase_bfs
            vertex_phase = lib.perform_vertex_phase_cc if app == 1 else lib.perform_vertex_phase_bfs
            for _ in range(10000):
                lib.phase_op_reset_global_accum()
                if vote > E // 5:
                    pull_phase(C.c_void_p(info.pull_list_device), info.pull_vectors)
                else:
                    push_phase(C.c_void_p(info.push_list_device), info.push_vectors)
                lib.phase_op_write_global_accum_to_buf(rbp)
                vote = lib.phase_op_combine_global_var_from_buf(rbp)
                if vote == 0:
                    break
                vertex_phase(0, info.num_vertices, None)
            assert lib.grz_phases_last_status() == 0
            np.testing.assert_array_equal(G.props(), ref)


@pytest.mark.parametrize("name", golden_names())
def test_graph_run_equals_host_loop(name):
    """grz_cc_run / grz_bfs_run execute the whole loop as one CUDA graph (engine choice and
    convergence on the device).  GRZ_FLAG_HOST_LOOP runs the same loop with a host round trip
    per iteration.  Both must give the same results for every engine flag set and for the
    learned policy, and BFS (level-synchronous) the same iterations and engine counts."""
    from grazelle import native
    from grazelle.switch import Switch
    rec, g = load_golden(name)
    with gpu_graph(g) as G:
        for policy in ("threshold", "learned"):
            if policy == "learned":
                G.set_policy(native.POLICY_LEARNED, Switch(0, seed=11))
            for _, flags in CC_VARIANTS:
                a, sa = G.connected_components(flags, stats=True)
                b, sb = G.connected_components(flags | native.FLAG_HOST_LOOP, stats=True)
                np.testing.assert_array_equal(a, b)
                np.testing.assert_array_equal(a, rec["cc_labels"])
                # CC updates labels in place (asynchronous, as the reference's CAS loop), so the
                # number of iterations may differ between runs; the labels may not
                for s_ in (sa, sb):
                    assert s_.iterations == s_.pull_iterations + s_.push_iterations
                    assert s_.iterations >= 1
            for _, flags in BFS_VARIANTS:
                for root in (0, g.num_vertices // 3):
                    pa, la, sa = G.bfs(root, flags, stats=True)
                    pb, lb, sb = G.bfs(root, flags | native.FLAG_HOST_LOOP, stats=True)
                    np.testing.assert_array_equal(la, lb)
                    np.testing.assert_array_equal(pa, pb)
                    assert (sa.iterations, sa.pull_iterations, sa.push_iterations) == \
                        (sb.iterations, sb.pull_iterations, sb.push_iterations), (policy, flags, root)
        G.set_policy(native.POLICY_THRESHOLD)


def test_graph_run_repeated_and_alternating():
    """The cached run graph survives alternating apps, roots and loops on one graph."""
    from grazelle import graphgen as gg, native
    g = gg.rmat(16, seed=77)
    push = g.push_order().pairs()
    with gpu_graph(g) as G:
        for k in range(3):
            for root in (1, 100, 5000):
                _, lv, st = G.bfs(root, stats=True)
                np.testing.assert_array_equal(lv, O.bfs_levels(push, g.num_vertices, root))
                _, lv2, st2 = G.bfs(root, native.FLAG_HOST_LOOP, stats=True)
                np.testing.assert_array_equal(lv2, lv)
                assert st.iterations == st2.iterations
            lab = G.connected_components()
            lab2 = G.connected_components(native.FLAG_HOST_LOOP)
            np.testing.assert_array_equal(lab, lab2)
        before = G.launch_count()
        G.bfs(1)
        assert G.launch_count() > before


def _digest_np(values_u32, degree, bfs):
    V = values_u32.shape[0]
    v = np.arange(V, dtype=np.uint64)
    odd = (v * np.uint64(0x9E3779B97F4A7C15)) | np.uint64(1)
    with np.errstate(over="ignore"):
        h = int(np.sum((values_u32.astype(np.uint64) + np.uint64(1)) * odd, dtype=np.uint64))
    if bfs:
        reached = values_u32 != 0xffffffff
        return int(reached.sum()), int(degree[reached].sum()), h
    return int((values_u32 == np.arange(V)).sum()), 0, h


@pytest.mark.parametrize("name", ["rmat10_s12", "rmat12_s13", "isolated_root70"])
def test_result_digest(name):
    rec, g = load_golden(name)
    deg = g.out_degrees().astype(np.int64)
    with gpu_graph(g) as G:
        par, lv = G.bfs(0)
        lv32 = np.where(lv < 0, 0xffffffff, lv).astype(np.uint32)
        assert G.digest() == _digest_np(lv32, deg, True)
        lab = G.connected_components()
        assert G.digest() == _digest_np(lab.astype(np.uint32), deg, False)


@pytest.mark.parametrize("name", ["rmat12_s13", "rmat10_sym_s21", "star_chain1001"])
def test_hub_encoding_and_kernel_shapes_do_not_change_results(name):
    """Hub sources (the pull list's high out-degree vertices served from shared memory) and the
    CC kernel's block size, cache size and grid change only speed: CC labels, BFS parents and
    levels, and PageRank props stay identical."""
    from grazelle.engine import Graph
    rec, g = load_golden(name)
    ref_lab = rec["cc_labels"]
    results = []
    for hubs, cache, threads, grid in ((0, 0, 512, 0), (49152, 49152, 1024, 0), (49152, 24576, 512, 0),
                                       (16, 8, 256, 3), (49152, 0, 256, 0), (4, 4, 512, 1)):
        with Graph(0) as G:
            G.tune(hubs=hubs, cc_cache=cache, cc_threads=threads, cc_grid=grid)
            G.load_pairs(g.num_vertices, g.pull_order().pairs(), g.push_order().pairs())
            t = G.tuning()
            assert t["hubs_loaded"] <= hubs
            if hubs == 0:
                assert t["hubs_loaded"] == 0
            lab = G.connected_components()
            lab2 = G.connected_components(O.FORCE_PULL)
            np.testing.assert_array_equal(lab, ref_lab)
            np.testing.assert_array_equal(lab2, rec["cc_pull_labels"])
            par, lv = G.bfs(0, O.FORCE_PULL)
            pr = G.pagerank(4)
            results.append((par, lv, pr))
    for par, lv, pr in results[1:]:
        np.testing.assert_array_equal(par, results[0][0])
        np.testing.assert_array_equal(lv, results[0][1])
        np.testing.assert_array_equal(pr, results[0][2])


@pytest.mark.parametrize("name", golden_names())
def test_bfs_pull_compacted_equals_scan(name):
    """The BFS pull forms give the same parents, levels, iterations and engine counts, all equal
    to the single-thread reference's: the early-exit pass over each wanted destination's first
    1, 2 or 64 vectors followed by the pass over the rest (1 is the default), the pass over every
    vector of the wanted destinations (compacted), and the scan of every vector."""
    rec, g = load_golden(name)
    forms = ((0, 1), (0, 0), (0, 2), (0, 64), (1, 1))
    with gpu_graph(g) as G:
        for variant, flags in BFS_VARIANTS:
            out = []
            for scan, first in forms:
                G.tune(bfs_pull_scan=scan, bfs_pull_first=first)
                par, lv, st = G.bfs(0, flags, stats=True)
                out.append((par, lv, (st.iterations, st.pull_iterations, st.push_iterations)))
            for o, form in zip(out[1:], forms[1:]):
                np.testing.assert_array_equal(out[0][0], o[0], err_msg="%s %s" % (variant, form))
                np.testing.assert_array_equal(out[0][1], o[1], err_msg="%s %s" % (variant, form))
                assert out[0][2] == o[2]
            np.testing.assert_array_equal(out[0][0], rec[variant + "_parents"], err_msg=variant)
        G.tune(bfs_pull_scan=0, bfs_pull_first=1)


@pytest.mark.parametrize("first", [0, 1, 3])
def test_bfs_pull_early_exit_graph_runs(first):
    """Whole BFS runs (one CUDA graph each) on an R-MAT 16 from 6 roots, forced pull, forced push
    and the default switch: levels equal to the oracle's and parents identical to the full pass's,
    for each length of the early-exit pass.  The big iterations touch more than V / 128
    destinations, so the touched list stops growing and the visit sweeps all vertices."""
    from grazelle import graphgen as gg
    from grazelle.engine import Graph
    g = gg.rmat(16, seed=71)
    pull, push = g.pull_order().pairs(), g.push_order().pairs()
    roots = [0, 1, 5, 77, 1000, 40000]
    with Graph(0) as G:
        G.load_pairs(g.num_vertices, pull, push)
        base = {}
        for flags in (O.FORCE_PULL, O.FORCE_PUSH, 0):
            G.tune(bfs_pull_first=0)
            for r in roots:
                base[(flags, r)] = G.bfs(r, flags)
            G.tune(bfs_pull_first=first)
            for r in roots:
                par, lv = G.bfs(r, flags)
                np.testing.assert_array_equal(par, base[(flags, r)][0], err_msg="root %d flags %d" % (r, flags))
                np.testing.assert_array_equal(lv, base[(flags, r)][1], err_msg="root %d flags %d" % (r, flags))
                np.testing.assert_array_equal(lv, O.bfs_levels(push, g.num_vertices, r), err_msg="root %d" % r)


def test_profiler_off_restores_the_graph_run():
    """Kernel profiling needs the host loop; once profiling is switched off again, whole runs go
    back to the single CUDA-graph launch (same launch accounting as a graph never profiled)."""
    from grazelle import graphgen as gg
    from grazelle.engine import Graph
    g = gg.rmat(14, seed=61, symmetric=True)
    counts = []
    for toggle in (False, True):
        with Graph(0) as G:
            G.load_pairs(g.num_vertices, g.pull_order().pairs(), g.push_order().pairs())
            G.cc_run()
            if toggle:
                G.profile(True)
                G.cc_run()
                G.profile(False)
            l0 = G.launch_count()
            G.cc_run()
            counts.append(G.launch_count() - l0)
    assert counts[0] == counts[1]


@pytest.mark.parametrize("host_loop", [False, True])
def test_run_bounds_return_timeout_and_leave_the_graph_usable(host_loop):
    """The iteration and time bounds of a CC/BFS run (the decision kernel's in a graph run, the
    host's in the host loop) stop a run that has not converged with GRZ_ERR_TIMEOUT; the next run
    with the default bounds gives the oracle's labels and levels."""
    from grazelle import graphgen as gg, native
    from grazelle.engine import Graph
    g = gg.rmat(14, seed=31, symmetric=True)
    V = g.num_vertices
    pull, push = g.pull_order().pairs(), g.push_order().pairs()
    flags = native.FLAG_HOST_LOOP if host_loop else 0
    L = O.layout(V, pull, push)
    with Graph(0) as G:
        G.load_pairs(V, pull, push)
        G.tune(run_max_iterations=1)
        st = native.RunStats()
        assert G.lib.grz_cc_run(G.h, flags, C.byref(st)) == native.GRZ_ERR_TIMEOUT
        assert b"iterations" in G.lib.grz_graph_last_error(G.h)
        assert G.lib.grz_bfs_run(G.h, 0, flags, C.byref(st)) == native.GRZ_ERR_TIMEOUT
        G.tune(run_max_iterations=0, run_limit_us=1)
        assert G.lib.grz_cc_run(G.h, flags, C.byref(st)) == native.GRZ_ERR_TIMEOUT
        assert b"time bound" in G.lib.grz_graph_last_error(G.h)
        G.tune(run_limit_us=0)
        np.testing.assert_array_equal(G.connected_components(flags), O.cc(L)[0])
        np.testing.assert_array_equal(G.bfs(0, flags)[1], O.bfs_levels(push, V, 0))


@pytest.mark.parametrize("threads", [256, 512, 1024])
def test_bulk_staged_pull_gives_the_same_labels(threads):
    """The CC pull with its edge stream staged by bulk copies (cp.async.bulk into shared memory,
    two tiles ahead, mbarrier completion with bounded waits) gives the oracle's labels under every
    block size, in the graph run and the host loop, including a list whose last tile is partial
    (served by plain loads)."""
    from grazelle import graphgen as gg, native
    from grazelle.engine import Graph
    g = gg.rmat(15, seed=41, symmetric=True)
    V = g.num_vertices
    pull, push = g.pull_order().pairs(), g.push_order().pairs()
    L = O.layout(V, pull, push)
    ref = O.cc(L)[0]
    with Graph(0) as G:
        G.load_pairs(V, pull, push)
        assert G.info().pull_vectors % threads != 0 or threads == 256
        G.tune(pull_staging=1, cc_threads=threads)
        np.testing.assert_array_equal(G.connected_components(), ref)
        np.testing.assert_array_equal(G.connected_components(native.FLAG_HOST_LOOP), ref)
        np.testing.assert_array_equal(G.connected_components(native.FORCE_PULL), ref)


def test_cc_full_pull_over_source_segments():
    """The CC run's full pull over the source-segmented lists (each segment's labels stay in L2;
    the later pulls with the converged-destination skip read the whole list, the device choosing
    which pass works) gives the oracle's labels: lists built for CC (GRZ_TUNE_CC_SEGMENTS = 2),
    lists left by grz_pr_init, in the graph run and the host loop, and the same labels with the
    segments turned off."""
    from grazelle import graphgen as gg, native
    from grazelle.engine import Graph
    for g in (gg.rmat(14, 16, seed=71, symmetric=True), gg.rmat(14, 8, seed=72)):
        V = g.num_vertices
        pull, push = g.pull_order().pairs(), g.push_order().pairs()
        ref = O.cc(O.layout(V, pull, push))[0]
        with Graph(0) as G:
            G.tune(cc_segments=2, pr_segment_bits=9)
            G.load_pairs(V, pull, push)
            np.testing.assert_array_equal(G.connected_components(), ref)
            np.testing.assert_array_equal(G.connected_components(native.FLAG_HOST_LOOP), ref)
            np.testing.assert_array_equal(G.connected_components(native.WITHOUT_COUNT), ref)
            G.tune(cc_segments=1)
            np.testing.assert_array_equal(G.connected_components(), ref)
        with Graph(0) as G:
            G.tune(pr_segment_bits=10)
            G.load_pairs(V, pull, push)
            np.testing.assert_array_equal(G.connected_components(), ref)   # no segments yet
            G.pagerank(2)                                                 # builds them
            np.testing.assert_array_equal(G.connected_components(), ref)   # the run graph is captured again
            np.testing.assert_array_equal(G.bfs(0)[1], O.bfs_levels(push, V, 0))


@pytest.mark.parametrize("first", [0, 1, 2, 3, 4])
def test_cc_first_vector_pass(first):
    """CC without the first-vector pass and with it in both forms (GRZ_TUNE_CC_PULL_FIRST: then
    the whole list without the destinations at 0, or the open destinations' remaining vectors):
    labels equal to the
    golden reference's on every golden graph and build variant, and to the oracle's on symmetric
    and directed R-MAT 16, through whole runs (graph path) and the host loop, with hub encoding too."""
    from grazelle import graphgen as gg
    from grazelle.engine import Graph
    for name in golden_names():
        rec, g = load_golden(name)
        with gpu_graph(g) as G:
            G.tune(cc_pull_first=first)
            for variant, flags in CC_VARIANTS:
                np.testing.assert_array_equal(G.connected_components(flags), rec[variant + "_labels"], err_msg="%s %s" % (name, variant))
    for sym in (True, False):
        g = gg.rmat(16, seed=91, symmetric=sym)
        pull, push = g.pull_order().pairs(), g.push_order().pairs()
        ref = O.cc_min_labels(pull, g.num_vertices).astype(np.float64)
        for hubs in (0, 256):
            with Graph(0) as G:
                G.tune(hubs=hubs, cc_cache=128, cc_pull_first=first)
                G.load_pairs(g.num_vertices, pull, push)
                for _ in range(2):
                    np.testing.assert_array_equal(G.connected_components(), ref, err_msg="sym %s hubs %d" % (sym, hubs))
                np.testing.assert_array_equal(G.connected_components(O.FORCE_PULL), ref)
                G.profile(True)  # the host loop, one launch per kernel
                np.testing.assert_array_equal(G.connected_components(), ref)
                G.profile(False)


def test_profile_work_counts_open_destination_vectors():
    """While profiling, grz_profile_work reports the vectors the CC open-destination pulls read
    (first pulls, later pulls) and resets them; with profiling off nothing is counted.  The counts
    are bounded by the pull list's length per pull, and the labels stay the oracle's."""
    from grazelle import graphgen as gg
    from grazelle.engine import Graph
    g = gg.rmat(16, seed=93, symmetric=True)
    pull, push = g.pull_order().pairs(), g.push_order().pairs()
    ref = O.cc_min_labels(pull, g.num_vertices).astype(np.float64)
    with Graph(0) as G:
        G.load_pairs(g.num_vertices, pull, push)
        nvec = G.info().pull_vectors
        G.profile(True)
        assert G.profile_work() == (0, 0)
        lab, st = G.connected_components(stats=True)
        first, later = G.profile_work()
        assert 0 <= first <= nvec and 0 <= later <= nvec * max(1, st.pull_iterations)
        assert G.profile_work() == (0, 0)
        G.profile_read()
        G.profile(False)
        np.testing.assert_array_equal(lab, ref)
        np.testing.assert_array_equal(G.connected_components(), ref)
        assert G.profile_work() == (0, 0)
