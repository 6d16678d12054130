"""The CPU oracle against the reference's own outputs (tests/golden, made by make_golden.py).

The oracle restates the reference's algorithm in portable C.  At -n 1 it must
reproduce the reference bit for bit: vector lists, vertex indices,
outdegrees, PageRank props, CC labels, BFS parents and iteration counts.
Only then is it trusted as the checker of the GPU engine.
"""
import hashlib

import numpy as np
import pytest

from conftest import golden_names, load_golden
from oracle import oracle as O

CASES = golden_names()


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


@pytest.fixture(scope="module", params=CASES)
def case(request):
    rec, g = load_golden(request.param)
    L = O.layout(g.num_vertices, g.pull_order().pairs(), g.push_order().pairs())
    return request.param, rec, g, L


def test_layout_matches_reference(case):
    name, rec, g, L = case
    assert L.pull_vec.shape[0] == int(rec["pull_nvec"])
    assert L.push_vec.shape[0] == int(rec["push_nvec"])
    assert sha(L.pull_vec) == str(rec["pull_list_sha"])
    assert sha(L.push_vec) == str(rec["push_list_sha"])
    assert sha(L.pull_index) == str(rec["pull_index_sha"])
    assert sha(L.push_index) == str(rec["push_index_sha"])
    np.testing.assert_array_equal(L.outdeg, rec["outdeg"])


def test_pagerank_bit_exact_single_thread(case):
    name, rec, g, L = case
    p = O.pr_pull(L, 16, damping=0.875, units=32)
    np.testing.assert_array_equal(p.view(np.uint64), rec["pr_n1"].view(np.uint64))


def test_pagerank_four_threads_within_tolerance(case):
    # with 4 threads the reference makes 128 units and sums S in a thread-dependent order
    name, rec, g, L = case
    p = O.pr_pull(L, 16, damping=0.875, units=128)
    assert O.relative_l1(p, rec["pr_n4"]) < 1e-12
    p_mt = O.pr_pull(L, 16, damping=0.875, units=128, threads=4, multithreaded=True)
    assert O.relative_l1(p_mt, rec["pr_n4"]) < 1e-12


def test_pagerank_sum_is_one(case):
    name, rec, g, L = case
    od = np.zeros(g.num_vertices + 8)
    od[:g.num_vertices] = L.outdeg
    pr = np.zeros(g.num_vertices + 8)
    pr[:g.num_vertices] = rec["pr_n1"]
    assert abs(O.lib().oracle_pr_sum(pr, od, g.num_vertices) - 1.0) < 1e-9


@pytest.mark.parametrize("variant,flags", [("cc", 0), ("cc_twc", O.WITHOUT_COUNT), ("cc_pull", O.FORCE_PULL), ("cc_push", O.FORCE_PUSH)])
def test_cc_matches_reference(case, variant, flags):
    name, rec, g, L = case
    labels, it, _ = O.cc(L, flags)
    np.testing.assert_array_equal(labels, rec[variant + "_labels"])
    np.testing.assert_array_equal(it, rec[variant + "_iters"])


@pytest.mark.parametrize("variant,flags", [("bfs", 0), ("bfs_twc", O.WITHOUT_COUNT), ("bfs_pull", O.FORCE_PULL), ("bfs_push", O.FORCE_PUSH)])
def test_bfs_matches_reference(case, variant, flags):
    name, rec, g, L = case
    parents, it, _ = O.bfs(L, flags)
    np.testing.assert_array_equal(parents, rec[variant + "_parents"])
    np.testing.assert_array_equal(it, rec[variant + "_iters"])


def test_bfs_reference_parents_form_legal_tree(case):
    name, rec, g, L = case
    push = g.push_order().pairs()
    lv = O.bfs_levels(push, g.num_vertices, 0)
    for variant in ("bfs", "bfs_pull", "bfs_push"):
        par = rec[variant + "_parents"].astype(np.int64)
        assert O.bfs_check_tree(push, g.num_vertices, 0, lv, par) == 0


def test_cc_labels_are_min_ancestor(case):
    # independent check: the fixed point is the minimum ID over each vertex's ancestors (and itself)
    name, rec, g, L = case
    V = g.num_vertices
    lab = np.arange(V, dtype=np.float64)
    src, dst = g.src.astype(np.int64), g.dst.astype(np.int64)
    while True:
        nxt = lab.copy()
        np.minimum.at(nxt, dst, lab[src])
        if np.array_equal(nxt, lab):
            break
        lab = nxt
    np.testing.assert_array_equal(lab, rec["cc_labels"])


def test_oracle_detects_planted_error(case):
    # a mistake planted in the oracle's output must be caught by the comparison used above
    name, rec, g, L = case
    p = O.pr_pull(L, 16, damping=0.875, units=32)
    p[len(p) // 2] *= 1.0 + 1e-9
    assert not np.array_equal(p.view(np.uint64), rec["pr_n1"].view(np.uint64))
    assert O.relative_l1(p, rec["pr_n1"]) > 0


def test_cc_min_labels_from_pairs_equal_the_reference_labels():
    """The pairs-based CC check used at sizes beyond a host layout gives the reference's labels
    bit for bit on every golden graph (directed and symmetric)."""
    for name in golden_names():
        rec, g = load_golden(name)
        lab = O.cc_min_labels(g.pull_order().pairs(), g.num_vertices, threads=4)
        np.testing.assert_array_equal(lab.astype(np.float64), rec["cc_labels"][:g.num_vertices], err_msg=name)


def test_pagerank_sample_iteration_matches_the_oracle():
    """The sampled one-iteration PageRank check used at R-MAT 27 agrees with the pinned oracle's
    first iteration at the sampled destinations (1e-14 relative; only the S sum order differs),
    including destinations without in-edges and dangling sources."""
    for name in ("rmat10_s12", "isolated_root70", "tiny13"):
        rec, g = load_golden(name)
        V = g.num_vertices
        pull = g.pull_order().pairs()
        L = O.layout(V, pull, g.push_order().pairs())
        ref = O.pr_pull(L, 1, 0.875)[:V]
        smp = np.arange(0, V, 3, dtype=np.uint64)
        got = O.pr_sample_iteration(pull, V, smp, 0.875, threads=3)
        assert O.relative_l1(got, ref[smp.astype(np.int64)]) < 1e-14, name
