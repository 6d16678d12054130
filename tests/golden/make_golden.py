#!/usr/bin/env python3
"""Generates tests/golden/*.npz: outputs of the unmodified Grazelle reference on small graphs.

Runs only where the reference builds (x86-64 with AVX2).  It needs the
binaries made by ``python oracle/build_ref.py``.  The fixtures travel with the
repository, so the oracle and GPU tests need no reference at run time.

Each fixture holds:
  * the graph: either the generator parameters (regenerated bit-identically by
    grazelle/graphgen.py) or, for hand-made edge cases, the pairs themselves;
  * sha256 digests of the reference's in-edge and out-edge vector lists and
    vertex indices (dumped by oracle/ref_driver.c), and the full lists for the
    smallest graphs;
  * PageRank props after 16 iterations at -n 1 and -n 4 (d = 0.875, fig11-pull build);
  * CC labels and iteration counts, and BFS parents and iteration counts, for
    the default, THRESHOLD_WITHOUT_COUNT, forced-pull and forced-push builds, at -n 1.

Usage: python tests/golden/make_golden.py
"""
from __future__ import annotations

import hashlib
import sys
import tempfile
from pathlib import Path

import numpy as np

REPO = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(REPO))
sys.path.insert(0, str(REPO / "grazelle-ppopp18_gb300"))

from grazelle import graphgen as gg  # noqa: E402
from oracle import oracle as O  # noqa: E402

OUT = Path(__file__).resolve().parent
PR_ITERS = 16


def sha(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def edge_cases() -> dict[str, gg.EdgeList]:
    cases = {}
    # V not a multiple of 64; vertex 3 has no in-edges, 5 no out-edges; 7 is isolated;
    # destination 0 has 9 in-edges (three vectors, split across work units)
    src = [1, 2, 3, 4, 6, 8, 9, 10, 11, 0, 0, 1, 2, 4, 6, 8, 9, 10, 11, 12, 12]
    dst = [0, 0, 0, 0, 0, 0, 0, 0, 0, 1, 2, 2, 4, 5, 5, 5, 5, 6, 12, 11, 5]
    cases["tiny13"] = gg.EdgeList(13, np.array(src, dtype=np.uint64), np.array(dst, dtype=np.uint64))
    # root 0 has no out-edges (BFS stops at once); 70 vertices
    rng = np.random.default_rng(7)
    s = rng.integers(1, 70, 300, dtype=np.uint64)
    d = rng.integers(0, 70, 300, dtype=np.uint64)
    e = gg._dedup(70, s, d)
    cases["isolated_root70"] = e
    # a star: one hub destination with 1000 in-edges, plus a chain
    hub_src = np.arange(1, 1001, dtype=np.uint64)
    hub_dst = np.zeros(1000, dtype=np.uint64)
    ch_src = np.arange(0, 1000, dtype=np.uint64)
    ch_dst = np.arange(1, 1001, dtype=np.uint64)
    cases["star_chain1001"] = gg._dedup(1001, np.concatenate([hub_src, ch_src]), np.concatenate([hub_dst, ch_dst]))
    return cases


def generated() -> dict[str, tuple[dict, gg.EdgeList]]:
    out = {}
    for scale, seed in ((8, 11), (10, 12), (12, 13)):
        out["rmat%d_s%d" % (scale, seed)] = ({"kind": "rmat", "scale": scale, "edge_factor": 16, "seed": seed}, gg.rmat(scale, seed=seed))
    out["rmat10_sym_s21"] = ({"kind": "rmat_sym", "scale": 10, "edge_factor": 16, "seed": 21}, gg.symmetrize(gg.rmat(10, seed=21)))
    out["er2000_d8_s31"] = ({"kind": "er", "n": 2000, "avg_degree": 8, "seed": 31}, gg.erdos_renyi(2000, 8, seed=31))
    return out


def run_case(name: str, g: gg.EdgeList, spec: dict | None, td: str) -> dict:
    base = str(Path(td) / name)
    gg.write_grazelle(g, base)
    rec: dict = {"name": np.array(name), "V": np.uint64(g.num_vertices), "E": np.uint64(g.num_edges)}
    if spec is None:
        rec["pairs_pull"] = g.pull_order().pairs()
    else:
        for k, v in spec.items():
            rec["spec_" + k] = np.array(v)
    run, (gl, gi, sl, si) = O.run_reference("pr_pull", base, threads=1, iters=PR_ITERS, lists=True)
    run_cc, (_, _, sl, si) = O.run_reference("cc", base, threads=1, lists=True)
    rec["pull_list_sha"] = np.array(sha(gl))
    rec["pull_index_sha"] = np.array(sha(gi))
    rec["push_list_sha"] = np.array(sha(sl))
    rec["push_index_sha"] = np.array(sha(si))
    rec["pull_nvec"] = np.uint64(gl.shape[0])
    rec["push_nvec"] = np.uint64(sl.shape[0])
    if gl.shape[0] <= 4096:
        rec["pull_list"] = gl
        rec["push_list"] = sl
        rec["pull_index"] = gi
        rec["push_index"] = si
    rec["outdeg"] = run.outdeg
    rec["pr_n1"] = run.props
    rec["pr_n4"] = O.run_reference("pr_pull", base, threads=4, iters=PR_ITERS).props
    for var in ("cc", "cc_twc", "cc_pull", "cc_push"):
        r = run_cc if var == "cc" else O.run_reference(var, base, threads=1)
        rec[var + "_labels"] = r.props
        rec[var + "_iters"] = np.array([r.iterations, r.pull_iterations, r.push_iterations], dtype=np.uint64)
    for var in ("bfs", "bfs_twc", "bfs_pull", "bfs_push"):
        r = O.run_reference(var, base, threads=1)
        rec[var + "_parents"] = r.props
        rec[var + "_iters"] = np.array([r.iterations, r.pull_iterations, r.push_iterations], dtype=np.uint64)
    return rec


def main() -> int:
    if not O.reference_available("pr_pull"):
        print("make_golden: reference binaries missing; run python oracle/build_ref.py first")
        return 1
    with tempfile.TemporaryDirectory() as td:
        for name, g in edge_cases().items():
            np.savez_compressed(OUT / (name + ".npz"), **run_case(name, g, None, td))
            print("wrote", name)
        for name, (spec, g) in generated().items():
            np.savez_compressed(OUT / (name + ".npz"), **run_case(name, g, spec, td))
            print("wrote", name)
    return 0


if __name__ == "__main__":
    sys.exit(main())
