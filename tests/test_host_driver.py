"""The C host driver (grazelle-gb300-{pr,cc,bfs}): command line, exit codes and outputs."""
import subprocess

import numpy as np
import pytest

from conftest import load_golden
from oracle import oracle as O


def exe(app):
    from grazelle import build
    build.build()
    return str(build.BUILD / ("grazelle-gb300-" + app))


def run(args, **kw):
    return subprocess.run(args, stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True, timeout=300, **kw)


@pytest.mark.parametrize("app", ["pr", "cc", "bfs"])
def test_exit_codes_without_gpu(app, tmp_path):
    e = exe(app)
    assert run([e, "-x"]).returncode == 1            # unknown option (cmdline.c:120-125)
    assert run([e, "-N", "zero", "-i", "g"]).returncode == 2   # invalid value
    assert run([e, "-i"]).returncode == 3            # missing value
    assert run([e, "-h", "x"]).returncode == 4       # extraneous value
    assert run([e]).returncode == 5                  # missing -i
    r = run([e, "-i", str(tmp_path / "nope")])
    assert r.returncode == 255 and "unable to read file" in r.stderr   # graphdata.c:963-967
    # truncated file: header promises more edges than the file holds
    base = tmp_path / "trunc"
    np.array([10, 5, 1, 2], dtype=np.uint64).tofile(str(base) + "-pull")
    assert run([e, "-i", str(base)]).returncode == 255
    v = run([e, "-V"])
    assert v.returncode == 0 and "ppopp18" in v.stdout


@pytest.mark.gpu
@pytest.mark.parametrize("app", ["pr", "cc", "bfs"])
def test_driver_output_matches_reference(app, tmp_path):
    from grazelle import graphgen as gg
    rec, g = load_golden("rmat10_s12")
    base = str(tmp_path / "g")
    gg.write_grazelle(g, base)
    out = tmp_path / "out.txt"
    r = run([exe(app), "-i", base, "-N", "16", "-o", str(out)])
    assert r.returncode == 0, r.stdout + r.stderr
    assert "EXECUTION STATISTICS" in r.stdout
    vals = np.loadtxt(out)
    assert vals.shape == (g.num_vertices, 2)
    np.testing.assert_array_equal(vals[:, 0], np.arange(g.num_vertices))
    if app == "pr":
        od = np.where(rec["outdeg"] == 0, g.num_vertices, rec["outdeg"])
        ranks = rec["pr_n1"] * od
        np.testing.assert_allclose(vals[:, 1], ranks, rtol=1e-5)   # %.5le in the file
        assert "PageRank Sum              = 1.0000000000" in r.stdout or "PageRank Sum              = 0.9999999999" in r.stdout
    elif app == "cc":
        np.testing.assert_array_equal(vals[:, 1], rec["cc_labels"])
        assert "Total Iterations" in r.stdout
    else:
        np.testing.assert_array_equal(vals[:, 1], rec["bfs_parents"])
        it = rec["bfs_iters"]
        assert "Total Iterations          = %d" % it[0] in r.stdout
        assert "Pull-Based Iterations     = %d" % it[1] in r.stdout


@pytest.mark.gpu
@pytest.mark.parametrize("app", ["cc", "bfs"])
def test_driver_derives_a_missing_push_file(app, tmp_path):
    """Without `<base>-push`, the CC and BFS drivers derive that list on the device and print the
    same output file and iteration counts as with both files."""
    import os
    from grazelle import graphgen as gg
    rec, g = load_golden("rmat10_s12")
    both, pull_only = str(tmp_path / "both"), str(tmp_path / "pull")
    gg.write_grazelle(g, both)
    gg.write_grazelle(g, pull_only)
    os.remove(pull_only + "-push")
    outs = []
    for base in (both, pull_only):
        out = tmp_path / (os.path.basename(base) + ".txt")
        r = run([exe(app), "-i", base, "-o", str(out)])
        assert r.returncode == 0, r.stdout + r.stderr
        outs.append((out.read_text(), [l for l in r.stdout.splitlines() if "Iterations" in l]))
    assert outs[0] == outs[1]


@pytest.mark.gpu
def test_driver_experiments_iteration_stats_and_long_vectors(tmp_path):
    """EXPERIMENT_ITERATION_STATS prints the reference's per-iteration CSV to stderr (one row per
    iteration); EXPERIMENT_MODEL_LONG_VECTORS prints the 8- and 16-lane vector counts and stops."""
    from grazelle import build
    from grazelle import graphgen as gg
    rec, g = load_golden("rmat10_s12")
    base = str(tmp_path / "g")
    gg.write_grazelle(g, base)
    build.build()
    r = run([str(build.build_driver("cc", ["ITERATION_STATS"])), "-i", base])
    assert r.returncode == 0, r.stdout + r.stderr
    rows = [l for l in r.stderr.splitlines() if l and l[0].isdigit()]
    assert r.stderr.splitlines()[0] == "Iteration,# Vectors,Packing Efficiency"
    total = int([l for l in r.stdout.splitlines() if l.startswith("Total Iterations")][0].split("=")[1])
    assert len(rows) == total
    for i, row in enumerate(rows):
        it, nv, eff = row.split(",")
        assert int(it) == i + 1 and int(nv) >= 0 and 0.0 <= float(eff) <= 1.0
    r = run([str(build.build_driver("bfs", ["MODEL_LONG_VECTORS"])), "-i", base])
    assert r.returncode == 0, r.stdout + r.stderr
    pull = g.pull_order().pairs()
    indeg = np.bincount(pull[1::2].astype(np.int64), minlength=g.num_vertices)
    for lanes in (8, 16):
        n = int(np.sum((indeg + lanes - 1) // lanes))
        assert "In-edges:  VL%d: created %d vectors" % (lanes, n) in r.stdout
    assert "Not executing application" in r.stdout and "EXECUTION STATISTICS" not in r.stdout
