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


def reference_output_file(app, rec, V):
    """The bytes graph_data_write_ranks_to_file (source/graphdata.c:1119-1138) writes from the
    reference's own props (the golden fixture, single-thread run): PageRank "%llu %.5le" of
    prop * deg', CC and BFS "%llu %.0lf" of the prop.  Python's %-formatting of a double is
    correctly rounded, as glibc's printf is, so the text is the reference's byte for byte."""
    if app == "pr":
        od = rec["outdeg"][:V]
        vals = rec["pr_n1"][:V] * np.where(od == 0.0, float(V), od)
        return "".join("%d %.5e\n" % (i, x) for i, x in enumerate(vals))
    vals = rec["cc_labels"][:V] if app == "cc" else rec["bfs_parents"][:V]
    return "".join("%d %.0f\n" % (i, x) for i, x in enumerate(vals))


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["rmat10_s12", "rmat10_sym_s21", "tiny13", "isolated_root70", "star_chain1001", "er2000_d8_s31"])
@pytest.mark.parametrize("app", ["pr", "cc", "bfs"])
def test_driver_output_file_is_the_reference_file(app, name, tmp_path):
    """The -o file equals, byte for byte, the one the reference writes on the same graph (16
    PageRank iterations); the stdout carries the reference's load, scheduler and statistics
    lines (source/graphdata.c:435-470, source/main.c:73-145)."""
    from grazelle import graphgen as gg
    rec, g = load_golden(name)
    V = g.num_vertices
    base = str(tmp_path / "g")
    gg.write_grazelle(g, base)
    out = tmp_path / "out.txt"
    r = run([exe(app), "-i", base, "-N", "16", "-n", "4", "-o", str(out)])
    assert r.returncode == 0, r.stdout + r.stderr
    assert out.read_text() == reference_output_file(app, rec, V)
    lines = r.stdout.splitlines()
    nvec = int(rec["pull_nvec"])
    assert "Vertices:  assigned using in-edge list" in lines
    assert "Vertices:  node 0 gets %d vertices (0 to %d, 100.00%% of total)" % (V, V - 1) in lines
    assert "Scheduler: total units = 128, vectors per unit = %d" % (nvec // 128) in lines
    assert lines.index("Scheduler: total units = 128, vectors per unit = %d" % (nvec // 128)) < \
        [i for i, l in enumerate(lines) if l.startswith("Loading graph took")][0]
    assert "EXECUTION STATISTICS" in r.stdout
    if app == "pr":
        assert "PageRank Sum              = 1.0000000000" in r.stdout or "PageRank Sum              = 0.9999999999" in r.stdout
    elif app == "bfs":
        it = rec["bfs_iters"]
        assert "Total Iterations          = %d" % it[0] in r.stdout
        assert "Pull-Based Iterations     = %d" % it[1] in r.stdout
    # -s: a granularity the graph is too small for (main.c:77-86)
    r = run([exe(app), "-i", base, "-s", str(nvec + 1)])
    assert r.returncode == 1 and "Unable to set requested scheduler granularity because the graph is too small." in r.stdout


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


@pytest.mark.gpu
@pytest.mark.parametrize("app,flags", [("cc", []), ("bfs", []), ("bfs", ["THRESHOLD_WITHOUT_COUNT"]), ("cc", ["THRESHOLD_WITHOUT_OUTDEGREES"])])
def test_driver_iteration_profile(app, flags, tmp_path):
    """EXPERIMENT_ITERATION_PROFILE (source/main.c:43-55,110-112, source/execution_bfs.c:127-215):
    a CSV on stderr with one row per iteration: its number, the engine, the edge phase's time
    (nanoseconds here, TSC cycles in the reference) and the vote it was chosen on over E (over V
    without outdegrees).  The engines and the first row's ratio follow the reference's rule."""
    from grazelle import build
    from grazelle import graphgen as gg
    rec, g = load_golden("rmat10_sym_s21")
    V, E = g.num_vertices, g.num_edges
    base = str(tmp_path / "g")
    gg.write_grazelle(g, base)
    build.build()
    r = run([str(build.build_driver(app, ["ITERATION_PROFILE"] + flags)), "-i", base])
    assert r.returncode == 0, r.stdout + r.stderr
    err = r.stderr.splitlines()
    col = {(): "HasInfo (Vertices + Edges) / Total Edges", ("THRESHOLD_WITHOUT_COUNT",): "HasInfo Edges / Total Edges",
           ("THRESHOLD_WITHOUT_OUTDEGREES",): "HasInfo Vertices / Total Vertices"}[tuple(flags)]
    assert err[0] == "Iteration,Selected Engine,Edge Phase Execution Time (ns)," + col
    rows = [l.split(",") for l in err[1:] if l and l[0].isdigit()]
    stat = {l.split("=")[0].strip(): int(l.split("=")[1]) for l in r.stdout.splitlines()
            if "Iterations" in l and "=" in l}
    assert len(rows) == stat["Total Iterations"]
    assert sum(1 for x in rows if x[1] == "Pull") == stat["Pull-Based Iterations"]
    assert [int(x[0]) for x in rows] == list(range(1, len(rows) + 1))
    assert all(int(x[2]) > 0 for x in rows)
    outdeg = rec["outdeg"][:V]
    if app == "cc":
        v0 = (V if "THRESHOLD_WITHOUT_COUNT" not in flags else 0) + (E if "THRESHOLD_WITHOUT_OUTDEGREES" not in flags else 0)
    else:
        v0 = (1 if "THRESHOLD_WITHOUT_COUNT" not in flags else 0) + (int(outdeg[0]) if "THRESHOLD_WITHOUT_OUTDEGREES" not in flags else 0)
    comparator = V if "THRESHOLD_WITHOUT_OUTDEGREES" in flags else E
    assert abs(float(rows[0][3]) - v0 / comparator) <= 1e-10  # printed with 10 decimals
    thr = V // 2 if "THRESHOLD_WITHOUT_OUTDEGREES" in flags else E // 5
    for x in rows:
        vote = float(x[3]) * comparator  # the vote the engine was chosen on (10 decimals of the ratio)
        if abs(vote - thr) > 1.0:
            assert (x[1] == "Pull") == (vote > thr)
