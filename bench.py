#!/usr/bin/env python3
"""Benchmark of the GB300 Grazelle engine: one JSON line per run.

Default workload: Connected Components, the configuration the metric is
quoted on.  The graph is a symmetrised R-MAT of scale 24 (edge factor 16,
a/b/c/d = .57/.19/.19/.05, seeded), run to convergence with the reference's
threshold engine switch.  One step is one full CC run.

  value     GTEPS = E x iterations / device time, graph resident in HBM (the reference's
            "Effective Processing Rate", source/main.c:129)
  e2e       the same metric through the C ABI from pinned HOST edge lists.  Each step does
            the H2D copy of the -pull pairs (grz_graph_load_pairs_ex with
            GRZ_LOAD_DERIVE_PUSH: the library derives the -push list on the device; --ingest
            both copies both lists instead), builds the vector-sparse layout on the device,
            runs CC and reads the labels back (D2H).
  roofline  the dominant kernel's algorithmic bytes per launch over its mean CUDA-event
            duration, against the measured HBM copy peak.  For CC the dominant record is a
            run's first pull; its bytes are those of the default pull form (row pointers, first
            vectors and labels, bitmaps, the vectors of the destinations still above 0, counted
            on the device), with the reference's full-pass bytes beside them (work_equivalent)
  apps      PageRank (R-MAT 20), BFS (R-MAT 26, 64 roots, both engine policies), the batch of
            PPR and multi-source BFS, the R-MAT 27 stress graph (PageRank and CC), each with
            parity, roofline, e2e and a CPU baseline where one fits
  cpu_baseline  the reference's algorithm on the host cores: the reference binary where it
            runs (x86-64 AVX2), else the OpenMP restatement in oracle/

`--impl reference` times only the CPU implementation, on all host threads.

Usage: python bench.py [--gpus N] [--steps K] [--warmup W] [--impl native|reference]
                       [--workload cc|pr|bfs|batch] [--scale S] [--no-tune]
Multi-GPU (torchrun): independent replicas, one graph per GPU ("replicas only"): nothing in
the path exchanges data between GPUs.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

REPO = Path(__file__).resolve().parent
sys.path.insert(0, str(REPO))
sys.path.insert(0, str(REPO / "grazelle-ppopp18_gb300"))

import numpy as np  # noqa: E402

FALLBACK_HBM_GBS = 6800.0
DEFAULT_SCALE = {"cc": 24, "pr": 20, "bfs": 24}


# ---------------------------------------------------------------------------------------------- helpers

def log(*a):
    print(*a, file=sys.stderr, flush=True)


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def combine_ranks(units: float, ms: float, dist=None, device: str = "cuda"):
    """Whole-job (units, ms) over the replicas: units summed over ranks, time the slowest rank's
    (max over ranks).  Without a process group the local values pass through."""
    if dist is None:
        return units, ms
    import torch
    t = torch.tensor([float(units), float(ms)], dtype=torch.float64, device=device)
    u = t[:1].clone()
    m = t[1:].clone()
    dist.all_reduce(u, op=dist.ReduceOp.SUM)
    dist.all_reduce(m, op=dist.ReduceOp.MAX)
    return float(u.item()), float(m.item())


def measured_hbm():
    p = REPO / "MEASURED_PEAKS.json"
    try:
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return FALLBACK_HBM_GBS, "fallback"


def profile_traffic(kernel: str, workload: str):
    """DRAM bytes per launch of `kernel` from the committed ncu summary, if one exists."""
    p = REPO / "profiles" / "traffic.json"
    try:
        d = json.loads(p.read_text())
        return d.get(workload, {}).get(kernel)
    except Exception:
        return None


def nonempty_destinations(G, V):
    """Vertices with in-vectors (the pull list's vertex index marks the others)."""
    vi = G.vertex_index()[:V]
    n = int(np.count_nonzero(vi < np.uint64(0x7fffffffffffffff)))
    del vi
    return n


def cc_first_pull_bytes(G, V, open_vectors=None):
    """Bytes the first CC pull of a run moves in its default form (GRZ_TUNE_CC_PULL_FIRST 4):
    row pointers 4(V+1); per destination with in-vectors its first vector (16) and its label read
    and written (8); HasInfo* V/8; the compaction's two bitmaps V/4; and per vector of the
    destinations still above 0 (counted on the device while profiling) its 16 bytes and its
    destination's label (4).  In form 1 or 3 the whole-list pass reads the 4N-byte destination
    stream and a label per destination instead of those vectors (a lower bound: the open
    destinations' vectors come on top).  Returns (bytes, basis)."""
    vne = nonempty_destinations(G, V)
    N = int(G.info().pull_vectors)
    base = 4 * (V + 1) + 24 * vne + V // 8
    if open_vectors is not None:
        return base + V // 4 + 20 * open_vectors, (
            "first-vector pass and open-destination pull: row pointers, each destination's first vector and label, "
            "HasInfo*, the compaction's bitmaps, and the %d vectors of the destinations still above 0 "
            "(%d destinations with in-vectors)" % (open_vectors, vne))
    return base + 4 * N + 4 * V, (
        "first-vector pass and whole-list pass: row pointers, each destination's first vector and label, HasInfo*, "
        "the destination stream and labels (%d destinations with in-vectors, %d vectors; the vectors of destinations "
        "still above 0 come on top)" % (vne, N))


def cc_first_pull_roofline(G, V, E, ms, hbm, hbm_kind, open_vectors=None):
    """Roofline entry of the first CC pull of a run (the dominant launch).  With the first-vector
    pass (the default), the algorithmic bytes are cc_first_pull_bytes; the bytes of the full pass
    over every vector (8E + 16V + V/4, the reference's pull) are reported as work-equivalent."""
    full = 8 * E + 16 * V + V // 4
    wk = full / (ms * 1e-3) / 1e9
    form = G.tuning().get("cc_pull_first", 0)
    if form:
        b, basis = cc_first_pull_bytes(G, V, open_vectors if form == 4 else None)
    else:
        b, basis = full, "full pass over every vector (8E + 16V + V/4)"
    ach = b / (ms * 1e-3) / 1e9
    return {"bound": "hbm", "kernel": "cc_pull", "achieved": round(ach, 1), "peak": hbm, "peak_kind": hbm_kind, "unit": "GB/s",
            "frac": round(ach / hbm, 4), "algorithmic_bytes": b, "basis": basis, "mean_launch_ms": round(ms, 4),
            "work_equivalent": {"bytes": full, "achieved": round(wk, 1), "frac": round(wk / hbm, 4),
                                "basis": "bytes of the reference's full pull pass; the skip reads fewer"}}


class ClockSampler:
    """nvidia-smi clock / throttle-reason samples every 200 ms while the timed region runs."""

    FIELDS = "index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown," \
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap"

    def __init__(self, gpu: int):
        self.gpu = gpu
        self.proc = None
        self.lines = []
        self.t = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.FIELDS,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
            time.sleep(0.3)
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for ln in self.proc.stdout:
            self.lines.append(ln.strip())

    def __exit__(self, *exc):
        if self.proc:
            time.sleep(0.25)
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [x.strip() for x in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx = max(mx, float(parts[2]))
            except ValueError:
                continue
            for k, n in enumerate(names):
                if parts[5 + k].lower().startswith("active"):
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sm)}


def make_graph(workload: str, scale: int, seed: int = 1, directed: bool = False):
    from grazelle import graphgen as gg
    g = gg.rmat(scale, 16, seed=seed, symmetric=workload in ("cc", "bfs") and not directed)
    push = g.push_order().pairs()
    pull = g.pull_order().pairs()
    return g, pull, push


def make_graph_lean(workload: str, scale: int, seed: int = 1, directed: bool = False):
    """Large graphs: only the -pull pairs stay on the host (the library derives the -push list on
    the device), and the generator's arrays are dropped as soon as they are used."""
    from grazelle import graphgen as gg
    g = gg.rmat(scale, 16, seed=seed, symmetric=workload in ("cc", "bfs") and not directed)
    V, E = g.num_vertices, g.num_edges
    p = g.pull_order()
    del g
    pull = p.pairs()
    del p
    return V, E, pull


def pick_roots(g, n: int, seed: int = 7):
    deg = g.out_degrees()
    cand = np.nonzero(deg)[0]
    rng = np.random.default_rng(seed)
    return [int(x) for x in rng.choice(cand, size=min(n, cand.shape[0]), replace=False)]


# ---------------------------------------------------------------------------------------------- native arm

class Timer:
    """CUDA events on the graph's (torch) stream."""

    def __init__(self, torch, stream):
        self.torch = torch
        self.stream = stream

    def __enter__(self):
        self.e0 = self.torch.cuda.Event(enable_timing=True)
        self.e1 = self.torch.cuda.Event(enable_timing=True)
        self.torch.cuda.synchronize()
        self.e0.record(self.stream)
        return self

    def __exit__(self, *exc):
        self.e1.record(self.stream)
        self.torch.cuda.synchronize()
        self.ms = self.e0.elapsed_time(self.e1)


def kernel_stats(records):
    agg = {}
    for k, ms in records:
        agg.setdefault(k, []).append(ms)
    return {k: {"n": len(v), "mean_ms": sum(v) / len(v), "total_ms": sum(v)} for k, v in agg.items()}


def run_native(a):
    import torch

    from grazelle.engine import Graph

    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    stream = torch.cuda.Stream()
    wl = a.workload
    scale = a.scale or DEFAULT_SCALE[wl]
    t0 = time.time()
    lean = a.lean or scale >= 26
    if lean:
        g, push = None, None
        V, E, pull = make_graph_lean(wl, scale, a.seed, a.directed)
    else:
        g, pull, push = make_graph(wl, scale, a.seed, a.directed)
        V, E = g.num_vertices, g.num_edges
    log("graph: %s scale %d V=%d E=%d (%.1fs)%s" % (wl, scale, V, E, time.time() - t0, " lean" if lean else ""))
    pin_pull = torch.from_numpy(pull.view(np.int64)).pin_memory()
    # the e2e leg hands the library the -pull pairs only (it derives the -push list on the device)
    # unless --ingest both, which copies both lists as the reference reads both files
    derive = lean or a.ingest == "pull"
    pin_push = torch.from_numpy(push.view(np.int64)).pin_memory() if (push is not None and not derive) else None
    pull_bytes, push_bytes = int(pull.nbytes), (int(push.nbytes) if pin_push is not None else 0)
    if lean:
        deg_lean = np.bincount(pull[0::2].astype(np.int64), minlength=V) if wl == "bfs" else None
        del pull
    G = Graph(local, stream=stream.cuda_stream)

    def load():
        if derive:
            G.load_pull_derive_push(V, E, pin_pull.data_ptr())
        else:
            G.load_pointers(V, E, pin_pull.data_ptr(), pin_push.data_ptr())

    if a.pr_props:
        G.tune(pr_props=a.pr_props)
    for kv in a.tune:
        k, v = kv.split("=", 1)
        G.tune(**{k: int(v)})
    load()
    hbm, hbm_kind = measured_hbm()
    # kernel shapes for this graph, chosen by timing (outside every timed region)
    tuned = None
    if not a.no_tune:
        from grazelle import autotune
        tuned = autotune.tune_cc(G, device=local) if wl in ("cc", "bfs") else autotune.tune_pr(G, device=local)
        tuned.pop("trials", None)
        tuned["gain"] = round(tuned["default_ms"] / tuned["best_ms"], 4) if tuned.get("default_ms") else None

    def barrier():
        if dist:
            dist.barrier()
        torch.cuda.synchronize()


    # one step of the workload, graph resident; returns (teps units, iterations)
    if wl == "bfs":
        roots = pick_roots(g, 8) if g is not None else [int(x) for x in np.random.default_rng(7).choice(np.nonzero(deg_lean)[0], 8, replace=False)]
    else:
        roots = []

    # (results stay on the device; the e2e loop below reads them back)
    def step(i):
        if wl == "cc":
            st = G.cc_run()
            return E * st.iterations, st.iterations
        if wl == "pr":
            G.pr_init(0.875).pr_iterate(16)
            G.sync()
            return E * 16, 16
        root = roots[i % len(roots)]
        st = G.bfs_run(root)
        _, reached_edges, _ = G.digest()
        return reached_edges, st.iterations

    for i in range(a.warmup):
        step(i)
    barrier()
    l0 = G.launch_count()
    units = 0
    iters = 0
    with ClockSampler(local) as clk:
        with Timer(torch, stream) as tm:
            for i in range(a.steps):
                u, it = step(i)
                units += u
                iters += it
    launches = G.launch_count() - l0
    units_all, ms = combine_ranks(units, tm.ms, dist)
    value = units_all / (ms * 1e-3) / 1e9

    # Per-kernel CUDA-event durations for the roofline: the same K steps once more with kernel
    # profiling on.  The event pairs need host-launched kernels, so CC/BFS run their host loop
    # here (the same kernels as the graph the headline region launches).
    G.profile(True)
    G.profile_work()
    recs, first_pull = [], []
    with Timer(torch, stream) as tprof:
        for i in range(a.steps):
            step(i)
            r = G.profile_read()
            recs += r
            # the first pull record of a CC run (no previous minimum to skip by yet)
            fp = [ms for k, ms in r if k == "cc_pull"]
            if fp:
                first_pull.append(fp[0])
    open_vectors = G.profile_work()[0] // max(1, len(first_pull))
    G.profile(False)
    ks = kernel_stats(recs)
    dominant = max(ks.items(), key=lambda kv: kv[1]["total_ms"])[0] if ks else None

    # algorithmic bytes per launch of the dominant kernel (8E + 16V for a pull pass; V/4 more for
    # the two CC bitmaps)
    alg = {"pr_gather": 8 * E + 16 * V, "cc_pull": 8 * E + 16 * V + V // 4, "bfs_pull": 8 * E + 16 * V + V // 4}
    roof = None
    if dominant:
        mean_ms = ks[dominant]["mean_ms"]
        region = "profiled pass of the same %d steps" % a.steps
        if dominant == "cc_pull" and first_pull:
            mean_ms = sum(first_pull) / len(first_pull)
            region += ", first pull of each run"
        mean_s = mean_ms * 1e-3
        if dominant == "cc_pull" and first_pull:
            roof = cc_first_pull_roofline(G, V, E, mean_ms, hbm, hbm_kind, open_vectors)
            roof.update({"share_of_profiled_pass": round(ks[dominant]["total_ms"] / tprof.ms, 4), "region": region,
                         "traffic": profile_traffic(dominant, "%s%d" % (wl, scale)) if not a.tune else None})
        elif dominant in alg:
            achieved = alg[dominant] / mean_s / 1e9
            roof = {"bound": "hbm", "kernel": dominant, "achieved": round(achieved, 1), "peak": hbm, "peak_kind": hbm_kind,
                    "unit": "GB/s", "frac": round(achieved / hbm, 4), "algorithmic_bytes": alg[dominant],
                    "mean_launch_ms": round(mean_ms, 4),
                    "share_of_profiled_pass": round(ks[dominant]["total_ms"] / tprof.ms, 4),
                    "region": region,
                    "traffic": profile_traffic(dominant, "%s%d" % (wl, scale)) if not a.tune else None}

    # end to end through the C ABI from pinned host buffers
    e2e_units = 0
    # the results come back into pinned host memory, as the pairs go out of it
    d2h_t = torch.zeros(V, dtype=torch.float64).pin_memory()
    d2h = d2h_t.numpy()
    for i in range(max(1, min(2, a.warmup))):
        load()
        step(i)
    barrier()
    with Timer(torch, stream) as te:
        for i in range(a.steps):
            load()
            u, _ = step(i)
            e2e_units += u
            G.lib.grz_read_props(G.h, d2h.ctypes.data, V)
    e2e_units_all, e2e_ms = combine_ranks(e2e_units, te.ms, dist)
    e2e = {"value": round(e2e_units_all / (e2e_ms * 1e-3) / 1e9, 3), "unit": "GTEPS",
           "h2d_bytes_per_step": pull_bytes + push_bytes, "d2h_bytes_per_step": int(d2h.nbytes),
           "ingest": ("the -pull pairs; the -push list derived on the device" if derive else "both lists"),
           "ms_per_step": round(e2e_ms / a.steps, 3)}

    apps = {}
    if rank == 0 and not a.no_apps and wl == "cc" and not lean:
        apps = extra_apps(a, G, g, torch, stream, hbm, hbm_kind)
    cpu = None
    parity = {}
    if rank == 0 and not a.no_cpu and not lean:
        cpu, ref_out = cpu_baseline(wl, g, pull, push, scale, sample=True)
        if wl == "cc":
            # the labels of the last e2e step (read back through the C ABI) against the CPU run's
            parity["cc_labels_exact"] = bool(np.array_equal(d2h, ref_out[:V]))
            parity["cc_labels_checked"] = "all %d vertices, the GPU run of the last e2e step against the OpenMP restatement" % V
        del ref_out
    elif rank == 0 and lean:
        cpu = {"value": None, "unit": "GTEPS", "cores": os.cpu_count(), "kind": "port",
               "sample": "not run: the CPU restatement's layout of a graph this size does not fit a bounded sample"}
    if dist:
        dist.barrier()
    if rank != 0:
        return
    line = {
        "metric": "GTEPS (%s, E x iterations / time)" % {"cc": "connected components", "pr": "pagerank pull", "bfs": "bfs"}[wl],
        "value": round(value, 3), "unit": "GTEPS", "n_gpus": world, "steps": a.steps, "warmup": a.warmup,
        "ms_per_step": round(ms / a.steps, 3), "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": {"cc": "u32", "pr": "u128 fixed point + f64", "bfs": "u32"}[wl], "data": "synthetic (seeded R-MAT)",
        "config": {"workload": "%s-rmat%d%s" % (wl, scale, "-sym" if wl != "pr" and not a.directed else ""), "scale": scale, "edge_factor": 16,
                   "rmat_abcd": [0.57, 0.19, 0.19, 0.05], "seed": a.seed, "V": V, "E": E,
                   "engine": "threshold heuristic (E/5)" if wl != "pr" else "pull", "iterations_per_step": iters / a.steps,
                   "l2": "inputs larger than L2 (%.1f GB of edge vectors)" % (G.info().pull_vectors * 20 / 1e9),
                   "parallelism": "replicas" if world > 1 else "single GPU", "autotuned": tuned},
        "roofline": roof, "kernels": {k: {"n": v["n"], "mean_us": round(v["mean_ms"] * 1e3, 2)} for k, v in ks.items()},
        "e2e": e2e, "gpu_launches": int(launches), "clocks": clk.summary(), "cpu_baseline": cpu, "parity": parity,
        "apps": apps,
    }
    for name, app in apps.items():
        if isinstance(app, dict) and "parity" in app:
            parity[name] = app["parity"]
    print(json.dumps(line), flush=True)


def extra_apps(a, G_cc, g_cc, torch, stream, hbm, hbm_kind):
    """CC under the learned switch on the headline graph, the BFS switch study (directed R-MAT
    26, 64 roots, threshold vs learned), and PageRank on R-MAT 20 (16 pull iterations)."""
    from grazelle import native
    from grazelle import switch as sw
    from grazelle.engine import Graph
    out = {}
    dev = torch.cuda.current_device()
    net = sw.pretrained(dev)
    # CC on the headline graph under both policies (device time per run, identical labels)
    cc = {}
    for name, policy, mlp in (("threshold", native.POLICY_THRESHOLD, None), ("learned", native.POLICY_LEARNED, net)):
        G_cc.set_policy(policy, mlp)
        G_cc.cc_run()
        tot, digs = 0.0, set()
        for _ in range(max(1, a.steps)):
            st = G_cc.cc_run()
            tot += st.ms
            digs.add(G_cc.digest())
        cc[name] = {"ms_per_run": round(tot / max(1, a.steps), 3), "iterations_pull_push": [st.iterations, st.pull_iterations,
                                                                                           st.push_iterations]}
        cc[name]["digest"] = sorted(digs)
    G_cc.set_policy(native.POLICY_THRESHOLD)
    cc["identical_labels"] = cc["threshold"]["digest"] == cc["learned"]["digest"]
    for k in ("threshold", "learned"):
        cc[k].pop("digest")
    cc["learned_speedup"] = round(cc["threshold"]["ms_per_run"] / cc["learned"]["ms_per_run"], 4)
    out["cc_switch"] = cc
    if a.bfs_scale:
        out["bfs_switch"] = bfs_switch_study(a, torch, stream, net, dev, hbm, hbm_kind)
    if not a.no_batch:
        out["batch"] = batch_study(a, torch, stream, dev)
    if a.stress_scale:
        out["stress"] = stress_study(a, torch, stream, dev, hbm, hbm_kind)
    out["pagerank"] = pagerank_study(a, torch, stream, hbm, hbm_kind)
    return out


def pagerank_study(a, torch, stream, hbm, hbm_kind, scale=20):
    """PageRank on R-MAT `scale` (16 pull iterations, d = 0.875, FP64 props): device-resident
    GTEPS, the gather kernel's roofline, e2e through the C ABI (the -pull pairs from pinned host
    memory, layout build, 16 iterations, props back), the OpenMP restatement on the host cores,
    and parity of the props with the serial oracle (relative L1, bound 1e-12)."""
    from grazelle.engine import Graph
    from oracle import oracle as O
    g, pull, push = make_graph("pr", scale, a.seed)
    V, E = g.num_vertices, g.num_edges
    res = {"workload": "pr-rmat%d, 16 iterations, d=0.875" % scale, "V": V, "E": E}
    pin_pull = torch.from_numpy(pull.view(np.int64)).pin_memory()
    d2h_t = torch.zeros(V, dtype=torch.float64).pin_memory()
    d2h = d2h_t.numpy()
    n = max(2, a.steps // 2)
    with Graph(torch.cuda.current_device(), stream=stream.cuda_stream) as G:
        G.load_pairs(V, pull, push)
        if not a.no_tune:
            from grazelle import autotune
            t = autotune.tune_pr(G, device=torch.cuda.current_device())
            res["autotuned"] = {"best": t["best"], "best_ms": round(t["best_ms"], 4),
                                "default_ms": round(t["default_ms"], 4) if t["default_ms"] else None,
                                "candidates": t["candidates"], "objective": t["objective"]}
        G.pr_init(0.875).pr_iterate(16)
        with Timer(torch, stream) as tp:
            for _ in range(n):
                G.pr_init(0.875).pr_iterate(16)
        G.profile(True)
        for _ in range(n):
            G.pr_init(0.875).pr_iterate(16)
        G.sync()
        ks = kernel_stats(G.profile_read())
        G.profile(False)
        props = G.pr_init(0.875).pr_iterate(16).props()
        alg = 8 * E + 16 * V
        gm = ks.get("pr_gather", {}).get("mean_ms", 0)
        it_ms = tp.ms / (16 * n)
        res.update({"gteps": round(E * 16 * n / (tp.ms * 1e-3) / 1e9, 3), "us_per_iteration": round(it_ms * 1e3, 2),
                    "kernels_us": {k: round(v["mean_ms"] * 1e3, 2) for k, v in ks.items()}})
        res["roofline"] = {"bound": "hbm", "kernel": "pr_gather", "algorithmic_bytes": alg,
                           "achieved": round(alg / (gm * 1e-3) / 1e9, 1) if gm else None, "peak": hbm, "peak_kind": hbm_kind,
                           "unit": "GB/s", "frac": round(alg / (gm * 1e-3) / 1e9 / hbm, 4) if gm else None,
                           "mean_launch_us": round(gm * 1e3, 2),
                           "iteration_frac": round(alg / (it_ms * 1e-3) / 1e9 / hbm, 4),
                           "traffic": profile_traffic("pr_gather", "pr%d" % scale) if not a.tune else None}
        # e2e: the -pull pairs cross the link each step (PageRank pull needs no -push list)
        for _ in range(2):
            G.load_pointers(V, E, pin_pull.data_ptr(), None)
            G.pr_init(0.875).pr_iterate(16)
            G.lib.grz_read_props(G.h, d2h.ctypes.data, V)
        with Timer(torch, stream) as te:
            for _ in range(n):
                G.load_pointers(V, E, pin_pull.data_ptr(), None)
                G.pr_init(0.875).pr_iterate(16)
                G.lib.grz_read_props(G.h, d2h.ctypes.data, V)
        res["e2e"] = {"value": round(E * 16 * n / (te.ms * 1e-3) / 1e9, 3), "unit": "GTEPS", "h2d_bytes_per_step": int(pull.nbytes),
                      "d2h_bytes_per_step": int(d2h.nbytes), "ms_per_step": round(te.ms / n, 3),
                      "ingest": "the -pull pairs (the pull engine needs no -push list)"}
        e2e_err = O.relative_l1(d2h, props[:V])
    L = O.layout(V, pull, push)
    ref = O.pr_pull(L, 16, 0.875)[:V]
    del L
    res["parity"] = {"props_rel_l1_vs_oracle": O.relative_l1(props[:V], ref), "bound": 1e-12,
                     "e2e_props_equal_resident": e2e_err == 0.0}
    res["parity"]["ok"] = res["parity"]["props_rel_l1_vs_oracle"] < 1e-12 and res["parity"]["e2e_props_equal_resident"]
    cpu, _ = cpu_baseline("pr", g, pull, push, scale, sample=True)
    res["cpu_baseline"] = cpu
    return res


def bfs_kernel_rooflines(G, roots, outdeg, indeg, hbm, hbm_kind):
    """Algorithmic bytes over CUDA-event time of the BFS edge kernels, from profiled host-loop
    runs: iteration k's push reads the frontier F = {level k-1}: 8 x (out-edges of F) + 8|F| +
    16|U|, U = {level k} the updates; its pull reads every vector of the wanted destinations W
    (unvisited, with in-edges): 8 x (in-edges of W) + 8|W| + 16|U|.  That is the reference's
    pull, which scans them all; the early-exit pass stops at each destination's first vector with
    a frontier source and reads far fewer, so the pull's figure is work-equivalent bandwidth (its
    DRAM traffic is in the launch-list summary), marked by `basis`."""
    agg = {"bfs_pull": [0, 0.0, 0], "bfs_push": [0, 0.0, 0]}
    G.profile(True)
    for r in roots:
        G.bfs_run(r)
        recs = [(k, ms) for k, ms in G.profile_read() if k in agg]
        lv = G.levels()
        nl = int(lv.max()) + 2
        key = np.where(lv < 0, nl, lv)  # unreached last
        cnt = np.bincount(key, minlength=nl + 1)
        out_by = np.bincount(key, weights=outdeg, minlength=nl + 1)
        has_in = indeg > 0
        w_cnt = np.bincount(key, weights=has_in.astype(np.float64), minlength=nl + 1)
        in_by = np.bincount(key, weights=indeg, minlength=nl + 1)
        for i, (kind, ms) in enumerate(recs):
            k = i + 1  # iteration k visits level k
            upd = cnt[k] if k < nl else 0
            if kind == "bfs_push":
                b = 8 * out_by[k - 1] + 8 * cnt[k - 1] + 16 * upd
            else:
                b = 8 * in_by[k:].sum() + 8 * w_cnt[k:].sum() + 16 * upd
            agg[kind][0] += 1
            agg[kind][1] += ms
            agg[kind][2] += int(b)
    G.profile(False)
    out = {}
    for kind, (n, ms, b) in agg.items():
        if n:
            gbs = b / (ms * 1e-3) / 1e9
            out[kind] = {"launches": n, "total_ms": round(ms, 3), "algorithmic_bytes": b, "achieved": round(gbs, 1),
                         "peak": hbm, "peak_kind": hbm_kind, "unit": "GB/s", "frac": round(gbs / hbm, 4),
                         "basis": "bytes the reference's full pass over the wanted destinations reads (the early exit "
                                  "reads fewer: work-equivalent)" if kind == "bfs_pull" else "bytes the push reads"}
    return out


def bfs_switch_study(a, torch, stream, net, dev, hbm=None, hbm_kind=None):
    """BFS on a directed R-MAT (default scale 26, edge factor 16) from 64 seeded non-isolated
    roots under the threshold rule and the learned switch: GTEPS from the device time of each
    run, identical levels checked by an on-device digest, and the edge-phase regret of both
    policies against the best engine per iteration on 4 of the roots.  Also: parity of 4 roots
    (levels equal to the oracle's, parents a legal BFS tree), the BFS kernels' rooflines, e2e
    through the C ABI (the -pull pairs from pinned host memory, the -push list derived on the
    device, 64 roots, a digest read back per root) and the OpenMP restatement on the host."""
    from grazelle import graphgen as gg
    from grazelle import native
    from grazelle import switch as sw
    from grazelle.engine import Graph
    from oracle import oracle as O
    t0 = time.time()
    g = gg.rmat(a.bfs_scale, 16, seed=a.seed + 26)
    V, E = g.num_vertices, g.num_edges
    roots = pick_roots(g, 64, seed=a.seed + 64)
    pull, push = g.pull_order().pairs(), g.push_order().pairs()
    del g
    log("bfs graph: scale %d V=%d E=%d (%.1fs)" % (a.bfs_scale, V, E, time.time() - t0))
    res = {"workload": "bfs-rmat%d (directed), %d roots" % (a.bfs_scale, len(roots)), "V": V, "E": E}
    with Graph(dev, stream=stream.cuda_stream) as G:
        G.load_pairs(V, pull, push)
        digests = {}
        for name, policy, mlp in (("threshold", native.POLICY_THRESHOLD, None), ("learned", native.POLICY_LEARNED, net)):
            G.set_policy(policy, mlp)
            for r in roots[:3]:
                G.bfs_run(r)
            ms, teps, npull, npush, dg = 0.0, 0, 0, 0, []
            for r in roots:
                st = G.bfs_run(r)
                reached, edges, h = G.digest()
                ms += st.ms
                teps += edges
                npull += st.pull_iterations
                npush += st.push_iterations
                dg.append((reached, edges, h))
            digests[name] = dg
            res[name] = {"ms_total": round(ms, 3), "ms_per_root": round(ms / len(roots), 4),
                         "gteps": round(teps / (ms * 1e-3) / 1e9, 3), "pull_iterations": npull, "push_iterations": npush}
        res["identical_levels"] = digests["threshold"] == digests["learned"]
        res["learned_speedup"] = round(res["threshold"]["ms_total"] / res["learned"]["ms_total"], 4)
        # parity: 4 roots under the learned switch against the oracle's levels, parents a legal tree
        chk = roots[:4]
        ref = O.bfs_levels_multi(push, V, chk)
        lv_ok, tree_ok = True, True
        for k, r in enumerate(chk):
            par, lv = G.bfs(r)
            lv_ok &= bool(np.array_equal(lv, ref[k]))
            tree_ok &= O.bfs_check_tree(push, V, r, lv, par.astype(np.int64)) == 0
        del ref
        res["parity"] = {"roots_checked": len(chk), "levels_exact": lv_ok, "parents_legal_bfs_tree": tree_ok,
                         "policies_identical_levels_64_roots": res["identical_levels"], "ok": lv_ok and tree_ok and res["identical_levels"]}
        G.set_policy(native.POLICY_THRESHOLD)
        d = sw.Samples()
        d.extend(sw.collect(G, native.APP_BREADTH_FIRST_SEARCH, roots[:4]))
        e = sw.edge_totals(d, net)
        res["edge_phase_regret_4_roots"] = {"threshold_ms": round(e["threshold_ms"], 4), "learned_ms": round(e["learned_ms"], 4),
                                            "best_per_iteration_ms": round(e["best_ms"], 4), "iterations": e["iterations"],
                                            "learned_regret": round(e["learned_ms"] / e["best_ms"] - 1, 4),
                                            "threshold_regret": round(e["threshold_ms"] / e["best_ms"] - 1, 4)}
        if hbm:
            outdeg = np.bincount(pull[0::2].astype(np.int64), minlength=V).astype(np.float64)
            indeg = np.bincount(pull[1::2].astype(np.int64), minlength=V).astype(np.float64)
            res["roofline"] = bfs_kernel_rooflines(G, roots[:4], outdeg, indeg, hbm, hbm_kind)
            del outdeg, indeg
        # e2e through the C ABI: load from pinned -pull pairs, 64 roots under the learned switch
        G.set_policy(native.POLICY_LEARNED, net)
        pin_pull = torch.from_numpy(pull.view(np.int64)).pin_memory()

        def e2e_step():
            G.load_pull_derive_push(V, E, pin_pull.data_ptr())
            u = 0
            for r in roots:
                G.bfs_run(r)
                u += G.digest()[1]
            return u
        e2e_step()
        with Timer(torch, stream) as te:
            units = e2e_step()
        res["e2e"] = {"value": round(units / (te.ms * 1e-3) / 1e9, 3), "unit": "GTEPS", "h2d_bytes_per_step": int(pull.nbytes),
                      "d2h_bytes_per_step": 24 * len(roots), "ms_per_step": round(te.ms, 3),
                      "step": "load of the -pull pairs (the -push list derived on the device), 64 BFS runs under the "
                              "learned switch, each run's digest (reached vertices, reached edges, level checksum) read back"}
        del pin_pull
        G.set_policy(native.POLICY_THRESHOLD)
    if not a.no_cpu:
        cpu, _ = cpu_baseline("bfs", None, pull, push, a.bfs_scale, sample=True, V=V)
        res["cpu_baseline"] = cpu
    return res


def stress_study(a, torch, stream, dev, hbm, hbm_kind):
    """Large power-law stress (directed R-MAT 27 by default, V = 2^27, E ~ 2.1e9, held in HBM):
    PageRank (16 pull iterations, d = 0.875) and CC to convergence on the same graph.  Only the
    -pull pairs stay on the host; the library derives the -push list on the device.  Reports
    device-resident GTEPS, the pull kernels' rooflines (the PageRank gather also against the
    gather-inclusive 8E + 8E + 16V, since the gathered props exceed L2), e2e through the C ABI,
    and parity: one PageRank iteration on a seeded sample of 10^5 destinations recomputed on
    the host in FP64 from the pairs, and all CC labels against the host's label propagation
    over the pairs."""
    from grazelle.engine import Graph
    from oracle import oracle as O
    scale = a.stress_scale
    t0 = time.time()
    V, E, pull = make_graph_lean("pr", scale, a.seed, True)
    log("stress graph: scale %d V=%d E=%d (%.1fs)" % (scale, V, E, time.time() - t0))
    res = {"workload": "rmat%d directed: pr 16 iterations d=0.875, cc to convergence" % scale, "V": V, "E": E}
    pin_pull = torch.from_numpy(pull.view(np.int64)).pin_memory()
    n = 2
    with Graph(dev, stream=stream.cuda_stream) as G:
        G.load_pull_derive_push(V, E, pin_pull.data_ptr())
        # PageRank
        G.pr_init(0.875).pr_iterate(16)
        with Timer(torch, stream) as tp:
            for _ in range(n):
                G.pr_init(0.875).pr_iterate(16)
        G.profile(True)
        G.pr_init(0.875).pr_iterate(16)
        G.sync()
        ks = kernel_stats(G.profile_read())
        G.profile(False)
        gm = ks.get("pr_gather", {}).get("mean_ms", 0)
        alg, alg_g = 8 * E + 16 * V, 16 * E + 16 * V
        pr = {"gteps": round(E * 16 * n / (tp.ms * 1e-3) / 1e9, 3), "ms_per_iteration": round(tp.ms / (16 * n), 3),
              "kernels_us": {k: round(v["mean_ms"] * 1e3, 1) for k, v in ks.items()}}
        if gm:
            pr["roofline"] = {"bound": "hbm", "kernel": "pr_gather", "mean_launch_ms": round(gm, 3), "peak": hbm,
                              "peak_kind": hbm_kind, "unit": "GB/s",
                              "algorithmic_bytes": alg, "achieved": round(alg / (gm * 1e-3) / 1e9, 1),
                              "frac": round(alg / (gm * 1e-3) / 1e9 / hbm, 4),
                              "gather_inclusive_bytes": alg_g, "gather_inclusive_achieved": round(alg_g / (gm * 1e-3) / 1e9, 1),
                              "gather_inclusive_frac": round(alg_g / (gm * 1e-3) / 1e9 / hbm, 4),
                              "traffic": profile_traffic("pr_gather", "pr%d" % scale) if not a.tune else None}
        # parity: one iteration at a seeded sample of destinations
        rng = np.random.default_rng(a.seed + 27)
        smp = np.sort(rng.choice(V, size=100000, replace=False)).astype(np.uint64)
        p1 = G.pr_init(0.875).pr_iterate(1).props()
        t1 = time.time()
        ref = O.pr_sample_iteration(pull, V, smp, 0.875)
        err = O.relative_l1(p1[smp.astype(np.int64)], ref)
        pr["parity"] = {"destinations_sampled": int(smp.shape[0]), "iterations": 1, "rel_l1": err, "bound": 1e-12,
                        "ok": err < 1e-12, "check_s": round(time.time() - t1, 1)}
        del p1, ref
        # CC on the same (directed) graph
        G.cc_run()
        ms, its = [], None
        for _ in range(n):
            st = G.cc_run()
            ms.append(st.ms)
            its = (st.iterations, st.pull_iterations, st.push_iterations)
        G.profile(True)
        G.profile_work()
        G.cc_run()
        recs = G.profile_read()
        open_vectors = G.profile_work()[0]
        G.profile(False)
        fp = [m for k, m in recs if k == "cc_pull"]
        cc = {"gteps": round(E * its[0] / (np.mean(ms) * 1e-3) / 1e9, 3), "ms_per_run": round(float(np.mean(ms)), 3),
              "iterations_pull_push": list(its),
              "kernels_us": {k: round(v["mean_ms"] * 1e3, 1) for k, v in kernel_stats(recs).items()}}
        if fp:
            cc["roofline"] = cc_first_pull_roofline(G, V, E, fp[0], hbm, hbm_kind, open_vectors)
            cc["roofline"]["launch"] = "first pull of the run"
        lab = G.props()
        # e2e: load + 16 PageRank iterations + props back; load + CC + labels back
        d2h = torch.zeros(V, dtype=torch.float64).pin_memory().numpy()
        with Timer(torch, stream) as te:
            G.load_pull_derive_push(V, E, pin_pull.data_ptr())
            G.pr_init(0.875).pr_iterate(16)
            G.lib.grz_read_props(G.h, d2h.ctypes.data, V)
        pr["e2e"] = {"value": round(E * 16 / (te.ms * 1e-3) / 1e9, 3), "unit": "GTEPS", "h2d_bytes_per_step": int(pull.nbytes),
                     "d2h_bytes_per_step": int(d2h.nbytes), "ms_per_step": round(te.ms, 3)}
        with Timer(torch, stream) as te:
            G.load_pull_derive_push(V, E, pin_pull.data_ptr())
            st = G.cc_run()
            G.lib.grz_read_props(G.h, d2h.ctypes.data, V)
        cc["e2e"] = {"value": round(E * st.iterations / (te.ms * 1e-3) / 1e9, 3), "unit": "GTEPS",
                     "h2d_bytes_per_step": int(pull.nbytes), "d2h_bytes_per_step": int(d2h.nbytes), "ms_per_step": round(te.ms, 3)}
        e2e_same = bool(np.array_equal(d2h, lab))
        del d2h
    del pin_pull
    t1 = time.time()
    ref = O.cc_min_labels(pull, V)
    ok = bool(np.array_equal(lab, ref.astype(np.float64)))
    cc["parity"] = {"labels_checked": V, "labels_exact": ok, "e2e_labels_equal_resident": e2e_same, "ok": ok and e2e_same,
                    "check": "label propagation over the -pull pairs on the host (oracle_cc_min_labels)",
                    "check_s": round(time.time() - t1, 1)}
    del ref, lab, pull
    res["pagerank"] = pr
    res["cc"] = cc
    res["parity"] = {"ok": pr["parity"]["ok"] and cc["parity"]["ok"]}
    res["cpu_baseline"] = {"value": None, "unit": "GTEPS", "cores": os.cpu_count(), "kind": "port",
                           "sample": "not run: the CPU restatement's vector layout of a graph this size does not fit a "
                                     "bounded sample; the parity checks above run on the host from the pairs"}
    return res


def batch_graphs(seed: int):
    """32 seeded graphs of uneven size: R-MAT scales 14-22 and Erdos-Renyi with average degree
    4-64."""
    from grazelle import graphgen as gg
    out = []
    for i in range(32):
        if i % 2 == 0:
            s = 14 + (i // 2) % 9
            out.append(("rmat%d" % s, gg.rmat(s, 16, seed=seed + 1000 + i)))
        else:
            ln, d = 14 + (i // 2) % 7, 4 << ((i // 2) % 5)
            out.append(("er%d_d%d" % (ln, d), gg.erdos_renyi(1 << ln, d, seed=seed + 1000 + i)))
    return out


def assign_graphs(edges, world: int):
    """Splits the batch's graphs over `world` ranks: longest first, each to the rank with the
    fewest edges so far (ties to the lower rank).  Returns the sorted graph indices per rank."""
    load = [0] * world
    out = [[] for _ in range(world)]
    for i in sorted(range(len(edges)), key=lambda j: (-edges[j], j)):
        r = min(range(world), key=lambda k: (load[k], k))
        out[r].append(i)
        load[r] += edges[i]
    return [sorted(x) for x in out]


def batch_study(a, torch, stream, dev, graph_ids=None):
    """256 personalized-PageRank instances (8 seeds per graph, 20 iterations, d = 0.85, FP64
    ranks) and 256 BFS instances (8 roots per graph) over the 32 graphs, each run one CUDA graph
    launch of the batch; every instance of every graph checked against the CPU oracles."""
    from grazelle.batch import Batch
    from oracle import oracle as O
    t0 = time.time()
    gs = batch_graphs(a.seed)
    seeds = [pick_roots(g, 8, seed=a.seed + 7 * i) for i, (_, g) in enumerate(gs)]
    if graph_ids is not None:
        gs = [gs[i] for i in graph_ids]
        seeds = [seeds[i] for i in graph_ids]
    E_tot = sum(g.num_edges for _, g in gs)
    log("batch graphs: %d, E=%d (%.1fs)" % (len(gs), E_tot, time.time() - t0))
    res = {"workload": "32 graphs (R-MAT 14-22, ER degree 4-64), 256 PPR x 20 iterations + 256 BFS",
           "graphs": len(gs), "edges": E_tot}
    with Batch(dev, stream=stream.cuda_stream) as B:
        t1 = time.time()
        for _, g in gs:
            B.add_graph(g.num_vertices, g.pull_order().pairs())
        B.build()
        res["build_s"] = round(time.time() - t1, 2)
        if not a.no_tune:
            from grazelle import autotune
            tb = autotune.tune_batch(B, seeds)
            res["autotuned"] = {k: {"best": v["best"], "best_ms": round(v["best_ms"], 3),
                                    "default_ms": round(v["default_ms"], 3) if v["default_ms"] else None} for k, v in tb.items()}
        B.ppr(seeds, 20, 0.85, ranks=False)
        ms = []
        for _ in range(max(1, a.steps)):
            _, st = B.ppr(seeds, 20, 0.85, ranks=False)
            ms.append(st.ms)
        ranks, _ = B.ppr(seeds, 20, 0.85)
        ppr_ms = float(np.median(ms))
        n_inst = sum(len(s) for s in seeds)
        # edge-instance updates: every instance traverses its graph's edges once per iteration
        upd = sum(g.num_edges * len(s) for (_, g), s in zip(gs, seeds)) * 20
        res["ppr"] = {"instances": n_inst, "ms": round(ppr_ms, 3), "gteps": round(upd / (ppr_ms * 1e-3) / 1e9, 2),
                      "ms_per_instance": round(ppr_ms / n_inst, 4)}
        B.msbfs(seeds, levels=False)
        ms = []
        for _ in range(max(1, a.steps)):
            _, st = B.msbfs(seeds, levels=False)
            ms.append(st.ms)
        levels, st = B.msbfs(seeds)
        bfs_ms = float(np.median(ms))
        reached = 0
        for (_, g), lv in zip(gs, levels):
            deg = g.out_degrees()
            for i in range(lv.shape[1]):
                reached += int(deg[lv[:, i] >= 0].sum())
        res["msbfs"] = {"instances": n_inst, "ms": round(bfs_ms, 3), "iterations": st.iterations,
                        "gteps": round(reached / (bfs_ms * 1e-3) / 1e9, 2)}
        # both in one CUDA graph launch, the two loops side by side (results equal the separate
        # runs': tests/test_gpu_batch.py)
        B.run(seeds, seeds, 20, 0.85, results=False)
        tots, sps, sbs = [], [], []
        for _ in range(max(1, a.steps)):
            _, _, sp, sb, tot = B.run(seeds, seeds, 20, 0.85, results=False)
            tots.append(tot)
            sps.append(sp.ms)
            sbs.append(sb.ms)
        one = float(np.median(tots))
        res["one_launch"] = {"ms": round(one, 3), "ppr_branch_ms": round(float(np.median(sps)), 3),
                             "bfs_branch_ms": round(float(np.median(sbs)), 3), "separate_ms": round(ppr_ms + bfs_ms, 3),
                             "gteps_ppr_plus_bfs": round((upd + reached) / (one * 1e-3) / 1e9, 2), "launches_per_run": 1}
        res["units"] = {"ppr_updates": upd, "bfs_reached_edges": reached}
        # every instance of every graph against the oracles (C, OpenMP): PPR within 1e-12
        # relative L1 of oracle/ppr.py's definition, BFS levels exactly
        t2 = time.time()
        worst, exact = 0.0, True
        for gi, (_, g) in enumerate(gs):
            pull, push = g.pull_order().pairs(), g.push_order().pairs()
            ref = O.ppr_multi(g.num_vertices, pull, seeds[gi], 20, 0.85)
            refl = O.bfs_levels_multi(push, g.num_vertices, seeds[gi])
            for i in range(len(seeds[gi])):
                worst = max(worst, O.relative_l1(ranks[gi][:, i], ref[:, i]))
                exact &= bool(np.array_equal(levels[gi][:, i].astype(np.int64), refl[i]))
        res["parity"] = {"graphs_checked": len(gs), "instances_checked": n_inst, "ppr_max_rel_l1": worst, "ppr_bound": 1e-12,
                         "bfs_levels_exact": exact, "ok": worst < 1e-12 and exact, "check_s": round(time.time() - t2, 1)}
        res["gpu_launches_per_run"] = {"ppr": 1 + 2 * 20, "msbfs": 1 + 3 * st.iterations}
    return res


def run_batch(a):
    """The batched workload on its own: 256 PPR and 256 BFS instances over 32 graphs.  Value:
    PPR edge-instance updates plus BFS reached edges per second of the one-launch run (GTEPS).
    Under torchrun the 32 graphs (and their instances) are split over the ranks
    (assign_graphs); units are summed and the slowest rank's time is taken."""
    import torch

    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    stream = torch.cuda.Stream()
    ids = None
    if world > 1:
        edges = [g.num_edges for _, g in batch_graphs(a.seed)]
        ids = assign_graphs(edges, world)[rank]
    res = batch_study(a, torch, stream, local, graph_ids=ids)
    units = res["units"]["ppr_updates"] + res["units"]["bfs_reached_edges"]
    u_all, ms = combine_ranks(units, res["one_launch"]["ms"], dist)
    if dist:
        dist.barrier()
    if rank != 0:
        return
    line = {"metric": "GTEPS (batched personalized PageRank and multi-source BFS, edge-instance updates / time)",
            "value": round(u_all / (ms * 1e-3) / 1e9, 2), "unit": "GTEPS", "n_gpus": world, "steps": a.steps, "warmup": a.warmup,
            "ms_per_step": ms, "higher_is_better": True, "scaling": "strong" if world > 1 else "weak", "vs_baseline": None,
            "dtype": "u128 fixed point + f64", "data": "synthetic (seeded R-MAT and Erdos-Renyi)",
            "config": {"workload": res["workload"], "graphs_per_rank": "split over ranks" if world > 1 else "all"}, "batch": res}
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------------------------------------- CPU

def cpu_baseline(wl, g, pull, push, scale, sample=True, threads=0, steps=1, V=None):
    """The reference's algorithm on the host cores.  The reference binary runs only on x86-64
    with AVX2, so this uses oracle/'s OpenMP restatement with the same work-unit scheme;
    `kind` says which.  Returns (baseline record, the last run's props as the reference stores
    them: PageRank rank/outdeg', CC labels, BFS parents)."""
    from oracle import oracle as O
    V = g.num_vertices if g is not None else V
    t0 = time.time()
    L = O.layout(V, pull, push)
    build_s = time.time() - t0
    cores = os.cpu_count() or 1
    vals = []
    n_used = 0
    it_total = 0
    out = None
    for _ in range(steps):
        t = time.time()
        if wl == "pr":
            iters = 4 if sample else 16
            out = O.pr_pull(L, iters, 0.875, units=32 * cores, threads=threads, multithreaded=True)
            units = L.E * iters
            it_total = iters
        elif wl == "cc":
            out, it, n_used = O.frontier_mt(L, 1, 0, threads=threads)
            units = L.E * int(it[0])
            it_total = int(it[0])
        else:
            out, it, n_used = O.frontier_mt(L, 2, 0, threads=threads)
            reached = out >= 0
            reached[0] = True
            units = int(L.outdeg[reached].sum())
            it_total = int(it[0])
        dt = time.time() - t
        vals.append(units / dt / 1e9)
    del L
    rec = {"value": round(max(vals), 4), "unit": "GTEPS", "cores": threads or cores, "kind": "port",
           "sample": "%s on the same graph, %d iteration(s) per run, best of %d, OpenMP restatement with the "
                     "reference's work units (oracle/grz_oracle.c); layout build %.1fs not timed" % (
                         {"pr": "PageRank pull", "cc": "CC to convergence", "bfs": "BFS from root 0"}[wl], it_total,
                         steps, build_s)}
    return rec, out


def run_reference(a):
    rank, world, local = dist_env()
    if rank != 0:
        return
    wl = a.workload
    scale = a.scale or DEFAULT_SCALE[wl]
    g, pull, push = make_graph(wl, scale, a.seed, a.directed)
    for _ in range(a.warmup):
        pass  # the CPU run has no warm-up state beyond the layout, which is built once
    res, _ = cpu_baseline(wl, g, pull, push, scale, sample=False, steps=max(1, a.steps))
    line = {
        "impl": "reference", "metric": "GTEPS (%s, E x iterations / time)" % {"cc": "connected components", "pr": "pagerank pull",
                                                                               "bfs": "bfs"}[wl],
        "value": res["value"], "unit": "GTEPS", "n_gpus": world, "steps": a.steps, "warmup": a.warmup,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded R-MAT)",
        "config": {"workload": "%s-rmat%d%s" % (wl, scale, "-sym" if wl != "pr" and not a.directed else ""), "scale": scale, "edge_factor": 16,
                   "seed": a.seed, "V": g.num_vertices, "E": g.num_edges},
        "cpu_baseline": res, "e2e": {"value": res["value"], "unit": "GTEPS", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["native", "reference"], default="native")
    ap.add_argument("--workload", choices=["cc", "pr", "bfs", "batch"], default="cc",
                    help="batch: only the batched PPR / multi-source BFS workload (its own JSON line)")
    ap.add_argument("--scale", type=int, default=0)
    ap.add_argument("--seed", type=int, default=1)
    ap.add_argument("--no-apps", action="store_true")
    ap.add_argument("--bfs-scale", type=int, default=26, help="R-MAT scale of the BFS switch study (0: skip)")
    ap.add_argument("--no-batch", action="store_true", help="skip the batched PPR / multi-source BFS study")
    ap.add_argument("--stress-scale", type=int, default=27,
                    help="R-MAT scale of the large power-law stress study, PageRank and CC on a directed graph (0: skip)")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-tune", action="store_true", help="keep the default kernel shapes (no autotuning pass)")
    ap.add_argument("--lean", action="store_true", help="host keeps only the -pull pairs (default from scale 26)")
    ap.add_argument("--ingest", choices=["pull", "both"], default="pull",
                    help="e2e input: the -pull pairs (the library derives the -push list) or both lists")
    ap.add_argument("--tune", action="append", default=[], metavar="KNOB=VALUE",
                    help="kernel-shape knob applied before the load (grazelle.engine.Graph.tune), e.g. pull_staging=1; repeatable")
    ap.add_argument("--pr-props", type=int, default=0, choices=[0, 1, 2],
                    help="props the PageRank gather reads: 0 by size, 1 fixed point, 2 doubles (results identical)")
    ap.add_argument("--directed", action="store_true", help="CC/BFS on the directed R-MAT (no symmetrisation), as the scale-27 stress configuration")
    a = ap.parse_args()
    if a.warmup < 3:
        log("warm-up raised to 3 steps (timing rule)")
        a.warmup = 3
    if a.impl == "reference":
        run_reference(a)
    elif a.workload == "batch":
        run_batch(a)
    else:
        run_native(a)


if __name__ == "__main__":
    main()
