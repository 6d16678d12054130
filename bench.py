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
            duration, against the measured HBM copy peak
  apps      PageRank (R-MAT scale 20, 16 pull iterations) and BFS on the same graph
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

    load()
    hbm, hbm_kind = measured_hbm()
    # kernel shapes for this graph, chosen by timing (outside every timed region)
    tuned = None
    if not a.no_tune:
        from grazelle import autotune
        tuned = autotune.tune_cc(G, device=local) if wl in ("cc", "bfs") else autotune.tune_pr(G, device=local)
        tuned.pop("trials", None)

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
    with Timer(torch, stream) as tprof:
        for i in range(a.steps):
            step(i)
    recs = G.profile_read()
    G.profile(False)
    ks = kernel_stats(recs)
    dominant = max(ks.items(), key=lambda kv: kv[1]["total_ms"])[0] if ks else None

    # algorithmic bytes per launch of the dominant kernel (8E + 16V for a pull pass; V/4 more for
    # the two CC bitmaps)
    alg = {"pr_gather": 8 * E + 16 * V, "cc_pull": 8 * E + 16 * V + V // 4, "bfs_pull": 8 * E + 16 * V + V // 4}
    roof = None
    if dominant:
        mean_s = ks[dominant]["mean_ms"] * 1e-3
        if dominant in alg:
            achieved = alg[dominant] / mean_s / 1e9
            roof = {"bound": "hbm", "kernel": dominant, "achieved": round(achieved, 1), "peak": hbm, "peak_kind": hbm_kind,
                    "unit": "GB/s", "frac": round(achieved / hbm, 4), "algorithmic_bytes": alg[dominant],
                    "mean_launch_ms": round(ks[dominant]["mean_ms"], 4),
                    "share_of_profiled_pass": round(ks[dominant]["total_ms"] / tprof.ms, 4),
                    "region": "profiled pass of the same %d steps" % a.steps,
                    "traffic": profile_traffic(dominant, "%s%d" % (wl, scale))}

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
    if rank == 0 and not a.no_cpu and not lean:
        cpu = cpu_baseline(wl, g, pull, push, scale, sample=True)
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
        "e2e": e2e, "gpu_launches": int(launches), "clocks": clk.summary(), "cpu_baseline": cpu, "apps": apps,
    }
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
        out["bfs_switch"] = bfs_switch_study(a, torch, stream, net, dev)
    if not a.no_batch:
        out["batch"] = batch_study(a, torch, stream, dev)
    # PageRank
    g, pull, push = make_graph("pr", 20, a.seed)
    V, E = g.num_vertices, g.num_edges
    with Graph(torch.cuda.current_device(), stream=stream.cuda_stream) as G:
        G.load_pairs(V, pull, push)
        G.pr_init(0.875).pr_iterate(16)
        n = max(1, a.steps // 2)
        with Timer(torch, stream) as tp:
            for _ in range(n):
                G.pr_init(0.875).pr_iterate(16)
        G.profile(True)
        for _ in range(n):
            G.pr_init(0.875).pr_iterate(16)
        G.sync()
        ks = kernel_stats(G.profile_read())
        G.profile(False)
        alg = 8 * E + 16 * V
        gm = ks.get("pr_gather", {}).get("mean_ms", 0)
        it_ms = tp.ms / (16 * n)
        out["pagerank"] = {"workload": "pr-rmat20, 16 iterations, d=0.875", "gteps": round(E * 16 * n / (tp.ms * 1e-3) / 1e9, 3),
                           "us_per_iteration": round(it_ms * 1e3, 2),
                           "roofline_iteration": {"achieved": round(alg / (it_ms * 1e-3) / 1e9, 1), "peak": hbm,
                                                  "peak_kind": hbm_kind, "frac": round(alg / (it_ms * 1e-3) / 1e9 / hbm, 4),
                                                  "algorithmic_bytes": alg},
                           "kernels_us": {k: round(v["mean_ms"] * 1e3, 2) for k, v in ks.items()},
                           "gather_roofline_frac": round(alg / (gm * 1e-3) / 1e9 / hbm, 4) if gm else None}
    return out


def bfs_switch_study(a, torch, stream, net, dev):
    """BFS on a directed R-MAT (default scale 26, edge factor 16) from 64 seeded non-isolated
    roots under the threshold rule and the learned switch: GTEPS from the device time of each
    run, identical levels checked by an on-device digest, and the edge-phase regret of both
    policies against the best engine per iteration on 4 of the roots."""
    from grazelle import graphgen as gg
    from grazelle import native
    from grazelle import switch as sw
    from grazelle.engine import Graph
    t0 = time.time()
    g = gg.rmat(a.bfs_scale, 16, seed=a.seed + 26)
    V, E = g.num_vertices, g.num_edges
    roots = pick_roots(g, 64, seed=a.seed + 64)
    log("bfs graph: scale %d V=%d E=%d (%.1fs)" % (a.bfs_scale, V, E, time.time() - t0))
    res = {"workload": "bfs-rmat%d (directed), %d roots" % (a.bfs_scale, len(roots)), "V": V, "E": E}
    with Graph(dev, stream=stream.cuda_stream) as G:
        G.load_pairs(V, g.pull_order().pairs(), g.push_order().pairs())
        del g
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
        G.set_policy(native.POLICY_THRESHOLD)
        res["identical_levels"] = digests["threshold"] == digests["learned"]
        res["learned_speedup"] = round(res["threshold"]["ms_total"] / res["learned"]["ms_total"], 4)
        d = sw.Samples()
        d.extend(sw.collect(G, native.APP_BREADTH_FIRST_SEARCH, roots[:4]))
        e = sw.edge_totals(d, net)
        res["edge_phase_regret_4_roots"] = {"threshold_ms": round(e["threshold_ms"], 4), "learned_ms": round(e["learned_ms"], 4),
                                            "best_per_iteration_ms": round(e["best_ms"], 4), "iterations": e["iterations"],
                                            "learned_regret": round(e["learned_ms"] / e["best_ms"] - 1, 4),
                                            "threshold_regret": round(e["threshold_ms"] / e["best_ms"] - 1, 4)}
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


def batch_study(a, torch, stream, dev):
    """256 personalized-PageRank instances (8 seeds per graph, 20 iterations, d = 0.85, FP64
    ranks) and 256 BFS instances (8 roots per graph) over the 32 graphs, each run one CUDA graph
    launch of the batch; every instance of two graphs checked against the CPU oracles."""
    from grazelle.batch import Batch
    from oracle import oracle as O
    from oracle import ppr as P
    t0 = time.time()
    gs = batch_graphs(a.seed)
    E_tot = sum(g.num_edges for _, g in gs)
    log("batch graphs: %d, E=%d (%.1fs)" % (len(gs), E_tot, time.time() - t0))
    seeds = [pick_roots(g, 8, seed=a.seed + 7 * i) for i, (_, g) in enumerate(gs)]
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
        worst, exact = 0.0, True
        for gi in (0, 1):
            g = gs[gi][1]
            pull, push = g.pull_order().pairs(), g.push_order().pairs()
            for i, s in enumerate(seeds[gi]):
                ref = P.ppr(g.num_vertices, pull, s, 20, 0.85)
                worst = max(worst, float(np.abs(ranks[gi][:, i] - ref).sum() / np.abs(ref).sum()))
                exact &= bool(np.array_equal(levels[gi][:, i].astype(np.int64), O.bfs_levels(push, g.num_vertices, s)))
        res["parity_sample"] = {"ppr_max_rel_l1": worst, "bfs_levels_exact": exact, "graphs_checked": [gs[0][0], gs[1][0]]}
        res["gpu_launches_per_run"] = {"ppr": 1 + 2 * 20, "msbfs": 1 + 3 * st.iterations}
    return res


def run_batch(a):
    """The batched workload on its own: 256 PPR and 256 BFS instances over 32 graphs, one CUDA
    graph launch per run.  Value: PPR edge-instance updates per second (GTEPS).  Under torchrun
    every rank runs its own replica of the batch; rank 0 reports its own numbers."""
    import torch

    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    stream = torch.cuda.Stream()
    res = batch_study(a, torch, stream, local)
    if rank != 0:
        return
    line = {"metric": "GTEPS (batched personalized PageRank, edge-instance updates / time)", "value": res["ppr"]["gteps"],
            "unit": "GTEPS", "n_gpus": 1, "steps": a.steps, "warmup": a.warmup, "ms_per_step": res["ppr"]["ms"],
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u128 fixed point + f64",
            "data": "synthetic (seeded R-MAT and Erdos-Renyi)", "config": {"workload": res["workload"]}, "batch": res}
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------------------------------------- CPU

def cpu_baseline(wl, g, pull, push, scale, sample=True, threads=0, steps=1):
    """The reference's algorithm on the host cores.  The reference binary runs only on x86-64
    with AVX2, so this uses oracle/'s OpenMP restatement with the same work-unit scheme;
    `kind` says which."""
    from oracle import oracle as O
    t0 = time.time()
    L = O.layout(g.num_vertices, pull, push)
    build_s = time.time() - t0
    cores = os.cpu_count() or 1
    vals = []
    n_used = 0
    it_total = 0
    for _ in range(steps):
        t = time.time()
        if wl == "pr":
            iters = 4 if sample else 16
            O.pr_pull(L, iters, 0.875, units=32 * cores, threads=threads, multithreaded=True)
            units = L.E * iters
            it_total = iters
        elif wl == "cc":
            lab, it, n_used = O.frontier_mt(L, 1, 0, threads=threads)
            units = L.E * int(it[0])
            it_total = int(it[0])
        else:
            par, it, n_used = O.frontier_mt(L, 2, 0, threads=threads)
            reached = par >= 0
            reached[0] = True
            units = int(L.outdeg[reached].sum())
            it_total = int(it[0])
        dt = time.time() - t
        vals.append(units / dt / 1e9)
    return {"value": round(max(vals), 4), "unit": "GTEPS", "cores": threads or cores, "kind": "port",
            "sample": "%s on the same graph, %d iteration(s) per run, best of %d, OpenMP restatement with the "
                      "reference's work units (oracle/grz_oracle.c); layout build %.1fs not timed" % (
                          {"pr": "PageRank pull", "cc": "CC to convergence", "bfs": "BFS from root 0"}[wl], it_total,
                          steps, build_s)}


def run_reference(a):
    rank, world, local = dist_env()
    if rank != 0:
        return
    wl = a.workload
    scale = a.scale or DEFAULT_SCALE[wl]
    g, pull, push = make_graph(wl, scale, a.seed, a.directed)
    for _ in range(a.warmup):
        pass  # the CPU run has no warm-up state beyond the layout, which is built once
    res = cpu_baseline(wl, g, pull, push, scale, sample=False, steps=max(1, a.steps))
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
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-tune", action="store_true", help="keep the default kernel shapes (no autotuning pass)")
    ap.add_argument("--lean", action="store_true", help="host keeps only the -pull pairs (default from scale 26)")
    ap.add_argument("--ingest", choices=["pull", "both"], default="pull",
                    help="e2e input: the -pull pairs (the library derives the -push list) or both lists")
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
