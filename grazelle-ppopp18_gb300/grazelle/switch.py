"""The learned push/pull switch: per-iteration timing data, training, and evaluation.

The reference picks the engine with a threshold on the vote (pull iff vote > E/5,
source/execution_bfs.c:146-168, source/execution_cc.c:120-142).  Here, before each
iteration, an MLP with hand-written CUDA kernels (csrc/grz_switch.cu) predicts whether pull
will beat push on this GPU.  Its features come from the frontier state.

Data: for every iteration of CC and BFS runs on seeded training graphs, the state is
snapshotted and both engines are timed from it with CUDA events.  The run then continues
along the faster one, so the collection also gives the best-per-iteration ("oracle") time.
Training: weighted binary cross-entropy (label: pull faster; weight: |t_pull - t_push|),
Adam, all on the GPU.  Evaluation: whole-run device time with the threshold policy, with the
learned policy, and the oracle bound.  Results (CC labels, BFS levels) are the same for all.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field

import numpy as np

import json
import os
import sys
import time

from . import graphgen as gg
from . import native
from .engine import Graph

NF = native.MLP_FEATURES
# weights trained on a GB300 by `python -m grazelle.switch train` (see main below)
PRETRAINED = os.path.join(os.path.dirname(os.path.abspath(__file__)), "switch_gb300.npy")


@dataclass
class Samples:
    X: list = field(default_factory=list)
    t_pull: list = field(default_factory=list)
    t_push: list = field(default_factory=list)
    heuristic: list = field(default_factory=list)
    tag: list = field(default_factory=list)

    def arrays(self):
        X = np.asarray(self.X, dtype=np.float32).reshape(-1, NF)
        tp = np.asarray(self.t_pull, dtype=np.float64)
        tq = np.asarray(self.t_push, dtype=np.float64)
        return X, tp, tq

    def labels(self):
        X, tp, tq = self.arrays()
        y = (tp < tq).astype(np.float32)
        gap = np.abs(tp - tq)
        w = (gap / max(gap.mean(), 1e-9)).astype(np.float32)
        return X, y, w

    def extend(self, other: "Samples"):
        for k in ("X", "t_pull", "t_push", "heuristic", "tag"):
            getattr(self, k).extend(getattr(other, k))


def _features(G: Graph):
    f = np.zeros(NF, dtype=np.float32)
    choice = C.c_int()
    G._ck(G.lib.grz_frontier_features(G.h, f.ctypes.data, NF, C.byref(choice)))
    return f, choice.value


def _step_timed(G: Graph, engine: int):
    used = C.c_int()
    vote = C.c_uint64()
    ms = C.c_float()
    rc = G.lib.grz_frontier_next_timed(G.h, engine, C.byref(used), C.byref(vote), C.byref(ms))
    if rc < 0:
        native.check(rc, G.h)
    return rc == 1, float(ms.value)


def collect(G: Graph, app: int, roots=(0,), tag: str = "", max_iters: int = 500) -> Samples:
    """Both engines timed from each iteration's state; the run continues along the faster."""
    out = Samples()
    G._ck(G.lib.grz_frontier_set_policy(G.h, native.POLICY_THRESHOLD, None))
    for root in roots:
        G.frontier_begin(app, root)
        for _ in range(max_iters):
            f, heur = _features(G)
            G._ck(G.lib.grz_frontier_snapshot(G.h))
            run_pull, t_pull = _step_timed(G, 1)
            G._ck(G.lib.grz_frontier_restore(G.h))
            run_push, t_push = _step_timed(G, 0)
            out.X.append(f)
            out.t_pull.append(t_pull)
            out.t_push.append(t_push)
            out.heuristic.append(heur)
            out.tag.append(tag)
            running = run_push
            if t_pull < t_push:
                G._ck(G.lib.grz_frontier_restore(G.h))
                running, _ = _step_timed(G, 1)
            if not running:
                break
    return out


class Switch:
    """The MLP on the GPU (grz_mlp)."""

    def __init__(self, device: int = 0, seed: int = 1):
        self.lib = native.load()
        h = C.c_void_p()
        native.check(self.lib.grz_mlp_create(C.byref(h), device, seed))
        self.h = h

    def close(self):
        if self.h:
            self.lib.grz_mlp_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def params(self) -> np.ndarray:
        p = np.zeros(native.MLP_PARAMS, dtype=np.float32)
        native.check(self.lib.grz_mlp_get_params(self.h, p.ctypes.data, p.shape[0]))
        return p

    def set_params(self, p: np.ndarray):
        p = np.ascontiguousarray(p, dtype=np.float32)
        native.check(self.lib.grz_mlp_set_params(self.h, p.ctypes.data, p.shape[0]))

    def gradients(self, X, Y, W):
        X, Y, W = (np.ascontiguousarray(a, dtype=np.float32) for a in (X, Y, W))
        g = np.zeros(native.MLP_PARAMS, dtype=np.float32)
        loss = C.c_float()
        native.check(self.lib.grz_mlp_gradients(self.h, X.ctypes.data, Y.ctypes.data, W.ctypes.data, Y.shape[0],
                                                g.ctypes.data, C.byref(loss)))
        return float(loss.value), g

    def train(self, X, Y, W, epochs: int = 400, lr: float = 3e-3) -> float:
        X, Y, W = (np.ascontiguousarray(a, dtype=np.float32) for a in (X, Y, W))
        loss = C.c_float()
        native.check(self.lib.grz_mlp_train(self.h, X.ctypes.data, Y.ctypes.data, W.ctypes.data, Y.shape[0], epochs,
                                            C.c_float(lr), C.byref(loss)))
        return float(loss.value)

    def predict(self, X) -> np.ndarray:
        X = np.ascontiguousarray(X, dtype=np.float32)
        z = np.zeros(X.shape[0], dtype=np.float32)
        native.check(self.lib.grz_mlp_predict(self.h, X.ctypes.data, X.shape[0], z.ctypes.data))
        return z


def training_graphs(scales=(18, 19, 20, 21, 22, 23), er_degrees=(8, 16, 32), er_log2n=(18, 20), seed: int = 100):
    """Seeded R-MAT (scales 18-23) and Erdős–Rényi (average degree 8-32) training graphs."""
    out = []
    for i, s in enumerate(scales):
        out.append(("rmat%d" % s, gg.rmat(s, seed=seed + i)))
    for j, d in enumerate(er_degrees):
        for k, ln in enumerate(er_log2n):
            out.append(("er%d_d%d" % (ln, d), gg.erdos_renyi(1 << ln, d, seed=seed + 50 + 7 * j + k)))
    return out


def roots_of(g, n: int, seed: int):
    deg = g.out_degrees()
    cand = np.nonzero(deg)[0]
    rng = np.random.default_rng(seed)
    return [int(x) for x in rng.choice(cand, size=min(n, cand.shape[0]), replace=False)]


def run_time(G: Graph, app: int, root: int, policy: int, mlp: "Switch | None"):
    """Whole-run device time (ms) and (iterations, pull, push) under a policy."""
    G.set_policy(policy, mlp)
    st = native.RunStats()
    try:
        if app == native.APP_CONNECTED_COMPONENTS:
            G._ck(G.lib.grz_cc_run(G.h, 0, C.byref(st)))
        else:
            G._ck(G.lib.grz_bfs_run(G.h, root, 0, C.byref(st)))
    finally:
        G.set_policy(native.POLICY_THRESHOLD, None)
    return float(st.ms), (st.iterations, st.pull_iterations, st.push_iterations)


def result_of(G: Graph, app: int) -> np.ndarray:
    """What must not depend on the engine: CC labels, BFS levels."""
    return G.levels() if app == native.APP_BREADTH_FIRST_SEARCH else G.props()


def edge_totals(samples: Samples, net: Switch) -> dict:
    """Edge-phase time summed over the sampled iterations, had each policy chosen the engine.

    For BFS every engine leaves the same frontier, so the sum is exactly what that policy's
    run spends in its edge phases.  For CC the pull and push engines propagate labels in a
    different order within an iteration, so the trajectory is the collected one."""
    X, tp, tq = samples.arrays()
    z = net.predict(X)
    heur = np.asarray(samples.heuristic)
    return {"threshold_ms": float(np.where(heur == 1, tp, tq).sum()),
            "learned_ms": float(np.where(z > 0, tp, tq).sum()),
            "best_ms": float(np.minimum(tp, tq).sum()),
            "iterations": int(X.shape[0]),
            "learned_agrees_with_best": float(np.mean((z > 0) == (tp < tq)))}


def compare_runs(G: Graph, app: int, roots, net: Switch, repeats: int = 1) -> dict:
    """Whole-run device time under the threshold and the learned policy; results must match."""
    thr = mlp = 0.0
    identical = True
    it_thr, it_mlp = [], []
    for r in roots:
        run_time(G, app, r, native.POLICY_THRESHOLD, None)
        run_time(G, app, r, native.POLICY_LEARNED, net)
        for _ in range(repeats):
            t, it = run_time(G, app, r, native.POLICY_THRESHOLD, None)
            thr += t
        a = result_of(G, app)
        for _ in range(repeats):
            t2, it2 = run_time(G, app, r, native.POLICY_LEARNED, net)
            mlp += t2
        b = result_of(G, app)
        identical &= bool(np.array_equal(a, b))
        it_thr.append(it)
        it_mlp.append(it2)
    return {"threshold_ms": thr / repeats, "learned_ms": mlp / repeats, "identical_results": identical,
            "iterations_pull_push_threshold": it_thr, "iterations_pull_push_learned": it_mlp}


def load_graph(G: Graph, g):
    G.load_pairs(g.num_vertices, g.pull_order().pairs(), g.push_order().pairs())
    return G


def train(device: int = 0, seed: int = 3, graphs=None, roots_per_graph: int = 4, log=None) -> tuple[Switch, Samples]:
    """Collects per-iteration timings of both engines on the training graphs and trains the MLP
    on the GPU (two Adam phases, 600 epochs each, full batch)."""
    data = Samples()
    t0 = time.time()
    for name, g in (graphs if graphs is not None else training_graphs()):
        with Graph(device) as G:
            load_graph(G, g)
            data.extend(collect(G, native.APP_BREADTH_FIRST_SEARCH, roots_of(g, roots_per_graph, 1), tag=name + "/bfs"))
            data.extend(collect(G, native.APP_CONNECTED_COMPONENTS, (0,), tag=name + "/cc"))
    if log:
        log("collected %d iterations in %.1f s" % (len(data.X), time.time() - t0))
    X, y, w = data.labels()
    net = Switch(device, seed=seed)
    for lr in (3e-3, 1e-3):
        loss = net.train(X, y, w, epochs=600, lr=lr)
    if log:
        log("trained: loss %.5f" % loss)
    return net, data


def pretrained(device: int = 0, path: str = PRETRAINED) -> Switch:
    net = Switch(device)
    net.set_params(np.load(path))
    return net


def held_out_graphs(seed: int = 990):
    return [("rmat21", gg.rmat(21, seed=seed + 9)), ("rmat22sym", gg.rmat(22, seed=seed + 8, symmetric=True)),
            ("rmat23", gg.rmat(23, seed=seed + 6)), ("er20_d12", gg.erdos_renyi(1 << 20, 12, seed=seed + 7)),
            ("er21_d24", gg.erdos_renyi(1 << 21, 24, seed=seed + 5))]


def evaluate(net: Switch, device: int = 0, graphs=None, roots_per_graph: int = 4, log=None) -> dict:
    """Per held-out graph: edge-phase totals (threshold / learned / best per iteration) and
    whole-run device times of both policies, with the check that results are identical."""
    report = {}
    for name, g in (graphs if graphs is not None else held_out_graphs()):
        with Graph(device) as G:
            load_graph(G, g)
            roots = roots_of(g, roots_per_graph, 5)
            d = Samples()
            d.extend(collect(G, native.APP_BREADTH_FIRST_SEARCH, roots))
            d.extend(collect(G, native.APP_CONNECTED_COMPONENTS, (0,)))
            rec = {"edge": edge_totals(d, net),
                   "bfs": compare_runs(G, native.APP_BREADTH_FIRST_SEARCH, roots, net),
                   "cc": compare_runs(G, native.APP_CONNECTED_COMPONENTS, (0,), net)}
        report[name] = rec
        if log:
            e = rec["edge"]
            log("%-10s edge ms thr %.3f learned %.3f best %.3f | run ms bfs %.3f -> %.3f, cc %.3f -> %.3f, identical %s"
                % (name, e["threshold_ms"], e["learned_ms"], e["best_ms"], rec["bfs"]["threshold_ms"],
                   rec["bfs"]["learned_ms"], rec["cc"]["threshold_ms"], rec["cc"]["learned_ms"],
                   rec["bfs"]["identical_results"] and rec["cc"]["identical_results"]))
    return report


def main(argv=None):
    """python -m grazelle.switch train [--out PATH] [--report PATH]: collect, train, evaluate on
    held-out graphs, write the weights (float32 .npy) and a JSON report."""
    import argparse
    ap = argparse.ArgumentParser(prog="python -m grazelle.switch")
    ap.add_argument("command", choices=["train", "evaluate"])
    ap.add_argument("--out", default=PRETRAINED)
    ap.add_argument("--report", default="")
    ap.add_argument("--device", type=int, default=0)
    ap.add_argument("--seed", type=int, default=3)
    a = ap.parse_args(argv)

    def log(msg):
        print(msg, file=sys.stderr, flush=True)

    if a.command == "train":
        net, data = train(a.device, a.seed, log=log)
        np.save(a.out, net.params())
        log("weights -> %s" % a.out)
    else:
        net = pretrained(a.device, a.out)
    report = evaluate(net, a.device, log=log)
    if a.report:
        with open(a.report, "w") as fh:
            json.dump(report, fh, indent=1)


if __name__ == "__main__":
    main()
