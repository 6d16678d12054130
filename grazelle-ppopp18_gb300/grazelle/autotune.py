"""Autotuner: kernel shapes chosen per loaded graph (or batch) by timing them on the device.

The knobs (include/grazelle_gb300.h, GRZ_TUNE_* and GRZ_BATCH_TUNE_*) change only speed:
block size and persistent grid of the CC pull kernel, persistent grid of the PageRank gather,
resident blocks per SM of the batch kernels, and the optional hub-source encoding.  Each
candidate is timed with the library's CUDA-event kernel profiler (or the run statistics), the
median of a few trials is kept, and the fastest candidate is applied.  The default shape is
always one of the candidates, so tuning never makes a kernel slower than the default by more
than the measurement noise.
"""
from __future__ import annotations

import statistics

from . import native


def _sms(device: int = 0) -> int:
    try:
        import torch
        return int(torch.cuda.get_device_properties(device).multi_processor_count)
    except Exception:
        return 152


def _kernel_ms(G, kind: str, run, trials: int) -> float:
    vals = []
    for _ in range(trials):
        G.profile(True)
        run()
        G.sync()
        recs = [ms for k, ms in G.profile_read() if k == kind]
        G.profile(False)
        if recs:
            vals.append(sum(recs) / len(recs))
    return statistics.median(vals) if vals else float("inf")


def tune_cc(G, trials: int = 3, threads=(256, 512, 1024), grids_per_sm=(0, 1, 2, 4), caches=(0,), device: int = 0) -> dict:
    """CC pull kernel: block size x persistent grid (x hub-label cache when hubs are loaded).
    Times the pull edge phase of a full CC run with the pull engine forced."""
    sms = _sms(device)
    start = G.tuning()
    flags = native.FORCE_PULL | native.FLAG_HOST_LOOP

    def run():
        G.cc_run(flags)

    run()  # warm-up
    trials_out = []
    for th in threads:
        for gps in grids_per_sm:
            for cache in caches:
                if cache and start["hubs_loaded"] == 0:
                    continue
                G.tune(cc_threads=th, cc_grid=gps * sms, cc_cache=cache)
                ms = _kernel_ms(G, "cc_pull", run, trials)
                trials_out.append({"cc_threads": th, "cc_grid": gps * sms, "cc_cache": cache, "ms": ms})
    default = next((t for t in trials_out if t["cc_threads"] == start["cc_threads"] and t["cc_grid"] == start["cc_grid"]
                    and t["cc_cache"] == (start["cc_cache"] if start["hubs_loaded"] else 0)), None)
    best = min(trials_out, key=lambda t: t["ms"])
    G.tune(cc_threads=best["cc_threads"], cc_grid=best["cc_grid"], cc_cache=best["cc_cache"])
    return {"kernel": "cc_pull", "best": {k: best[k] for k in ("cc_threads", "cc_grid", "cc_cache")},
            "best_ms": best["ms"], "default_ms": default["ms"] if default else None, "candidates": len(trials_out),
            "trials": trials_out}


def tune_pr(G, trials: int = 3, grids_per_sm=(0, 1, 2, 4, 8), iterations: int = 4, device: int = 0) -> dict:
    """PageRank gather: persistent grid.  Times `iterations` fused iterations."""
    sms = _sms(device)
    start = G.tuning()

    def run():
        G.pr_init(0.875).pr_iterate(iterations)

    run()
    trials_out = []
    for gps in grids_per_sm:
        G.tune(pr_grid=gps * sms)
        trials_out.append({"pr_grid": gps * sms, "ms": _kernel_ms(G, "pr_gather", run, trials)})
    default = next((t for t in trials_out if t["pr_grid"] == start["pr_grid"]), None)
    best = min(trials_out, key=lambda t: t["ms"])
    G.tune(pr_grid=best["pr_grid"])
    return {"kernel": "pr_gather", "best": {"pr_grid": best["pr_grid"]}, "best_ms": best["ms"],
            "default_ms": default["ms"] if default else None, "candidates": len(trials_out), "trials": trials_out}


def tune_batch(B, seeds, iterations: int = 5, trials: int = 2, blocks=(2, 4, 8, 16)) -> dict:
    """Batch kernels: resident blocks per SM of the PPR gather/apply and of the multi-source
    BFS pull, each timed over whole runs (one CUDA graph launch each)."""
    start = B.tuning()
    out = {}
    for key, run in (("ppr_blocks", lambda: B.ppr(seeds, iterations, 0.85, ranks=False)[1].ms),
                     ("bfs_blocks", lambda: B.msbfs(seeds, levels=False)[1].ms)):
        trials_out = []
        for nb in blocks:
            B.tune(**{key: nb})
            run()  # capture + warm-up
            trials_out.append({key: nb, "ms": statistics.median(run() for _ in range(trials))})
        default = next((t for t in trials_out if t[key] == start[key]), None)
        best = min(trials_out, key=lambda t: t["ms"])
        B.tune(**{key: best[key]})
        out[key] = {"best": best[key], "best_ms": best["ms"], "default_ms": default["ms"] if default else None,
                    "trials": trials_out}
    return out
