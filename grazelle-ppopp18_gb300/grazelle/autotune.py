"""Autotuner: kernel shapes chosen per loaded graph (or batch) by timing them on the device.

The knobs (include/grazelle_gb300.h, GRZ_TUNE_* and GRZ_BATCH_TUNE_*) change only speed:
block size, persistent grid and edge-stream staging of the CC pull kernel, the PageRank
iteration's form (two kernels or one persistent launch) and gather grid, resident blocks per SM
of the batch kernels, and the optional hub-source encoding.  Each candidate is timed on the
device (the run statistics' or CUDA-event times of the whole run or iteration sequence), the
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


def _median_ms(run, trials: int) -> float:
    return statistics.median(run() for _ in range(trials))


def tune_cc(G, trials: int = 3, threads=(256, 512, 1024), grids_per_sm=(0, 1, 2, 4), caches=(0,), stagings=(0, 1),
            forms=(4, 3, 1, 0), device: int = 0) -> dict:
    """CC: the pull form (GRZ_TUNE_CC_PULL_FIRST: 4 open destinations in every pull, 3 and 1 the
    first-vector pass then the whole list, 0 the full first pull), and for the full pull the
    kernel's block size x persistent grid x edge-stream staging (streaming loads or bulk copies
    into shared memory) (x hub-label cache when hubs are loaded); the forms that read the whole
    list in fewer pulls run at the starting shape.  The objective is the whole run to convergence
    (one CUDA graph launch, device time), which is what the knobs are for."""
    sms = _sms(device)
    start = G.tuning()

    def run():
        return G.cc_run().ms

    run()  # warm-up
    trials_out = []

    def trial(form, th, grid, cache, stg):
        G.tune(cc_pull_first=form, cc_threads=th, cc_grid=grid, cc_cache=cache, pull_staging=stg)
        run()  # the run graph is captured again for a new shape
        trials_out.append({"cc_pull_first": form, "cc_threads": th, "cc_grid": grid, "cc_cache": cache, "pull_staging": stg,
                           "ms": _median_ms(run, trials)})

    start_cache = start["cc_cache"] if start["hubs_loaded"] else 0
    for form in forms:
        if form != 0:
            trial(form, start["cc_threads"], start["cc_grid"], start_cache, start["pull_staging"])
            continue
        for th in threads:
            for gps in grids_per_sm:
                for stg in stagings:
                    for cache in caches:
                        if cache and start["hubs_loaded"] == 0:
                            continue
                        trial(0, th, gps * sms, cache, stg)
    keys = ("cc_pull_first", "cc_threads", "cc_grid", "cc_cache", "pull_staging")
    default = next((t for t in trials_out if t["cc_pull_first"] == start["cc_pull_first"] and t["cc_threads"] == start["cc_threads"]
                    and t["cc_grid"] == start["cc_grid"] and t["cc_cache"] == start_cache
                    and t["pull_staging"] == start["pull_staging"]), None)
    best = min(trials_out, key=lambda t: t["ms"])
    G.tune(**{k: best[k] for k in keys})
    return {"objective": "cc run to convergence", "best": {k: best[k] for k in keys},
            "best_ms": best["ms"], "default_ms": default["ms"] if default else None, "candidates": len(trials_out),
            "trials": trials_out}


def tune_pr(G, trials: int = 3, grids_per_sm=(0, 1, 2, 4, 8), forms=(1, 2, 3), iterations: int = 8, device: int = 0) -> dict:
    """PageRank: the iteration's form (two kernels, or one persistent cooperative launch with 6
    or 8 blocks per SM) and, for two kernels, the gather's persistent grid.  The objective is the
    device time of `iterations` iterations."""
    sms = _sms(device)
    start = G.tuning()

    def run():
        G.pr_init(0.875)
        return G.pr_time(iterations)

    run()
    cands = []
    for form in forms:
        cands += [(1, gps) for gps in grids_per_sm] if form == 1 else [(form, 0)]
    trials_out = []
    for form, gps in cands:
        G.tune(pr_persistent=form, pr_grid=gps * sms)
        run()
        trials_out.append({"pr_persistent": form, "pr_grid": gps * sms, "ms": _median_ms(run, trials)})
    keys = ("pr_persistent", "pr_grid")
    default = next((t for t in trials_out if t["pr_grid"] == start["pr_grid"] and t["pr_persistent"] == (start["pr_persistent"] or 1)),
                   None)
    best = min(trials_out, key=lambda t: t["ms"])
    G.tune(**{k: best[k] for k in keys})
    return {"objective": "%d PageRank iterations" % iterations, "best": {k: best[k] for k in keys},
            "best_ms": best["ms"], "default_ms": default["ms"] if default else None, "candidates": len(trials_out),
            "trials": trials_out}


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
