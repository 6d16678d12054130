"""Batches: many personalized-PageRank and multi-source BFS instances over many graphs.

Wraps grz_batch (csrc/grz_batch.cu).  Graphs of uneven size are added with their -pull
pairs; the device holds them as one block-diagonal union graph, and each run processes up
to BATCH_K instances of every graph in one CUDA graph launch.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import native

NONE = 0xFFFFFFFF


class Batch:
    def __init__(self, device: int = 0, stream: int | None = None):
        self.lib = native.load()
        h = C.c_void_p()
        native.check(self.lib.grz_batch_create(C.byref(h), device, C.c_void_p(stream) if stream else None))
        self.h = h
        self.sizes: list[int] = []
        self.voff = [0]

    def close(self):
        if self.h:
            self.lib.grz_batch_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _ck(self, rc):
        if rc != 0:
            raise native.GrzError(rc, self.lib.grz_batch_last_error(self.h).decode())

    def add_graph(self, num_vertices: int, pull_pairs: np.ndarray):
        """pull_pairs: interleaved (src, dst) uint64, sorted by (dst, src)."""
        p = np.ascontiguousarray(pull_pairs, dtype=np.uint64)
        self._ck(self.lib.grz_batch_add_graph(self.h, num_vertices, p.shape[0] // 2, p.ctypes.data))
        self.sizes.append(int(num_vertices))
        self.voff.append(self.voff[-1] + int(num_vertices))
        return self

    def build(self):
        self._ck(self.lib.grz_batch_build(self.h))
        return self

    def info(self):
        vals = [C.c_uint64() for _ in range(4)]
        self._ck(self.lib.grz_batch_info(self.h, *[C.byref(v) for v in vals]))
        return {"graphs": vals[0].value, "vertices": vals[1].value, "edges": vals[2].value, "vectors": vals[3].value}

    def _ids(self, per_graph):
        k = max(len(r) for r in per_graph)
        a = np.full((len(self.sizes), k), NONE, dtype=np.uint32)
        for g, r in enumerate(per_graph):
            a[g, :len(r)] = r
        return a, k

    def ppr(self, seeds, iterations: int = 20, damping: float = 0.85, ranks: bool = True):
        """seeds: per graph a list of up to BATCH_K local seed vertices.  Returns (per-graph
        [V_g, k] float64 ranks or None, RunStats)."""
        a, k = self._ids(seeds)
        out = np.zeros((self.voff[-1], k), dtype=np.float64) if ranks else None
        st = native.RunStats()
        self._ck(self.lib.grz_batch_ppr(self.h, a.ctypes.data, k, iterations, C.c_double(damping),
                                        out.ctypes.data if ranks else None, C.byref(st)))
        return ([out[self.voff[g]:self.voff[g + 1]] for g in range(len(self.sizes))] if ranks else None), st

    def msbfs(self, roots, levels: bool = True):
        """roots: per graph a list of up to BATCH_K local roots.  Returns (per-graph [V_g, k] int32
        levels, -1 = unreached, or None, RunStats)."""
        a, k = self._ids(roots)
        out = np.zeros((self.voff[-1], k), dtype=np.int32) if levels else None
        st = native.RunStats()
        self._ck(self.lib.grz_batch_msbfs(self.h, a.ctypes.data, k, out.ctypes.data if levels else None, C.byref(st)))
        return ([out[self.voff[g]:self.voff[g + 1]] for g in range(len(self.sizes))] if levels else None), st

    def run(self, seeds, roots, iterations: int = 20, damping: float = 0.85, results: bool = True):
        """PPR from `seeds` and multi-source BFS from `roots` in one CUDA graph launch (the two loops
        run side by side).  Returns (ranks or None, levels or None, PPR RunStats, BFS RunStats,
        total device ms of the launch)."""
        a, k = self._ids(seeds)
        r, kb = self._ids(roots)
        ranks = np.zeros((self.voff[-1], k), dtype=np.float64) if results else None
        levels = np.zeros((self.voff[-1], kb), dtype=np.int32) if results else None
        sp, sb, tot = native.RunStats(), native.RunStats(), C.c_float()
        self._ck(self.lib.grz_batch_run(self.h, a.ctypes.data, k, iterations, C.c_double(damping), r.ctypes.data, kb,
                                        ranks.ctypes.data if results else None, levels.ctypes.data if results else None,
                                        C.byref(sp), C.byref(sb), C.byref(tot)))
        split = (lambda x: [x[self.voff[g]:self.voff[g + 1]] for g in range(len(self.sizes))]) if results else (lambda x: None)
        return split(ranks), split(levels), sp, sb, tot.value

    def tune(self, ppr_blocks: int | None = None, bfs_blocks: int | None = None, ppr_props: int | None = None):
        """Resident blocks per SM of the persistent batch kernels, and the props the PPR gather
        reads (0 or 1 fixed point, 2 doubles); results never depend on them."""
        for p, v in ((native.BATCH_TUNE_PPR_BLOCKS, ppr_blocks), (native.BATCH_TUNE_BFS_BLOCKS, bfs_blocks),
                     (native.BATCH_TUNE_PPR_PROPS, ppr_props)):
            if v is not None:
                self._ck(self.lib.grz_batch_tune_set(self.h, p, int(v)))
        return self

    def tuning(self) -> dict:
        out = {}
        for k, p in (("ppr_blocks", native.BATCH_TUNE_PPR_BLOCKS), ("bfs_blocks", native.BATCH_TUNE_BFS_BLOCKS),
                     ("ppr_props", native.BATCH_TUNE_PPR_PROPS)):
            v = C.c_int64()
            self._ck(self.lib.grz_batch_tune_get(self.h, p, C.byref(v)))
            out[k] = v.value
        return out

    def launch_count(self) -> int:
        return int(self.lib.grz_batch_launch_count(self.h))
