"""Python front end of the GB300 engine: one ``Graph`` wraps one ``grz_graph``.

Mirrors the reference's driver flow (source/main.c:62-117): load a graph from
its -pull/-push edge lists, run one application, then read the vertex props
back in the reference's format (PR: rank/outdegree', CC: labels, BFS: parents,
all float64).
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import native


def _ptr(a: np.ndarray) -> C.c_void_p:
    return C.c_void_p(a.ctypes.data)


class Graph:
    def __init__(self, device: int = 0, stream: int | None = None):
        self.lib = native.load()
        h = C.c_void_p()
        native.check(self.lib.grz_graph_create(C.byref(h), device, C.c_void_p(stream) if stream else None))
        self.h = h
        self.V = 0
        self.E = 0

    # ------------------------------------------------------------------ lifecycle
    def close(self):
        if self.h:
            self.lib.grz_graph_destroy(self.h)
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
        native.check(rc, self.h)

    def set_stream(self, stream: int | None):
        self._ck(self.lib.grz_graph_set_stream(self.h, C.c_void_p(stream) if stream else None))

    def sync(self):
        self._ck(self.lib.grz_sync(self.h))

    # ------------------------------------------------------------------ profiling
    def profile(self, on: bool = True):
        self._ck(self.lib.grz_profile_enable(self.h, 1 if on else 0))
        return self

    def profile_read(self, capacity: int = 8192):
        """[(kernel kind name, milliseconds)] in launch order since the last read."""
        kinds = (C.c_int * capacity)()
        ms = (C.c_float * capacity)()
        n = self.lib.grz_profile_read(self.h, kinds, ms, capacity)
        if n < 0:
            native.check(n, self.h)
        return [(self.lib.grz_profile_kind_name(kinds[i]).decode(), ms[i]) for i in range(n)]

    def profile_work(self) -> tuple[int, int]:
        """Vectors the CC open-destination pulls read while profiling (first pulls, later pulls)
        since the last call."""
        a, b = C.c_uint64(), C.c_uint64()
        self._ck(self.lib.grz_profile_work(self.h, C.byref(a), C.byref(b)))
        return a.value, b.value

    def tune(self, **kw):
        """Set kernel shapes: hubs=, cc_cache=, cc_threads=, cc_grid=, pr_grid=, bfs_pull_scan=, bfs_pull_first=, cc_pull_first=,
        pr_props=, ingest_chunks=, pr_persistent=, pull_staging=, pr_segment_bits=, cc_segments= (results never depend on them; hubs and ingest_chunks take effect
        at the next load), and the bounds of the device-side waits: pr_wait_limit_us=, run_max_iterations=,
        run_limit_us= (pr_withhold= injects a barrier fault for tests)."""
        keys = {"hubs": native.TUNE_HUBS, "cc_cache": native.TUNE_CC_CACHE, "cc_threads": native.TUNE_CC_THREADS,
                "cc_grid": native.TUNE_CC_GRID, "pr_grid": native.TUNE_PR_GRID, "bfs_pull_scan": native.TUNE_BFS_PULL_SCAN,
                "pr_props": native.TUNE_PR_PROPS, "ingest_chunks": native.TUNE_INGEST_CHUNKS,
                "pr_persistent": native.TUNE_PR_PERSISTENT, "pr_wait_limit_us": native.TUNE_PR_WAIT_LIMIT_US,
                "pr_withhold": native.TUNE_PR_WITHHOLD, "run_max_iterations": native.TUNE_RUN_MAX_ITERATIONS,
                "run_limit_us": native.TUNE_RUN_LIMIT_US, "pull_staging": native.TUNE_PULL_STAGING,
                "pr_segment_bits": native.TUNE_PR_SEGMENT_BITS,
                "cc_segments": native.TUNE_CC_SEGMENTS, "bfs_pull_first": native.TUNE_BFS_PULL_FIRST, "cc_pull_first": native.TUNE_CC_PULL_FIRST}
        for k, v in kw.items():
            self._ck(self.lib.grz_tune_set(self.h, keys[k], int(v)))
        return self

    def tuning(self) -> dict:
        out = {}
        for k, p in (("hubs", native.TUNE_HUBS), ("cc_cache", native.TUNE_CC_CACHE), ("cc_threads", native.TUNE_CC_THREADS),
                     ("cc_grid", native.TUNE_CC_GRID), ("pr_grid", native.TUNE_PR_GRID),
                     ("bfs_pull_scan", native.TUNE_BFS_PULL_SCAN), ("pr_props", native.TUNE_PR_PROPS),
                     ("ingest_chunks", native.TUNE_INGEST_CHUNKS), ("pr_persistent", native.TUNE_PR_PERSISTENT),
                     ("pr_wait_limit_us", native.TUNE_PR_WAIT_LIMIT_US), ("pr_withhold", native.TUNE_PR_WITHHOLD),
                     ("run_max_iterations", native.TUNE_RUN_MAX_ITERATIONS), ("run_limit_us", native.TUNE_RUN_LIMIT_US), ("pull_staging", native.TUNE_PULL_STAGING), ("pr_segment_bits", native.TUNE_PR_SEGMENT_BITS), ("cc_segments", native.TUNE_CC_SEGMENTS), ("bfs_pull_first", native.TUNE_BFS_PULL_FIRST), ("cc_pull_first", native.TUNE_CC_PULL_FIRST),
                     ("hubs_loaded", native.TUNE_HUBS_LOADED)):
            v = C.c_int64()
            self._ck(self.lib.grz_tune_get(self.h, p, C.byref(v)))
            out[k] = v.value
        return out

    def launch_count(self) -> int:
        return int(self.lib.grz_launch_count(self.h))

    # ------------------------------------------------------------------ ingest
    def load_pairs(self, num_vertices: int, pull_pairs, push_pairs=None):
        """Interleaved (src, dst) uint64 pairs in file order.  numpy arrays (host) or raw device pointers (int)."""
        def arg(x):
            if x is None:
                return None, 0
            if isinstance(x, int):
                return C.c_void_p(x), None
            x = np.ascontiguousarray(x, dtype=np.uint64)
            return _ptr(x), x
        pp, keep1 = arg(pull_pairs)
        sp, keep2 = arg(push_pairs)
        if isinstance(pull_pairs, int):
            raise ValueError("pass the edge count with load_device_pairs for device pointers")
        E = keep1.shape[0] // 2
        self._ck(self.lib.grz_graph_load_pairs(self.h, num_vertices, E, pp, sp))
        self.V, self.E = num_vertices, E
        return self

    def load_pointers(self, num_vertices: int, num_edges: int, pull_ptr: int, push_ptr: int | None = None):
        """Edge lists given as raw pointers (pinned host or device memory), 2*E uint64 each."""
        self._ck(self.lib.grz_graph_load_pairs(self.h, num_vertices, num_edges, C.c_void_p(pull_ptr),
                                               C.c_void_p(push_ptr) if push_ptr else None))
        self.V, self.E = num_vertices, num_edges
        return self

    def load_pull_derive_push(self, num_vertices: int, num_edges: int, pull_ptr: int):
        """Only the -pull list (raw pointer, pinned host or device); the -push list is built on the
        device from it (GRZ_LOAD_DERIVE_PUSH)."""
        self._ck(self.lib.grz_graph_load_pairs_ex(self.h, num_vertices, num_edges, C.c_void_p(pull_ptr), None,
                                                  native.LOAD_DERIVE_PUSH))
        self.V, self.E = num_vertices, num_edges
        return self

    def load_device_pairs(self, num_vertices: int, num_edges: int, pull_ptr: int, push_ptr: int | None = None):
        self._ck(self.lib.grz_graph_load_pairs(self.h, num_vertices, num_edges, C.c_void_p(pull_ptr),
                                               C.c_void_p(push_ptr) if push_ptr else None))
        self.V, self.E = num_vertices, num_edges
        return self

    def load_files(self, base: str, derive_push: bool = False):
        """`<base>-pull` (and `<base>-push`, or with derive_push the -push list built on the device)."""
        self._ck(self.lib.grz_graph_load_files_ex(self.h, base.encode(), native.LOAD_DERIVE_PUSH if derive_push else 0))
        info = self.info()
        self.V, self.E = info.num_vertices, info.num_edges
        return self

    def info(self) -> native.GraphInfo:
        out = native.GraphInfo()
        self._ck(self.lib.grz_graph_get_info(self.h, C.byref(out)))
        return out

    def list_vectors(self, which: int = native.LIST_PULL) -> np.ndarray:
        info = self.info()
        n = info.pull_vectors if which == native.LIST_PULL else info.push_vectors
        out = np.zeros((n, 4), dtype=np.uint64)
        self._ck(self.lib.grz_graph_copy_list(self.h, which, _ptr(out), n))
        return out

    def vertex_index(self, which: int = native.LIST_PULL) -> np.ndarray:
        out = np.zeros(self.V + 64, dtype=np.uint64)
        self._ck(self.lib.grz_graph_copy_vertex_index(self.h, which, _ptr(out), out.shape[0]))
        return out

    def outdegrees(self) -> np.ndarray:
        out = np.zeros(self.V, dtype=np.float64)
        self._ck(self.lib.grz_graph_copy_outdegrees(self.h, _ptr(out), out.shape[0]))
        return out

    def vector_model(self, list_id: int, lanes: int) -> int:
        """Vectors the list would need with `lanes`-wide vectors (the reference's MODEL_LONG_VECTORS)."""
        n = C.c_uint64()
        self._ck(self.lib.grz_graph_vector_model(self.h, list_id, lanes, C.byref(n)))
        return n.value

    def stats_enable(self, on: bool = True):
        """Per-phase counts of processed vectors and their edges (the reference's ITERATION_STATS)."""
        self._ck(self.lib.grz_stats_enable(self.h, 1 if on else 0))
        return self

    def stats_take(self) -> tuple[int, int]:
        v, e = C.c_uint64(), C.c_uint64()
        self._ck(self.lib.grz_stats_take(self.h, C.byref(v), C.byref(e)))
        return v.value, e.value

    # ------------------------------------------------------------------ PageRank
    def pr_init(self, damping: float = 0.875):
        self._ck(self.lib.grz_pr_init(self.h, damping))
        return self

    def pr_iterate(self, iterations: int):
        self._ck(self.lib.grz_pr_iterate(self.h, iterations))
        return self

    def pr_time(self, iterations: int) -> float:
        ms = C.c_float()
        self._ck(self.lib.grz_pr_time_iterations(self.h, iterations, C.byref(ms)))
        return ms.value

    def pagerank(self, iterations: int, damping: float = 0.875) -> np.ndarray:
        """Props (rank / outdegree') after `iterations` pull iterations, as the reference stores them."""
        self.pr_init(damping).pr_iterate(iterations)
        return self.props()

    def props(self) -> np.ndarray:
        out = np.zeros(self.V, dtype=np.float64)
        self._ck(self.lib.grz_read_props(self.h, _ptr(out), out.shape[0]))
        return out

    # ------------------------------------------------------------------ CC / BFS
    def connected_components(self, flags: int = 0, stats: bool = False):
        """CC labels (float64, as the reference stores them) after running to convergence."""
        st = native.RunStats()
        self._ck(self.lib.grz_cc_run(self.h, flags, C.byref(st)))
        lab = self.props()
        return (lab, st) if stats else lab

    def cc_run(self, flags: int = 0) -> native.RunStats:
        """CC to convergence without reading the labels back."""
        st = native.RunStats()
        self._ck(self.lib.grz_cc_run(self.h, flags, C.byref(st)))
        return st

    def bfs_run(self, root: int = 0, flags: int = 0) -> native.RunStats:
        """BFS from `root` without reading the result back (see digest / levels / props)."""
        st = native.RunStats()
        self._ck(self.lib.grz_bfs_run(self.h, root, flags, C.byref(st)))
        return st

    def bfs(self, root: int = 0, flags: int = 0, stats: bool = False):
        """(parents float64 with -1 for unvisited/root, levels int64 with -1 for unreached)."""
        st = native.RunStats()
        self._ck(self.lib.grz_bfs_run(self.h, root, flags, C.byref(st)))
        par = self.props()
        lv = np.zeros(self.V, dtype=np.int64)
        self._ck(self.lib.grz_read_levels(self.h, _ptr(lv), lv.shape[0]))
        return (par, lv, st) if stats else (par, lv)

    def set_policy(self, policy: int, switch=None):
        """Engine choice for CC/BFS runs: native.POLICY_THRESHOLD (the reference's rule) or
        native.POLICY_LEARNED with a grazelle.switch.Switch."""
        self._ck(self.lib.grz_frontier_set_policy(self.h, policy, switch.h if switch is not None else None))
        self._switch = switch  # keeps the network alive while the graph refers to it
        return self

    def frontier_begin(self, app: int, root: int = 0, flags: int = 0):
        self._ck(self.lib.grz_frontier_begin(self.h, app, root, flags))
        return self

    def frontier_next(self, engine: int = -1):
        """One iteration; returns (running, engine used, vote)."""
        e = C.c_int()
        v = C.c_uint64()
        rc = self.lib.grz_frontier_next(self.h, engine, C.byref(e), C.byref(v))
        if rc < 0:
            native.check(rc, self.h)
        return rc == 1, e.value, v.value

    def frontier_vote(self):
        v = C.c_uint64()
        e = C.c_int()
        self._ck(self.lib.grz_frontier_current_vote(self.h, C.byref(v), C.byref(e)))
        return v.value, e.value

    def digest(self):
        """(reached vertices or CC components, reached out-edges, checksum of levels/labels),
        computed on the device."""
        out = np.zeros(3, dtype=np.uint64)
        self._ck(self.lib.grz_result_digest(self.h, _ptr(out)))
        return int(out[0]), int(out[1]), int(out[2])

    def levels(self) -> np.ndarray:
        lv = np.zeros(self.V, dtype=np.int64)
        self._ck(self.lib.grz_read_levels(self.h, _ptr(lv), lv.shape[0]))
        return lv
