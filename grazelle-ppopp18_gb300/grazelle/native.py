"""ctypes binding of ``libgrazelle_gb300.so`` (the C ABI of ``include/grazelle_gb300.h`` and
``include/grazelle_phases.h``).

There is no fallback: if the library is missing, or a call reports a CUDA error,
an exception is raised.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

from . import build as _build

GRZ_OK = 0
GRZ_ERR_ARG, GRZ_ERR_CUDA, GRZ_ERR_NOMEM, GRZ_ERR_UNSORTED = -1, -2, -3, -4
GRZ_ERR_RANGE, GRZ_ERR_STATE, GRZ_ERR_IO, GRZ_ERR_TIMEOUT = -5, -6, -7, -8
ERRORS = {
    -1: "GRZ_ERR_ARG", -2: "GRZ_ERR_CUDA", -3: "GRZ_ERR_NOMEM", -4: "GRZ_ERR_UNSORTED",
    -5: "GRZ_ERR_RANGE", -6: "GRZ_ERR_STATE", -7: "GRZ_ERR_IO", -8: "GRZ_ERR_TIMEOUT",
}
APP_PAGERANK, APP_CONNECTED_COMPONENTS, APP_BREADTH_FIRST_SEARCH = 0, 1, 2
LIST_PULL, LIST_PUSH = 0, 1


class GrzError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__("%s (%d): %s" % (ERRORS.get(code, "GRZ_ERR"), code, msg))
        self.code = code


FORCE_PULL, FORCE_PUSH, WITHOUT_COUNT, WITHOUT_OUTDEG = 1, 2, 4, 8
BATCH_K = 8
LOAD_DERIVE_PUSH = 1
TUNE_HUBS, TUNE_CC_CACHE, TUNE_CC_THREADS, TUNE_CC_GRID, TUNE_PR_GRID, TUNE_BFS_PULL_SCAN, TUNE_PR_PROPS = 0, 1, 2, 3, 4, 5, 6
TUNE_INGEST_CHUNKS, TUNE_HUBS_LOADED = 7, 100
TUNE_PR_PERSISTENT, TUNE_PR_WAIT_LIMIT_US, TUNE_PR_WITHHOLD = 8, 9, 10
TUNE_RUN_MAX_ITERATIONS, TUNE_RUN_LIMIT_US, TUNE_PULL_STAGING, TUNE_PR_SEGMENT_BITS = 11, 12, 13, 14
TUNE_CC_SEGMENTS = 16
TUNE_BFS_PULL_FIRST = 17
TUNE_CC_PULL_FIRST = 18
BATCH_TUNE_PPR_BLOCKS, BATCH_TUNE_BFS_BLOCKS, BATCH_TUNE_PPR_PROPS = 0, 1, 2
FLAG_HOST_LOOP = 16  # grz_cc_run / grz_bfs_run: host round trip per iteration instead of one CUDA graph
MLP_FEATURES, MLP_HIDDEN, MLP_PARAMS = 12, 32, 1505
POLICY_THRESHOLD, POLICY_LEARNED = 0, 1


class RunStats(C.Structure):
    _fields_ = [("iterations", C.c_uint32), ("pull_iterations", C.c_uint32), ("push_iterations", C.c_uint32),
                ("ms", C.c_float)]


class GraphInfo(C.Structure):
    _fields_ = [
        ("num_vertices", C.c_uint64), ("num_edges", C.c_uint64),
        ("pull_vectors", C.c_uint64), ("push_vectors", C.c_uint64),
        ("pull_index_start", C.c_uint64), ("pull_index_end", C.c_uint64),
        ("push_index_start", C.c_uint64), ("push_index_end", C.c_uint64),
        ("pull_list_device", C.c_void_p), ("push_list_device", C.c_void_p),
        ("device_bytes", C.c_uint64),
    ]


# every exported symbol with (restype, argtypes); the headers in include/ declare the same set
_VP, _U64, _U32, _I, _D = C.c_void_p, C.c_uint64, C.c_uint32, C.c_int, C.c_double
_PU64, _PD = C.POINTER(C.c_uint64), C.POINTER(C.c_double)
SIGNATURES = {
    # grazelle_gb300.h
    "grz_error_string": (C.c_char_p, [_I]),
    "grz_graph_last_error": (C.c_char_p, [_VP]),
    "grz_graph_create": (_I, [C.POINTER(_VP), _I, _VP]),
    "grz_graph_set_stream": (_I, [_VP, _VP]),
    "grz_graph_destroy": (None, [_VP]),
    "grz_sync": (_I, [_VP]),
    "grz_graph_load_pairs": (_I, [_VP, _U64, _U64, _VP, _VP]),
    "grz_graph_load_files": (_I, [_VP, C.c_char_p]),
    "grz_graph_load_files_ex": (_I, [_VP, C.c_char_p, _I]),
    "grz_stats_enable": (_I, [_VP, _I]),
    "grz_stats_take": (_I, [_VP, C.POINTER(_U64), C.POINTER(_U64)]),
    "grz_graph_vector_model": (_I, [_VP, _I, C.c_uint32, C.POINTER(_U64)]),
    "grz_graph_get_info": (_I, [_VP, C.POINTER(GraphInfo)]),
    "grz_graph_copy_list": (_I, [_VP, _I, _VP, _U64]),
    "grz_graph_copy_vertex_index": (_I, [_VP, _I, _VP, _U64]),
    "grz_graph_copy_outdegrees": (_I, [_VP, _VP, _U64]),
    "grz_pr_init": (_I, [_VP, _D]),
    "grz_pr_iterate": (_I, [_VP, _U32]),
    "grz_read_props": (_I, [_VP, _VP, _U64]),
    "grz_pr_time_iterations": (_I, [_VP, _U32, C.POINTER(C.c_float)]),
    "grz_cc_run": (_I, [_VP, _I, _VP]),
    "grz_bfs_run": (_I, [_VP, _U32, _I, _VP]),
    "grz_read_levels": (_I, [_VP, _VP, _U64]),
    "grz_result_digest": (_I, [_VP, _VP]),
    "grz_tune_set": (_I, [_VP, _I, C.c_int64]),
    "grz_graph_load_pairs_ex": (_I, [_VP, _U64, _U64, _VP, _VP, _I]),
    "grz_batch_create": (_I, [C.POINTER(_VP), _I, _VP]),
    "grz_batch_destroy": (None, [_VP]),
    "grz_batch_last_error": (C.c_char_p, [_VP]),
    "grz_batch_add_graph": (_I, [_VP, _U64, _U64, _VP]),
    "grz_batch_build": (_I, [_VP]),
    "grz_batch_info": (_I, [_VP, _VP, _VP, _VP, _VP]),
    "grz_batch_ppr": (_I, [_VP, _VP, _U32, _U32, _D, _VP, _VP]),
    "grz_batch_msbfs": (_I, [_VP, _VP, _U32, _VP, _VP]),
    "grz_batch_run": (_I, [_VP, _VP, _U32, _U32, _D, _VP, _U32, _VP, _VP, _VP, _VP, _VP]),
    "grz_batch_launch_count": (C.c_ulonglong, [_VP]),
    "grz_batch_tune_set": (_I, [_VP, _I, C.c_int64]),
    "grz_batch_tune_get": (_I, [_VP, _I, _VP]),
    "grz_tune_get": (_I, [_VP, _I, _VP]),
    "grz_frontier_begin": (_I, [_VP, _I, _U32, _I]),
    "grz_frontier_next": (_I, [_VP, _I, C.POINTER(C.c_int), C.POINTER(C.c_uint64)]),
    "grz_frontier_current_vote": (_I, [_VP, C.POINTER(C.c_uint64), C.POINTER(C.c_int)]),
    "grz_mlp_create": (_I, [C.POINTER(_VP), _I, _U64]),
    "grz_mlp_destroy": (None, [_VP]),
    "grz_mlp_get_params": (_I, [_VP, _VP, _U64]),
    "grz_mlp_set_params": (_I, [_VP, _VP, _U64]),
    "grz_mlp_gradients": (_I, [_VP, _VP, _VP, _VP, _U64, _VP, C.POINTER(C.c_float)]),
    "grz_mlp_train": (_I, [_VP, _VP, _VP, _VP, _U64, _U32, C.c_float, C.POINTER(C.c_float)]),
    "grz_mlp_predict": (_I, [_VP, _VP, _U64, _VP]),
    "grz_frontier_set_policy": (_I, [_VP, _I, _VP]),
    "grz_frontier_features": (_I, [_VP, _VP, _U64, C.POINTER(C.c_int)]),
    "grz_frontier_last_features": (_I, [_VP, _VP, _U64]),
    "grz_frontier_snapshot": (_I, [_VP]),
    "grz_frontier_restore": (_I, [_VP]),
    "grz_frontier_next_timed": (_I, [_VP, _I, C.POINTER(C.c_int), C.POINTER(C.c_uint64), C.POINTER(C.c_float)]),
    "grz_profile_enable": (_I, [_VP, _I]),
    "grz_profile_read": (_I, [_VP, C.POINTER(C.c_int), C.POINTER(C.c_float), _I]),
    "grz_profile_kind_name": (C.c_char_p, [_I]),
    "grz_profile_work": (_I, [_VP, _PU64, _PU64]),
    "grz_launch_count": (C.c_ulonglong, [_VP]),
    "grz_fixed_point_roundtrip": (_I, [_D, _PD]),
    "grz_pr_step_noalloc": (_I, [_VP, _U64, _U64, _VP, _VP, _D, _VP, _VP]),
    "grz_pr_step_noalloc_max_vertices": (_U64, []),
    "grz_fixed_point_sum": (_I, [_VP, _U64, _PD]),
    # grazelle_phases.h
    "grz_phases_bind": (_I, [_VP, _I]),
    "grz_phases_last_status": (_I, []),
    "phase_op_reset_global_accum": (None, []),
    "phase_op_write_global_accum_to_buf": (None, [_VP]),
    "phase_op_combine_global_var_from_buf": (_U64, [_VP]),
    "edge_pull_op_merge_with_merge_buffer": (None, [_VP, _U64, _VP]),
    "perform_edge_pull_phase_pr": (None, [_VP, _U64]),
    "perform_edge_pull_phase_cc": (None, [_VP, _U64]),
    "perform_edge_pull_phase_bfs": (None, [_VP, _U64]),
    "perform_edge_push_phase_pr": (None, [_VP, _U64]),
    "perform_edge_push_phase_cc": (None, [_VP, _U64]),
    "perform_edge_push_phase_bfs": (None, [_VP, _U64]),
    "perform_vertex_phase_pr": (None, [_U64, _U64, _VP]),
    "perform_vertex_phase_cc": (None, [_U64, _U64, _VP]),
    "perform_vertex_phase_bfs": (None, [_U64, _U64, _VP]),
}

_lib = None


def library_path() -> Path:
    return _build.LIB


def load(build_if_missing: bool = True):
    """Loads libgrazelle_gb300.so (building it first if asked); raises if it cannot."""
    global _lib
    if _lib is not None:
        return _lib
    path = library_path()
    if not path.exists():
        if not build_if_missing:
            raise RuntimeError("libgrazelle_gb300.so is not built (%s); run __graft_entry__.build()" % path)
        _build.build()
    lib = C.CDLL(str(path))
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def check(rc: int, graph_handle=None):
    if rc != GRZ_OK:
        lib = load()
        msg = lib.grz_graph_last_error(graph_handle).decode() if graph_handle else lib.grz_error_string(rc).decode()
        raise GrzError(rc, msg)
