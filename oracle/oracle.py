"""ctypes front end of the CPU oracle (``oracle/grz_oracle.c``) and of the reference binaries.

TEST INFRASTRUCTURE ONLY.  Imported by ``tests/``, ``__graft_entry__.smoke()``
and the CPU-baseline legs of ``bench.py``, where it checks or times the GPU
product.  The product itself never imports it.

Two sources of truth are reachable from here:

* the C restatement (``build()`` compiles it with gcc into ``oracle/_build``);
* the unmodified reference, compiled by ``oracle/build_ref.py`` into
  ``oracle/_ref/<variant>/grazelle_ref``.  It runs on x86-64 with AVX2 only.
  ``run_reference`` drives it through ``oracle/ref_driver.c``.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
import tempfile
from dataclasses import dataclass
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
BUILD = HERE / "_build"
LIB = BUILD / "libgrz_oracle.so"
REF = HERE / "_ref"

FORCE_PULL, FORCE_PUSH, WITHOUT_COUNT, WITHOUT_OUTDEG = 1, 2, 4, 8

_u64p = np.ctypeslib.ndpointer(np.uint64, flags="C_CONTIGUOUS")
_f64p = np.ctypeslib.ndpointer(np.float64, flags="C_CONTIGUOUS")
_i64p = np.ctypeslib.ndpointer(np.int64, flags="C_CONTIGUOUS")
_u8p = np.ctypeslib.ndpointer(np.uint8, flags="C_CONTIGUOUS")


def build(force: bool = False) -> Path:
    """Compile the oracle library (gcc, OpenMP) if it is missing or stale."""
    src = HERE / "grz_oracle.c"
    if force or not LIB.exists() or LIB.stat().st_mtime < src.stat().st_mtime:
        BUILD.mkdir(parents=True, exist_ok=True)
        tmp = LIB.with_suffix(".so.tmp%d" % os.getpid())
        subprocess.check_call(["gcc", "-O2", "-fPIC", "-shared", "-fopenmp", "-std=c11", "-o", str(tmp), str(src), "-lm"])
        os.replace(tmp, LIB)
    return LIB


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(str(LIB))
        L.oracle_shared_id.restype = C.c_uint64
        L.oracle_shared_id.argtypes = [_u64p]
        L.oracle_pack_vectors.restype = C.c_uint64
        L.oracle_pack_vectors.argtypes = [_u64p, C.c_uint64, C.c_int, _u64p]
        L.oracle_vertex_index.argtypes = [_u64p, C.c_uint64, _u64p, C.c_uint64, C.POINTER(C.c_uint64), C.POINTER(C.c_uint64)]
        L.oracle_outdegrees.argtypes = [_u64p, C.c_uint64, C.c_uint64, _f64p]
        L.oracle_pr_init.argtypes = [C.c_uint64, _f64p, _f64p, _f64p]
        L.oracle_pr_pull.argtypes = [_u64p, C.c_uint64, _f64p, C.c_uint64, C.c_uint32, C.c_double, C.c_uint64, _f64p, _f64p]
        L.oracle_pr_pull_mt.restype = C.c_int
        L.oracle_pr_pull_mt.argtypes = [_u64p, C.c_uint64, _f64p, C.c_uint64, C.c_uint32, C.c_double, C.c_uint64, C.c_int, _f64p, _f64p]
        L.oracle_pr_push.argtypes = [_u64p, C.c_uint64, _f64p, C.c_uint64, C.c_uint32, C.c_double, _f64p, _f64p]
        L.oracle_pr_sum.restype = C.c_double
        L.oracle_pr_sum.argtypes = [_f64p, _f64p, C.c_uint64]
        L.oracle_cc.argtypes = [_u64p, C.c_uint64, _u64p, C.c_uint64, _f64p, C.c_uint64, C.c_uint64, C.c_uint64, C.c_int,
                                _f64p, _u64p, _u8p, C.c_uint64]
        L.oracle_bfs.argtypes = [_u64p, C.c_uint64, _u64p, C.c_uint64, _f64p, C.c_uint64, C.c_uint64, C.c_int,
                                 _f64p, _u64p, _u8p, C.c_uint64]
        L.oracle_frontier_mt.restype = C.c_int
        L.oracle_frontier_mt.argtypes = [_u64p, C.c_uint64, _u64p, _u64p, C.c_uint64, _u64p, _f64p, C.c_uint64, C.c_uint64,
                                         C.c_int, C.c_int, C.c_int, _f64p, _u64p]
        L.oracle_bfs_levels.argtypes = [_u64p, C.c_uint64, C.c_uint64, C.c_uint64, _i64p]
        L.oracle_ppr_multi.argtypes = [_u64p, C.c_uint64, C.c_uint64, np.ctypeslib.ndpointer(np.uint32, flags="C_CONTIGUOUS"),
                                       C.c_uint32, C.c_uint32, C.c_double, C.c_int, _f64p]
        L.oracle_bfs_levels_multi.argtypes = [_u64p, C.c_uint64, C.c_uint64, _u64p, C.c_uint32, C.c_int, _i64p]
        L.oracle_cc_min_labels.restype = C.c_uint32
        L.oracle_cc_min_labels.argtypes = [_u64p, C.c_uint64, C.c_uint64, C.c_int,
                                           np.ctypeslib.ndpointer(np.uint32, flags="C_CONTIGUOUS")]
        L.oracle_pr_sample_iteration.argtypes = [_u64p, C.c_uint64, C.c_uint64, C.c_double, C.c_int, _u64p, C.c_uint64, _f64p]
        L.oracle_bfs_check_tree.restype = C.c_uint64
        L.oracle_bfs_check_tree.argtypes = [_u64p, C.c_uint64, C.c_uint64, C.c_uint64, _i64p, _i64p]
        _lib = L
    return _lib


# ------------------------------------------------------------------------------------------------

@dataclass
class Layout:
    """The reference's in-memory graph: both vector lists, vertex indices and outdegrees."""
    V: int
    E: int
    pull_vec: np.ndarray     # uint64[nvec, 4]
    push_vec: np.ndarray     # uint64[nvec, 4]
    pull_index: np.ndarray   # uint64[V+64]
    push_index: np.ndarray   # uint64[V+64]
    outdeg: np.ndarray       # float64[V]


def pack_vectors(pairs: np.ndarray, shared_is_dst: bool) -> np.ndarray:
    pairs = np.ascontiguousarray(pairs, dtype=np.uint64)
    e = pairs.shape[0] // 2
    out = np.zeros((max(e, 1), 4), dtype=np.uint64)
    n = lib().oracle_pack_vectors(pairs, e, 1 if shared_is_dst else 0, out.reshape(-1))
    return out[:n].copy()


def vertex_index(vec: np.ndarray, V: int) -> tuple[np.ndarray, int, int]:
    idx = np.zeros(V + 64, dtype=np.uint64)
    s, e = C.c_uint64(), C.c_uint64()
    lib().oracle_vertex_index(np.ascontiguousarray(vec).reshape(-1), vec.shape[0], idx, V + 64, C.byref(s), C.byref(e))
    return idx, s.value, e.value


def outdegrees(pull_pairs: np.ndarray, V: int) -> np.ndarray:
    out = np.zeros(V, dtype=np.float64)
    lib().oracle_outdegrees(np.ascontiguousarray(pull_pairs, dtype=np.uint64), pull_pairs.shape[0] // 2, V, out)
    return out


def layout(V: int, pull_pairs: np.ndarray, push_pairs: np.ndarray) -> Layout:
    pv = pack_vectors(pull_pairs, True)
    sv = pack_vectors(push_pairs, False)
    pi, _, _ = vertex_index(pv, V)
    si, _, _ = vertex_index(sv, V)
    return Layout(V, pull_pairs.shape[0] // 2, pv, sv, pi, si, outdegrees(pull_pairs, V))


def pr_pull(L: Layout, iters: int, damping: float = 0.875, units: int = 32, threads: int = 0,
            multithreaded: bool = False) -> np.ndarray:
    """PageRank props (rank / outdegree', as the reference stores them) after `iters` pull iterations."""
    prop = np.zeros(L.V + 8, dtype=np.float64)
    acc = np.zeros(L.V + 8, dtype=np.float64)
    od = np.zeros(L.V + 8, dtype=np.float64)
    od[:L.V] = L.outdeg
    lib().oracle_pr_init(L.V, od, prop, acc)
    flat = np.ascontiguousarray(L.pull_vec).reshape(-1)
    if multithreaded:
        lib().oracle_pr_pull_mt(flat, L.pull_vec.shape[0], od, L.V, iters, damping, units, threads, prop, acc)
    else:
        lib().oracle_pr_pull(flat, L.pull_vec.shape[0], od, L.V, iters, damping, units, prop, acc)
    return prop[:L.V].copy()


def pr_push(L: Layout, iters: int, damping: float = 0.875) -> np.ndarray:
    prop = np.zeros(L.V + 8, dtype=np.float64)
    acc = np.zeros(L.V + 8, dtype=np.float64)
    od = np.zeros(L.V + 8, dtype=np.float64)
    od[:L.V] = L.outdeg
    lib().oracle_pr_init(L.V, od, prop, acc)
    lib().oracle_pr_push(np.ascontiguousarray(L.push_vec).reshape(-1), L.push_vec.shape[0], od, L.V, iters, damping, prop, acc)
    return prop[:L.V].copy()


def cc(L: Layout, flags: int = 0, units: int = 32):
    labels = np.zeros(L.V, dtype=np.float64)
    it = np.zeros(3, dtype=np.uint64)
    log = np.zeros(1 << 16, dtype=np.uint8)
    lib().oracle_cc(np.ascontiguousarray(L.pull_vec).reshape(-1), L.pull_vec.shape[0],
                    np.ascontiguousarray(L.push_vec).reshape(-1), L.push_vec.shape[0],
                    np.ascontiguousarray(L.outdeg), L.V, L.E, units, flags, labels, it, log, log.shape[0])
    return labels, it, log[:int(it[0])].copy()


def bfs(L: Layout, flags: int = 0):
    parent = np.zeros(L.V, dtype=np.float64)
    it = np.zeros(3, dtype=np.uint64)
    log = np.zeros(1 << 16, dtype=np.uint8)
    lib().oracle_bfs(np.ascontiguousarray(L.pull_vec).reshape(-1), L.pull_vec.shape[0],
                     np.ascontiguousarray(L.push_vec).reshape(-1), L.push_vec.shape[0],
                     np.ascontiguousarray(L.outdeg), L.V, L.E, flags, parent, it, log, log.shape[0])
    return parent, it, log[:int(it[0])].copy()


def frontier_mt(L: Layout, app: int, flags: int = 0, threads: int = 0):
    """Multi-threaded CC (app 1) or BFS (app 2) with the reference's SPMD semantics; (props, iters, threads)."""
    props = np.zeros(L.V, dtype=np.float64)
    it = np.zeros(3, dtype=np.uint64)
    n = lib().oracle_frontier_mt(np.ascontiguousarray(L.pull_vec).reshape(-1), L.pull_vec.shape[0], L.pull_index,
                                 np.ascontiguousarray(L.push_vec).reshape(-1), L.push_vec.shape[0], L.push_index,
                                 np.ascontiguousarray(L.outdeg), L.V, L.E, app, flags, threads, props, it)
    return props, it, n


def bfs_levels(push_pairs: np.ndarray, V: int, root: int = 0) -> np.ndarray:
    lv = np.zeros(V, dtype=np.int64)
    lib().oracle_bfs_levels(np.ascontiguousarray(push_pairs, dtype=np.uint64), push_pairs.shape[0] // 2, V, root, lv)
    return lv


def bfs_levels_multi(push_pairs: np.ndarray, V: int, roots, threads: int = 0) -> np.ndarray:
    """BFS levels from several roots at once (one CSR, the roots on parallel threads): [n, V]."""
    r = np.ascontiguousarray(np.asarray(roots, dtype=np.uint64))
    lv = np.zeros((r.shape[0], V), dtype=np.int64)
    lib().oracle_bfs_levels_multi(np.ascontiguousarray(push_pairs, dtype=np.uint64), push_pairs.shape[0] // 2, V, r,
                                  r.shape[0], threads, lv)
    return lv


def ppr_multi(V: int, pull_pairs: np.ndarray, seeds, iterations: int, damping: float, threads: int = 0) -> np.ndarray:
    """Personalized PageRank of several seeds side by side (oracle/ppr.py's definition, in C with
    OpenMP): ranks [V, K]; a seed >= V leaves its column zero."""
    s = np.ascontiguousarray(np.asarray(seeds, dtype=np.uint32))
    assert 0 < s.shape[0] <= 64
    out = np.zeros((V, s.shape[0]), dtype=np.float64)
    lib().oracle_ppr_multi(np.ascontiguousarray(pull_pairs, dtype=np.uint64), pull_pairs.shape[0] // 2, V, s, s.shape[0],
                           iterations, damping, threads, out)
    return out


def cc_min_labels(pull_pairs: np.ndarray, V: int, threads: int = 0) -> np.ndarray:
    """CC labels from the -pull pairs alone: the smallest vertex ID reaching each vertex (uint32[V])."""
    lab = np.zeros(V, dtype=np.uint32)
    lib().oracle_cc_min_labels(np.ascontiguousarray(pull_pairs, dtype=np.uint64), pull_pairs.shape[0] // 2, V, threads, lab)
    return lab


def pr_sample_iteration(pull_pairs: np.ndarray, V: int, samples, damping: float = 0.875, threads: int = 0) -> np.ndarray:
    """PageRank props after one iteration from the initial props, at the sampled destinations only."""
    smp = np.ascontiguousarray(np.asarray(samples, dtype=np.uint64))
    out = np.zeros(smp.shape[0], dtype=np.float64)
    lib().oracle_pr_sample_iteration(np.ascontiguousarray(pull_pairs, dtype=np.uint64), pull_pairs.shape[0] // 2, V, damping,
                                     threads, smp, smp.shape[0], out)
    return out


def bfs_check_tree(push_pairs: np.ndarray, V: int, root: int, level: np.ndarray, parent: np.ndarray) -> int:
    """0 if `parent` is a legal BFS tree for `level`, else 1 + the first bad vertex."""
    return int(lib().oracle_bfs_check_tree(np.ascontiguousarray(push_pairs, dtype=np.uint64), push_pairs.shape[0] // 2,
                                           V, root, np.ascontiguousarray(level, dtype=np.int64),
                                           np.ascontiguousarray(parent, dtype=np.int64)))


def relative_l1(a: np.ndarray, b: np.ndarray) -> float:
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    den = np.abs(b).sum()
    return float(np.abs(a - b).sum() / den) if den else float(np.abs(a - b).sum())


# ------------------------------------------------------------------------------------------------
# The reference binary (x86-64 only)

def reference_exe(variant: str) -> Path:
    return REF / variant / "grazelle_ref"


def reference_available(variant: str = "pr_pull") -> bool:
    return reference_exe(variant).exists()


@dataclass
class RefRun:
    props: np.ndarray
    outdeg: np.ndarray
    iterations: int
    pull_iterations: int
    push_iterations: int
    elapsed_ns: int
    threads: int
    stdout: str


def run_reference(variant: str, graph_base: str, threads: int = 1, iters: int = 1, lists: bool = False,
                  extra_args=()):
    """Run oracle/_ref/<variant>/grazelle_ref on <graph_base>-pull/-push and read its binary dump."""
    exe = reference_exe(variant)
    with tempfile.TemporaryDirectory() as td:
        env = dict(os.environ)
        env["GRZ_REF_DUMP"] = os.path.join(td, "dump.bin")
        if lists:
            env["GRZ_REF_DUMP_LISTS"] = os.path.join(td, "lists.bin")
        cmd = [str(exe), "-i", graph_base, "-n", str(threads), "-N", str(iters)] + list(extra_args)
        r = subprocess.run(cmd, env=env, stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True, timeout=3600)
        if r.returncode != 0:
            raise RuntimeError("reference exited %d: %s %s" % (r.returncode, r.stdout[-2000:], r.stderr[-2000:]))
        raw = np.fromfile(env["GRZ_REF_DUMP"], dtype=np.uint64)
        V = int(raw[1])
        props = raw[8:8 + V].view(np.float64).copy()
        outdeg = raw[8 + V:8 + 2 * V].view(np.float64).copy()
        run = RefRun(props, outdeg, int(raw[3]), int(raw[4]), int(raw[5]), int(raw[6]), int(raw[7]), r.stdout)
        if not lists:
            return run
        lr = np.fromfile(env["GRZ_REF_DUMP_LISTS"], dtype=np.uint64)
        nv, ng, ns = int(lr[0]), int(lr[2]), int(lr[3])
        off = 4
        gl = lr[off:off + 4 * ng].reshape(ng, 4).copy(); off += 4 * ng
        gi = lr[off:off + nv + 64].copy(); off += nv + 64
        sl = si = None
        if ns:
            sl = lr[off:off + 4 * ns].reshape(ns, 4).copy(); off += 4 * ns
            si = lr[off:off + nv + 64].copy()
        return run, (gl, gi, sl, si)
