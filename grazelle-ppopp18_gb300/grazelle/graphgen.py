"""Seeded synthetic graphs in Grazelle's binary edge-list format.

Grazelle reads a graph as two files (the reference's README.md, "Datasets"): ``<name>-pull`` with
edges grouped by destination in ascending order, and ``<name>-push`` grouped by
source.  Each file is a 64-bit header ``{V, E}`` followed by ``E`` pairs of
64-bit ``(source, destination)`` IDs.  The header is read by
source/graphdata.c:533-568 and the pairs by graphdata.c:577-593.

The paper's datasets are not available here, so seeded R-MAT and Erdős–Rényi
graphs stand in for them.  Every random draw is a splitmix64 hash of
``(seed, edge index, bit level)`` compared against 64-bit integer thresholds.
The same seed therefore yields the same bytes on any machine and with any numpy
build, so a graph written in one place can be regenerated anywhere else.

Generation is plain numpy: this is input synthesis, not the measured path.
"""
from __future__ import annotations

import ctypes as C
import os
from dataclasses import dataclass
from pathlib import Path

import numpy as np

_M64 = (1 << 64) - 1
_GOLDEN = np.uint64(0x9E3779B97F4A7C15)


def _splitmix64(x: np.ndarray) -> np.ndarray:
    """splitmix64 finaliser (Steele, Lea & Flood 2014), element-wise on uint64."""
    with np.errstate(over="ignore"):
        z = x + _GOLDEN
        z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        return z ^ (z >> np.uint64(31))


_TOOLS = None


def _tools():
    """libgrazelle_tools.so (the same draws in C with OpenMP) if it has been built, else None."""
    global _TOOLS
    if _TOOLS is None:
        path = Path(__file__).resolve().parent.parent / "build" / "libgrazelle_tools.so"
        if not path.exists():
            return None
        lib = C.CDLL(str(path))
        u64p = np.ctypeslib.ndpointer(np.uint64, flags="C_CONTIGUOUS")
        lib.grz_gen_rmat_raw.argtypes = [C.c_int, C.c_uint64, C.c_uint64, C.c_uint64, C.c_uint64, C.c_uint64, u64p, u64p]
        lib.grz_gen_er_raw.argtypes = [C.c_uint64, C.c_uint64, C.c_uint64, u64p, u64p]
        lib.grz_radix_sort_u64.argtypes = [u64p, u64p, C.c_uint64, C.c_int]
        lib.grz_radix_sort_u64_mt.argtypes = [u64p, u64p, C.c_uint64, C.c_int]
        lib.grz_sym_keys.argtypes = [u64p, u64p, C.c_uint64, u64p]
        lib.grz_keys_to_pairs.argtypes = [u64p, C.c_uint64, C.c_int, u64p]
        lib.grz_unique_no_loops.restype = C.c_uint64
        lib.grz_unique_no_loops.argtypes = [u64p, C.c_uint64]
        _TOOLS = lib
    return _TOOLS


def _seed_key(seed: int, stream: int) -> np.uint64:
    k = _splitmix64(np.array([(seed * 0x100000001B3 + stream) & _M64], dtype=np.uint64))
    return np.uint64(int(k[0]))


@dataclass
class EdgeList:
    """A directed graph: ``V`` vertices and ``E`` (src, dst) pairs, deduplicated, no self-loops."""
    num_vertices: int
    src: np.ndarray  # uint64[E]
    dst: np.ndarray  # uint64[E]
    push_sorted: bool = False  # edges already in (src, dst) order

    @property
    def num_edges(self) -> int:
        return int(self.src.shape[0])

    def _sorted_by(self, major: np.ndarray, minor: np.ndarray, major_is_src: bool) -> "EdgeList":
        if major_is_src and self.push_sorted:
            return self
        lib = _tools()
        if lib is not None and self.num_vertices <= (1 << 32):
            key = (major.astype(np.uint64) << np.uint64(32)) | minor.astype(np.uint64)
            tmp = np.empty_like(key)
            lib.grz_radix_sort_u64_mt(key, tmp, key.shape[0], max(1, 32 + int(max(self.num_vertices - 1, 1)).bit_length()))
            hi, lo = key >> np.uint64(32), key & np.uint64(0xFFFFFFFF)
            return EdgeList(self.num_vertices, hi, lo, True) if major_is_src else EdgeList(self.num_vertices, lo, hi)
        o = np.lexsort((minor, major))
        return EdgeList(self.num_vertices, self.src[o], self.dst[o], major_is_src)

    def pull_order(self) -> "EdgeList":
        """Edges sorted by (dst, src): the ``-pull`` file order."""
        return self._sorted_by(self.dst, self.src, False)

    def push_order(self) -> "EdgeList":
        """Edges sorted by (src, dst): the ``-push`` file order."""
        return self._sorted_by(self.src, self.dst, True)

    def pairs(self) -> np.ndarray:
        """Interleaved uint64[2E] (src0, dst0, src1, dst1, ...), the on-disk pair layout."""
        out = np.empty(2 * self.num_edges, dtype=np.uint64)
        out[0::2] = self.src
        out[1::2] = self.dst
        return out

    def out_degrees_fast(self) -> np.ndarray:
        return self.out_degrees()

    def out_degrees(self) -> np.ndarray:
        return np.bincount(self.src.astype(np.int64), minlength=self.num_vertices).astype(np.uint64)

    def in_degrees(self) -> np.ndarray:
        return np.bincount(self.dst.astype(np.int64), minlength=self.num_vertices).astype(np.uint64)


def _dedup_keys(num_vertices: int, key: np.ndarray) -> EdgeList:
    lib = _tools()
    tmp = np.empty_like(key)
    bits = max(1, 32 + int(max(num_vertices - 1, 1)).bit_length())
    lib.grz_radix_sort_u64_mt(key, tmp, key.shape[0], bits)
    del tmp
    n = int(lib.grz_unique_no_loops(key, key.shape[0]))
    key = key[:n]
    return EdgeList(num_vertices, key >> np.uint64(32), key & np.uint64(0xFFFFFFFF), True)


def _dedup(num_vertices: int, src: np.ndarray, dst: np.ndarray) -> EdgeList:
    lib = _tools()
    if lib is not None and num_vertices <= (1 << 32):
        return _dedup_keys(num_vertices, (src << np.uint64(32)) | dst)
    keep = src != dst
    src, dst = src[keep], dst[keep]
    if num_vertices <= (1 << 32):
        key = np.unique((src << np.uint64(32)) | dst)
        return EdgeList(num_vertices, key >> np.uint64(32), key & np.uint64(0xFFFFFFFF))
    pairs = np.unique(np.stack([src, dst], axis=1), axis=0)
    return EdgeList(num_vertices, pairs[:, 0].copy(), pairs[:, 1].copy())


def rmat(scale: int, edge_factor: int = 16, a: float = 0.57, b: float = 0.19, c: float = 0.19,
         seed: int = 1, chunk: int = 1 << 24, use_native: bool = True, symmetric: bool = False) -> EdgeList:
    """Directed R-MAT graph (Chakrabarti, Zhan & Faloutsos 2004) with per-bit quadrant sampling.

    ``edge_factor * 2**scale`` edges are drawn.  At bit level ``i`` (MSB first) the
    quadrant is chosen with probabilities a, b, c, 1-a-b-c.  Quadrant b sets the
    destination bit, c sets the source bit, and d sets both.  Self-loops and
    duplicates are then removed, so E is a little below the drawn count.
    """
    n = 1 << scale
    m = edge_factor * n
    ta = np.uint64(min(int(a * 2.0 ** 64), _M64))
    tb = np.uint64(min(int((a + b) * 2.0 ** 64), _M64))
    tc = np.uint64(min(int((a + b + c) * 2.0 ** 64), _M64))
    key = _seed_key(seed, 0x524D4154)  # "RMAT"
    lib = _tools() if use_native else None
    if lib is not None:
        s = np.empty(m, dtype=np.uint64)
        d = np.empty(m, dtype=np.uint64)
        lib.grz_gen_rmat_raw(scale, m, int(key), int(ta), int(tb), int(tc), s, d)
        if symmetric:
            keys = np.empty(2 * m, dtype=np.uint64)
            lib.grz_sym_keys(s, d, m, keys)
            del s, d
            return _dedup_keys(n, keys)
        return _dedup(n, s, d)
    srcs, dsts = [], []
    for lo in range(0, m, chunk):
        hi = min(m, lo + chunk)
        idx = np.arange(lo, hi, dtype=np.uint64)
        s = np.zeros(hi - lo, dtype=np.uint64)
        d = np.zeros(hi - lo, dtype=np.uint64)
        with np.errstate(over="ignore"):
            base = idx * np.uint64(64) + key
        for lvl in range(scale):
            with np.errstate(over="ignore"):
                u = _splitmix64(base + np.uint64(lvl))
            bit = np.uint64(1) << np.uint64(scale - 1 - lvl)
            qb = (u >= ta) & (u < tb)
            qc = (u >= tb) & (u < tc)
            qd = u >= tc
            d |= np.where(qb | qd, bit, np.uint64(0))
            s |= np.where(qc | qd, bit, np.uint64(0))
        srcs.append(s)
        dsts.append(d)
    g = _dedup(n, np.concatenate(srcs), np.concatenate(dsts))
    return symmetrize(g) if symmetric else g


def erdos_renyi(num_vertices: int, avg_degree: float, seed: int = 1, use_native: bool = True) -> EdgeList:
    """Directed G(n, m) graph with m = avg_degree * n uniformly drawn pairs (dedup, no self-loops)."""
    m = int(round(avg_degree * num_vertices))
    key = _seed_key(seed, 0x45524447)  # "ERDG"
    lib = _tools() if use_native else None
    if lib is not None:
        s = np.empty(m, dtype=np.uint64)
        d = np.empty(m, dtype=np.uint64)
        lib.grz_gen_er_raw(num_vertices, m, int(key), s, d)
        return _dedup(num_vertices, s, d)
    idx = np.arange(m, dtype=np.uint64)
    with np.errstate(over="ignore"):
        u = _splitmix64(idx * np.uint64(2) + key)
        w = _splitmix64(idx * np.uint64(2) + np.uint64(1) + key)
    nv = np.uint64(num_vertices)
    # multiply-high maps a uniform 32-bit draw onto [0, n) (n < 2^32)
    s = ((u >> np.uint64(32)) * nv) >> np.uint64(32)
    d = ((w >> np.uint64(32)) * nv) >> np.uint64(32)
    return _dedup(num_vertices, s, d)


def symmetrize(g: EdgeList) -> EdgeList:
    """Union of both edge directions (deduplicated); used for the undirected CC workload."""
    return _dedup(g.num_vertices, np.concatenate([g.src, g.dst]), np.concatenate([g.dst, g.src]))


def relabel_swap(g: EdgeList, root: int) -> EdgeList:
    """Swap vertex IDs ``root`` and 0.

    The reference's BFS always starts at vertex 0 (source/execution_bfs.c:28),
    so another root is run by swapping it with vertex 0 first.
    """
    if root == 0:
        return EdgeList(g.num_vertices, g.src.copy(), g.dst.copy())
    r = np.uint64(root)
    z = np.uint64(0)

    def sw(x):
        y = x.copy()
        y[x == r] = z
        y[x == z] = r
        return y

    return EdgeList(g.num_vertices, sw(g.src), sw(g.dst))


def write_grazelle(g: EdgeList, base: str) -> tuple[str, str]:
    """Write ``base-pull`` (dst-sorted) and ``base-push`` (src-sorted) binary edge lists."""
    paths = (base + "-pull", base + "-push")
    for path, ordered in zip(paths, (g.pull_order(), g.push_order())):
        os.makedirs(os.path.dirname(os.path.abspath(path)), exist_ok=True)
        with open(path, "wb") as f:
            np.array([g.num_vertices, g.num_edges], dtype=np.uint64).tofile(f)
            ordered.pairs().tofile(f)
    return paths


def read_grazelle(path: str) -> EdgeList:
    """Read one Grazelle binary edge-list file (either order); raises ValueError on a bad file."""
    raw = np.fromfile(path, dtype=np.uint64)
    if raw.shape[0] < 2:
        raise ValueError("%s: missing {V, E} header" % path)
    v, e = int(raw[0]), int(raw[1])
    if raw.shape[0] != 2 + 2 * e:
        raise ValueError("%s: header says %d edges but file holds %d words of pairs" % (path, e, raw.shape[0] - 2))
    return EdgeList(v, raw[2::2].copy(), raw[3::2].copy())
