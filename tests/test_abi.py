"""The C-ABI library loads without a GPU and exports every function that include/*.h declares."""
import ctypes as C
import math
import re

import numpy as np
import pytest

from conftest import REPO


def declared_functions():
    names = set()
    for h in sorted((REPO / "include").glob("*.h")):
        text = re.sub(r"/\*.*?\*/", "", h.read_text(), flags=re.S)
        text = re.sub(r"//[^\n]*", "", text)
        for m in re.finditer(r"^[A-Za-z_][\w \*]*?\b([a-z_][a-z0-9_]*)\s*\([^;{]*\)\s*;", text, flags=re.M):
            names.add(m.group(1))
    return sorted(names)


def test_headers_declare_the_reference_phase_api():
    names = set(declared_functions())
    for app in ("pr", "cc", "bfs"):
        for ph in ("perform_edge_pull_phase_", "perform_edge_push_phase_", "perform_vertex_phase_"):
            assert ph + app in names
    for f in ("phase_op_reset_global_accum", "phase_op_write_global_accum_to_buf",
              "phase_op_combine_global_var_from_buf", "edge_pull_op_merge_with_merge_buffer"):
        assert f in names


def test_library_exports_every_declared_symbol():
    from grazelle import native
    lib = native.load()
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing
    # and the Python binding describes each of them
    assert set(declared_functions()) <= set(native.SIGNATURES)


def test_no_gpu_calls_fail_cleanly():
    from grazelle import native
    lib = native.load()
    assert lib.grz_error_string(-4).decode().startswith("edge list")
    assert lib.grz_graph_last_error(None).decode() == "no graph"


def test_fixed_point_roundtrip_is_exact():
    from grazelle import native
    lib = native.load()
    rng = np.random.default_rng(0)
    xs = np.concatenate([rng.random(2000), rng.random(2000) * 1e-9, 2.0 ** rng.integers(-70, 3, 2000) * rng.random(2000),
                         [0.0, 1.0, 15.999999, 2.0 ** -72, 1.0 / 3.0]])
    out = C.c_double()
    for x in xs:
        assert lib.grz_fixed_point_roundtrip(float(x), C.byref(out)) == 0
        assert out.value == float(x)


def test_fixed_point_sum_is_correctly_rounded():
    """The exact u128 sum rounded once equals math.fsum (the correctly rounded exact sum)."""
    from grazelle import native
    lib = native.load()
    rng = np.random.default_rng(1)
    out = C.c_double()
    for n in (1, 2, 7, 100, 5000):
        # totals stay below 16, the range of the 4.124 format (PageRank sums stay below ~1)
        xs = np.ascontiguousarray(rng.random(n) * (2.0 ** rng.integers(-40, 0, n)) * (8.0 / n))
        assert lib.grz_fixed_point_sum(xs.ctypes.data, n, C.byref(out)) == 0
        assert out.value == math.fsum(xs.tolist())
    bad = np.array([-1.0])
    assert lib.grz_fixed_point_sum(bad.ctypes.data, 1, C.byref(out)) == -5
    over = np.full(5, 15.0)
    assert lib.grz_fixed_point_sum(over.ctypes.data, 5, C.byref(out)) == -5


def _defines(path):
    out = {}
    for m in re.finditer(r"^#define (GRZ_\w+)\s+(-?\d+)u?\b", path.read_text(), flags=re.M):
        out[m.group(1)] = int(m.group(2))
    return out


def test_constants_agree_across_headers_and_the_binding():
    """The public header, the library's internal header and the Python binding give every shared
    constant (error codes, flags, tuning parameters, load flags) the same value."""
    from grazelle import native
    pub = {}
    for h in sorted((REPO / "include").glob("*.h")):
        pub.update(_defines(h))
    internal = _defines(REPO / "grazelle-ppopp18_gb300" / "csrc" / "grz_internal.cuh")
    shared = sorted(set(pub) & set(internal))
    assert len(shared) >= 20
    for name in shared:
        assert pub[name] == internal[name], name
    checked = 0
    for name, value in pub.items():
        short = name[len("GRZ_"):]
        for cand in (short, short.replace("FLAG_", "", 1) if short.startswith("FLAG_") and not short.endswith("HOST_LOOP") else None):
            if cand and hasattr(native, cand) and isinstance(getattr(native, cand), int):
                assert getattr(native, cand) == value, name
                checked += 1
                break
    assert checked >= 15, checked
    for code, label in native.ERRORS.items():
        assert pub[label] == code, label
