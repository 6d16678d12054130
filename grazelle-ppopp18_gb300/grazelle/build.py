"""Builds the native libraries in-tree.

* ``build/libgrazelle_gb300.so``: the CUDA kernels and the C ABI of ``include/*.h``.
  It is compiled with nvcc for sm_103a only
  (``-gencode arch=compute_103a,code=sm_103a -lineinfo``), one object per
  translation unit, in parallel.
* ``build/libgrazelle_tools.so``: the host-side graph generator (gcc, OpenMP).
* ``build/grazelle-gb300-{pr,cc,bfs}``: the C host driver, compiled once per
  application as the reference selects its application at compile time
  (Makefile:179-223).

Objects are rebuilt when a source or header is newer.  nvcc cross-compiles, so
this also works on a machine without a GPU.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
from pathlib import Path

PKG = Path(__file__).resolve().parent.parent          # grazelle-ppopp18_gb300/
REPO = PKG.parent
CSRC = PKG / "csrc"
HOST = PKG / "host"
INCLUDE = REPO / "include"
BUILD = PKG / "build"
LIB = BUILD / "libgrazelle_gb300.so"
TOOLS = BUILD / "libgrazelle_tools.so"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-fvisibility=default",
              "--expt-relaxed-constexpr", "-I", str(INCLUDE)]
APPS = {"pr": "PAGERANK", "cc": "CONNECTED_COMPONENTS", "bfs": "BREADTH_FIRST_SEARCH"}


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libgrazelle_gb300.so")


def _newer(target: Path, deps) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(Path(d).stat().st_mtime > t for d in deps)


def _run(cmd):
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed: %s\n%s" % (" ".join(map(str, cmd)), r.stdout[-6000:]))
    return r.stdout


def build(verbose: bool = False, jobs: int | None = None, ptxas_verbose: bool = False) -> Path:
    BUILD.mkdir(parents=True, exist_ok=True)
    headers = list(CSRC.glob("*.cuh")) + list(INCLUDE.glob("*.h"))
    cus = sorted(CSRC.glob("*.cu"))
    objs, cmds = [], []
    nv = nvcc()
    extra = ["-Xptxas", "-v"] if ptxas_verbose else []
    for cu in cus:
        o = BUILD / (cu.stem + ".o")
        objs.append(o)
        if ptxas_verbose or _newer(o, [cu] + headers):
            cmds.append([nv] + ARCH + NVCC_FLAGS + extra + ["-c", str(cu), "-o", str(o)])
    outs = []
    with cf.ThreadPoolExecutor(max_workers=jobs or min(8, os.cpu_count() or 4)) as ex:
        outs = list(ex.map(_run, cmds))
    if verbose or ptxas_verbose:
        for o in outs:
            print(o)
    if cmds or _newer(LIB, objs):
        tmp = BUILD / ("libgrazelle_gb300.so.tmp%d" % os.getpid())
        _run([nv] + ARCH + ["-shared", "-o", str(tmp)] + [str(o) for o in objs] + ["-lcudart_static"])
        os.replace(tmp, LIB)
    gen = CSRC / "grz_graphgen.c"
    if _newer(TOOLS, [gen]):
        tmp = BUILD / ("libgrazelle_tools.so.tmp%d" % os.getpid())
        _run(["gcc", "-O3", "-fPIC", "-shared", "-fopenmp", "-std=c11", "-o", str(tmp), str(gen)])
        os.replace(tmp, TOOLS)
    build_drivers()
    return LIB


def build_driver(app: str, experiments=()) -> Path:
    """The C host driver of one application, with the reference's EXPERIMENTS as
    -DEXPERIMENT_<name> (Makefile:59-176), e.g. build_driver("cc", ["ITERATION_STATS"])."""
    srcs = sorted(HOST.glob("*.c"))
    hdrs = list(HOST.glob("*.h")) + list(INCLUDE.glob("*.h"))
    exps = sorted(experiments)
    exe = BUILD / ("grazelle-gb300-" + app + "".join("-" + e.lower() for e in exps))
    if _newer(exe, srcs + hdrs + [LIB]):
        _run(["gcc", "-O2", "-std=c11", "-D_GNU_SOURCE", "-D" + APPS[app]] + ["-DEXPERIMENT_" + e for e in exps]
             + ["-I", str(INCLUDE), "-I", str(HOST), "-o", str(exe)]
             + [str(s) for s in srcs] + ["-L", str(BUILD), "-lgrazelle_gb300", "-Wl,-rpath," + str(BUILD), "-lm"])
    return exe


def build_drivers() -> list[Path]:
    """C host driver, one binary per application (compile-time selection as in the reference)."""
    if not sorted(HOST.glob("*.c")):
        return []
    return [build_driver(app) for app in APPS]


if __name__ == "__main__":
    import sys
    build(verbose=True, ptxas_verbose="-v" in sys.argv)
    print("built", LIB)
