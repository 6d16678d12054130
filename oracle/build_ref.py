#!/usr/bin/env python3
"""Recipe that compiles the unmodified Grazelle reference into ``oracle/_ref/``.

Test infrastructure only: the binaries it makes are the golden source the
C restatement in ``oracle/grz_oracle.c`` is pinned against.  Nothing in the
product links or runs them.

The reference is x86-64 C plus MASM-syntax AVX2 assembly (the reference's README.md, "Requirements").
This script does not run the reference's Makefile.  Instead it:

1. Translates each ``source/*.asm`` and ``include/*.inc`` to GNU ``as`` syntax
   into ``oracle/_ref/<variant>/asm``.  The text rules are the ones that
   ``buildhelpers/x-as.mk`` and ``buildhelpers/x-as-macros.sh`` apply, written
   here in Python.  Running them in Python also avoids ``/bin/sh`` being dash,
   whose ``echo`` mangles backslashes.
2. Compiles ``source/*.c`` (except ``main.c``) in place with the reference's
   CFLAGS (Makefile:40), one ``-D<APP>`` and ``-DEXPERIMENT_*`` per flag
   (Makefile:70-83, 201-210).  ``oracle/ref_shim/numa.h`` stands in for
   libnuma, which is absent here.
3. Assembles with the reference's ASFLAGS (Makefile:45) plus ``--defsym`` per flag.
4. Links ``oracle/ref_driver.c`` with ``-no-pie`` (the assembly uses absolute 32-bit relocations).

It only builds where the reference does: x86-64 with AVX2
(include/versioninfo.h:33-47).  Elsewhere it says so and exits 0.

Usage: python oracle/build_ref.py [--ref DIR] [--variant NAME ...]

The reference tree is DIR, else the environment variable GRZ_REFERENCE, else
the one place this recipe knows it is mounted read-only (``KNOWN_TREE``).  When
none of them holds the reference the recipe says so and exits 0 (nothing else
needs the binaries: the committed fixtures under tests/golden/ were made by them).
"""
from __future__ import annotations

import argparse
import concurrent.futures as cf
import os
import platform
import re
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
OUT = HERE / "_ref"
KNOWN_TREE = "/root/reference"


def locate(explicit: str | None = None) -> Path | None:
    """The reference tree: the explicit path, GRZ_REFERENCE, or KNOWN_TREE; None if absent."""
    for cand in (explicit, os.environ.get("GRZ_REFERENCE"), KNOWN_TREE):
        if cand and (Path(cand) / "source" / "main.c").exists():
            return Path(cand)
    return None

# variant name -> (ALGORITHM, EXPERIMENTS); mirrors the Makefile's figure targets minus TSX (Makefile:277-355)
VARIANTS = {
    "pr_pull": ("PAGERANK", ["EDGE_FORCE_PULL"]),                      # fig11-pull
    "pr_push": ("PAGERANK", ["EDGE_FORCE_PUSH"]),                      # fig11-push without HTM
    "cc": ("CONNECTED_COMPONENTS", []),                               # default CC build (CAS)
    "cc_twc": ("CONNECTED_COMPONENTS", ["THRESHOLD_WITHOUT_COUNT"]),   # fig12 minus HTM / FORCE_MERGE
    "cc_pull": ("CONNECTED_COMPONENTS", ["EDGE_FORCE_PULL"]),
    "cc_push": ("CONNECTED_COMPONENTS", ["EDGE_FORCE_PUSH"]),
    "bfs": ("BREADTH_FIRST_SEARCH", []),
    "bfs_twc": ("BREADTH_FIRST_SEARCH", ["THRESHOLD_WITHOUT_COUNT"]),  # fig13
    "bfs_pull": ("BREADTH_FIRST_SEARCH", ["EDGE_FORCE_PULL"]),
    "bfs_push": ("BREADTH_FIRST_SEARCH", ["EDGE_FORCE_PUSH"]),
}

CFLAGS = ["-g", "-O3", "-Wall", "-std=c11", "-march=core-avx2", "-masm=intel", "-mno-vzeroupper",
          "-pthread", "-D_GNU_SOURCE", "-Wno-unused-variable", "-Wno-unused-but-set-variable"]
ASFLAGS = ["--64", "-mmnemonic=intel", "-msyntax=intel", "-mnaked-reg"]


# ----------------------------------------------------------------------------------------------
# MASM -> GNU as translation.  Each stage maps a list of lines to a list of lines, like one
# stage of the reference's sed pipeline (a stage may emit embedded newlines; they split lines
# for the next stage exactly as the next sed process would see them).
# ----------------------------------------------------------------------------------------------

def _stage(lines, fn):
    out = []
    for ln in lines:
        out.extend(fn(ln).split("\n"))
    return out


def _sub1(pat, rep):
    rx = re.compile(pat)
    return lambda ln: rx.sub(rep, ln, count=1)


def masm_to_gas(text: str) -> str:
    lines = text.split("\n")
    if lines and lines[-1] == "":
        lines = lines[:-1]
    # egrep -v 'END[SP]?$'
    lines = [ln for ln in lines if not re.search(r"END[SP]?$", ln)]
    stages = [
        lambda ln: ln.replace(";", "#"),
        _sub1(r"INCLUDE (.*)\.inc", r'.include "\1.S"'),
        lambda ln: re.sub(r"^IF([^ ]*) *(.*)", lambda m: ".if" + m.group(1).lower() + " " + m.group(2), ln, count=1),
        _sub1(r"^ELSE", ".else"),
        _sub1(r"^ENDIF", ".endif"),
        _sub1(r"^([^ ]*) *EQU *(.*)$", r".equ \1, \2"),
        _sub1(r"^([^ ]*) *TEXTEQU *<([^>]*)>", r".equ \1, \2"),
        _sub1(r"^EXTRN ([^:]*).*", r".extern \1"),
        _sub1(r"ALIGN\(([0-9]*).*", "\n.align \\1"),
        _sub1(r"_TEXT *SEGMENT.*", ".section .text"),
        _sub1(r"DATA *SEGMENT.*", ".section .data"),
        _sub1(r"CONST *SEGMENT.*", ".section .rodata"),
        _sub1(r"^([^ ]*) *PROC PUBLIC", "\\1:".join([".globl \\1\n", ""])),
        _sub1(r"^([^ ]*) *PROC$", r"\1:"),
        _sub1(r"^PUBLIC *([^ ]*).*", r".globl \1"),
        _sub1(r"^ *([^ ]+) +(DB|DW|DD|DQ|REAL8) (.*)", "\\1:\n\\2 \\3"),
        _sub1(r"^.*DW +([^Hh]*).*", r".word 0x\1"),
        _sub1(r"^.*DQ +([^Hh]*).*", r".8byte 0x\1"),
        _sub1(r"^.*REAL8 +([^Hh]*).*", r".double \1"),
        _sub1(r"(, *)([a-fA-F0-9]*)[hH]", r"\g<1>0x\2"),
    ]
    for st in stages:
        lines = _stage(lines, st)
    # macro conversion (x-as-macros.sh): `read` strips surrounding blanks, unquoted echo
    # collapses internal runs of blanks; parameters inside a macro body become \param.
    out = []
    inmacro = False
    params: list[str] = []
    for raw in lines:
        line = " ".join(raw.split())
        if re.search(r"^[^ ]* *MACRO", line):
            inmacro = True
            name = line.split()[0]
            params = re.sub(r"^.*MACRO *", "", line).replace(",", "").split()
            out.append(".macro " + name + ((" " + " ".join(params)) if params else ""))
        elif "ENDM" in line:
            inmacro = False
            params = []
            out.append(".endm")
        else:
            if inmacro:
                for p in params:
                    line = re.sub(p, lambda m: "\\" + m.group(0), line)
            out.append(line)
    return "\n".join(out) + "\n"


# ----------------------------------------------------------------------------------------------

def run(cmd, cwd=None):
    r = subprocess.run(cmd, cwd=cwd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("command failed: %s\n%s" % (" ".join(map(str, cmd)), r.stdout[-4000:]))
    return r.stdout


def build_variant(ref: Path, name: str, algo: str, exps: list[str], jobs: int) -> Path:
    vdir = OUT / name
    asm_src = vdir / "asm" / "source"
    asm_inc = vdir / "asm" / "include"
    obj = vdir / "obj"
    for d in (asm_src, asm_inc, obj):
        d.mkdir(parents=True, exist_ok=True)
    for inc in sorted((ref / "include").glob("*.inc")):
        (asm_inc / (inc.stem + ".S")).write_text(masm_to_gas(inc.read_text()))
    asm_files = []
    for src in sorted((ref / "source").glob("*.asm")):
        dst = asm_src / (src.stem + ".s")
        dst.write_text(masm_to_gas(src.read_text()))
        asm_files.append(dst)

    dflags = ["-D" + algo] + ["-DEXPERIMENT_" + e for e in exps]
    if exps:
        dflags.append('-DEXPERIMENT_STR="%s"' % " ".join(exps))
    asflags = ASFLAGS + ["-I", str(asm_inc), "--defsym", algo + "=1"]
    for e in exps:
        asflags += ["--defsym", "EXPERIMENT_%s=1" % e]
    inc = ["-I", str(ref / "include"), "-I", str(HERE / "ref_shim")]

    cmds = []
    objs = []
    for c in sorted((ref / "source").glob("*.c")):
        if c.name == "main.c":
            continue
        o = obj / (c.name + ".o")
        cmds.append(["gcc"] + CFLAGS + inc + dflags + ["-c", "-o", str(o), str(c)])
        objs.append(o)
    for s in asm_files:
        o = obj / (s.name + ".o")
        cmds.append(["as"] + asflags + [str(s), "-o", str(o)])
        objs.append(o)
    for extra in (HERE / "ref_driver.c", HERE / "ref_shim" / "numa_stub.c"):
        o = obj / (extra.name + ".o")
        cmds.append(["gcc"] + CFLAGS + inc + dflags + ["-c", "-o", str(o), str(extra)])
        objs.append(o)
    with cf.ThreadPoolExecutor(max_workers=jobs) as ex:
        list(ex.map(run, cmds))
    exe = vdir / "grazelle_ref"
    run(["gcc", "-g", "-no-pie", "-o", str(exe)] + [str(o) for o in objs] + ["-lpthread", "-lrt", "-lm"])
    return exe


def reference_buildable() -> tuple[bool, str]:
    if platform.machine() not in ("x86_64", "AMD64"):
        return False, "reference is x86-64 AVX2 only (include/versioninfo.h:33-47); host is %s" % platform.machine()
    try:
        flags = Path("/proc/cpuinfo").read_text()
    except OSError:
        flags = ""
    if " avx2" not in flags:
        return False, "host CPU lacks AVX2"
    return True, ""


def main(argv=None) -> int:
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default=None, help="reference tree (default: GRZ_REFERENCE, then KNOWN_TREE)")
    ap.add_argument("--variant", action="append")
    ap.add_argument("-j", type=int, default=os.cpu_count() or 4)
    a = ap.parse_args(argv)
    ok, why = reference_buildable()
    if not ok:
        print("build_ref: skipped:", why)
        return 0
    ref = locate(a.ref)
    if ref is None:
        print("build_ref: skipped: no reference tree (give --ref DIR or set GRZ_REFERENCE)")
        return 0
    names = a.variant or list(VARIANTS)
    for n in names:
        algo, exps = VARIANTS[n]
        exe = build_variant(ref, n, algo, exps, a.j)
        print("built", exe)
    return 0


if __name__ == "__main__":
    sys.exit(main())
