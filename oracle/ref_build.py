"""ORACLE build recipe (test infrastructure): compiles PeleC's own hot-path
source code, where it lies in the reference tree, into
``oracle/_ref/libpc_ref_ns{1,9,21}.so`` — one library per species count,
since NUM_SPECIES is a compile-time constant of the reference — and, on
request, the flop-counting builds ``libpc_ref_count_ns{1,9}.so``.

What is compiled from the reference (unchanged): Source/MOL.cpp (with MOL.H
and Riemann.H), Source/Diffterm.H, Source/Utilities.H, Source/TransCoeff.H,
Source/IndexDefines.H, Source/Constants.H, Source/EBStencilTypes.H.  The
reference's build system is not used: g++ compiles two files of this
directory (ref_harness.cpp includes the reference sources, ref_physics.cpp
supplies the equation of state and transport) against ``ref_shim/``, which
stands in for the absent AMReX and PelePhysics headers and for the
reference headers that only pull those in (PeleC.H, EB.H, GradUtil.H,
Godunov.H, prob.H).  ``-I-`` turns off the search of an including file's own
directory, so ``#include "PeleC.H"`` inside Source/ finds the stand-in
first; everything else resolves in Source/ itself.  ``-I-`` also stops
libstdc++'s parallel-algorithm headers from finding their siblings, so their
directory is named explicitly (``_pstl_dir``).

Outputs go only to oracle/_ref/ (git-ignored).  The reference tree exists
only where the tests are developed, not on the GPU machines; ``available()``
says whether it is here.
"""
from __future__ import annotations

import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
REF_ROOT = os.environ.get("PC_REFERENCE_ROOT", "/root/reference")
REF_SRC = os.path.join(REF_ROOT, "Source")
OUTDIR = os.path.join(HERE, "_ref")
SPECIES = (1, 9, 21)
COUNT_SPECIES = (1, 9)
REF_FILES = ("MOL.cpp", "MOL.H", "Riemann.H", "Diffterm.H", "Utilities.H", "TransCoeff.H", "Timestep.H", "IndexDefines.H",
             "Constants.H", "EBStencilTypes.H")


def available() -> bool:
    return all(os.path.exists(os.path.join(REF_SRC, f)) for f in REF_FILES)


def lib_path(ns: int, count: bool = False) -> str:
    return os.path.join(OUTDIR, f"libpc_ref_{'count_' if count else ''}ns{ns}.so")


def _deps():
    shim = os.path.join(HERE, "ref_shim")
    out = [os.path.join(HERE, f) for f in ("ref_harness.cpp", "ref_physics.cpp", "pc_oracle.hpp")]
    out += [os.path.join(shim, f) for f in os.listdir(shim)]
    out += [os.path.join(REF_SRC, f) for f in REF_FILES]
    out += [os.path.join(ROOT, "include", "pelec_mol.h"), __file__]
    out += [os.path.join(ROOT, "pelec_gb300", "csrc", f) for f in ("pc_exp.h", "pc_exp_tables.h")]
    return out


def _pstl_dir() -> list:
    """The libstdc++ directory holding pstl/ (from g++'s own search list)."""
    r = subprocess.run(["g++", "-x", "c++", "-E", "-v", "-"], input="", capture_output=True, text=True)
    for line in r.stderr.splitlines():
        d = os.path.join(line.strip(), "pstl")
        if line.startswith(" ") and os.path.isfile(os.path.join(d, "glue_algorithm_defs.h")):
            return ["-I", d]
    return []


def build(force: bool = False, count: bool = False) -> list:
    """The reference-source libraries, one per species count; with count,
    the flop-counting builds instead (amrex::Real a counting double,
    ref_shim/flop_count.hpp; exported ref_count_mol_rhs)."""
    if not available():
        raise FileNotFoundError(f"reference sources not found under {REF_SRC}")
    os.makedirs(OUTDIR, exist_ok=True)
    newest = max(os.path.getmtime(p) for p in _deps())
    procs, outs = [], []
    pstl = _pstl_dir()
    # the counting build runs serially (no -fopenmp): its tallies are plain counters
    extra = ["-DPC_COUNT_FLOPS", "-fno-strict-aliasing"] if count else ["-fopenmp"]
    for ns in (COUNT_SPECIES if count else SPECIES):
        out = lib_path(ns, count)
        outs.append(out)
        if not force and os.path.exists(out) and os.path.getmtime(out) >= newest:
            continue
        cmd = ["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-fPIC", "-shared", "-w", *extra,
               f"-DPC_REF_NS={ns}", "-I-", *pstl, "-I", os.path.join(HERE, "ref_shim"), "-I", REF_SRC,
               "-I", os.path.join(ROOT, "include"), "-I", HERE, "-I", os.path.join(ROOT, "pelec_gb300", "csrc"),
               "-o", out + ".tmp", os.path.join(HERE, "ref_harness.cpp"), os.path.join(HERE, "ref_physics.cpp")]
        # g++ notes that -I- is obsolete on every run; show its output only on failure
        procs.append((subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True), out))
    for p, out in procs:
        log, _ = p.communicate()
        if p.returncode != 0:
            raise RuntimeError(f"g++ failed building {out}:\n{log}")
        os.replace(out + ".tmp", out)
    return outs


if __name__ == "__main__":
    import sys

    for o in build(force="--force" in sys.argv, count="--count" in sys.argv):
        print(o)
