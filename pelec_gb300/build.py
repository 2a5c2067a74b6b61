"""Build recipe of the CUDA library ``pelec_gb300/_lib/libpelec_mol.so``.

One translation unit per library, compiled by nvcc for sm_103a only, with no
torch headers: the library is a plain C ABI (include/pelec_mol.h).
"""
from __future__ import annotations

import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
LIBDIR = os.path.join(HERE, "_lib")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]

LIBS = {
    "libpelec_mol.so": ["pc_mol.cu"],
}


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if cand and (os.path.sep not in cand or os.path.exists(cand)):
            return cand
    return "nvcc"


def _deps():
    out = [os.path.join(ROOT, "include", "pelec_mol.h"), __file__]
    for f in os.listdir(CSRC):
        if f.endswith((".cu", ".cuh", ".h")):
            out.append(os.path.join(CSRC, f))
    return out


def build(force: bool = False, verbose: bool = False) -> list:
    os.makedirs(LIBDIR, exist_ok=True)
    newest = max(os.path.getmtime(p) for p in _deps())
    procs, outs = [], []
    for lib, srcs in LIBS.items():
        out = os.path.join(LIBDIR, lib)
        outs.append(out)
        if not force and os.path.exists(out) and os.path.getmtime(out) >= newest:
            continue
        # -fmad=false: the FP64 kernels evaluate a fixed sequence of IEEE
        # operations (explicit fma() only where written), so they reproduce
        # the CPU restatement's arithmetic exactly; host code likewise.
        cmd = [nvcc(), *ARCH, "-O3", "-std=c++17", "-lineinfo", "-fmad=false", "-Xcompiler", "-fPIC",
               "-Xcompiler", "-ffp-contract=off", "-shared",
               "-I", os.path.join(ROOT, "include"), "-o", out + ".tmp"]
        if verbose:
            cmd += ["-Xptxas", "-v"]
        cmd += [os.path.join(CSRC, s) for s in srcs]
        procs.append((subprocess.Popen(cmd), out))
    for p, out in procs:
        if p.wait() != 0:
            raise RuntimeError(f"nvcc failed building {os.path.basename(out)}")
        os.replace(out + ".tmp", out)
    return outs


if __name__ == "__main__":
    import sys

    for o in build(force="--force" in sys.argv, verbose="-v" in sys.argv):
        print(o)
