"""Build recipe of the CUDA library ``pelec_gb300/_lib/libpelec_mol.so``.

Translation units compiled by nvcc for sm_103a only (in parallel) and
linked into one shared library with a plain C ABI (include/pelec_mol.h), no
torch headers; the kernels are instantiated for 1, 9 and 21 species:

* pc_mol.cu — the ABI, the host side and the FP64 kernels, compiled with
  ``-fmad=false``: the FP64 kernels evaluate a fixed sequence of IEEE
  operations (explicit fma() only where written), so they reproduce the CPU
  restatement's arithmetic exactly; host code is built without contraction
  too.
* pc_mol_mixed.cu — the mixed-precision kernels, with contraction on.
* pc_tiles_fp64.cu / pc_tiles_mixed.cu — the flux pass of each precision at
  the tile shapes other than the default, compiled like the unit above them
  (pc_tiles_fp64.cu once per species count, like the two below).
* pc_adjoint.cu — the vector-Jacobian product passes, without contraction
  (their re-evaluated forward quantities must be the forward's own).
* pc_tangent.cu — the Jacobian-vector product (the forward passes on dual
  numbers), without contraction for the same reason.
* pc_rhs_rcp.cu — the FP64 passes a second time, with quotients by a shared
  divisor as products with its reciprocal (PC_PRECISION_FP64_RCP), without
  contraction like pc_mol.cu.

libpc_peaks.so (pc_peaks.cu) measures the FP64/FP32 FMA rates that bench.py
uses as roofline denominators.
"""
from __future__ import annotations

import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
LIBDIR = os.path.join(HERE, "_lib")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off"]

MIXED_FLAGS = ["-fmad=true", "-prec-div=false", "-prec-sqrt=false"]

# The units with the heaviest kernels are compiled once per species count
# (pc_unit_ns.h), so that the compilations run in parallel.
_PER_NS = [(src, ["-fmad=false", f"-DPC_UNIT_NS={ns}"]) for src in ("pc_tiles_fp64.cu", "pc_adjoint.cu", "pc_tangent.cu")
           for ns in (1, 9, 21)]
_PER_NS_MIXED = [("pc_tiles_mixed.cu", MIXED_FLAGS + [f"-DPC_UNIT_NS={ns}"]) for ns in (1, 9, 21)]
LIBS = {
    # The mixed-precision units are checked by error norms, not bit for bit:
    # their FP32 divisions and square roots may be the approximate forms
    # (the double-float arithmetic uses explicit round-to-nearest intrinsics,
    # and denormals are kept).
    "libpelec_mol.so": [("pc_mol.cu", ["-fmad=false"]), ("pc_mol_mixed.cu", MIXED_FLAGS),
                        ("pc_rhs_rcp.cu", ["-fmad=false"])] + _PER_NS + _PER_NS_MIXED,
    # arithmetic peak rates for bench.py's roofline (not part of the ABI)
    "libpc_peaks.so": [("pc_peaks.cu", ["-fmad=true"])],
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
    outs = []
    for lib, units in LIBS.items():
        out = os.path.join(LIBDIR, lib)
        outs.append(out)
        if not force and os.path.exists(out) and os.path.getmtime(out) >= newest:
            continue
        procs, objs = [], []
        for src, flags in units:
            tag = "".join("_ns" + f.split("=")[1] for f in flags if f.startswith("-DPC_UNIT_NS="))
            obj = os.path.join(LIBDIR, os.path.splitext(src)[0] + tag + ".o")
            cmd = [nvcc(), *ARCH, *COMMON, *flags, "-I", os.path.join(ROOT, "include"), "-c", "-o", obj,
                   os.path.join(CSRC, src)]
            if verbose:
                cmd += ["-Xptxas", "-v"]
            procs.append(subprocess.Popen(cmd))
            objs.append(obj)
        for p in procs:
            if p.wait() != 0:
                raise RuntimeError(f"nvcc failed building {lib}")
        subprocess.run([nvcc(), *ARCH, "-shared", "-o", out + ".tmp", *objs], check=True)
        os.replace(out + ".tmp", out)
    return outs


if __name__ == "__main__":
    import sys

    for o in build(force="--force" in sys.argv, verbose="-v" in sys.argv):
        print(o)
