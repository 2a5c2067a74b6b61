"""ORACLE build recipe (test infrastructure): compiles the CPU restatement
``pc_oracle.cpp`` into ``oracle/_build/libpc_oracle.so`` with g++ and OpenMP.

``-ffp-contract=off`` keeps the oracle's arithmetic free of fused
multiply-adds on every host (aarch64 GCC contracts by default), so its results
do not depend on the machine it is built on.  No -march flags: the same
recipe builds on x86_64 and aarch64.
"""
from __future__ import annotations

import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
OUT = os.path.join(HERE, "_build", "libpc_oracle.so")


def build(force: bool = False) -> str:
    src = os.path.join(HERE, "pc_oracle.cpp")
    hdr = os.path.join(HERE, "pc_oracle.hpp")
    api = os.path.join(ROOT, "include", "pelec_mol.h")
    # exp/log of the transport: one implementation shared with the kernels
    shared = [os.path.join(ROOT, "pelec_gb300", "csrc", f) for f in ("pc_exp.h", "pc_exp_tables.h")]
    if not force and os.path.exists(OUT):
        newest = max(os.path.getmtime(p) for p in [src, hdr, api, __file__] + shared)
        if os.path.getmtime(OUT) >= newest:
            return OUT
    os.makedirs(os.path.dirname(OUT), exist_ok=True)
    tmp = OUT + ".tmp"
    cmd = ["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-fopenmp", "-fPIC", "-shared",
           "-I", os.path.join(ROOT, "include"), "-I", os.path.join(ROOT, "pelec_gb300", "csrc"), "-o", tmp, src]
    subprocess.run(cmd, check=True)
    os.replace(tmp, OUT)
    return OUT


if __name__ == "__main__":
    print(build(force=True))
