"""Regenerate tests/golden/mol_rhs_golden.npz with the oracle.

The reference ships no RHS-level golden vectors and cannot be built here, so
these fixtures freeze the oracle's own output on two small seeded cases (an
8^3 Taylor-Green box and a 6^3 flame box, inputs included).  They pin the
oracle against regressions and give the GPU tests a fixed target; they are
not reference outputs.

    python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from oracle import build, pyoracle  # noqa: E402
from pelec_gb300 import problems  # noqa: E402


def main():
    build.build()
    out = {}
    mech, st = problems.tgv(8, seed=11)
    R, = pyoracle.mol_rhs(problems.make_config(mech), [st])
    out.update(tgv8_S=st.S, tgv8_R=R, tgv8_dx=np.array(st.dx))
    mech, st, _ = problems.flame((6, 6, 6), seed=12)
    R, = pyoracle.mol_rhs(problems.make_config(mech), [st])
    out.update(flame6_S=st.S, flame6_R=R, flame6_dx=np.array(st.dx))
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "mol_rhs_golden.npz")
    np.savez_compressed(path, **out)
    print(path, os.path.getsize(path), "bytes")


if __name__ == "__main__":
    main()
