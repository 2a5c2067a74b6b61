"""Regenerate tests/golden/mol_rhs_golden.npz with PeleC's OWN hot-path code.

The RHS values are computed by the reference's source files compiled where
they lie in the reference tree (oracle/ref_build.py, oracle/ref_harness.cpp:
pc_ctoprim, pc_transcoeff, pc_diffusion_flux, pc_compute_hyp_mol_flux and
pc_flux_div, called in getMOLSrcTerm's order).  PelePhysics is absent, so
the EOS and transport behind those calls are the oracle's restatement and
the 9-species table is synthetic: everything else in these numbers is the
reference's own arithmetic.  The reference tree is needed only to run this
script; the GPU machines use the committed file.

Cases: an 8^3 Taylor-Green box (C1 physics) and a 6^3 flame box (C2
physics) with the default flags, the flame box under the rest of the flag
matrix, a ragged 5x7x6 flame box, and the face fluxes of the flame box.

    python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from oracle import refharness  # noqa: E402
from pelec_gb300 import problems  # noqa: E402

# name -> make_config flags; the flame box runs each of them
FLAME_FLAGS = {
    "laxf": dict(use_laxf_flux=1),
    "first_order": dict(plm_iorder=1),
    "arithmetic_mean": dict(harmonic=0),
    "hydro_only": dict(diffuse=0),
    "diffusion_only": dict(do_hydro=0),
}


def main():
    out = {}
    mech, st = problems.tgv(8, seed=11)
    R, = refharness.mol_rhs(problems.make_config(mech), [st])
    out.update(tgv8_S=st.S, tgv8_R=R, tgv8_dx=np.array(st.dx))
    mech, st, _ = problems.flame((6, 6, 6), seed=12)
    cfg = problems.make_config(mech)
    (R, F), = refharness.mol_rhs(cfg, [st], fluxes=True)
    out.update(flame6_S=st.S, flame6_R=R, flame6_dx=np.array(st.dx))
    out.update({f"flame6_F{d}": F[d] for d in range(3)})
    for name, flags in FLAME_FLAGS.items():
        R, = refharness.mol_rhs(problems.make_config(mech, **flags), [st])
        out[f"flame6_{name}_R"] = R
    mech, st, _ = problems.flame((5, 7, 6), seed=13)
    R, = refharness.mol_rhs(problems.make_config(mech), [st])
    out.update(flame576_S=st.S, flame576_R=R, flame576_dx=np.array(st.dx))
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "mol_rhs_golden.npz")
    np.savez_compressed(path, **out)
    print(path, os.path.getsize(path), "bytes")


if __name__ == "__main__":
    main()
