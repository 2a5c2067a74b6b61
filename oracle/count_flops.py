"""ORACLE — test infrastructure: the algorithmic floating-point work of one
RHS of each benchmark workload, counted exactly.

The reference's own hot-path sources (ref_harness.cpp: getMOLSrcTerm's
regular-box body with pc_ctoprim, the transport call, pc_diffusion_flux,
pc_compute_hyp_mol_flux with mol_slope and riemann, pc_flux_div) and the
oracle's equation of state and transport are compiled with amrex::Real a
counting double (ref_shim/flop_count.hpp, oracle/ref_build.py count=True)
and run once on the workload's box: every +, -, *, /, fma, sqrt, exp, log
and pow is tallied by class.  flops = add + mul + div + sqrt + 2 fma (a
fused multiply-add counted as two, as the GPU's DFMA is in the ncu counts);
exp, log and pow are reported beside them as transcendentals.  The counts
are the algorithm's (one IEEE operation each), not what a GPU executes to
perform them (a division or an exp is several instructions there).

    python oracle/count_flops.py [c1 c2 c4] [--out profiles/algorithmic_flops.txt]

C4 (256^3) takes about 10 minutes on one core.
"""
from __future__ import annotations

import os
import sys
import time

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

from oracle import refharness  # noqa: E402
from pelec_gb300 import problems  # noqa: E402

WORKLOADS = {
    "c1": "64^3 Taylor-Green vortex, 1 species, GammaLaw, constant transport",
    "c2": "128^3 premixed flame, 9 species, ideal mixture, mixture-averaged transport",
    "c4": "256^3 premixed flame, 9 species, ideal mixture, mixture-averaged transport",
}


def state(name: str):
    if name == "c1":
        mech, st = problems.tgv(64, seed=0)
    else:
        n = 256 if name == "c4" else 128
        mech, st, _ = problems.flame((n, n, n), seed=1)
    return mech, st


def count(name: str) -> dict:
    mech, st = state(name)
    cfg = problems.make_config(mech)
    t0 = time.time()
    c, _ = refharness.count_mol_rhs(cfg, [st])
    cells = st.ncells
    flops = c["add"] + c["mul"] + c["div"] + c["sqrt"] + 2 * c["fma"]
    out = {f"{name}_{k}": v for k, v in c.items()}
    out[f"{name}_cells"] = cells
    out[f"{name}_flops_per_rhs"] = flops
    out[f"{name}_flops_per_cell"] = round(flops / cells, 2)
    out[f"{name}_transcendentals_per_cell"] = round((c["exp"] + c["log"] + c["pow"]) / cells, 3)
    print(f"{name}: {flops / cells:.1f} flops per cell ({time.time() - t0:.0f} s)", flush=True)
    return out


def main(argv):
    names = [a for a in argv if a in WORKLOADS] or list(WORKLOADS)
    out_path = os.path.join(ROOT, "profiles", "algorithmic_flops.txt")
    if "--out" in argv:
        out_path = argv[argv.index("--out") + 1]
    res = {}
    for n in names:
        res.update(count(n))
    lines = [
        "# Algorithmic floating-point work of one RHS (getMOLSrcTerm's regular-box body) per workload,",
        "# counted exactly by running the reference's own hot-path sources and the oracle's EOS and",
        "# transport with amrex::Real a counting double (oracle/ref_shim/flop_count.hpp), from",
        "#   python oracle/count_flops.py " + " ".join(names),
        "# flops = add + mul + div + sqrt + 2 fma; exp, log, pow are the transcendentals; cmp are",
        "# comparisons, min and max (not floating-point work).  Per valid cell of the box; the",
        "# counts include the ghost-cell work of grow(valid, 4) as getMOLSrcTerm does it.",
    ]
    for n in names:
        lines.append(f"# {n}: {WORKLOADS[n]}")
    lines += [f"{k}: {v}" for k, v in res.items()]
    with open(out_path, "w") as f:
        f.write("\n".join(lines) + "\n")
    print("wrote", out_path)


if __name__ == "__main__":
    main(sys.argv[1:])
