"""Finite differences of the C5 objective along the oracle's CPU trajectory,
saved as tests/golden/c5_fd.npz for tests/test_gpu_trajectory.py.

C5: the 64^3 premixed flame (9 species, FP64, periodic x/y, outflow z),
50 SSP-RK2 steps at CFL 0.3 with the time steps frozen along the base
trajectory (estTimeStep before each step), J = sum over valid cells of T dV
after the last computeTemp.  The trajectory is the oracle's
(oracle/pyoracle.ssprk2_step: ghost fill, RHS, LinComb, computeTemp), the
CPU path pinned bit for bit to the reference's own code.

Saved for two initial states, the configuration's (w and p uniform) and the
same with N(0, 1 cm/s) noise on w:
  * the frozen time steps and J of the base trajectory;
  * for 20 seeded directions v (each conserved component of U0 scaled by a
    seeded N(0,1) factor; UEINT, UTEMP and ghost cells 0), J(U0 +- h v) with
    h = 1e-6 (a relative step of the state);
and for the configuration state and the first three wrinkle amplitudes,
J(a_m + s) - J(a_m - s) at s = h_a and 2 h_a (h_a = 1e-8 cm), each summed
cell by cell from the difference of the two final temperature fields with
an exactly rounded sum (math.fsum), so that the rounding of the two sums of
T does not enter.  A step in a moves the flame, and with it some limiter
arguments across their min/max switches; each crossing adds an error of
order s to the difference quotient (1.7e-6 of dJ/da at 1e-7 cm, 5e-8 at
1e-8 cm for the first mode), which no Richardson step removes, so the step
is small rather than extrapolated.

About 94 trajectories: 20 minutes on 16 cores.  With --amp-only, only the
amplitude differences (12 trajectories) are computed again and written into
the existing fixture.

    python tests/golden/make_c5_fd.py [--amp-only] [out.npz]
"""
import dataclasses
import math
import os
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from oracle import build, pyoracle  # noqa: E402
from pelec_gb300 import abi, problems  # noqa: E402

SHAPE = (64, 64, 64)
SEED = 5
NSTEPS = 50
CFL = 0.3
NDIRS = 20
H_STATE = 1e-6
H_AMP = 1e-8  # cm
DIR_SEED = 2024


def geometry(st):
    return abi.geometry(st.lo, st.hi, (0, 0, abi.PC_BC_OUTFLOW), (0, 0, abi.PC_BC_OUTFLOW))


def objective(st) -> float:
    T = st.valid(st.S)[abi.UTEMP]
    return float(T.sum()) * float(np.prod(st.dx))


def final_state(cfg, st, dts=None):
    """(final BoxState, dts): the trajectory from st (not modified); with dts
    None the time steps are estimated before each step and returned."""
    geom = geometry(st)
    boxes = [problems.BoxState(st.lo, st.hi, st.S.copy(), st.dx)]
    out = []
    for n in range(NSTEPS):
        if dts is None:
            pyoracle.fill_ghosts(boxes, geom, boxes[0].ng)
            dt, _ = pyoracle.est_dt(cfg, boxes, CFL)
            out.append(dt)
        else:
            dt = dts[n]
        boxes = pyoracle.ssprk2_step(cfg, boxes, geom, dt)
    return boxes[0], (out if dts is None else list(dts))


def trajectory(cfg, st, dts=None):
    """(J, dts) of the trajectory from st."""
    fin, dts = final_state(cfg, st, dts)
    return objective(fin), dts


def objective_difference(a, b) -> float:
    """J(a) - J(b), summed cell by cell from T(a) - T(b), exactly rounded."""
    dT = st_T(a) - st_T(b)
    return math.fsum(dT.ravel().tolist()) * float(np.prod(a.dx))


def st_T(st):
    return st.valid(st.S)[abi.UTEMP]


def amplitude_fd(cfg, st, fp, dts, log):
    """(3, 2): J(a_m + s) - J(a_m - s) for the first three wrinkle
    amplitudes at s = H_AMP and 2 H_AMP."""
    dJ = np.zeros((3, 2))
    for m in range(3):
        for c, step in enumerate((H_AMP, 2 * H_AMP)):
            fins = []
            for sgn in (1.0, -1.0):
                amps = fp.amps.copy()
                amps[m] += sgn * step
                _, stp, _ = problems.flame(SHAPE, seed=SEED, params=dataclasses.replace(fp, amps=amps))
                fins.append(final_state(cfg, stp, dts)[0])
            dJ[m, c] = objective_difference(*fins)
        log(f"wrinkle mode {m}: central FD {dJ[m, 0] / (2 * H_AMP):.12e} (step {H_AMP:g} cm), "
            f"{dJ[m, 1] / (4 * H_AMP):.12e} (step {2 * H_AMP:g} cm)")
    return dJ


def directions(st, n=NDIRS, seed=DIR_SEED):
    """The seeded state directions: per-component factors (n, NVAR)."""
    rng = np.random.default_rng(seed)
    sc = rng.normal(size=(n, st.S.shape[0]))
    sc[:, abi.UEINT] = 0.0
    sc[:, abi.UTEMP] = 0.0
    return sc


def direction_field(st, s):
    v = s[:, None, None, None] * st.S
    mask = np.zeros(st.S.shape[1:], bool)
    g = st.ng
    mask[g:-g, g:-g, g:-g] = True
    return v * mask


def state_fd(cfg, st, dts, tag, log):
    sc = directions(st)
    Jp, Jm = [], []
    for d in range(NDIRS):
        v = direction_field(st, sc[d])
        for sgn, acc in ((1.0, Jp), (-1.0, Jm)):
            pert = problems.BoxState(st.lo, st.hi, st.S + sgn * H_STATE * v, st.dx)
            acc.append(trajectory(cfg, pert, dts)[0])
        log(f"{tag}: direction {d}: FD {(Jp[-1] - Jm[-1]) / (2 * H_STATE):.12e}")
    return sc, np.array(Jp), np.array(Jm)


def main(out=None):
    build.build()
    t0 = time.time()

    def log(msg):
        print(f"[{time.time() - t0:7.1f} s] {msg}", flush=True)

    res = {"nsteps": NSTEPS, "cfl": CFL, "h_state": H_STATE, "h_amp": H_AMP, "shape": np.array(SHAPE),
           "seed": SEED, "dir_seed": DIR_SEED}
    for tag, w_noise in (("config", 0.0), ("wnoise", 1.0)):
        mech, st, fp = problems.flame(SHAPE, seed=SEED, w_noise=w_noise)
        cfg = problems.make_config(mech)
        J0, dts = trajectory(cfg, st)
        log(f"{tag}: J = {J0!r}, dt {dts[0]:.6e} .. {dts[-1]:.6e}")
        sc, Jp, Jm = state_fd(cfg, st, dts, tag, log)
        res.update({f"{tag}_J0": J0, f"{tag}_dts": np.array(dts), f"{tag}_scales": sc, f"{tag}_Jp": Jp,
                    f"{tag}_Jm": Jm})
        if tag == "config":
            res.update({"config_amps": fp.amps.copy(), "config_dJamp": amplitude_fd(cfg, st, fp, dts, log)})
    out = out or DEFAULT_OUT
    np.savez_compressed(out, **res)
    log(f"wrote {out}")


def main_amp_only(out=None):
    """Recompute the amplitude differences of an existing fixture (the base
    trajectory's time steps are read from it)."""
    build.build()
    t0 = time.time()

    def log(msg):
        print(f"[{time.time() - t0:7.1f} s] {msg}", flush=True)

    out = out or DEFAULT_OUT
    with np.load(out) as f:
        res = {k: f[k] for k in f.files if k not in ("config_Jamp", "config_dJamp", "h_amp")}
    mech, st, fp = problems.flame(SHAPE, seed=SEED)
    np.testing.assert_array_equal(fp.amps, res["config_amps"])
    cfg = problems.make_config(mech)
    res["h_amp"] = H_AMP
    res["config_dJamp"] = amplitude_fd(cfg, st, fp, [float(v) for v in res["config_dts"]], log)
    np.savez_compressed(out, **res)
    log(f"wrote {out}")


DEFAULT_OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "c5_fd.npz")

if __name__ == "__main__":
    args = [a for a in sys.argv[1:] if a != "--amp-only"]
    if "--amp-only" in sys.argv[1:]:
        main_amp_only(args[0] if args else None)
    else:
        main(args[0] if args else None)
