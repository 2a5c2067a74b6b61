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
and for the configuration state, J at the first three wrinkle amplitudes
a_m +- h_a and a_m +- 2 h_a (h_a = 1e-7 cm), for central and Richardson
differences in a.

About 94 trajectories: 20 minutes on 16 cores.

    python tests/golden/make_c5_fd.py [out.npz]
"""
import dataclasses
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
H_AMP = 1e-7  # cm
DIR_SEED = 2024


def geometry(st):
    return abi.geometry(st.lo, st.hi, (0, 0, abi.PC_BC_OUTFLOW), (0, 0, abi.PC_BC_OUTFLOW))


def objective(st) -> float:
    T = st.valid(st.S)[abi.UTEMP]
    return float(T.sum()) * float(np.prod(st.dx))


def trajectory(cfg, st, dts=None):
    """(J, dts): the trajectory from st (not modified); with dts None the
    time steps are estimated before each step and returned."""
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
    return objective(boxes[0]), (out if dts is None else list(dts))


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
            Ja = np.zeros((3, 4))  # a+h, a-h, a+2h, a-2h
            for m in range(3):
                for c, step in enumerate((H_AMP, -H_AMP, 2 * H_AMP, -2 * H_AMP)):
                    amps = fp.amps.copy()
                    amps[m] += step
                    _, stp, _ = problems.flame(SHAPE, seed=SEED, w_noise=w_noise,
                                               params=dataclasses.replace(fp, amps=amps))
                    Ja[m, c] = trajectory(cfg, stp, dts)[0]
                log(f"wrinkle mode {m}: central FD {(Ja[m, 0] - Ja[m, 1]) / (2 * H_AMP):.12e}")
            res.update({"config_amps": fp.amps.copy(), "config_Jamp": Ja})
    out = out or os.path.join(os.path.dirname(os.path.abspath(__file__)), "c5_fd.npz")
    np.savez_compressed(out, **res)
    log(f"wrote {out}")


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else None)
