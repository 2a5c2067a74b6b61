"""Seeded synthetic states for the MOL right-hand side.

Each state is a FAB with ``NG = 4`` ghost layers (PeleC::numGrow(), Source/
PeleC.H:877-900) in Array4 layout: a numpy array of shape
``(NVAR, nz + 2 NG, ny + 2 NG, nx + 2 NG)``.  The reference initialisers these
mirror are Exec/RegTests/TG/prob.H:22-77 (Taylor-Green) and the premixed-flame
problems (Exec/RegTests/PMF); the workloads are:

* ``tgv``   — one periodic box on a cube of side 2 pi cm, GammaLaw gas, Mach
  0.1 Taylor-Green vortex with the standard pressure field, isothermal
  density as the reference initialiser (PYT2RE(p, Y, T0)), and seeded uniform
  noise of relative amplitude 1e-3 on rho and on the velocity (relative to U0).
* ``flame`` — a planar premixed H2/air flame along z, T = 300 + 1700
  (1 + tanh((z - z0 - a(x,y))/0.02 cm))/2, a(x,y) a seeded sum of 8 Fourier
  modes with total amplitude at most 0.01 cm, mass fractions blended between
  unburnt phi = 0.8 H2/air and its complete-combustion products, seeded 1e-6
  positive noise on H, O, OH, HO2, H2O2, renormalised; p = 1 atm, w = 100 cm/s,
  u, v ~ N(0, 1 cm/s).  Periodic in x and y, first-order extrapolation in z.
* ``level_boxes`` — a BoxArray of boxes with seeded edges from
  {8,16,24,32,48,64}, each holding the flame at its own seeded offset.
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np

from . import abi
from .mechanism import P_ATM, RU, Mechanism, gamma_law_single, h2_air_synthetic

NG = 4


@dataclass
class BoxState:
    lo: tuple  # valid box smallEnd
    hi: tuple  # valid box bigEnd
    S: np.ndarray  # (NVAR, nz+2NG, ny+2NG, nx+2NG), FP64
    dx: tuple
    ng: int = NG

    @property
    def shape(self):
        return tuple(h - l + 1 for l, h in zip(self.lo, self.hi))

    @property
    def begin(self):
        return tuple(l - self.ng for l in self.lo)

    @property
    def ncells(self) -> int:
        n = 1
        for s in self.shape:
            n *= s
        return n

    def valid(self, A: np.ndarray) -> np.ndarray:
        g = self.ng
        return A[:, g:-g, g:-g, g:-g]


def conserved(mech: Mechanism, rho, u, v, w, T, Y) -> np.ndarray:
    """Conserved FAB components (URHO..UFS+ns-1) from primitives."""
    ns = mech.nspec
    e = mech.mixture_e(T, Y)
    S = np.empty((7 + ns,) + rho.shape)
    S[abi.URHO] = rho
    S[abi.UMX] = rho * u
    S[abi.UMY] = rho * v
    S[abi.UMZ] = rho * w
    S[abi.UEINT] = rho * e
    S[abi.UEDEN] = rho * (e + 0.5 * (u * u + v * v + w * w))
    S[abi.UTEMP] = T
    for k in range(ns):
        S[abi.UFS + k] = rho * Y[k]
    return S


def fill_ghosts(S: np.ndarray, ng: int, bc=("periodic", "periodic", "periodic")) -> None:
    """Single-box ghost fill in place: 'periodic' (int_dir) or 'foextrap'
    (copy of the nearest valid cell), per axis x, y, z (Source/Setup.cpp:34-56)."""
    for d, kind in enumerate(bc):
        ax = 3 - d  # array axes: (n, z, y, x)
        n = S.shape[ax] - 2 * ng
        idx_lo = [slice(None)] * 4
        idx_hi = [slice(None)] * 4
        src_lo = [slice(None)] * 4
        src_hi = [slice(None)] * 4
        idx_lo[ax] = slice(0, ng)
        idx_hi[ax] = slice(ng + n, 2 * ng + n)
        if kind == "periodic":
            src_lo[ax] = slice(n, n + ng)
            src_hi[ax] = slice(ng, 2 * ng)
        elif kind == "foextrap":
            src_lo[ax] = slice(ng, ng + 1)
            src_hi[ax] = slice(ng + n - 1, ng + n)
        else:
            raise ValueError(f"unknown boundary kind {kind!r}")
        S[tuple(idx_lo)] = S[tuple(src_lo)]
        S[tuple(idx_hi)] = S[tuple(src_hi)]


def tgv(n: int = 64, seed: int = 0, mech: Mechanism | None = None, noise: float = 1e-3) -> tuple:
    """Mach-0.1 Taylor-Green vortex on [0, 2 pi)^3 with periodic ghosts."""
    mech = mech or gamma_law_single()
    W = mech.mw[0]
    gamma = mech.gamma
    rho0, p0 = 1.17e-3, 1.01325e6
    T0 = p0 * W / (rho0 * RU)
    c0 = np.sqrt(gamma * p0 / rho0)
    U0 = 0.1 * c0
    dx = 2.0 * np.pi / n
    x = (np.arange(n) + 0.5) * dx
    Z, Yg, X = np.meshgrid(x, x, x, indexing="ij")
    u = U0 * np.sin(X) * np.cos(Yg) * np.cos(Z)
    v = -U0 * np.cos(X) * np.sin(Yg) * np.cos(Z)
    w = np.zeros_like(u)
    p = p0 + rho0 * U0 * U0 / 16.0 * (np.cos(2 * X) + np.cos(2 * Yg)) * (np.cos(2 * Z) + 2.0)
    rho = p * W / (RU * T0)
    rng = np.random.default_rng(seed)
    rho = rho * (1.0 + noise * rng.uniform(-1.0, 1.0, rho.shape))
    u = u + noise * U0 * rng.uniform(-1.0, 1.0, u.shape)
    v = v + noise * U0 * rng.uniform(-1.0, 1.0, u.shape)
    w = w + noise * U0 * rng.uniform(-1.0, 1.0, u.shape)
    T = p * W / (rho * RU)
    Y = np.ones((1,) + rho.shape)
    Sv = conserved(mech, rho, u, v, w, T, Y)
    S = np.zeros((Sv.shape[0], n + 2 * NG, n + 2 * NG, n + 2 * NG))
    S[:, NG:-NG, NG:-NG, NG:-NG] = Sv
    fill_ghosts(S, NG, ("periodic",) * 3)
    st = BoxState(lo=(0, 0, 0), hi=(n - 1, n - 1, n - 1), S=S, dx=(dx, dx, dx))
    return mech, st


# ---------------------------------------------------------------------------
# Premixed H2/air flame
# ---------------------------------------------------------------------------
def _h2air_endpoints(mech: Mechanism, phi: float = 0.8):
    """Unburnt phi H2/air and complete-combustion products, mass fractions."""
    idx = {n: i for i, n in enumerate(mech.names)}
    nu = np.zeros(mech.nspec)
    nb = np.zeros(mech.nspec)
    nu[idx["H2"]] = 2.0 * phi
    nu[idx["O2"]] = 1.0
    nu[idx["N2"]] = 3.76
    nb[idx["H2O"]] = 2.0 * phi
    nb[idx["O2"]] = 1.0 - phi
    nb[idx["N2"]] = 3.76
    yu = nu * mech.mw
    yb = nb * mech.mw
    return yu / yu.sum(), yb / yb.sum()


@dataclass
class FlameParams:
    amps: np.ndarray  # (8,) mode amplitudes, cm
    kx: np.ndarray  # (8,) integer wavenumbers along x
    ky: np.ndarray
    phase: np.ndarray
    Lx: float
    Ly: float
    z0: float
    delta: float = 0.02
    phi: float = 0.8


def flame_params(Lx: float, Ly: float, z0: float, seed: int) -> FlameParams:
    rng = np.random.default_rng(seed)
    kx = rng.integers(0, 4, 8)
    ky = rng.integers(0, 4, 8)
    both0 = (kx == 0) & (ky == 0)
    kx[both0] = 1
    amps = rng.uniform(0.0, 0.01 / 8.0, 8)
    phase = rng.uniform(0.0, 2.0 * np.pi, 8)
    return FlameParams(amps=amps, kx=kx, ky=ky, phase=phase, Lx=Lx, Ly=Ly, z0=z0)


def wrinkle(fp: FlameParams, x, y):
    a = np.zeros(np.broadcast(x, y).shape)
    for m in range(8):
        a = a + fp.amps[m] * np.cos(2 * np.pi * (fp.kx[m] * x / fp.Lx + fp.ky[m] * y / fp.Ly) + fp.phase[m])
    return a


def flame_primitives(mech: Mechanism, fp: FlameParams, X, Yc, Z, rng, w_noise: float = 0.0):
    """Primitive flame fields at cell centres (X, Yc, Z), with seeded noise.
    w_noise > 0 adds seeded Gaussian noise of that std (cm/s) to w as well."""
    s = 0.5 * (1.0 + np.tanh((Z - fp.z0 - wrinkle(fp, X, Yc)) / fp.delta))
    T = 300.0 + 1700.0 * s
    yu, yb = _h2air_endpoints(mech, fp.phi)
    Y = (1.0 - s)[None] * yu[:, None, None, None] + s[None] * yb[:, None, None, None]
    idx = {n: i for i, n in enumerate(mech.names)}
    for r in ("H", "O", "OH", "HO2", "H2O2"):
        if r in idx:
            Y[idx[r]] = Y[idx[r]] + 1e-6 * rng.uniform(0.0, 1.0, T.shape)
    # species a larger mechanism adds (hydrocarbons, argon): seeded traces
    for n in mech.names:
        if n not in ("H2", "O2", "H2O", "N2", "H", "O", "OH", "HO2", "H2O2"):
            Y[idx[n]] = Y[idx[n]] + 1e-6 * rng.uniform(0.0, 1.0, T.shape)
    Y = Y / Y.sum(axis=0, keepdims=True)
    p = np.full(T.shape, P_ATM)
    rho = p * mech.wbar(Y) / (RU * T)
    u = rng.normal(0.0, 1.0, T.shape)
    v = rng.normal(0.0, 1.0, T.shape)
    w = np.full(T.shape, 100.0)
    if w_noise > 0.0:
        w = w + rng.normal(0.0, w_noise, T.shape)
    return rho, u, v, w, T, Y


def flame(shape=(128, 128, 128), dx: float = 1e-3, seed: int = 1, mech: Mechanism | None = None,
          params: FlameParams | None = None, w_noise: float = 0.0) -> tuple:
    """Flame box with periodic x/y ghosts and first-order-extrapolated z ghosts.

    With the default w_noise = 0 the pressure and w are exactly uniform, so
    the MOL limiter's acoustic slopes and the slopes of w sit exactly at the
    limiter's non-differentiable point mc(0, 0); derivative checks against
    finite differences use w_noise > 0."""
    mech = mech or h2_air_synthetic()
    nx, ny, nz = shape
    Lx, Ly, Lz = nx * dx, ny * dx, nz * dx
    fp = params or flame_params(Lx, Ly, 0.5 * Lz, seed)
    rng = np.random.default_rng(seed + 1000)
    x = (np.arange(nx) + 0.5) * dx
    y = (np.arange(ny) + 0.5) * dx
    z = (np.arange(nz) + 0.5) * dx
    Z, Yc, X = np.meshgrid(z, y, x, indexing="ij")
    prims = flame_primitives(mech, fp, X, Yc, Z, rng, w_noise)
    Sv = conserved(mech, *prims)
    S = np.zeros((Sv.shape[0], nz + 2 * NG, ny + 2 * NG, nx + 2 * NG))
    S[:, NG:-NG, NG:-NG, NG:-NG] = Sv
    fill_ghosts(S, NG, ("periodic", "periodic", "foextrap"))
    st = BoxState(lo=(0, 0, 0), hi=(nx - 1, ny - 1, nz - 1), S=S, dx=(dx, dx, dx))
    return mech, st, fp


def level_boxes(nboxes: int = 400, seed: int = 3, dx: float = 1e-3, mech: Mechanism | None = None,
                edges=(8, 16, 24, 32, 48, 64)) -> tuple:
    """BoxArray of independent boxes, each the flame at a seeded offset.

    Boxes are laid out side by side along x in index space (disjoint, as in
    an AMReX BoxArray); each box's state including its ghost cells is the
    analytic flame field at its own offset plus its own noise.
    """
    mech = mech or h2_air_synthetic()
    rng = np.random.default_rng(seed)
    fp = flame_params(0.128, 0.128, 0.0, seed + 7)
    boxes = []
    x0 = 0
    for b in range(nboxes):
        nx, ny, nz = (int(rng.choice(edges)) for _ in range(3))
        off = np.array([rng.uniform(0.0, 0.128), rng.uniform(0.0, 0.128),
                        rng.uniform(-0.5 * nz * dx, 0.5 * nz * dx)])
        lo = (x0, 0, 0)
        hi = (x0 + nx - 1, ny - 1, nz - 1)
        x0 += nx
        xs = off[0] + (np.arange(-NG, nx + NG) + 0.5) * dx
        ys = off[1] + (np.arange(-NG, ny + NG) + 0.5) * dx
        zs = off[2] + (np.arange(-NG, nz + NG) + 0.5 - 0.5 * nz) * dx
        Z, Yc, X = np.meshgrid(zs, ys, xs, indexing="ij")
        prims = flame_primitives(mech, fp, X, Yc, Z, np.random.default_rng(seed * 100003 + b))
        S = conserved(mech, *prims)
        boxes.append(BoxState(lo=lo, hi=hi, S=np.ascontiguousarray(S), dx=(dx, dx, dx)))
    return mech, boxes


def make_config(mech: Mechanism, precision: int = abi.PC_PRECISION_FP64, do_hydro: int = 1,
                diffuse: int = 1, plm_iorder: int = 4, use_laxf_flux: int = 0, harmonic: int = 1,
                check_output: int = 1, newton_max_iter: int = 50, time_passes: int = 0,
                mixed_p_ref: float = 0.0, **flags) -> abi.PcMolConfig:
    """pc_mol_config for a mechanism; ``diffuse`` sets all four diffuse_* flags
    unless individual ones are given in ``flags``."""
    c = abi.PcMolConfig()
    c.nspec = mech.nspec
    c.eos = mech.eos
    c.transport = mech.transport
    c.precision = precision
    c.do_hydro = do_hydro
    c.diffuse_vel = flags.get("diffuse_vel", diffuse)
    c.diffuse_temp = flags.get("diffuse_temp", diffuse)
    c.diffuse_spec = flags.get("diffuse_spec", diffuse)
    c.diffuse_enth = flags.get("diffuse_enth", diffuse)
    c.plm_iorder = plm_iorder
    c.use_laxf_flux = use_laxf_flux
    c.transport_harmonic_mean = harmonic
    c.check_output = check_output
    c.newton_max_iter = newton_max_iter
    c.time_passes = time_passes
    c.mixed_p_ref = mixed_p_ref
    c.mech = mech.to_ctypes()
    return c
