"""Species tables for the two physics models of the MOL path.

The reference selects its EOS, transport model and mechanism at compile time
from PelePhysics (Exec/Make.PeleC:74-115).  PelePhysics is not part of the
reference tree, so its data cannot be used here; this module supplies:

* ``gamma_law_single(...)`` — the GammaLaw EOS with one species and Constant
  transport (the Taylor-Green vortex setup, Exec/RegTests/TG/GNUmakefile and
  TG/prob.cpp:39-57: conductivity = mu * cp / Pr, bulk viscosity 0).  The
  molecular weight is a stated parameter (default 28.97 g/mol); the RHS does
  not depend on it because conductivity scales with cp = gamma/(gamma-1) R/W.

* ``h2_air_synthetic()`` — a SYNTHETIC 9-species table in the species order
  of the LiDryer H2/air mechanism (H2, O2, H2O, H, O, OH, HO2, H2O2, N2).  It
  is NOT LiDryer data: the NASA-7 coefficients, formation enthalpies and
  transport fits below are generated from smooth, physically plausible
  parametric forms so that every code path of the ideal-mixture EOS and the
  mixture-averaged transport is exercised with realistic magnitudes.
  Molecular weights are sums of standard atomic weights.  A real mechanism
  plugs in through the same ``pc_mechanism`` structure.

* ``drm_synthetic()`` — a SYNTHETIC 21-species table in the species order of
  the DRM19 methane mechanism (the size of a common hydrocarbon mechanism),
  with the same kind of generated data (cp/R and transport from each
  species' atom count and molecular weight); not DRM19 data.  It exercises
  the kernels at NUM_SPECIES = 21.

Host-side thermodynamics (numpy) for building initial states lives here too.
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

from . import abi

RU = 8.31446261815324e7  # erg / (mol K)
P_ATM = 1013250.0  # dyn / cm^2

SPECIES_9 = ("H2", "O2", "H2O", "H", "O", "OH", "HO2", "H2O2", "N2")
SPECIES_21 = ("H2", "H", "O", "O2", "OH", "H2O", "HO2", "CH2", "CH2(S)", "CH3", "CH4", "CO", "CO2", "HCO", "CH2O",
              "CH3O", "C2H4", "C2H5", "C2H6", "N2", "AR")
_ATOMIC = {"H": 1.008, "O": 15.999, "N": 14.007, "C": 12.011, "AR": 39.948}
_COMPOSITION = {
    "H2": {"H": 2}, "O2": {"O": 2}, "H2O": {"H": 2, "O": 1}, "H": {"H": 1}, "O": {"O": 1},
    "OH": {"O": 1, "H": 1}, "HO2": {"H": 1, "O": 2}, "H2O2": {"H": 2, "O": 2}, "N2": {"N": 2},
    "CH2": {"C": 1, "H": 2}, "CH2(S)": {"C": 1, "H": 2}, "CH3": {"C": 1, "H": 3}, "CH4": {"C": 1, "H": 4},
    "CO": {"C": 1, "O": 1}, "CO2": {"C": 1, "O": 2}, "HCO": {"H": 1, "C": 1, "O": 1},
    "CH2O": {"C": 1, "H": 2, "O": 1}, "CH3O": {"C": 1, "H": 3, "O": 1}, "C2H4": {"C": 2, "H": 4},
    "C2H5": {"C": 2, "H": 5}, "C2H6": {"C": 2, "H": 6}, "AR": {"AR": 1},
}


@dataclass
class Mechanism:
    """Species data in the layout of ``pc_mechanism`` (numpy, float64)."""

    names: tuple
    mw: np.ndarray
    eos: int
    transport: int
    gamma: float = 1.4
    nasa_tmid: np.ndarray = None
    nasa_lo: np.ndarray = None
    nasa_hi: np.ndarray = None
    visc_fit: np.ndarray = None
    cond_fit: np.ndarray = None
    diff_fit: np.ndarray = None
    bulk_ratio: np.ndarray = None
    diff_pref: float = P_ATM
    const_mu: float = 0.0
    const_xi: float = 0.0
    const_lambda: float = 0.0
    const_rhoD: float = 0.0
    notes: dict = field(default_factory=dict)

    @property
    def nspec(self) -> int:
        return len(self.names)

    def to_ctypes(self) -> abi.PcMechanism:
        m = abi.PcMechanism()
        ns = self.nspec
        m.nspec = ns
        m.gamma = float(self.gamma)
        for k in range(ns):
            m.mw[k] = float(self.mw[k])
        if self.nasa_lo is not None:
            for k in range(ns):
                m.nasa_tmid[k] = float(self.nasa_tmid[k])
                for n in range(7):
                    m.nasa_lo[k][n] = float(self.nasa_lo[k, n])
                    m.nasa_hi[k][n] = float(self.nasa_hi[k, n])
        if self.visc_fit is not None:
            for k in range(ns):
                for n in range(4):
                    m.visc_fit[k][n] = float(self.visc_fit[k, n])
                    m.cond_fit[k][n] = float(self.cond_fit[k, n])
                m.bulk_ratio[k] = float(self.bulk_ratio[k])
                for j in range(ns):
                    for n in range(4):
                        m.diff_fit[k][j][n] = float(self.diff_fit[k, j, n])
        m.diff_pref = float(self.diff_pref)
        m.const_mu = float(self.const_mu)
        m.const_xi = float(self.const_xi)
        m.const_lambda = float(self.const_lambda)
        m.const_rhoD = float(self.const_rhoD)
        return m

    # ---- host thermodynamics (numpy), used to build initial states ----
    def wbar(self, Y: np.ndarray) -> np.ndarray:
        """Mean molecular weight; Y has the species on axis 0."""
        return 1.0 / np.tensordot(1.0 / self.mw, Y, axes=(0, 0))

    def _coef(self, k: int, T: np.ndarray):
        lo = self.nasa_lo[k][:, None]
        hi = self.nasa_hi[k][:, None]
        sel = (T.reshape(-1) < self.nasa_tmid[k])[None, :]
        return np.where(sel, lo, hi).reshape((7,) + T.shape)

    def species_e(self, T: np.ndarray) -> np.ndarray:
        """Specific internal energy of each species, erg/g, shape (ns,)+T.shape."""
        T = np.asarray(T, dtype=np.float64)
        if self.eos == abi.PC_EOS_GAMMA_LAW:
            return np.stack([RU / self.mw[k] / (self.gamma - 1.0) * T for k in range(self.nspec)])
        out = []
        for k in range(self.nspec):
            a = self._coef(k, T)
            hRT = a[0] + T * (a[1] / 2.0 + T * (a[2] / 3.0 + T * (a[3] / 4.0 + T * (a[4] / 5.0)))) + a[5] / T
            out.append(RU / self.mw[k] * T * (hRT - 1.0))
        return np.stack(out)

    def mixture_e(self, T: np.ndarray, Y: np.ndarray) -> np.ndarray:
        return np.sum(Y * self.species_e(T), axis=0)

    def cp_mass(self, T: np.ndarray, Y: np.ndarray) -> np.ndarray:
        T = np.asarray(T, dtype=np.float64)
        if self.eos == abi.PC_EOS_GAMMA_LAW:
            return self.gamma / (self.gamma - 1.0) * RU / self.wbar(Y)
        cp = np.zeros_like(T)
        for k in range(self.nspec):
            a = self._coef(k, T)
            cpR = a[0] + T * (a[1] + T * (a[2] + T * (a[3] + T * a[4])))
            cp = cp + Y[k] * RU / self.mw[k] * cpR
        return cp


def _mw(name: str) -> float:
    return sum(_ATOMIC[a] * n for a, n in _COMPOSITION[name].items())


def gamma_law_single(gamma: float = 1.4, mw: float = 28.97, mu: float = 1.0e-4, prandtl: float = 0.72,
                     bulk: float = 0.0) -> Mechanism:
    """One species, GammaLaw EOS, Constant transport: lambda = mu cp / Pr."""
    cp = gamma / (gamma - 1.0) * RU / mw
    return Mechanism(
        names=("AIR",), mw=np.array([mw]), eos=abi.PC_EOS_GAMMA_LAW, transport=abi.PC_TRANSPORT_CONSTANT,
        gamma=gamma, const_mu=mu, const_xi=bulk, const_lambda=mu * cp / prandtl, const_rhoD=0.0,
        notes={"mw": "stated parameter; RHS independent of it", "prandtl": prandtl},
    )


# Synthetic cp/R polynomials in T' = T/1000 K: cp/R = b0 + b1 T' + ... + b4 T'^4.
_CP_B = {
    "H2": (3.25, 0.35, -0.06, 0.006, -0.0002),
    "O2": (3.30, 0.60, -0.12, 0.010, -0.0003),
    "H2O": (3.80, 0.90, -0.10, 0.006, -0.0002),
    "H": (2.50, 0.0, 0.0, 0.0, 0.0),
    "O": (2.60, -0.12, 0.06, -0.010, 0.0005),
    "OH": (3.40, 0.20, 0.02, -0.002, 0.00005),
    "HO2": (3.95, 1.10, -0.18, 0.012, -0.0003),
    "H2O2": (4.50, 2.00, -0.35, 0.025, -0.0007),
    "N2": (3.25, 0.45, -0.08, 0.007, -0.0002),
}
# Synthetic formation enthalpies h(298.15 K)/R in K.
_HF_R = {"H2": 0.0, "O2": 0.0, "H2O": -29000.0, "H": 26200.0, "O": 29900.0, "OH": 4500.0,
         "HO2": 1500.0, "H2O2": -16300.0, "N2": 0.0}
# Synthetic pure-species transport magnitudes at 300 K.
_MU300 = {"H2": 0.89e-4, "O2": 2.06e-4, "H2O": 1.00e-4, "H": 0.65e-4, "O": 1.50e-4, "OH": 1.55e-4,
          "HO2": 2.00e-4, "H2O2": 1.10e-4, "N2": 1.78e-4}
_LAM300 = {"H2": 1.8e4, "O2": 2.65e3, "H2O": 1.9e3, "H": 1.6e4, "O": 2.9e3, "OH": 2.6e3, "HO2": 2.3e3,
           "H2O2": 1.9e3, "N2": 2.6e3}
_BULK = {"H2": 0.25, "O2": 0.25, "H2O": 0.5, "H": 0.0, "O": 0.0, "OH": 0.25, "HO2": 0.5, "H2O2": 0.5, "N2": 0.25}


def _power_fit(q300: float, expo: float, c2: float, c3: float) -> np.ndarray:
    """ln q = c0 + c1 L + c2 L^2 + c3 L^3 with q(300 K) = q300, c1 = expo."""
    L3 = np.log(300.0)
    c0 = np.log(q300) - (expo * L3 + c2 * L3 ** 2 + c3 * L3 ** 3)
    return np.array([c0, expo, c2, c3])


def _generic_species(name: str):
    """Synthetic (cp/R coefficients, h_f/R, mu300, lambda300, bulk ratio) of a
    species not in the 9-species tables, from its atom count and weight."""
    natoms = sum(_COMPOSITION[name].values())
    w = _mw(name)
    b = (2.5 + 0.9 * (natoms - 1), 0.25 * (natoms - 1) + 0.05, -0.04 * (natoms - 1), 0.004 * (natoms - 1),
         -0.00012 * (natoms - 1))
    hf = -4000.0 * (len(name) % 5) + 2500.0 * ((natoms * 7) % 5)
    mu = 1.0e-4 * np.sqrt(w / 16.0)
    lam = 2.5e3 * np.sqrt(16.0 / w) * (1.0 + 0.1 * natoms)
    bulk = 0.0 if natoms == 1 else 0.25 + 0.05 * min(natoms, 5)
    return b, hf, mu, lam, bulk


def h2_air_synthetic(tmid: float = 1000.0, names=SPECIES_9) -> Mechanism:
    """SYNTHETIC 9-species H2/air table (see module docstring); with another
    species list, the same construction over those species."""
    ns = len(names)
    mw = np.array([_mw(n) for n in names])
    nasa_lo = np.zeros((ns, 7))
    nasa_hi = np.zeros((ns, 7))
    d = -0.03  # high range: cp_hi = cp_lo + d (T'-1)^2, continuous with slope at tmid
    scale = np.array([1.0, 1e-3, 1e-6, 1e-9, 1e-12])

    def h_int(a, T):  # integral of cp/R dT without the constant
        return T * (a[0] + T * (a[1] / 2 + T * (a[2] / 3 + T * (a[3] / 4 + T * a[4] / 5))))

    gen = {n: _generic_species(n) for n in names if n not in _CP_B}
    cpb = {n: (_CP_B[n] if n in _CP_B else gen[n][0]) for n in names}
    hfr = {n: (_HF_R[n] if n in _HF_R else gen[n][1]) for n in names}
    mu300 = {n: (_MU300[n] if n in _MU300 else gen[n][2]) for n in names}
    lam300 = {n: (_LAM300[n] if n in _LAM300 else gen[n][3]) for n in names}
    bulkr = {n: (_BULK[n] if n in _BULK else gen[n][4]) for n in names}
    for k, n in enumerate(names):
        b = np.array(cpb[n], dtype=np.float64)
        bh = b.copy()
        bh[0] += d
        bh[1] -= 2 * d
        bh[2] += d
        alo = b * scale
        ahi = bh * scale
        a5_lo = hfr[n] - h_int(alo, 298.15)
        a5_hi = h_int(alo, tmid) + a5_lo - h_int(ahi, tmid)
        nasa_lo[k, :5] = alo
        nasa_lo[k, 5] = a5_lo
        nasa_hi[k, :5] = ahi
        nasa_hi[k, 5] = a5_hi
    visc = np.stack([_power_fit(mu300[n], 0.70, 0.004, -0.0002) for n in names])
    cond = np.stack([_power_fit(lam300[n], 0.80, 0.004, -0.0002) for n in names])
    diff = np.zeros((ns, ns, 4))
    for i in range(ns):
        for j in range(ns):
            mij = 2.0 * mw[i] * mw[j] / (mw[i] + mw[j])
            diff[i, j] = _power_fit(0.3 * np.sqrt(28.0 / mij), 1.75, 0.002, -0.0001)
    bulk = np.array([bulkr[n] for n in names])
    return Mechanism(
        names=names, mw=mw, eos=abi.PC_EOS_IDEAL_MIX, transport=abi.PC_TRANSPORT_SIMPLE,
        nasa_tmid=np.full(ns, tmid), nasa_lo=nasa_lo, nasa_hi=nasa_hi, visc_fit=visc, cond_fit=cond,
        diff_fit=diff, bulk_ratio=bulk, diff_pref=P_ATM,
        notes={"synthetic": True, "order": names},
    )


def drm_synthetic(tmid: float = 1000.0) -> Mechanism:
    """SYNTHETIC 21-species table in the DRM19 species order (see the module
    docstring); the H2/air species keep the 9-species table's data."""
    return h2_air_synthetic(tmid, SPECIES_21)
