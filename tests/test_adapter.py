"""The reference-side adapter (pelec_gb300/adapter/PeleC_GB300.H) compiles
and reaches the C ABI.

The adapter is what a PeleC maintainer adds to Source/Diffusion.cpp: the
getMOLSrcTerm replacement over amrex::MultiFab / MFIter / Array4, and
fill_mechanism, which restates the compiled PelePhysics mechanism as
pc_mechanism.  Here it is compiled with g++ against stand-ins for the absent
AMReX and PelePhysics headers (tests/adapter_shim, oracle/ref_shim); the
PelePhysics stand-in evaluates the synthetic 9-species table, written out by
this test, through the entry points the adapter reads (get_mw, cp_R,
speciesEnthalpy, the Simple transport fits).  Checks: the NASA-7
coefficients recovered by sampling equal the table's, the Array4 mapping is
the ABI's, and the handle creation goes through libpelec_mol.so (on a
machine without a GPU it ends in the library's PC_ERR_NO_DEVICE message).
"""
import os
import subprocess

import numpy as np
import pytest

from pelec_gb300 import mechanism

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIB = os.path.join(ROOT, "pelec_gb300", "_lib", "libpelec_mol.so")


def _table(mech) -> str:
    ns = mech.nspec
    f = lambda v: repr(float(v))
    rows = lambda a: ", ".join("{" + ", ".join(f(x) for x in r) + "}" for r in a)
    out = [f"#pragma once\n#define NUM_SPECIES {ns}",
           f"static const double kMW[{ns}] = {{{', '.join(f(x) for x in mech.mw)}}};",
           f"static const double kTMID[{ns}] = {{{', '.join(f(x) for x in mech.nasa_tmid)}}};",
           f"static const double kLO[{ns}][7] = {{{rows(mech.nasa_lo)}}};",
           f"static const double kHI[{ns}][7] = {{{rows(mech.nasa_hi)}}};",
           f"static const double kVISC[{ns}][4] = {{{rows(mech.visc_fit)}}};",
           f"static const double kCOND[{ns}][4] = {{{rows(mech.cond_fit)}}};",
           f"static const double kDIFF[{ns}][{ns}][4] = {{{', '.join('{' + rows(m) + '}' for m in mech.diff_fit)}}};"]
    return "\n".join(out) + "\n"


@pytest.fixture(scope="module")
def driver(tmp_path_factory):
    if not os.path.exists(LIB):
        from pelec_gb300 import build

        build.build()
    d = tmp_path_factory.mktemp("adapter")
    (d / "mechanism_table.H").write_text(_table(mechanism.h2_air_synthetic()))
    exe = d / "adapter_driver"
    cmd = ["g++", "-std=c++17", "-O1", "-Wall", "-I", str(d), "-I", os.path.join(ROOT, "tests", "adapter_shim"),
           "-I", os.path.join(ROOT, "oracle", "ref_shim"), "-I", os.path.join(ROOT, "pelec_gb300", "adapter"),
           "-I", os.path.join(ROOT, "include"), os.path.join(ROOT, "tests", "adapter_shim", "adapter_driver.cpp"),
           "-o", str(exe), LIB, "-Wl,-rpath," + os.path.dirname(LIB)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    out = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    assert out.returncode == 0, out.stderr
    return out.stdout


def test_fill_mechanism_recovers_the_table(driver):
    line = next(ln for ln in driver.splitlines() if ln.startswith("fill_mechanism"))
    f = line.split()
    assert int(f[2]) == 0, line
    mw_err, nasa_err, fit_err, tmid = float(f[4]), float(f[6]), float(f[8]), float(f[10])
    assert mw_err == 0.0 and fit_err == 0.0, line
    assert nasa_err <= 1e-9, line  # coefficient contributions to cp/R at 1000 K
    assert tmid == 1000.0


def test_array4_mapping(driver):
    line = next(ln for ln in driver.splitlines() if ln.startswith("array4"))
    v = line.split()
    # valid box (2,3,4)-(9,7,13) with 4 ghosts: begin lo-4, end hi+1+4, 16 components
    assert v[2:5] == ["-2", "-1", "0"] and v[6:9] == ["14", "12", "18"], line
    nx, ny, nz = 16, 13, 18
    assert (int(v[10]), int(v[12]), int(v[14]), int(v[16])) == (nx, nx * ny, nx * ny * nz, 16), line
    assert v[18:21] == ["2", "3", "4"], line


def test_handle_creation_reaches_the_library(driver):
    import torch

    line = next(ln for ln in driver.splitlines() if ln.startswith(("abort", "create")))
    if torch.cuda.is_available():
        assert line.startswith("create ok") or "no CUDA device" not in line, line
    else:
        assert line.startswith("abort") and "no CUDA device" in line, line
