"""CPU tests of the flop-counting build of the reference harness
(oracle/ref_shim/flop_count.hpp, oracle/count_flops.py): it computes the same
RHS bit for bit as the plain build, its counts are deterministic, and they
match what the code must do where that is known exactly."""
import numpy as np
import pytest

from oracle import refharness
from pelec_gb300 import problems

pytestmark = pytest.mark.skipif(not refharness.available(), reason="reference sources not present")


def test_counting_build_computes_the_same_rhs_and_counts_deterministically():
    mech, st, _ = problems.flame((6, 5, 4), seed=3)
    cfg = problems.make_config(mech)
    c1, R1 = refharness.count_mol_rhs(cfg, [st])
    c2, _ = refharness.count_mol_rhs(cfg, [st])
    assert c1 == c2
    np.testing.assert_array_equal(R1[0], refharness.mol_rhs(cfg, [st])[0])
    assert all(c1[k] > 0 for k in ("add", "mul", "div", "fma", "sqrt", "exp", "log"))


def test_transport_transcendentals_are_counted_per_grown_cell():
    """Mixture-averaged transport (9 species) on every cell of grow(valid, 4):
    9 viscosity and 9 conductivity fits, the mixture viscosity's 1/6 power
    (one exp, one log), and 9 x 8 binary diffusion fits are exponentials, and
    ln T is one more log; nothing else on the path calls exp or log."""
    mech, st, _ = problems.flame((4, 4, 4), seed=1)
    c, _ = refharness.count_mol_rhs(problems.make_config(mech), [st])
    grown = 12 ** 3
    assert c["exp"] == (9 + 9 + 1 + 9 * 8) * grown
    assert c["log"] == 2 * grown


def test_single_species_tgv_has_no_transcendentals():
    mech, st = problems.tgv(8, seed=0)
    c, _ = refharness.count_mol_rhs(problems.make_config(mech), [st])
    assert c["exp"] == 0 and c["log"] == 0 and c["pow"] == 0
    assert c["sqrt"] > 0
