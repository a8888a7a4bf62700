"""Fixed-rank BUG on the GB300 against the reference's FixedBUG fixtures."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

from golden_util import BUG_CASES, fidelity_and_dist, oracle_state, run_bug_case


@pytest.mark.parametrize("name", BUG_CASES)
def test_gpu_fixed_bug_matches_reference(name):
    c, st, z = run_bug_case(name)
    assert np.max(np.abs(z - c["z"])) < 1e-10
    one_minus_f, _ = fidelity_and_dist(oracle_state(c, "final"), st)
    assert one_minus_f < 1e-12


@pytest.mark.parametrize("name", ["binary7_tfim_bug", "ternary2_xxz_bug"])
def test_gpu_adaptive_bug_matches_reference(name):
    from golden_util import run_adaptive_bug_case
    c, st, z, bonds, ref_bonds = run_adaptive_bug_case(name)
    assert np.array_equal(bonds, ref_bonds)
    assert np.max(np.abs(z - c["z"])) < 1e-9
    one_minus_f, _ = fidelity_and_dist(oracle_state(c, "final"), st)
    assert one_minus_f < 1e-11
