"""Time-dependent Hamiltonians on the GB300: a driven field through
TimeDependentTTNO and config.time_dep against the reference's own run."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

from golden_util import DRIVEN_CASES, fidelity_and_dist, oracle_state, run_driven_case


@pytest.mark.parametrize("name", DRIVEN_CASES)
@pytest.mark.parametrize("precision", ["plain", "mixed"])
def test_gpu_time_dependent_hamiltonian(name, precision):
    c, st, z = run_driven_case(name, precision=precision)
    one_minus_f, _ = fidelity_and_dist(oracle_state(c, "final"), st)
    if precision == "plain":
        assert np.max(np.abs(z - c["z"].real)) < 1e-10
        assert one_minus_f < 1e-12
    else:
        assert np.max(np.abs(z - c["z"].real)) < 1e-5
        assert one_minus_f < 1e-9
