"""One-site TDVP on the GPU against the reference's own runs on the trees and
Hamiltonian families of the 61-site T-tree (Heisenberg + fields) and the
31-site binary TFIM with one field per site, at chi 8 (full-rank states)."""
import numpy as np
import pytest

import oracle as O
from golden_util import CONFIG_SHAPE_CASES, build_ttn, load_case, oracle_state, fidelity_and_dist

pytestmark = pytest.mark.gpu
Zm = np.diag([1.0, -1.0]).astype(complex)


@pytest.mark.parametrize("name", CONFIG_SHAPE_CASES)
def test_gpu_config_shape_one_site(name):
    import pytreenet_gb300 as P
    c = load_case(name)
    assert c["order"] == 1
    st = build_ttn(P.TTNS, c["spec"], c["init"])
    H = build_ttn(P.TTNO, c["spec"], c["ttno"])
    algo = P.FirstOrderOneSiteTDVP(st, H, c["dt"], c["dt"] * c["steps"], {},
                                   config=P.TDVPConfig(time_evo_mode=P.TimeEvoMode.KRYLOV),
                                   solver_options={"krylov_tol": c["krylov_tol"]})
    assert algo.update_path == c["update_path"]
    zerr = 0.0
    for k in range(c["steps"]):
        algo.run_one_time_step()
        z = [algo.evaluate_operator({nid: Zm}) for nid, _ in c["spec"]]
        zerr = max(zerr, float(np.max(np.abs(np.array(z) - c["z"][k]))))
    got = O.OState(oracle_state(c).tree, {nid: algo.state.get_phys_numpy(nid) for nid, _ in c["spec"]})
    one_minus_f, _ = fidelity_and_dist(oracle_state(c, "final"), got)
    # ~120 Krylov solves per run: a stop test that falls within rounding of
    # its threshold may add or drop one basis vector (<= krylov_tol each)
    assert zerr < 1e-9
    assert one_minus_f < 1e-12
