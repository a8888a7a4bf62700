"""Hand-written TDVP adjoint on the GB300: gradients against the torch
oracle (CPU autograd through dense exponentials) and against central finite
differences of the engine's driver."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

# bounds of the mixed-precision adjoint against the FP64 one on the 31-site,
# chi=16, 10-step workload; measured on a GB300: |value difference| 1.6e-7,
# gradient difference 1.9e-6 of the gradient's norm
MIXED_VALUE_TOL = 1e-6
MIXED_GRAD_TOL = 1e-5


def test_gpu_tdvp_gradient_matches_oracle_and_fd():
    import oracle as O
    import oracle.adjoint_oracle as AO
    from pytreenet_gb300.adjoint import OneSiteTDVPAdjoint, coupling_gradient
    from pytreenet_gb300.tdvp import FirstOrderOneSiteTDVP, TDVPConfig, TimeEvoMode, TensorProduct
    from pytreenet_gb300.workloads import binary_tfim_random_state
    from pytreenet_gb300.operators import tfim_ttno
    st, spec, tensors, g, J = binary_tfim_random_state(n=7, chi=4, seed=3)
    theta = np.array([g[nid] for nid, _ in spec] + [J])

    def ham(th):
        return tfim_ttno(st, J=float(th[-1]), g={nid: float(th[i]) for i, (nid, _) in enumerate(spec)})
    dt, steps = 0.1, 4
    ops = {"s0": np.diag([1.0, -1.0]).astype(complex)}
    adj = OneSiteTDVPAdjoint(st, ham(theta), dt, steps, krylov_tol=1e-14)
    val, grad = coupling_gradient(adj, ham, theta, ops)
    val2, gW, gA = adj.expectation_and_gradient(ops, wrt_state=True)
    # torch autograd through the oracle's dense sweep, from the engine's canonical tensors
    tree = O.OTree()
    for nid, p in spec:
        tree.add_root(nid) if p is None else tree.add_child(nid, p)
    otd = AO.FirstOrderOneSiteTDVPTorch(O.OState(tree, {k: v.copy() for k, v in tensors.items()}), dt)
    A0 = {k: adj.A0[k].cpu().clone().requires_grad_(True) for k in adj.order}
    W0 = {k: adj.W0[k].cpu().clone().requires_grad_(True) for k in adj.order}
    ov = otd.expectation(A0, W0, steps, ops).real
    ref = torch.autograd.grad(ov, [A0[k] for k in adj.order] + [W0[k] for k in adj.order])
    assert abs(val2 - float(ov.detach())) < 1e-11
    n = len(adj.order)
    for k, r in zip(adj.order, ref[:n]):
        assert torch.allclose(gA[k].cpu(), r, atol=1e-9), k
    for k, r in zip(adj.order, ref[n:]):
        assert torch.allclose(gW[k].cpu(), r, atol=1e-9), k

    def run(th_):
        s = st.copy_structure()
        s._phys = {k: np.array(v, copy=True) for k, v in tensors.items()}
        algo = FirstOrderOneSiteTDVP(s, ham(th_), dt, dt * steps, {},
                                     config=TDVPConfig(time_evo_mode=TimeEvoMode.KRYLOV),
                                     solver_options={"krylov_tol": 1e-14})
        for _ in range(steps):
            algo.run_one_time_step()
        return float(np.real(algo.evaluate_operator(TensorProduct(ops))))
    assert abs(run(theta) - val) < 1e-11
    h = 1e-5
    fd = np.array([(run(theta + h * np.eye(theta.size)[j]) - run(theta - h * np.eye(theta.size)[j])) / (2 * h)
                   for j in range(theta.size)])
    assert np.linalg.norm(grad) > 1e-4
    assert np.linalg.norm(grad - fd) < 1e-6 * np.linalg.norm(grad)


def test_gpu_second_order_tdvp_gradient_matches_oracle():
    """The second-order adjoint on the GB300 against torch autograd through the
    oracle's dense second-order sweep."""
    import oracle as O
    import oracle.adjoint_oracle as AO
    from pytreenet_gb300.adjoint import OneSiteTDVPAdjoint
    from pytreenet_gb300.workloads import binary_tfim_random_state
    from pytreenet_gb300.operators import tfim_ttno
    st, spec, tensors, g, J = binary_tfim_random_state(n=7, chi=4, seed=6)
    H = tfim_ttno(st, J=J, g=g)
    dt, steps = 0.1, 3
    ops = {"s0": np.diag([1.0, -1.0]).astype(complex)}
    adj = OneSiteTDVPAdjoint(st, H, dt, steps, krylov_tol=1e-14, second_order=True)
    val, gW, gA = adj.expectation_and_gradient(ops, wrt_state=True)
    tree = O.OTree()
    for nid, p in spec:
        tree.add_root(nid) if p is None else tree.add_child(nid, p)
    otd = AO.SecondOrderOneSiteTDVPTorch(O.OState(tree, {k: v.copy() for k, v in tensors.items()}), dt)
    A0 = {k: adj.A0[k].cpu().clone().requires_grad_(True) for k in adj.order}
    W0 = {k: adj.W0[k].cpu().clone().requires_grad_(True) for k in adj.order}
    ov = otd.expectation(A0, W0, steps, ops).real
    ref = torch.autograd.grad(ov, [A0[k] for k in adj.order] + [W0[k] for k in adj.order])
    assert abs(val - float(ov.detach())) < 1e-11
    n = len(adj.order)
    for k, r in zip(adj.order, ref[:n]):
        assert torch.allclose(gA[k].cpu(), r, atol=1e-9), k
    for k, r in zip(adj.order, ref[n:]):
        assert torch.allclose(gW[k].cpu(), r, atol=1e-9), k


def test_gpu_gradient_31_sites_chi16_matches_central_differences():
    """The coupling gradient of <Z_root>(T) on the 31-site binary tree of the
    gradient workload (chi = 16, 10 first-order steps, dt = 0.02, state
    normalised) against central differences (h = 1e-5) of the engine's driver,
    on the root's field, a middle field, a leaf's field and J: every checked
    component within 1e-6 of the gradient's norm."""
    from pytreenet_gb300.adjoint import OneSiteTDVPAdjoint, coupling_gradient
    from pytreenet_gb300.tdvp import FirstOrderOneSiteTDVP, TDVPConfig, TimeEvoMode, TensorProduct
    from pytreenet_gb300.workloads import binary_tfim_random_state
    from pytreenet_gb300.operators import tfim_ttno
    st, spec, tensors, g, J = binary_tfim_random_state(n=31, chi=16, seed=0)
    theta = np.array([g[nid] for nid, _ in spec] + [J])

    def ham(th):
        return tfim_ttno(st, J=float(th[-1]), g={nid: float(th[i]) for i, (nid, _) in enumerate(spec)})
    dt, steps, tol = 0.02, 10, 1e-14
    ops = {"s0": np.diag([1.0, -1.0]).astype(complex)}
    adj = OneSiteTDVPAdjoint(st, ham(theta), dt, steps, krylov_tol=tol, normalise=True)
    val, grad = coupling_gradient(adj, ham, theta, ops)

    def run(th_):
        s = st.copy_structure()
        s._phys = {k: np.array(v, copy=True) for k, v in tensors.items()}
        algo = FirstOrderOneSiteTDVP(s, ham(th_), dt, dt * steps, {},
                                     config=TDVPConfig(time_evo_mode=TimeEvoMode.KRYLOV),
                                     solver_options={"krylov_tol": tol})
        algo.net.normalise_center()
        for _ in range(steps):
            algo.run_one_time_step()
        return float(np.real(algo.evaluate_operator(TensorProduct(ops))))
    assert abs(run(theta) - val) < 1e-10
    h = 1e-5
    idx = [0, 7, 30, theta.size - 1]
    fd = np.array([(run(theta + h * np.eye(theta.size)[j]) - run(theta - h * np.eye(theta.size)[j])) / (2 * h)
                   for j in idx])
    assert np.linalg.norm(grad) > 1e-3
    assert np.max(np.abs(grad[idx] - fd)) < 1e-6 * np.linalg.norm(grad), (grad[idx], fd)


def test_gpu_gradient_31_sites_mixed_precision():
    """The mixed-precision adjoint (BF16x6 tensor-core contractions forward and
    backward; FP64 Krylov, QR and phi-integral) on the 31-site workload of the
    test above, against the FP64 adjoint: the value and the gradient within
    the bounds measured for the BF16x6 path (MIXED_VALUE_TOL absolute,
    MIXED_GRAD_TOL relative to the gradient's norm)."""
    from pytreenet_gb300.adjoint import OneSiteTDVPAdjoint, coupling_gradient
    from pytreenet_gb300.workloads import binary_tfim_random_state
    from pytreenet_gb300.operators import tfim_ttno
    st, spec, tensors, g, J = binary_tfim_random_state(n=31, chi=16, seed=0)
    theta = np.array([g[nid] for nid, _ in spec] + [J])

    def ham(th):
        return tfim_ttno(st, J=float(th[-1]), g={nid: float(th[i]) for i, (nid, _) in enumerate(spec)})
    dt, steps, tol = 0.02, 10, 1e-14
    ops = {"s0": np.diag([1.0, -1.0]).astype(complex)}
    val, grad = coupling_gradient(OneSiteTDVPAdjoint(st, ham(theta), dt, steps, krylov_tol=tol, normalise=True),
                                  ham, theta, ops)
    adj_m = OneSiteTDVPAdjoint(st, ham(theta), dt, steps, krylov_tol=tol, normalise=True, precision="mixed")
    val_m, grad_m = coupling_gradient(adj_m, ham, theta, ops)
    assert abs(val_m - val) < MIXED_VALUE_TOL, (val_m, val)
    assert np.linalg.norm(grad_m - grad) < MIXED_GRAD_TOL * np.linalg.norm(grad)
