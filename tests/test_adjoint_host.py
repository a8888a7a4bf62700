"""Hand-written adjoint of one-site TDVP on CPU (engine calls served by the
NumPy stand-in of the library): each primitive against torch autograd, and
the gradient of a whole evolution against the torch oracle and against
central finite differences of the engine's own driver."""
import numpy as np
import pytest
import torch

import fake_ptn

RNG = np.random.default_rng(5)


def crandn(*shape):
    return torch.from_numpy(RNG.normal(size=shape) + 1j * RNG.normal(size=shape))


@pytest.fixture
def fake(monkeypatch):
    return fake_ptn.install(monkeypatch)


def test_coupling_matrix_matches_quadrature():
    from pytreenet_gb300.adjoint import coupling_matrix
    rng = np.random.default_rng(1)

    def herm(m):
        a = rng.normal(size=(m, m)) + 1j * rng.normal(size=(m, m))
        return a + a.conj().T
    Tv, Tw = herm(5), herm(4)
    z = -0.3j
    M = coupling_matrix(Tv, 1.7, Tw, 0.6, z)
    import scipy.linalg
    xs, ws = np.polynomial.legendre.leggauss(40)
    xs, ws = 0.5 * (xs + 1), 0.5 * ws
    ref = np.zeros((4, 5), dtype=complex)
    for s, w in zip(xs, ws):
        b = 1.7 * scipy.linalg.expm(s * z * Tv)[:, 0]
        a = 0.6 * scipy.linalg.expm(-(1 - s) * z * Tw)[:, 0]
        ref += w * np.outer(a.conj(), b)
    assert np.max(np.abs(M - ref)) < 1e-13


@pytest.mark.parametrize("conj_b", [False, True])
def test_contract_adjoint_matches_torch(fake, conj_b):
    from pytreenet_gb300.adjoint import contract
    a = crandn(3, 4, 5).requires_grad_(True)
    b = crandn(5, 6, 3).requires_grad_(True)
    c = contract(a, ["i", "j", "k"], b, ["k", "l", "i"], ["l", "j"], conj_b=conj_b)
    g = crandn(6, 4)
    ga, gb = torch.autograd.grad(c, [a, b], grad_outputs=g)
    a2, b2 = a.detach().clone().requires_grad_(True), b.detach().clone().requires_grad_(True)
    c2 = torch.einsum("ijk,kli->lj", a2, b2.conj() if conj_b else b2)
    assert torch.allclose(c, c2, atol=1e-12)
    ra, rb = torch.autograd.grad(c2, [a2, b2], grad_outputs=g)
    assert torch.allclose(ga, ra, atol=1e-12) and torch.allclose(gb, rb, atol=1e-12)


@pytest.mark.parametrize("shape,ax", [((6, 4, 2), 1), ((3, 5, 2), 0), ((4, 4), 0), ((2, 3, 2, 2), 3)])
def test_qr_adjoint_matches_torch(fake, shape, ax):
    from pytreenet_gb300.adjoint import qr
    A = crandn(*shape).requires_grad_(True)
    Q, R = qr(A, ax)
    gQ, gR = crandn(*Q.shape), crandn(*R.shape)
    # a gauge-invariant loss is needed for comparison only if the gauges differ;
    # both follow LAPACK's (real diagonal of R), so the factors agree directly
    (gA,) = torch.autograd.grad([Q, R], [A], grad_outputs=[gQ, gR])
    A2 = A.detach().clone().requires_grad_(True)
    perm = [j for j in range(A2.dim()) if j != ax] + [ax]
    q, r = torch.linalg.qr(A2.permute(perm).reshape(-1, shape[ax]))
    Q2 = q.reshape([shape[j] for j in perm]).permute(list(np.argsort(perm)))
    assert torch.allclose(Q, Q2, atol=1e-12) and torch.allclose(R, r, atol=1e-12)
    (rA,) = torch.autograd.grad([Q2, r], [A2], grad_outputs=[gQ, gR])
    assert torch.allclose(gA, rA, atol=1e-10)


def test_krylov_adjoint_matches_dense_exponential(fake):
    """Site with three neighbours: y = exp(-i dt H(E, W)) x; gradients with
    respect to x, the three environments and W against torch.matrix_exp."""
    from pytreenet_gb300.adjoint import krylov_expm, _SiteOp, site_apply
    import oracle.adjoint_oracle as AO
    dims, w, d = [3, 2, 2], [2, 3, 2], 2

    def herm_env(chi, ww):
        e = crandn(chi, ww, chi)
        return (e + e.permute(2, 1, 0).conj()) / 2          # Hermitian in (ket, bra) per ham index
    envs = [herm_env(c, ww) for c, ww in zip(dims, w)]
    W = crandn(*w, d, d)
    W = (W + W.transpose(-1, -2).conj()) / 2
    x = crandn(*dims, d)
    x = x / torch.linalg.norm(x)
    leaves = [t.clone().requires_grad_(True) for t in envs + [W, x]]
    y = krylov_expm(leaves[-1], _SiteOp(3), leaves[:4], 0.07, -1j, tol=1e-14)
    g = crandn(*y.shape)
    got = torch.autograd.grad(y, leaves, grad_outputs=g)
    ref_leaves = [t.detach().clone().requires_grad_(True) for t in leaves]
    H = AO.heff_matrix(list(x.shape), ref_leaves[:3], ref_leaves[3])
    # the engine's matvec and the oracle's dense matrix are the same operator
    assert torch.allclose(H @ x.reshape(-1), site_apply(x, envs, W).reshape(-1), atol=1e-12)
    y2 = (torch.matrix_exp(-0.07j * H) @ ref_leaves[4].reshape(-1)).reshape(y.shape)
    assert torch.allclose(y, y2, atol=1e-12)
    ref = torch.autograd.grad(y2, ref_leaves, grad_outputs=g)
    for a, b in zip(got, ref):
        assert torch.allclose(a, b, atol=1e-10), float((a - b).abs().max())


def _seven_site_problem(seed=3):
    from pytreenet_gb300.workloads import binary_tfim_random_state
    from pytreenet_gb300.operators import tfim_ttno
    st, spec, tensors, g, J = binary_tfim_random_state(n=7, chi=4, seed=seed)
    theta = np.array([g[nid] for nid, _ in spec] + [J])

    def ham(th):
        return tfim_ttno(st, J=float(th[-1]), g={nid: float(th[i]) for i, (nid, _) in enumerate(spec)})
    return st, spec, tensors, theta, ham


def test_tdvp_gradient_matches_oracle_and_finite_differences(fake):
    """d<Z_root>(T)/d(g_1..g_7, J) after 3 first-order one-site TDVP steps:
    the engine's adjoint equals torch autograd through the oracle's dense
    sweep, and central differences of the engine's own driver."""
    import oracle as O
    import oracle.adjoint_oracle as AO
    from pytreenet_gb300.adjoint import OneSiteTDVPAdjoint, coupling_gradient
    from pytreenet_gb300.engine import ttno_site_tensors
    from pytreenet_gb300.tdvp import FirstOrderOneSiteTDVP, TDVPConfig, TimeEvoMode, TensorProduct
    st, spec, tensors, theta, ham = _seven_site_problem()
    dt, steps = 0.05, 3
    Z = np.diag([1.0, -1.0]).astype(complex)
    ops = {"s0": Z}
    adj = OneSiteTDVPAdjoint(st, ham(theta), dt, steps, krylov_tol=1e-14)
    val, grad = coupling_gradient(adj, ham, theta, ops)

    # oracle: torch autograd through dense exponentials
    tree = O.OTree()
    for nid, p in spec:
        tree.add_root(nid) if p is None else tree.add_child(nid, p)
    otd = AO.FirstOrderOneSiteTDVPTorch(O.OState(tree, {k: v.copy() for k, v in tensors.items()}), dt)
    th = torch.tensor(theta, requires_grad=True)
    base = {k: torch.from_numpy(v) for k, v in ttno_site_tensors(st, ham(theta)).items()}
    D = []
    for j in range(theta.size):
        e = np.zeros_like(theta)
        e[j] = 1.0
        Wj = ttno_site_tensors(st, ham(theta + e))
        D.append({k: torch.from_numpy(Wj[k]) - base[k] for k in base})
    Wt = {k: base[k] + sum((th[j] - float(theta[j])) * D[j][k] for j in range(theta.size)) for k in base}
    ov = AO.FirstOrderOneSiteTDVPTorch.expectation(otd, dict(otd.A0), Wt, steps, ops).real
    (og,) = torch.autograd.grad(ov, [th])
    assert abs(val - float(ov.detach())) < 1e-11
    assert np.linalg.norm(grad - og.numpy()) < 1e-9 * np.linalg.norm(grad)

    # central differences of the engine's driver (same semantics, its own code path)
    def run(th_):
        s = st.copy_structure()
        s._phys = {k: np.array(v, copy=True) for k, v in tensors.items()}
        algo = FirstOrderOneSiteTDVP(s, ham(th_), dt, dt * steps, {}, config=TDVPConfig(time_evo_mode=TimeEvoMode.KRYLOV),
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


def test_tdvp_state_gradient_matches_oracle(fake):
    """Gradient with respect to the canonical initial tensors (torch's complex
    convention) against the oracle's autograd."""
    import oracle as O
    import oracle.adjoint_oracle as AO
    from pytreenet_gb300.adjoint import OneSiteTDVPAdjoint
    st, spec, tensors, theta, ham = _seven_site_problem(seed=4)
    dt, steps = 0.04, 2
    X = np.array([[0, 1], [1, 0]], dtype=complex)
    ops = {"s1": X, "s5": np.diag([1.0, -1.0]).astype(complex)}
    adj = OneSiteTDVPAdjoint(st, ham(theta), dt, steps, krylov_tol=1e-14)
    val, gW, gA = adj.expectation_and_gradient(ops, wrt_state=True)
    tree = O.OTree()
    for nid, p in spec:
        tree.add_root(nid) if p is None else tree.add_child(nid, p)
    otd = AO.FirstOrderOneSiteTDVPTorch(O.OState(tree, {k: v.copy() for k, v in tensors.items()}), dt)
    # the two canonical forms agree up to the QR gauge only where it is fixed
    # (LAPACK's), so compare on the engine's canonical tensors
    A0 = {k: adj.A0[k].detach().clone().requires_grad_(True) for k in adj.order}
    W0 = {k: adj.W0[k].detach().clone().requires_grad_(True) for k in adj.order}
    ov = otd.expectation(A0, W0, steps, ops).real
    grads = torch.autograd.grad(ov, [A0[k] for k in adj.order] + [W0[k] for k in adj.order])
    assert abs(val - float(ov.detach())) < 1e-11
    for k, g in zip(adj.order, grads[:len(adj.order)]):
        assert torch.allclose(gA[k], g, atol=1e-9), k
    for k, g in zip(adj.order, grads[len(adj.order):]):
        assert torch.allclose(gW[k], g, atol=1e-9), k


def test_second_order_tdvp_gradient_matches_oracle_and_fd(fake):
    """The second-order schedule: coupling gradient against torch autograd
    through the oracle's dense second-order sweep and against central
    differences of the engine's SecondOrderOneSiteTDVP driver."""
    import oracle as O
    import oracle.adjoint_oracle as AO
    from pytreenet_gb300.adjoint import OneSiteTDVPAdjoint, coupling_gradient
    from pytreenet_gb300.tdvp import SecondOrderOneSiteTDVP, TDVPConfig, TimeEvoMode, TensorProduct
    st, spec, tensors, theta, ham = _seven_site_problem(seed=6)
    dt, steps = 0.1, 3
    ops = {"s0": np.diag([1.0, -1.0]).astype(complex)}
    adj = OneSiteTDVPAdjoint(st, ham(theta), dt, steps, krylov_tol=1e-14, second_order=True)
    val, grad = coupling_gradient(adj, ham, theta, ops)
    _, gW, gA = adj.expectation_and_gradient(ops, wrt_state=True)
    tree = O.OTree()
    for nid, p in spec:
        tree.add_root(nid) if p is None else tree.add_child(nid, p)
    otd = AO.SecondOrderOneSiteTDVPTorch(O.OState(tree, {k: v.copy() for k, v in tensors.items()}), dt)
    A0 = {k: adj.A0[k].detach().clone().requires_grad_(True) for k in adj.order}
    W0 = {k: adj.W0[k].detach().clone().requires_grad_(True) for k in adj.order}
    ov = otd.expectation(A0, W0, steps, ops).real
    ref = torch.autograd.grad(ov, [A0[k] for k in adj.order] + [W0[k] for k in adj.order])
    assert abs(val - float(ov.detach())) < 1e-11
    n = len(adj.order)
    for k, r in zip(adj.order, ref[:n]):
        assert torch.allclose(gA[k], r, atol=1e-9), k
    for k, r in zip(adj.order, ref[n:]):
        assert torch.allclose(gW[k], r, atol=1e-9), k

    def run(th_):
        s = st.copy_structure()
        s._phys = {k: np.array(v, copy=True) for k, v in tensors.items()}
        algo = SecondOrderOneSiteTDVP(s, ham(th_), dt, dt * steps, {},
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


def test_mixed_precision_adjoint_close_to_fp64(fake):
    """The adjoint with every contraction (forward and backward) as BF16-split
    tensor-core products, the stand-in accumulating in FP32: value and coupling
    gradient within the FP32 level of the complex128 adjoint's."""
    from pytreenet_gb300.adjoint import OneSiteTDVPAdjoint, coupling_gradient
    st, spec, tensors, theta, ham = _seven_site_problem()
    ops = {"s0": np.diag([1.0, -1.0]).astype(complex)}
    adj = OneSiteTDVPAdjoint(st, ham(theta), 0.05, 3, krylov_tol=1e-14)
    val, grad = coupling_gradient(adj, ham, theta, ops)
    adj_m = OneSiteTDVPAdjoint(st, ham(theta), 0.05, 3, krylov_tol=1e-14, precision="mixed")
    val_m, grad_m = coupling_gradient(adj_m, ham, theta, ops)
    assert abs(val_m - val) < 1e-6
    assert 0 < np.linalg.norm(grad_m - grad) < 1e-5 * np.linalg.norm(grad)
