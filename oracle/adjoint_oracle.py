"""FP64 torch-autograd restatement of first-order one-site TDVP (oracle, test infrastructure).

Only ``tests/`` may use this module. It restates the sweep of
``FirstOrderOneSiteTDVPOracle`` (``tdvp_algorithms/firstorderonesite.py:92-104``,
``onesitetdvp.py:29-127``) with ``torch.tensordot`` contractions, dense local
exponentials (``torch.matrix_exp`` of the effective Hamiltonian, as the
reference's EXPM mode builds it, ``effective_hamiltonians.py:109-131``) and
``torch.linalg.qr``, so that torch's own autograd gives the gradients the GPU
engine's hand-written adjoint must reproduce. Small trees only (the local
Hamiltonians are formed as dense matrices).
"""
from __future__ import annotations

import numpy as np
import torch

from .ptn_oracle import OState, canonical_form, leaf_to_root_path, orthogonalisation_paths


def _td(a, la, b, lb, lc, conj_b=False):
    k = [l for l in la if l in lb]
    t = torch.tensordot(a, b.conj() if conj_b else b, dims=([la.index(l) for l in k], [lb.index(l) for l in k]))
    cur = [l for l in la if l not in k] + [l for l in lb if l not in k]
    return t.permute([cur.index(l) for l in lc]) if lc else t


def _chain(x, lx, envs, W, n, open_k=None):
    """All environments except ``open_k``, then W (``contract_ket_ham_with_envs``,
    ``state_operator_contraction.py:227-273``, which contracts the
    environments before the TTNO tensor)."""
    T, lT = x, list(lx)
    for k in range(n):
        if k == open_k:
            continue
        lnew = [l for l in lT if l != f"a{k}"] + [f"b{k}", f"c{k}"]
        T, lT = _td(T, lT, envs[k], [f"a{k}", f"b{k}", f"c{k}"], lnew), lnew
    lW = [f"b{k}" for k in range(n)] + ["t", "s"]
    cl = [f"b{k}" for k in range(n) if k != open_k] + ["s"]
    lnew = [l for l in lT if l not in cl] + [l for l in lW if l not in cl]
    return _td(T, lT, W, lW, lnew), lnew


def heff_matrix(shape, envs, W):
    n = len(shape) - 1
    N = int(np.prod(shape))
    eye = torch.eye(N, dtype=torch.complex128, device=W.device).reshape([N] + list(shape))
    T, lT = _chain(eye, ["r"] + [f"a{k}" for k in range(n)] + ["s"], envs, W, n)
    y = T.permute([lT.index(l) for l in ["r"] + [f"c{k}" for k in range(n)] + ["t"]]).reshape(N, N)
    return y.T


def env_update(A, envs, W, k0):
    n = A.dim() - 1
    T, lT = _chain(A, [f"a{k}" for k in range(n)] + ["s"], envs, W, n, open_k=k0)
    return _td(T, lT, A, [f"c{k}" if k != k0 else "z" for k in range(n)] + ["t"], [f"a{k0}", f"b{k0}", "z"],
               conj_b=True)


def bond_matrix(eq, en):
    ka, kc = eq.shape[0], en.shape[0]
    eye = torch.eye(ka * kc, dtype=torch.complex128, device=eq.device).reshape(ka * kc, ka, kc)
    t = _td(eq, ["a", "b", "x"], eye, ["r", "a", "c"], ["r", "b", "x", "c"])
    y = _td(t, ["r", "b", "x", "c"], en, ["c", "b", "y"], ["r", "x", "y"]).reshape(ka * kc, ka * kc)
    return y.T


def qr_split(A, ax):
    perm = [j for j in range(A.dim()) if j != ax] + [ax]
    At = A.permute(perm)
    k = A.shape[ax]
    q, r = torch.linalg.qr(At.reshape(-1, k), mode="reduced")
    Q = q.reshape(At.shape).permute(list(np.argsort(perm)))
    return Q, r


def absorb(R, T, ax):
    return torch.movedim(torch.tensordot(R, T, dims=([1], [ax])), 0, ax)


def expect_product(A, nbrs, root, ops):
    def rec(nid, toward):
        T = A[nid]
        nb = nbrs[nid]
        n = len(nb)
        if nid in ops:
            O = torch.as_tensor(np.asarray(ops[nid], dtype=np.complex128))
            T = torch.movedim(torch.tensordot(O, T, dims=([1], [n])), 0, n)
        lT = [f"a{k}" for k in range(n)] + ["s"]
        for k, x in enumerate(nb):
            if x != toward:
                lnew = [l for l in lT if l != f"a{k}"] + [f"c{k}"]
                T, lT = _td(T, lT, rec(x, nid), [f"a{k}", f"c{k}"], lnew), lnew
        lB = [f"c{k}" if nb[k] != toward else "z" for k in range(n)] + ["s"]
        if toward is None:
            return _td(T, lT, A[nid], lB, [], conj_b=True)
        return _td(T, lT, A[nid], lB, [f"a{nb.index(toward)}", "z"], conj_b=True)
    return rec(root, None)


class FirstOrderOneSiteTDVPTorch:
    """The sweep as a differentiable function of the canonical site tensors and
    the TTNO tensors (physical leg layouts, as in :mod:`ptn_oracle`)."""

    def __init__(self, state: OState, dt: float):
        st = state.copy()
        self.tree = st.tree
        self.path = leaf_to_root_path(st.tree.copy())
        self.orth = orthogonalisation_paths(st.tree, self.path)
        bp = list(reversed(self.path))
        self.back_path = bp
        self.back_orth = [st.tree.path_from_to(nid, bp[i + 2])[:-1] for i, nid in enumerate(bp[1:-1])] + [[bp[-1]]]
        canonical_form(st, self.path[0])
        self.A0 = {k: torch.from_numpy(np.ascontiguousarray(v)) for k, v in st.tensors.items()}
        self.nbrs = {k: st.tree.neighbours(k) for k in st.tensors}
        self.dt = dt

    def _env(self, A, W, envs, nid, nxt):
        nb = self.nbrs[nid]
        return env_update(A[nid], [envs.get((x, nid)) for x in nb], W[nid], nb.index(nxt))

    def _hop(self, A, a, b):
        Q, R = qr_split(A[a], self.nbrs[a].index(b))
        A[a] = Q
        A[b] = absorb(R, A[b], self.nbrs[b].index(a))

    def step(self, A, W):
        A = dict(A)
        envs = {}
        path, op = self.path, self.orth

        def rec(nid, toward):
            for x in self.nbrs[nid]:
                if x != toward:
                    rec(x, nid)
            if toward is not None:
                envs[(nid, toward)] = self._env(A, W, envs, nid, toward)
        rec(path[0], None)
        for i, nid in enumerate(path):
            if i > 0:
                for prev, cur in zip(op[i - 1][:-1], op[i - 1][1:]):
                    self._hop(A, prev, cur)
                    envs[(prev, cur)] = self._env(A, W, envs, nid=prev, nxt=cur)
            nb = self.nbrs[nid]
            H = heff_matrix(list(A[nid].shape), [envs[(x, nid)] for x in nb], W[nid])
            A[nid] = (torch.matrix_exp(-1j * self.dt * H) @ A[nid].reshape(-1)).reshape(A[nid].shape)
            if i < len(path) - 1:
                nxt = op[i][0]
                Q, R = qr_split(A[nid], nb.index(nxt))
                A[nid] = Q
                envs[(nid, nxt)] = self._env(A, W, envs, nid, nxt)
                Hb = bond_matrix(envs[(nid, nxt)], envs[(nxt, nid)])
                R = (torch.matrix_exp(1j * self.dt * Hb) @ R.reshape(-1)).reshape(R.shape)
                A[nxt] = absorb(R, A[nxt], self.nbrs[nxt].index(nid))
            else:
                back = self.tree.path_from_to(nid, path[0])
                for a, b in zip(back[:-1], back[1:]):
                    self._hop(A, a, b)
        return A

    def expectation(self, A, W, steps, ops):
        for _ in range(steps):
            A = self.step(A, W)
        return expect_product(A, self.nbrs, self.tree.root, ops)


class SecondOrderOneSiteTDVPTorch(FirstOrderOneSiteTDVPTorch):
    """``SecondOrderOneSiteTDVPOracle`` (``secondorderonesite.py:60-193``) in torch;
    the environments carried between steps by the reference are rebuilt from
    the tensors at each step start (they point toward the centre and were
    computed from the tensors as they are, so the two agree)."""

    def _site(self, A, W, envs, nid, factor):
        nb = self.nbrs[nid]
        H = heff_matrix(list(A[nid].shape), [envs[(x, nid)] for x in nb], W[nid])
        A[nid] = (torch.matrix_exp(-1j * self.dt * factor * H) @ A[nid].reshape(-1)).reshape(A[nid].shape)

    def _link(self, A, W, envs, nid, nxt, factor):
        Q, R = qr_split(A[nid], self.nbrs[nid].index(nxt))
        A[nid] = Q
        envs[(nid, nxt)] = self._env(A, W, envs, nid, nxt)
        Hb = bond_matrix(envs[(nid, nxt)], envs[(nxt, nid)])
        R = (torch.matrix_exp(1j * self.dt * factor * Hb) @ R.reshape(-1)).reshape(R.shape)
        A[nxt] = absorb(R, A[nxt], self.nbrs[nxt].index(nid))

    def _move(self, A, W, envs, path):
        for prev, cur in zip(path[:-1], path[1:]):
            self._hop(A, prev, cur)
            envs[(prev, cur)] = self._env(A, W, envs, prev, cur)

    def step(self, A, W):
        A = dict(A)
        envs = {}
        path, op = self.path, self.orth

        def rec(nid, toward):
            for x in self.nbrs[nid]:
                if x != toward:
                    rec(x, nid)
            if toward is not None:
                envs[(nid, toward)] = self._env(A, W, envs, nid, toward)
        rec(path[0], None)
        for i, nid in enumerate(path[:-1]):
            if i > 0:
                self._move(A, W, envs, op[i - 1])
            self._site(A, W, envs, nid, 0.5)
            self._link(A, W, envs, nid, op[i][0], 0.5)
        center = op[-1][0]
        self._site(A, W, envs, path[-1], 1.0)
        bp, bo = self.back_path, self.back_orth
        self._link(A, W, envs, center, bp[1], 0.5)
        center = bp[1]
        for i, nid in enumerate(bp[1:-1]):
            idx = i + 1
            self._site(A, W, envs, nid, 0.5)
            if bo[idx - 1]:
                self._move(A, W, envs, bo[idx - 1])
                center = bo[idx - 1][-1]
            self._link(A, W, envs, center, bp[idx + 1], 0.5)
            center = bp[idx + 1]
        self._site(A, W, envs, bp[-1], 0.5)
        return A
