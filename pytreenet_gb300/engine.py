"""GPU engine: device-resident TTNS/TTNO/environment data and the local-update kernels.

Everything numerical runs in libptn_gb300 (hand-written CUDA for sm_103a); this
module only plans the calls. PyTorch provides device memory and the stream.

Data layout in HBM
------------------
* site tensor of node v: complex128, contiguous, legs (parent, children in
  attachment order, physical) -- one buffer per node, updated in place;
* TTNO tensor of node v: legs (parent, children, out, in), same neighbour order;
* environment E(u -> v) for every directed edge: (ket, ham, bra) =
  (chi_uv, w_uv, chi_uv), one persistent buffer per directed edge;
* workspace slots: contraction intermediates and Krylov basis, grown on demand
  and shared by all plans (one stream, so no two plans run at once).

A contraction step is ``ptn_zcontract``: tensordot semantics, but the legs are
addressed through strides, so no tensor is ever transposed in memory.
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass

import numpy as np
import torch

from . import _lib
from ._lib import ContractDesc, MAX_MODES, check

CDT = torch.complex128
DEFAULT_DEVICE = "cuda"


_RAW_STREAM = getattr(torch._C, "_cuda_getCurrentRawStream", None)
_CUR_DEVICE = getattr(torch._C, "_cuda_getDevice", None)


def _stream_ptr():
    """The current CUDA stream of the current device as a foreign-call
    argument. Called once per launch sequence: the direct lookup costs ~1 us
    where torch.cuda.current_stream() measured ~15 us per call."""
    if _RAW_STREAM is not None and _CUR_DEVICE is not None:
        return ctypes.c_void_p(_RAW_STREAM(_CUR_DEVICE()))
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


# ----------------------------------------------------------------------------
# workspace
# ----------------------------------------------------------------------------
class _BufferTable(dict):
    """The workspace's buffers; every replacement bumps the workspace's
    generation, so plans re-read their pointers only when one moved."""

    def __init__(self, ws):
        super().__init__()
        self._ws = ws

    def __setitem__(self, key, value):
        super().__setitem__(key, value)
        self._ws.gen += 1

    def __delitem__(self, key):
        super().__delitem__(key)
        self._ws.gen += 1

    def pop(self, *a):
        self._ws.gen += 1
        return super().pop(*a)


class Workspace:
    """Named device scratch buffers that only grow."""

    def __init__(self, device):
        self.device = device
        self.gen = 0                    # bumped whenever a buffer is replaced
        self.bufs: dict[str, torch.Tensor] = _BufferTable(self)

    def get(self, name: str, numel: int, dtype=CDT) -> torch.Tensor:
        b = self.bufs.get(name)
        if b is None or b.numel() < numel or b.dtype != dtype:
            b = torch.empty(max(numel, 1), dtype=dtype, device=self.device)
            self.bufs[name] = b
        return b[:numel]

    def ptr(self, name: str) -> int:
        return self.bufs[name].data_ptr()


# ----------------------------------------------------------------------------
# labelled operands and contraction steps
# ----------------------------------------------------------------------------
@dataclass
class Operand:
    """A tensor operand of a plan: how to find its pointer, and its legs."""
    ref: tuple               # ("fixed", tensor) | ("in",) | ("out",) | ("ws", name)
    labels: list
    dims: list
    strides: list

    @staticmethod
    def contiguous(ref, labels, dims):
        strides = [0] * len(dims)
        s = 1
        for i in range(len(dims) - 1, -1, -1):
            strides[i] = s
            s *= dims[i]
        return Operand(ref, list(labels), list(dims), strides)

    def numel(self):
        return int(np.prod(self.dims)) if self.dims else 1

    def permuted_to(self, order):
        """Same memory, legs listed in ``order``."""
        idx = [self.labels.index(x) for x in order]
        return Operand(self.ref, list(order), [self.dims[i] for i in idx], [self.strides[i] for i in idx])


def _merge_modes(dims, sa, sb):
    """Merge adjacent modes that are contiguous in both operands."""
    od, oa, ob = [], [], []
    for d, a, b in zip(dims, sa, sb):
        if d == 1:
            continue
        if od and oa[-1] == a * d and ob[-1] == b * d:
            od[-1] *= d
            oa[-1] = a
            ob[-1] = b
        else:
            od.append(d)
            oa.append(a)
            ob.append(b)
    return od, oa, ob


def _fill(modes, dims, s_first, s_second, which):
    dims, s1, s2 = _merge_modes(dims, s_first, s_second)
    if len(dims) > MAX_MODES:
        raise ValueError(f"contraction needs {len(dims)} modes in one group (max {MAX_MODES})")
    modes.n = len(dims)
    for i, (d, a, b) in enumerate(zip(dims, s1, s2)):
        modes.dim[i] = d
        if which == "m":
            modes.stride_a[i], modes.stride_c[i] = a, b
        elif which == "n":
            modes.stride_b[i], modes.stride_c[i] = a, b
        else:
            modes.stride_a[i], modes.stride_b[i] = a, b


class Step:
    """One ptn_zcontract call with prebuilt strides; pointers resolved at run time."""

    __slots__ = ("desc", "refs", "flops")

    def __init__(self, A: Operand, B: Operand, klabels, C: Operand, conj_a=False, conj_b=False,
                 alpha=1.0, beta=0.0):
        d = ContractDesc()
        mlab = [l for l in A.labels if l not in klabels]
        nlab = [l for l in B.labels if l not in klabels]
        if sorted(C.labels) != sorted(mlab + nlab):
            raise ValueError(f"output legs {C.labels} do not match {mlab + nlab}")

        def col(op, labs, what):
            return [getattr(op, what)[op.labels.index(l)] for l in labs]
        for l in klabels:
            if A.dims[A.labels.index(l)] != B.dims[B.labels.index(l)]:
                raise ValueError(f"dimension mismatch on leg {l}")
        # the output's legs must have the sizes of the operand legs they come
        # from: the kernel writes through C's strides over A's and B's ranges
        for op, labs in ((A, mlab), (B, nlab)):
            for l in labs:
                if C.dims[C.labels.index(l)] != op.dims[op.labels.index(l)]:
                    raise ValueError(f"output leg {l} has size {C.dims[C.labels.index(l)]}, "
                                     f"the operand's has {op.dims[op.labels.index(l)]}")
        _fill(d.m, col(A, mlab, "dims"), col(A, mlab, "strides"), col(C, mlab, "strides"), "m")
        _fill(d.n, col(B, nlab, "dims"), col(B, nlab, "strides"), col(C, nlab, "strides"), "n")
        _fill(d.k, col(A, klabels, "dims"), col(A, klabels, "strides"), col(B, klabels, "strides"), "k")
        d.alpha_re, d.alpha_im = float(np.real(alpha)), float(np.imag(alpha))
        d.beta_re, d.beta_im = float(np.real(beta)), float(np.imag(beta))
        d.conj_a, d.conj_b = int(conj_a), int(conj_b)
        self.desc = d
        self.refs = (A.ref, B.ref, C.ref)
        self.flops = 8 * int(np.prod(col(A, mlab, "dims") or [1])) * \
            int(np.prod(col(B, nlab, "dims") or [1])) * int(np.prod(col(A, klabels, "dims") or [1]))


class _NativeOps:
    """A fixed list of descriptors run by ``ptn_exec_ops`` in one foreign call.
    Operand references become indices into a pointer table filled per run:
    0 = the input vector, 1 = the output, then each distinct fixed tensor or
    workspace slot."""

    def __init__(self, items):
        slots: dict = {}
        self.refs = [("in",), ("out",)]

        def slot(ref):
            if ref is None:
                return -1
            kind = ref[0]
            if kind == "in":
                return 0
            if kind == "out":
                return 1
            key = (kind, id(ref[1])) if kind == "fixed" else (kind, ref[1])
            if key not in slots:
                slots[key] = len(self.refs)
                self.refs.append(ref)
            return slots[key]
        self.descs = [d for _, d, _ in items]
        self.ops = (_lib.ExecOp * max(len(items), 1))()
        for i, (kind, d, refs) in enumerate(items):
            a, b, c = refs[:3]
            self.ops[i].kind = kind
            self.ops[i].a, self.ops[i].b, self.ops[i].c = slot(a), slot(b), slot(c)
            self.ops[i].d = slot(refs[3]) if len(refs) > 3 else -1
            self.ops[i].desc = ctypes.addressof(d)
        self.n = len(items)
        self.ptrs = (ctypes.c_void_p * len(self.refs))()
        self._gen = -1
        # fixed operands that are not tensors (pointer holders whose address
        # changes between runs) are re-read on every run
        self._moving = [i for i in range(2, len(self.refs))
                        if self.refs[i][0] == "fixed" and not isinstance(self.refs[i][1], torch.Tensor)]

    def run(self, ws, x_ptr, y_ptr):
        p = self.ptrs
        p[0], p[1] = x_ptr or None, y_ptr or None
        # fixed tensors never move, workspace slots only when the workspace's
        # generation changed since the table was last filled
        if self._gen != ws.gen:
            for i in range(2, len(self.refs)):
                ref = self.refs[i]
                p[i] = ref[1].data_ptr() if ref[0] == "fixed" else ws.ptr(ref[1])
            self._gen = ws.gen
        else:
            for i in self._moving:
                p[i] = self.refs[i][1].data_ptr()
        check(_lib.load().ptn_exec_ops(self.ops, self.n, p, len(self.refs), _stream_ptr()), "ptn_exec_ops")


class Plan:
    """A sequence of contraction steps with one dynamic input and output."""

    def __init__(self, ws: Workspace, steps, ws_sizes):
        self.ws = ws
        self.steps = steps
        self.ws_sizes = ws_sizes  # name -> numel
        self.flops = sum(s.flops for s in steps)

    def run(self, x_ptr: int = 0, y_ptr: int = 0):
        ws = self.ws
        if getattr(self, "_sized_at", None) != ws.gen:
            for name, n in self.ws_sizes.items():
                ws.get(name, n)
            self._sized_at = ws.gen     # slots only grow: still large enough until one is replaced
        if not hasattr(self, "_exec"):
            self._exec = _NativeOps([(_lib.OP_ZCONTRACT, st.desc, st.refs) for st in self.steps])
        self._exec.run(ws, x_ptr, y_ptr)


class ChainBuilder:
    """Builds a Plan from tensordot-style steps on labelled operands."""

    def __init__(self, ws: Workspace):
        self.ws = ws
        self.steps = []
        self.logical = []
        self.sizes = {}
        self.slot = 0

    def contract(self, A: Operand, B: Operand, klabels, out: Operand | None = None, **kw) -> Operand:
        if out is None:
            mlab = [l for l in A.labels if l not in klabels]
            nlab = [l for l in B.labels if l not in klabels]
            dims = [A.dims[A.labels.index(l)] for l in mlab] + [B.dims[B.labels.index(l)] for l in nlab]
            name = f"chain{self.slot % 2}"
            self.slot += 1
            out = Operand.contiguous(("ws", name), mlab + nlab, dims)
            self.sizes[name] = max(self.sizes.get(name, 0), out.numel())
        self.steps.append(Step(A, B, klabels, out, **kw))
        self.logical.append((A, B, list(klabels), out, kw))
        return out

    def plan(self) -> Plan:
        return Plan(self.ws, self.steps, self.sizes)

    def mixed_plan(self, levels: int = 3, own_fixed: bool = False) -> "MixedPlan":
        return MixedPlan(self.ws, self.logical, levels, own_fixed)


def _modes_single(dims, strides):
    """Merge adjacent modes contiguous in one layout; drop unit modes."""
    od, os_ = [], []
    for d, st in zip(dims, strides):
        if d == 1:
            continue
        if od and os_[-1] == st * d:
            od[-1] *= d
            os_[-1] = st
        else:
            od.append(d)
            os_.append(st)
    return od, os_


def _set_modes(modes, dims, strides, field):
    dims, strides = _modes_single(dims, strides)
    if len(dims) > MAX_MODES:
        raise ValueError("too many modes")
    modes.n = len(dims)
    for i, (d, st) in enumerate(zip(dims, strides)):
        modes.dim[i] = d
        getattr(modes, field)[i] = st


def _round8(x):
    return (x + 7) // 8 * 8


# products that libptn_gb300 runs on its CUDA-core kernel instead of the
# tensor-core pipeline (ptn_cgemm_bf16x3: K <= 32 and N <= 128)
SMALLK_MAX_K = 32
SMALLK_MAX_N = 128


class MixedPlan:
    """The same contraction chain on the tensor cores (BF16 splits, FP32 accumulation).

    Every step is ``ptn_cgemm_bf16x3`` with both operands K-major. The running
    tensor is kept as BF16 hi/lo planes whose layout is chosen for the step that
    reads it: [rows = that step's free legs][cols = its contracted legs]; each
    GEMM's epilogue writes straight into that layout, and the last one writes
    complex128 into the destination. Small operands (environments, TTNO
    tensors, the conjugate site tensor) are expanded per call by
    ``ptn_expand_b``; the first operand is gathered by ``ptn_to_planes``.
    """

    def __init__(self, ws: Workspace, logical, levels: int = 3, own_fixed: bool = False):
        """``own_fixed``: operands that are fixed tensors (environments, TTNO
        tensors) are split into BF16 planes held by the plan and converted by
        ``prepare()`` only; a plan run many times on the same operands (the
        H_eff of one Krylov solve) then converts only the moving vector."""
        from ._lib import CgemmDesc, ConvertDesc
        self.ws = ws
        self.levels = L = int(levels)
        self.ops = []            # ("conv"|"expand"|"gemm", desc, refs)
        self.prep = []           # conversions of fixed operands into plan-owned planes
        self.owned = []          # plan-owned plane buffers
        self.hold = False        # True: run() skips the prep conversions (operands unchanged)
        self.sizes = {}          # ws name -> numel (bf16 planes)
        self.byte_sizes = {}     # ws name -> bytes (complex128 slots)
        self.flops = 0
        nsteps = len(logical)
        info = []
        for (A, B, kl, out, kw) in logical:
            mlab = [l for l in A.labels if l not in kl]
            nlab = [l for l in B.labels if l not in kl]
            dims = {**dict(zip(A.labels, A.dims)), **dict(zip(B.labels, B.dims))}
            info.append((mlab, list(kl), nlab, dims))
        # Layouts are assigned from the last step backwards. The output of step i
        # is the A operand of step i+1, laid out [rows][cols] with cols = the
        # legs step i+1 contracts (contiguous). Rows are ordered by the stride the
        # legs get in step i+1's own output (largest first), and cols put a leg
        # that step i's rows carry innermost: the epilogue maps one thread to one
        # row, so the row leg that varies fastest then writes consecutive
        # addresses.
        out_stride = [None] * nsteps          # label -> stride in step i's output
        A_layout = [None] * nsteps            # (rows order, cols order, lda, stride map)
        A_last, _, _, out_last, _ = logical[-1]
        out_stride[-1] = dict(zip(out_last.labels, out_last.strides))
        for i in range(nsteps - 1, -1, -1):
            mlab, kl, nlab, dims = info[i]
            ost = out_stride[i]
            rows = sorted(mlab, key=lambda l: -ost[l])
            if i > 0:
                prev_m = set(info[i - 1][0])
                cols = sorted(kl, key=lambda l: (l in prev_m, dims[l]))
            else:
                cols = list(kl)
            K = int(np.prod([dims[l] for l in cols] or [1]))
            Nn = int(np.prod([dims[l] for l in nlab] or [1]))
            # a product the CUDA-core kernel takes (K <= 32, N <= 128) reads its A
            # rows without TMA, so they are not padded to 8 entries: a padded row
            # would make the producing epilogue write partial sectors (read-modify-
            # write in L2) and the consumer read the padding
            lda = K if (K <= SMALLK_MAX_K and Nn <= SMALLK_MAX_N) else _round8(K)
            stride = {}
            s_ = 1
            for l in reversed(cols):
                stride[l] = s_
                s_ *= dims[l]
            s_ = lda
            for l in reversed(rows):
                stride[l] = s_
                s_ *= dims[l]
            A_layout[i] = (rows, cols, lda, stride)
            if i > 0:
                out_stride[i - 1] = stride
        for i, (A, B, kl, out, kw) in enumerate(logical):
            mlab, _, nlab, dims = info[i]
            rows, cols, lda, stride = A_layout[i]
            M = int(np.prod([dims[l] for l in rows] or [1]))
            N = int(np.prod([dims[l] for l in nlab] or [1]))
            K = int(np.prod([dims[l] for l in cols] or [1]))
            self.flops += 8 * M * N * K
            aslot = f"mp{i % 2}"
            plane = _round8(M * lda)
            if i == 0:
                d = ConvertDesc()
                _set_modes(d.rows, [dims[l] for l in rows], [A.strides[A.labels.index(l)] for l in rows], "stride_a")
                _set_modes(d.cols, [dims[l] for l in cols], [A.strides[A.labels.index(l)] for l in cols], "stride_a")
                d.ld, d.plane, d.conj, d.levels = lda, plane, int(kw.get("conj_a", False)), L
                if own_fixed and A.ref[0] == "fixed":
                    buf = torch.empty(2 * L * plane + 64, dtype=torch.bfloat16, device=ws.device)
                    self.owned.append(buf)
                    aref = ("fixed", buf)
                    self.prep.append(("conv", d, (A.ref, aref)))
                else:
                    aref = ("ws", aslot)
                    self.ops.append(("conv", d, (A.ref, aref)))
                    self._need(aslot, 2 * L * plane)
            else:
                aref = ("ws", aslot)
            ldb = _round8(K)
            d = ConvertDesc()
            _set_modes(d.rows, [dims[l] for l in nlab], [B.strides[B.labels.index(l)] for l in nlab], "stride_a")
            _set_modes(d.cols, [dims[l] for l in cols], [B.strides[B.labels.index(l)] for l in cols], "stride_a")
            d.ld, d.plane, d.conj, d.levels = ldb, 0, int(kw.get("conj_b", False)), L
            if own_fixed and B.ref[0] == "fixed":
                buf = torch.empty(3 * L * N * ldb + 64, dtype=torch.bfloat16, device=ws.device)
                self.owned.append(buf)
                bref = ("fixed", buf)
                self.prep.append(("expand", d, (B.ref, bref)))
            else:
                bref = ("ws", "bx")
                self.ops.append(("expand", d, (B.ref, bref)))
                self._need("bx", 3 * L * N * ldb)
            g = CgemmDesc()
            g.lda, g.a_plane, g.M, g.K, g.ldb, g.N = lda, plane, M, K, ldb, N
            g.levels = L
            # split-K scratch for outputs with few tiles (one shared slot)
            pb = int(_lib.load().ptn_cgemm_partial_bytes(M, N, K))
            g.partial_bytes = pb
            if pb:
                self._need_bytes("tc_partial", pb)
            ost = out_stride[i]
            if i < nsteps - 1:
                nrows, ncols, nlda, _ = A_layout[i + 1]
                nM = int(np.prod([info[i + 1][3][l] for l in nrows] or [1]))
                cslot = f"mp{(i + 1) % 2}"
                g.out_kind = 1
                g.c_plane = _round8(nM * nlda)
                self._need(cslot, 2 * L * g.c_plane)
                _set_modes(g.m_out, [dims[l] for l in rows], [ost[l] for l in rows], "stride_c")
                _set_modes(g.n_out, [dims[l] for l in nlab], [ost[l] for l in nlab], "stride_c")
                self.ops.append(("gemm", g, (aref, bref, ("ws", cslot))))
            else:
                g.out_kind = 0
                g.c_plane = 0
                _set_modes(g.m_out, [dims[l] for l in rows], [ost[l] for l in rows], "stride_c")
                _set_modes(g.n_out, [dims[l] for l in nlab], [ost[l] for l in nlab], "stride_c")
                self.ops.append(("gemm", g, (aref, bref, out.ref)))

    def _need(self, name, numel):
        self.sizes[name] = max(self.sizes.get(name, 0), numel)

    def _need_bytes(self, name, nbytes):
        self.byte_sizes[name] = max(self.byte_sizes.get(name, 0), int(nbytes))

    def _build_exec(self):
        ws = self.ws
        if getattr(self, "_sized_at", None) != ws.gen:
            for name, n in self.sizes.items():
                ws.get(name, n + 64, torch.bfloat16)
            for name, nb in self.byte_sizes.items():
                ws.get(name, (nb + 15) // 16, CDT)
            if ws.bufs.get("tc_status") is None:
                ws.bufs["tc_status"] = torch.zeros(1, dtype=torch.int32, device=ws.device)
            self._sized_at = ws.gen     # slots only grow: still large enough until one is replaced
        status = ws.bufs["tc_status"]
        if not hasattr(self, "_exec"):
            items = []
            for kind, d, refs in self.ops:
                if kind == "conv":
                    items.append((_lib.OP_TO_PLANES, d, (refs[0], None, refs[1])))
                elif kind == "expand":
                    items.append((_lib.OP_EXPAND_B, d, (refs[0], None, refs[1])))
                else:
                    d.status = status.data_ptr()
                    part = ("ws", "tc_partial") if d.partial_bytes else None
                    items.append((_lib.OP_CGEMM, d, tuple(refs) + (part,)))
            self._exec = _NativeOps(items)
            self._prep_exec = _NativeOps([(_lib.OP_TO_PLANES if kind == "conv" else _lib.OP_EXPAND_B, d,
                                           (refs[0], None, refs[1])) for kind, d, refs in self.prep])

    def run(self, x_ptr: int = 0, y_ptr: int = 0):
        self._build_exec()
        if self.prep and not self.hold:
            self._prep_exec.run(self.ws, 0, 0)
        self._exec.run(self.ws, x_ptr, y_ptr)

    def prepare(self):
        """Convert the fixed operands into the plan's own planes now; runs
        made while ``hold`` is set reuse them."""
        self._build_exec()
        if self.prep:
            self._prep_exec.run(self.ws, 0, 0)


# ----------------------------------------------------------------------------
# Krylov exponential (krylov_exp_action, time_evolution/time_evolution.py:721-821)
# ----------------------------------------------------------------------------
def small_propagator(T, dt, exp_factor, hermitian=True):
    """First column of exp(exp_factor dt T) for the m x m projection
    (``_krylov_small_propagator``, ``time_evolution/time_evolution.py:696-718``)."""
    if hermitian:
        H = 0.5 * (T + T.conj().T)
        ev, V = np.linalg.eigh(H)
        return V @ (np.exp(exp_factor * dt * ev) * V[0].conj())
    import scipy.linalg
    return scipy.linalg.expm(exp_factor * dt * T)[:, 0]


class KrylovSolver:
    @staticmethod
    def _proj(T, m, tridiagonal):
        if not tridiagonal:
            return T[:m, :m]
        P = np.zeros((m, m), dtype=complex)
        idx = np.arange(m)
        P[idx, idx] = T[idx, idx].real
        if m > 1:
            P[idx[1:], idx[:-1]] = T[idx[1:], idx[:-1]].real
            P[idx[:-1], idx[1:]] = T[idx[1:], idx[:-1]].real
        return P

    """Matrix-free Arnoldi/Lanczos exponential on the device.

    Two Gram-Schmidt passes per step (classical, each a multi-dot + multi-axpy
    kernel pair; the reference does the same projections one vector at a time).
    The adaptive stop, the happy-breakdown floors and the symmetrised ``eigh``
    propagator follow the reference; the m x m projection is tiny and is
    diagonalised on the host after each step.
    """

    # Krylov solves on vectors up to this length run speculative batches (the
    # matvec is cheap there, so a host round trip per step would dominate).
    SPECULATE_MAX_N = 1 << 21

    def __init__(self, ws: Workspace):
        self.ws = ws
        self.depths: list[int] = []
        self._host = None
        self._spec_depth: dict[int, int] = {}
        self._qcap = 0

    def _ensure_Q(self, x, n, cap):
        """Krylov basis of ``cap`` rows of length n (existing rows kept)."""
        cur = self.ws.bufs.get("kry_Q")
        if cur is not None and cur.numel() >= cap * n:
            self._qcap = cur.numel() // n
            return
        Qn = torch.empty((cap * n,), dtype=CDT, device=x.device)
        if cur is not None and self._qcap > 0:
            keep = min(cur.numel(), cap * n, self._qcap * n)
            Qn[:keep].copy_(cur[:keep])
        self.ws.bufs["kry_Q"] = Qn
        self._qcap = cap

    def _pinned(self, n, ns=2):
        if self._host is None or self._host[0].numel() < n or self._host[1].numel() < ns:
            pin = self.ws.device.type == "cuda"
            self._host = (torch.empty(max(n, 64), dtype=CDT, pin_memory=pin),
                          torch.empty(max(ns, 64), dtype=torch.float64, pin_memory=pin),
                          torch.zeros(1, dtype=torch.int32, pin_memory=pin))
        return self._host

    def expm(self, x: torch.Tensor, apply, dt: float, exp_factor: complex, krylov_tol=1e-10,
             max_krylov_dim=None, hermitian=True, out: torch.Tensor | None = None,
             tridiagonal: bool = False, basis: dict | None = None) -> torch.Tensor:
        """``tridiagonal``: project on the Lanczos tridiagonal (alpha_j, beta_j)
        only. Used with reduced-precision operators, whose rounding leaves
        entries far from the diagonal of the Arnoldi projection that the
        reference's full symmetrised projection would turn into a spurious
        first-order coupling (the adaptive stop then never triggers).

        ``apply(xp, yp)`` gets device pointers, or the basis row and the output
        as tensors when it carries ``takes_tensors = True``. ``basis``, when
        given, receives the Krylov basis (``Q``: m x n copy), the m x m
        projection used for the propagator (``T``) and the norm of x
        (``beta0``); the adjoint of the exponential reuses them."""
        lib = _lib.load()
        stream = _stream_ptr()
        n = x.numel()
        out = x if out is None else out
        part = self.ws.get("kry_part", int(lib.ptn_krylov_partials(n)) + 8)
        scal = self.ws.get("kry_scal", 8, torch.float64)
        check(lib.ptn_dznrm2(x.data_ptr(), n, scal.data_ptr(), part.data_ptr(), stream), "dznrm2")
        beta0 = float(scal[0].item())
        if beta0 == 0.0:
            if out.data_ptr() != x.data_ptr():
                out.copy_(x)
            if basis is not None:
                basis.update(Q=None, T=np.zeros((0, 0), dtype=complex), beta0=0.0, m=0)
            return out
        tensor_apply = getattr(apply, "takes_tensors", False)
        max_steps = n if max_krylov_dim is None else min(n, int(max_krylov_dim))
        floor_abs = np.finfo(float).eps * max(n, 1)
        T = np.zeros((min(max_steps, 64) + 1,) * 2, dtype=complex)
        # Speculation: for vectors up to SPECULATE_MAX_N the steps of a batch are
        # enqueued back to back and the host reads their coefficients once per
        # batch (the first batch as deep as the last solve of this size). The
        # decisions below are the same, taken on the same numbers, so the result
        # equals the one-step-at-a-time loop; vectors computed past the stop are
        # discarded.
        spec = self._spec_depth.get(n, 4) if n <= self.SPECULATE_MAX_N else 1
        self._ensure_Q(x, n, min(max_steps + 1, max(spec + 1, 8)))
        Q = self.ws.bufs["kry_Q"][:self._qcap * n].view(self._qcap, n)
        w = self.ws.get("kry_w", n)
        check(lib.ptn_zscal_inv(x.data_ptr(), scal.data_ptr(), Q[0].data_ptr(), n, stream), "zscal")
        m = 0
        j = 0
        done = False
        while not done and j < max_steps:
            batch = max(1, min(spec - j, max_steps - j)) if j < spec else 1
            if j + batch + 1 > self._qcap:
                self._ensure_Q(x, n, min(max_steps + 1, max(2 * self._qcap, j + batch + 1)))
                Q = self.ws.bufs["kry_Q"][:self._qcap * n].view(self._qcap, n)
            hs = self.ws.get("kry_hs", (j + batch) * 2 * (j + batch) + 8)
            sc = self.ws.get("kry_sc", 2 * (j + batch) + 8, torch.float64)
            for jj in range(j, j + batch):
                if tensor_apply:
                    apply(Q[jj], w)
                else:
                    apply(Q[jj].data_ptr(), w.data_ptr())
                nq = jj + 1
                base = hs[jj * 2 * (j + batch):]
                qnext = Q[jj + 1].data_ptr() if jj + 1 < self._qcap else None
                # |w|, two Gram-Schmidt passes, |w|, next basis vector: one foreign call
                check(lib.ptn_krylov_gs_step(Q.data_ptr(), n, nq, w.data_ptr(), n, base.data_ptr(), part.data_ptr(),
                                             sc[2 * jj:].data_ptr(), qnext, stream), "krylov_gs_step")
            # one synchronisation per batch: coefficients, norms and the status
            # word go to pinned host memory asynchronously, then the stream syncs
            nh = (j + batch) * 2 * (j + batch)
            hh_host, sc_host, st_host = self._pinned(nh, 2 * (j + batch))
            hh_host[:nh].copy_(hs[:nh], non_blocking=True)
            sc_host[:2 * (j + batch)].copy_(sc[:2 * (j + batch)], non_blocking=True)
            st = self.ws.bufs.get("tc_status")
            if st is not None:
                st_host.copy_(st[:1], non_blocking=True)
            if self.ws.device.type == "cuda":
                check(lib.ptn_stream_synchronize(stream), "stream synchronize")
            if st is not None and int(st_host[0]) != 0:
                code = int(st_host[0])
                st.zero_()
                raise _lib.PtnError(code, "tensor-core contraction inside the Krylov exponential")
            hh_all = hh_host[:nh].numpy()
            sc_all = sc_host[:2 * (j + batch)].numpy()
            for jj in range(j, j + batch):
                if jj + 2 > T.shape[0]:
                    T2 = np.zeros((2 * T.shape[0],) * 2, dtype=complex)
                    T2[:T.shape[0], :T.shape[0]] = T
                    T = T2
                nq = jj + 1
                hh = hh_all[jj * 2 * (j + batch):jj * 2 * (j + batch) + 2 * nq]
                w0, beta = float(sc_all[2 * jj]), float(sc_all[2 * jj + 1])
                T[:nq, jj] = hh[:nq] + hh[nq:]
                T[jj + 1, jj] = beta
                m = jj + 1
                if not np.isfinite(beta):
                    raise _lib.PtnError(3, "Krylov exponential: non-finite vector")
                if beta <= max(floor_abs, 1e-12 * w0):
                    done = True
                    break
                if krylov_tol > 0.0:
                    col = small_propagator(self._proj(T, m, tridiagonal), dt, exp_factor, hermitian)
                    if beta0 * beta * abs(col[m - 1]) < krylov_tol:
                        done = True
                        break
                if jj + 1 >= self._qcap:
                    done = True       # basis capacity reached (only with max_krylov_dim = capacity)
                    break
            j += batch
        if n <= self.SPECULATE_MAX_N:
            self._spec_depth[n] = m
        self.depths.append(m)
        if basis is not None:
            basis.update(Q=Q[:m].clone(), T=self._proj(T, m, tridiagonal).copy(), beta0=beta0, m=m)
        c = beta0 * small_propagator(self._proj(T, m, tridiagonal), dt, exp_factor, hermitian)
        cdev = self.ws.get("kry_h", m + 8)[:m]
        cdev.copy_(torch.from_numpy(np.ascontiguousarray(c)).to(x.device))
        for i0 in range(0, m, 64):
            cnt = min(64, m - i0)
            if i0 == 0:
                check(lib.ptn_zcombine(Q.data_ptr(), n, cnt, cdev.data_ptr(), out.data_ptr(), n, stream),
                      "zcombine")
            else:
                tmp = self.ws.get("kry_tmp", n)
                check(lib.ptn_zcombine(Q[i0:].data_ptr(), n, cnt, cdev[i0:].data_ptr(), tmp.data_ptr(), n,
                                       stream), "zcombine")
                out.view(-1).add_(tmp)
        return out


# ----------------------------------------------------------------------------
# device network
# ----------------------------------------------------------------------------
def ttno_site_tensors(state, hamiltonian) -> dict:
    """The TTNO's tensors as contiguous complex128 NumPy arrays with legs
    (the state's physical neighbour order, out, in)."""
    state._finalise()
    hamiltonian._finalise()
    out = {}
    for nid in state._order:
        Wn = hamiltonian.phys(nid)
        hn = hamiltonian.nodes[nid]
        order = state.nodes[nid].phys_neighbours()
        hax = [hn.phys_neighbours().index(x) for x in order]
        Wn = np.asarray(Wn.detach().cpu().numpy() if isinstance(Wn, torch.Tensor) else Wn)
        Wn = np.transpose(Wn, hax + [Wn.ndim - 2, Wn.ndim - 1])
        out[nid] = np.ascontiguousarray(Wn, dtype=np.complex128)
    return out


class DeviceNetwork:
    """Device copy of a TTNS (+ TTNO) with environment buffers and cached plans."""

    PRECISIONS = {"plain": 0, "bf16x3": 2, "bf16x6": 3, "mixed": 3}

    def __init__(self, state, hamiltonian=None, device=None, precision: str = "plain"):
        if precision not in self.PRECISIONS:
            raise ValueError("precision must be 'plain' (complex128), 'bf16x3', 'bf16x6' or 'mixed' "
                             "(= bf16x6) tensor-core contractions")
        self.precision = precision
        self.levels = self.PRECISIONS[precision]
        _lib.load()
        if not torch.cuda.is_available():
            raise RuntimeError("pytreenet_gb300 needs a CUDA device (no CPU fallback)")
        self.device = torch.device(device or DEFAULT_DEVICE)
        self.state = state
        self.ham = hamiltonian
        self.ws = Workspace(self.device)
        self.krylov = KrylovSolver(self.ws)
        # explicit Runge-Kutta options ({"method": "RK45", "atol": ..., ...})
        # when the local equations are integrated instead of exponentiated
        self.ode: dict | None = None
        self._rk = None
        state._finalise()
        self.t = {}
        for nid in state._order:
            t = state._phys[nid]
            if isinstance(t, np.ndarray):
                host = t
                t = torch.from_numpy(np.ascontiguousarray(t, dtype=np.complex128)).to(self.device, CDT)
                if t.device.type == "cpu" and np.shares_memory(t.numpy(), host):
                    t = t.clone()            # never evolve the caller's arrays in place
            t = t.to(self.device, CDT).contiguous()
            self.t[nid] = t
            state._phys[nid] = t
        self.W = {}
        if hamiltonian is not None:
            self.W = {nid: torch.from_numpy(Wn).to(self.device)
                      for nid, Wn in ttno_site_tensors(state, hamiltonian).items()}
        self.env: dict[tuple, torch.Tensor] = {}
        self.plans: dict = {}
        self.rowoff: dict = {}
        self.flops = 0
        # QR launch sequences are captured into CUDA graphs (one per node and
        # direction) after their first eager run; R and the work area then
        # must never move, so they are sized for the largest split up front.
        self.use_graphs = True
        self.qr_graphs: dict = {}
        self.qr_seen: set = set()
        self.cholqr_fails: set = set()
        self.cholqr_count = 0          # splits done by CholeskyQR2
        self.householder_count = 0     # splits done by Householder QR
        self.qr_rows_skipped = 0       # zero trailing rows the Householder QRs skipped
        self.graph_launches = 0
        # modification stamps: _mod[node] = clock at the last write of its tensor,
        # _env_at[(u, v)] = clock when E(u -> v) was computed, _w_at = clock of
        # the last TTNO refresh (init_cache_but_one(reuse=True) reads them)
        self._clock = 0
        self._mod: dict = {}
        self._env_at: dict = {}
        self._w_at = 0
        self._obs_sig = None           # tensors the cached observable plans were built on
        self._obs_plans: dict = {}
        self._ttno_nets: dict = {}     # id(TTNO) -> (TTNO, tensor signature, network)
        lib = _lib.load()
        kmax, wmax = 1, 1
        for nid in state._order:
            n = self.t[nid].numel()
            for k in self.t[nid].shape[:-1]:
                kmax = max(kmax, k)
                wmax = max(wmax, int(lib.ptn_zqr_work_bytes(n // k, k)))
        self.qr_R = torch.zeros((kmax * kmax,), dtype=CDT, device=self.device)
        self.qr_work = torch.zeros(((wmax + 15) // 16,), dtype=CDT, device=self.device)

    def refresh_hamiltonian(self, hamiltonian):
        """Copy a changed TTNO's tensors into the device buffers in place (every
        plan keeps pointing at them); the bond dimensions must not change."""
        new = ttno_site_tensors(self.state, hamiltonian)
        for nid, Wn in new.items():
            if tuple(Wn.shape) != tuple(self.W[nid].shape):
                raise ValueError(f"TTNO tensor of {nid} changed shape {tuple(self.W[nid].shape)} -> "
                                 f"{tuple(Wn.shape)}; the environments would not fit")
        for nid, Wn in new.items():
            self.W[nid].copy_(torch.from_numpy(Wn))
        self.ham = hamiltonian
        self._clock += 1
        self._w_at = self._clock

    def _finish(self, cb: "ChainBuilder", own_fixed: bool = False):
        """The chain as a tensor-core plan on the reduced-precision paths, else FP64.
        (Small chains stay on the tensor cores too: the FP64 kernel's 64 x 64
        tiles leave most of the GPU idle on skinny shapes such as a leaf's
        2 x 256 x 1280 step, measured 16x slower than the tensor-core plan.)
        ``own_fixed``: the plan keeps its fixed operands converted (see
        ``MixedPlan``), for the operators of a Krylov solve."""
        return cb.mixed_plan(self.levels, own_fixed) if self.levels else cb.plan()

    def _touch(self, *nids):
        """Record a write of these nodes' tensors (environment reuse)."""
        self._clock += 1
        for nid in nids:
            self._mod[nid] = self._clock

    # -- shapes ------------------------------------------------------------------
    def nbrs(self, nid):
        return self.state.nodes[nid].phys_neighbours()

    def shape(self, nid):
        return list(self.t[nid].shape)

    def env_buf(self, u, v):
        key = (u, v)
        if key not in self.env:
            chi = self.t[u].shape[self.state.phys_axis(u, v)]
            w = self.W[u].shape[self.state.phys_axis(u, v)]
            self.env[key] = torch.zeros((chi, w, chi), dtype=CDT, device=self.device)
        return self.env[key]

    def _env_op(self, u, v, labels):
        return Operand.contiguous(("fixed", self.env_buf(u, v)), labels, list(self.env_buf(u, v).shape))

    # -- site chain (shared by the matvec and the environment update) -------------
    def _site_chain(self, cb: ChainBuilder, x: Operand, nid: str, open_k=None) -> Operand:
        """Environments of the first half of the neighbours, then W, then the
        rest. Cost chi^{n+1} d (S(h) + S(n-h)) + chi^n d^2 w^n complex MAC;
        the reference contracts every environment before W (w^n larger)."""
        nb = self.nbrs(nid)
        n = len(nb)
        ks = [k for k in range(n) if k != open_k]
        half = len(ks) // 2
        T = x
        for k in ks[:half]:
            T = cb.contract(T, self._env_op(nb[k], nid, [f"a{k}", f"b{k}", f"c{k}"]), [f"a{k}"])
        Wop = Operand.contiguous(("fixed", self.W[nid]), [f"b{k}" for k in range(n)] + ["t", "s"],
                                 list(self.W[nid].shape))
        T = cb.contract(T, Wop, [f"b{k}" for k in ks[:half]] + ["s"])
        return T, ks[half:], nb

    def heff_plan(self, nid, fp64: bool = False) -> Plan:
        """y = H_eff x (``contract_ket_ham_with_envs``,
        ``contractions/state_operator_contraction.py:227-273``); ``fp64`` forces
        the complex128 chain on the reduced-precision path."""
        key = ("heff", nid) if not fp64 else ("heff", nid, "fp64")
        if key in self.plans:
            return self.plans[key]
        cb = ChainBuilder(self.ws)
        shape = self.shape(nid)
        n = len(shape) - 1
        x = Operand.contiguous(("in",), [f"a{k}" for k in range(n)] + ["s"], shape)
        y = Operand.contiguous(("out",), [f"c{k}" for k in range(n)] + ["t"], shape)
        T, rest, nb = self._site_chain(cb, x, nid)
        for i, k in enumerate(rest):
            E = self._env_op(nb[k], nid, [f"a{k}", f"b{k}", f"c{k}"])
            if i == len(rest) - 1:
                cb.contract(T, E, [f"a{k}", f"b{k}"], out=y)
            else:
                T = cb.contract(T, E, [f"a{k}", f"b{k}"])
        if not rest:
            raise RuntimeError("site without neighbours")
        p = cb.plan() if fp64 else self._finish(cb, own_fixed=True)
        self.plans[key] = p
        return p

    def env_plan(self, nid, nxt) -> Plan:
        """E(nid -> nxt) (``contract_any``, ``contractions/state_operator_contraction.py:407-694``)."""
        key = ("env", nid, nxt)
        if key in self.plans:
            return self.plans[key]
        cb = ChainBuilder(self.ws)
        shape = self.shape(nid)
        n = len(shape) - 1
        nb = self.nbrs(nid)
        k0 = nb.index(nxt)
        A = Operand.contiguous(("fixed", self.t[nid]), [f"a{k}" for k in range(n)] + ["s"], shape)
        T, rest, _ = self._site_chain(cb, A, nid, open_k=k0)
        for k in rest:
            T = cb.contract(T, self._env_op(nb[k], nid, [f"a{k}", f"b{k}", f"c{k}"]), [f"a{k}", f"b{k}"])
        B = Operand.contiguous(("fixed", self.t[nid]),
                               [f"c{k}" if k != k0 else "z" for k in range(n)] + ["t"], shape)
        E = self._env_op(nid, nxt, [f"a{k0}", f"b{k0}", "z"])
        cb.contract(T, B, [f"c{k}" for k in range(n) if k != k0] + ["t"], out=E, conj_b=True)
        p = self._finish(cb)
        self.plans[key] = p
        return p

    def bond_plan(self, nid, nxt) -> Plan:
        """Bond matvec on R (legs: nid side, nxt side) (``contract_bond_tensor``,
        ``contractions/state_operator_contraction.py:984-1040``)."""
        key = ("bond", nid, nxt)
        if key in self.plans:
            return self.plans[key]
        cb = ChainBuilder(self.ws)
        eq = self._env_op(nid, nxt, ["a", "b", "x"])
        en = self._env_op(nxt, nid, ["c", "b", "y"])
        chi_q, chi_n = eq.dims[0], en.dims[0]
        r = Operand.contiguous(("in",), ["a", "c"], [chi_q, chi_n])
        y = Operand.contiguous(("out",), ["x", "y"], [chi_q, chi_n])
        T = cb.contract(eq, r, ["a"])
        cb.contract(T, en, ["c", "b"], out=y)
        p = self._finish(cb, own_fixed=True)
        self.plans[key] = p
        return p

    # -- environment cache --------------------------------------------------------
    def update_env(self, nid, nxt):
        p = self.env_plan(nid, nxt)
        p.run()
        self.flops += p.flops
        self._env_at[(nid, nxt)] = self._clock

    def init_cache_but_one(self, left_out, reuse: bool = False):
        """All environments pointing toward ``left_out``
        (``SandwichCache.init_cache_but_one``, ``contractions/sandwich_caching.py:97-126``).
        ``reuse``: keep an environment computed after the last write of every
        tensor on its side of the edge (and of the TTNO) -- its inputs are
        unchanged, so recomputing it would give the same bits. Only for callers
        whose tensor writes all went through this network."""
        self.env_reused = getattr(self, "env_reused", 0)

        def rec(nid, toward):
            newest = self._mod.get(nid, 0)
            for nb in self.nbrs(nid):
                if nb != toward:
                    newest = max(newest, rec(nb, nid))
            if toward is not None:
                at = self._env_at.get((nid, toward))
                if (reuse and at is not None and (nid, toward) in self.env and at >= newest
                        and at >= self._w_at):
                    self.env_reused += 1
                else:
                    self.update_env(nid, toward)
            return newest
        rec(left_out, None)

    # -- local evolutions ------------------------------------------------------------
    @staticmethod
    def _held(p, fn):
        """Run ``fn`` with plan ``p``'s fixed operands converted once (its
        environments and TTNO tensor do not change during one local solve)."""
        if not isinstance(p, MixedPlan) or not p.prep:
            return fn()
        p.prepare()
        p.hold = True
        try:
            return fn()
        finally:
            p.hold = False

    def evolve_site(self, nid, dt, exp_factor, tol, maxdim, hermitian: bool = True):
        p = self.heff_plan(nid)

        def apply(xp, yp):
            p.run(xp, yp)
            self.flops += p.flops
        x = self.t[nid]
        self._held(p, lambda: self.local_exp(x, apply, dt, exp_factor, tol, maxdim, hermitian, out=x))
        self._touch(nid)
        self.check_device_status()

    def local_exp(self, x, apply, dt, exp_factor, tol, maxdim, hermitian=True, out=None):
        """exp(exp_factor dt H) x for the operator ``apply``: the Krylov
        exponential, or the adaptive Runge-Kutta integration of
        y' = exp_factor H y when ``self.ode`` names an ODE method."""
        if self.ode is not None:
            if self._rk is None:
                from .ode import RungeKuttaSolver
                self._rk = RungeKuttaSolver(self.ws)
            return self._rk.integrate(x, apply, dt, exp_factor, out=out, **self.ode)
        return self.krylov.expm(x, apply, dt, exp_factor, tol, maxdim, hermitian=hermitian, out=out,
                                tridiagonal=self.levels > 0)

    def check_device_status(self):
        st = self.ws.bufs.get("tc_status")
        if st is not None and int(st.item()) != 0:
            code = int(st.item())
            st.zero_()
            raise _lib.PtnError(code, "tensor-core contraction")

    def evolve_bond(self, r: torch.Tensor, nid, nxt, dt, exp_factor, tol, maxdim, hermitian: bool = True):
        p = self.bond_plan(nid, nxt)

        def apply(xp, yp):
            p.run(xp, yp)
            self.flops += p.flops
        return self._held(p, lambda: self.local_exp(r, apply, dt, exp_factor, tol, maxdim, hermitian, out=r))

    # -- QR split and R absorption ---------------------------------------------------
    # Reduced-precision path: tall splits (m >= 2k, k <= ptn_zchol_max_k) try
    # CholeskyQR2 first; the pivot test on the device decides, and a split that
    # is not of full numerical rank takes the Householder path.
    CHOLQR_MIN_ROWS = 64
    # Splits with at least this many entries are scanned for exactly-zero
    # trailing rows, which the Householder QR then skips (ptn_zqr_keep_rows).
    QR_SCAN_MIN = 1 << 15
    # CholeskyQR2 writes Q = A X with one tensor-core product, whose FP32
    # rounding (relative to |A||X|) puts ~6e-8 kappa(A) into Q R - A; splits
    # whose first Cholesky factor has a diagonal ratio below this (kappa above
    # ~10) take the backward-stable Householder path instead
    CHOLQR_PIVOT_RATIO = 0.1
    # second pass: first-order factor when ||Q1^H Q1 - I||_F is at most this
    CHOLQR_SERIES_TOL = 3e-4

    def _qr_words(self):
        """Device words written by the split probe ([0] rows in use, [1] the
        Cholesky status as int32) and their pinned host copy."""
        w = self.ws.bufs.get("qr_words")
        if w is None:
            w = torch.zeros(2, dtype=torch.int64, device=self.device)
            self.ws.bufs["qr_words"] = w
            self._qr_words_host = torch.zeros(2, dtype=torch.int64, pin_memory=self.device.type == "cuda")
        return w, self._qr_words_host

    def _cholqr_plans(self, nid, row_axes, col_axis):
        """Tensor-core plans of CholeskyQR2 for one split: the Gram matrix of the
        site matrix A, A times a k x k matrix B (into the ``cholqr_out`` slot),
        and the Gram matrix of that product. ``bufs``: k x k complex128 slots
        [G, B, R1, R2, R2^-1, X, R0]."""
        shape = self.shape(nid)
        n = len(shape) - 1
        labels = [f"a{i}" for i in range(n)] + ["s"]
        rows = [labels[a] for a in row_axes]
        col = labels[col_axis]
        k = shape[col_axis]
        key = ("cholqr", nid, tuple(shape), tuple(row_axes), col_axis)
        if key not in self.plans:
            bufs = torch.zeros((7, k, k), dtype=CDT, device=self.device)
            lp = [l if l != col else "p" for l in labels]
            lq = [l if l != col else "q" for l in labels]
            G = Operand.contiguous(("fixed", bufs[0]), ["p", "q"], [k, k])
            cb = ChainBuilder(self.ws)
            cb.contract(Operand.contiguous(("fixed", self.t[nid]), lp, shape),
                        Operand.contiguous(("fixed", self.t[nid]), lq, shape), rows, out=G, conj_a=True)
            gram_a = cb.mixed_plan(self.levels)
            cb = ChainBuilder(self.ws)
            cb.contract(Operand.contiguous(("fixed", self.t[nid]), lp, shape),
                        Operand.contiguous(("fixed", bufs[1]), ["p", "q"], [k, k]), ["p"],
                        out=Operand.contiguous(("ws", "cholqr_out"), lq, shape))
            apply_a = cb.mixed_plan(self.levels)
            cb = ChainBuilder(self.ws)
            cb.contract(Operand.contiguous(("ws", "cholqr_out"), lp, shape),
                        Operand.contiguous(("ws", "cholqr_out"), lq, shape), rows, out=G, conj_a=True)
            gram_q = cb.mixed_plan(self.levels)
            self.plans[key] = (gram_a, apply_a, gram_q, bufs)
        return self.plans[key]

    def _cholqr_finish(self, nid, gram_a, apply_a, gram_q, bufs, k) -> torch.Tensor:
        """CholeskyQR2 once the first factor R1 (of G1 = A^H A) passed its test:
        Q1 = A R1^-1, G2 = Q1^H Q1 = R2^H R2, X = R1^-1 R2^-1, Q = A X written
        over the site tensor, and R = X^-1 from R2 R1 by one FP64 Newton step,
        so that Q R = A to FP64 rounding plus the one tensor-core product A X
        (the FP32 error of the Cholesky factors only moves Q's gauge and its
        orthonormality). No host round trip."""
        lib = _lib.load()
        stream = _stream_ptr()
        numel = self.t[nid].numel()
        G, B, R1, R2, R2i, X, R0 = (bufs[i] for i in range(7))
        self.ws.get("cholqr_out", numel)
        apply_a.run()                                   # Q1 = A R1^-1 (B holds R1^-1)
        gram_q.run()                                    # G = Q1^H Q1
        # a failure here (not expected after the first pass) lands in the
        # tensor-core status word, which the next status check reports
        st = self.ws.bufs.get("tc_status")
        work = self.ws.get("chol_work", (int(lib.ptn_zchol_work_bytes(k)) + 15) // 16)
        check(lib.ptn_zchol_upper(G.data_ptr(), k, k, R2.data_ptr(), R2i.data_ptr(), 0.0, 1,
                                  self.CHOLQR_SERIES_TOL, st.data_ptr(), work.data_ptr(), stream), "zchol_upper")
        check(lib.ptn_ztri_mul_upper(B.data_ptr(), R2i.data_ptr(), X.data_ptr(), k, stream), "ztri_mul_upper")
        check(lib.ptn_ztri_mul_upper(R2.data_ptr(), R1.data_ptr(), R0.data_ptr(), k, stream), "ztri_mul_upper")
        B.copy_(X)
        Rd = self.qr_R[:k * k].view(k, k)
        check(lib.ptn_ztri_inv_newton(X.data_ptr(), R0.data_ptr(), Rd.data_ptr(), G.data_ptr(), k, stream),
              "ztri_inv_newton")
        apply_a.run()                                   # Q = A X
        self.t[nid].view(-1).copy_(self.ws.bufs["cholqr_out"][:numel])
        self.flops += 2 * gram_a.flops + 2 * apply_a.flops
        self.cholqr_count += 1
        return Rd

    def qr_split(self, nid, nbr) -> torch.Tensor:
        R = self._qr_split(nid, nbr)
        self._touch(nid)
        return R

    def _qr_split(self, nid, nbr) -> torch.Tensor:
        """tensor[nid] <- Q (KEEP), returns R (k x k; legs: new bond, nbr-side bond).
        Rows in the reference's logical order (``util/tensor_splitting.py:60-107``)."""
        st = self.state
        node = st.nodes[nid]
        if node.parent == nbr:
            row_nbrs = list(node.children)
        else:
            row_nbrs = ([node.parent] if node.parent is not None else []) + \
                [c for c in node.children if c != nbr]
        shape = self.shape(nid)
        row_axes = [st.phys_axis(nid, x) for x in row_nbrs] + [len(shape) - 1]
        col_axis = st.phys_axis(nid, nbr)
        key = (tuple(shape), tuple(row_axes), col_axis)
        strides = self.t[nid].stride()
        if key not in self.rowoff:
            idx = np.zeros(1, dtype=np.int64)
            for ax in row_axes:
                idx = (idx[:, None] + np.arange(shape[ax], dtype=np.int64)[None, :] * strides[ax]).reshape(-1)
            self.rowoff[key] = torch.from_numpy(idx).to(self.device)
        rowoff = self.rowoff[key]
        m = rowoff.numel()
        k = shape[col_axis]
        lib = _lib.load()
        stream = _stream_ptr()
        # two-site splits change bond dimensions, and with them the row count of
        # every other split of the two nodes: size R and the work area for this one
        self._ensure_qr_buffers(m, k)
        ckey = (nid, tuple(shape), tuple(row_axes), col_axis)
        use_chol = bool(self.levels) and m >= self.CHOLQR_MIN_ROWS and m >= 2 * k and \
            k <= int(lib.ptn_zchol_max_k()) and ckey not in self.cholqr_fails
        scan = m * k >= self.QR_SCAN_MIN and self.device.type == "cuda"
        m_used = m
        if use_chol or scan:
            # one probe, one synchronisation: the rows in use and, for a tall
            # split, the first Cholesky factor of the Gram matrix with its pivot test
            words, host = self._qr_words()
            words.zero_()
            A = self.t[nid]
            if scan:
                check(lib.ptn_znonzero_rows(A.data_ptr(), rowoff.data_ptr(), m, k, strides[col_axis],
                                            words.data_ptr(), stream), "znonzero_rows")
            if use_chol:
                gram_a, apply_a, gram_q, bufs = self._cholqr_plans(nid, row_axes, col_axis)
                gram_a.run()
                if self.ws.bufs.get("tc_status") is None:
                    self.ws.bufs["tc_status"] = torch.zeros(1, dtype=torch.int32, device=self.device)
                work = self.ws.get("chol_work", (int(lib.ptn_zchol_work_bytes(k)) + 15) // 16)
                check(lib.ptn_zchol_upper(bufs[0].data_ptr(), k, k, bufs[2].data_ptr(), bufs[1].data_ptr(),
                                          self.CHOLQR_PIVOT_RATIO, 0, 0.0, words.data_ptr() + 8,
                                          work.data_ptr(), stream), "zchol_upper")
            host.copy_(words, non_blocking=True)
            if self.device.type == "cuda":
                check(lib.ptn_stream_synchronize(stream), "stream synchronize")
            if scan:
                m_used = max(1, int(host[0]))
            if use_chol:
                if int(host[1]) == 0:
                    R = self._cholqr_finish(nid, gram_a, apply_a, gram_q, bufs, k)
                    if node.parent != nbr:
                        node.children = [nbr] + [c for c in node.children if c != nbr]
                    return R
                # not of full numerical rank (e.g. zero-padded bonds): keep
                # LAPACK's Householder complement, which one-site TDVP depends on
                self.cholqr_fails.add(ckey)
        R = self.qr_R[:k * k].view(k, k)
        work = self.qr_work
        if m_used < m:
            self.qr_rows_skipped += m - m_used

        def launch():
            if m_used < m:
                check(lib.ptn_zqr_keep_rows(self.t[nid].data_ptr(), rowoff.data_ptr(), m, m_used, k,
                                            strides[col_axis], R.data_ptr(), work.data_ptr(), _stream_ptr()),
                      "ptn_zqr_keep_rows")
            else:
                check(lib.ptn_zqr_keep(self.t[nid].data_ptr(), rowoff.data_ptr(), m, k, strides[col_axis],
                                       R.data_ptr(), work.data_ptr(), _stream_ptr()), "ptn_zqr_keep")
        gkey = (nid, nbr, key, m_used)
        # small splits run as one cooperative launch (ptn_zqr_path 1): nothing
        # to replay; the per-step launch sequences of larger ones are recorded
        one_launch = m <= 2048 and int(lib.ptn_zqr_path(m_used, k)) == 1
        if not self.use_graphs or self.device.type != "cuda" or one_launch:
            launch()
        elif gkey in self.qr_graphs:
            g, nlaunch = self.qr_graphs[gkey]
            g.replay()
            self.graph_launches += nlaunch
        elif gkey in self.qr_seen:
            g = torch.cuda.CUDAGraph()
            c0 = int(lib.ptn_launch_counter())
            with torch.cuda.graph(g):
                launch()
            nlaunch = int(lib.ptn_launch_counter()) - c0
            self.qr_graphs[gkey] = (g, nlaunch)
            g.replay()
            self.graph_launches += nlaunch
        else:
            self.qr_seen.add(gkey)
            launch()
        if node.parent != nbr:
            node.children = [nbr] + [c for c in node.children if c != nbr]
        self.flops += 8 * 2 * m_used * k * k
        self.householder_count += 1
        return R

    def absorb(self, R: torch.Tensor, src, dst, link_variant: bool, precise: bool = False):
        """dst[..., new, ...] = sum_a R[new, a] dst[..., a, ...] on dst's leg toward src.
        Logical order as in ``contract_nodes`` (``contractions/node_contraction.py:88-138``)."""
        st = self.state
        shape = self.shape(dst)
        n = len(shape) - 1
        ax = st.phys_axis(dst, src)
        key = ("absorb", dst, src, precise)
        if key not in self.plans:
            cb = ChainBuilder(self.ws)
            Rop = Operand.contiguous(("in",), ["new", f"a{ax}"], [shape[ax], shape[ax]])
            T = Operand.contiguous(("fixed", self.t[dst]), [f"a{k}" for k in range(n)] + ["s"], shape)
            labels = [f"a{k}" if k != ax else "new" for k in range(n)] + ["s"]
            out = Operand.contiguous(("ws", "absorb"), labels, shape)
            cb.sizes["absorb"] = out.numel()
            cb.contract(T, Rop, [f"a{ax}"], out=out)
            if self.levels and not precise:
                mp = cb.mixed_plan(self.levels)
                mp.sizes_c128 = dict(cb.sizes)
                self.plans[key] = mp
            else:
                self.plans[key] = cb.plan()
        p = self.plans[key]
        self.ws.get("absorb", self.t[dst].numel())
        p.run(R.data_ptr(), 0)
        self.t[dst].view(-1).copy_(self.ws.bufs["absorb"][:self.t[dst].numel()])
        self.flops += p.flops
        if isinstance(p, MixedPlan):
            # dst is an isometry toward src, so the new centre has exactly R's
            # norm; restore it in FP64 so the reduced-precision product cannot
            # drift the state norm (fidelity is unaffected either way)
            lib = _lib.load()
            t = self.t[dst]
            k = R.numel()
            part = self.ws.get("kry_part", int(lib.ptn_krylov_partials(max(t.numel(), k))) + 8)
            scal = self.ws.get("absorb_norms", 2, torch.float64)
            check(lib.ptn_dznrm2(R.data_ptr(), k, scal[0:].data_ptr(), part.data_ptr(), _stream_ptr()), "dznrm2")
            check(lib.ptn_dznrm2(t.data_ptr(), t.numel(), scal[1:].data_ptr(), part.data_ptr(), _stream_ptr()),
                  "dznrm2")
            check(lib.ptn_zscal_ratio(t.data_ptr(), scal[0:].data_ptr(), scal[1:].data_ptr(), t.data_ptr(),
                                      t.numel(), _stream_ptr()), "zscal_ratio")
        self._touch(dst)
        node = st.nodes[src]
        if node.parent == dst:
            dn = st.nodes[dst]
            others = [c for c in dn.children if c != src]
            dn.children = ([src] + others) if link_variant else (others + [src])

    def move_orth_one_hop(self, a, b, precise: bool = False):
        R = self.qr_split(a, b)
        self.absorb(R, a, b, link_variant=False, precise=precise)

    def move_orth_center(self, new_center):
        st = self.state
        if st.orthogonality_center_id is None:
            raise AssertionError("The TTN is not in canonical form, so the orth. center cannot be moved!")
        path = st.path_from_to(st.orthogonality_center_id, new_center)
        for a, b in zip(path[:-1], path[1:]):
            self.move_orth_one_hop(a, b)
        st.orthogonality_center_id = new_center

    # -- two-site update: merge, matvec, truncated SVD split -----------------------
    def _two_site_info(self, u, v) -> dict:
        """Leg bookkeeping of the merged pair. The merged tensor holds u's other
        neighbours (physical order) and u's physical leg ("u side", m entries),
        and the same for v ("v side", n entries). The larger side is stored
        first, so the SVD sees a tall column-major matrix T = M (m >= n) or
        T = M^T (m < n) without a transpose."""
        su, sv = self.shape(u), self.shape(v)
        key = ("2info", u, v, tuple(su), tuple(sv))
        info = self.plans.get(key)
        if info is not None:
            return info
        st = self.state
        nu = [x for x in self.nbrs(u) if x != v]
        nv = [x for x in self.nbrs(v) if x != u]
        du = [su[st.phys_axis(u, x)] for x in nu] + [su[-1]]
        dv = [sv[st.phys_axis(v, x)] for x in nv] + [sv[-1]]
        lu = [f"au{k}" for k in range(len(nu))] + ["su"]
        lv = [f"av{k}" for k in range(len(nv))] + ["sv"]
        m, n = int(np.prod(du)), int(np.prod(dv))
        vfirst = m >= n
        info = dict(nu=nu, nv=nv, du=du, dv=dv, lu=lu, lv=lv, m=m, n=n, vfirst=vfirst,
                    labels=(lv + lu) if vfirst else (lu + lv), dims=(dv + du) if vfirst else (du + dv))
        self.plans[key] = info
        return info

    def merge_plan(self, u, v) -> Plan:
        """The two site tensors contracted over their bond (``contract_nodes``,
        ``contractions/node_contraction.py:12-141``), written in the merged layout."""
        info = self._two_site_info(u, v)
        key = ("merge", u, v, tuple(info["dims"]))
        if key in self.plans:
            return self.plans[key]
        cb = ChainBuilder(self.ws)
        A = Operand.contiguous(("fixed", self.t[u]),
                               ["bond" if x == v else info["lu"][info["nu"].index(x)] for x in self.nbrs(u)]
                               + ["su"], self.shape(u))
        B = Operand.contiguous(("fixed", self.t[v]),
                               ["bond" if x == u else info["lv"][info["nv"].index(x)] for x in self.nbrs(v)]
                               + ["sv"], self.shape(v))
        cb.contract(A, B, ["bond"], out=Operand.contiguous(("out",), info["labels"], info["dims"]))
        # FP64 on every path: the merged tensor IS the state (a reduced-precision
        # product here would move its norm), and the merge is one contraction
        # against the several matvecs of the Krylov exponential
        p = cb.plan()
        self.plans[key] = p
        return p

    def heff2_plan(self, u, v) -> Plan:
        """H_eff of the merged pair (``effective_two_site_evolution``,
        ``time_evo_util/effective_time_evolution.py:326-410``). The reference joins
        the two TTNO tensors and contracts every environment before them; here
        each side runs the single-site order (half of its environments, its W,
        the rest), so no intermediate carries more than two TTNO bond legs."""
        info = self._two_site_info(u, v)
        key = ("heff2", u, v, tuple(info["dims"]))
        if key in self.plans:
            return self.plans[key]
        cb = ChainBuilder(self.ws)
        out_labels = [l.replace("au", "cu").replace("av", "cv").replace("su", "tu").replace("sv", "tv")
                      for l in info["labels"]]
        x = Operand.contiguous(("in",), info["labels"], info["dims"])
        y = Operand.contiguous(("out",), out_labels, info["dims"])
        ops = []
        for side, node, other, nbl in (("u", u, v, info["nu"]), ("v", v, u, info["nv"])):
            half = len(nbl) // 2
            envs = [self._env_op(nb, node, [f"a{side}{k}", f"b{side}{k}", f"c{side}{k}"])
                    for k, nb in enumerate(nbl)]
            for k in range(half):
                ops.append((envs[k], [f"a{side}{k}"]))
            wl = ["bw" if x_ == other else f"b{side}{nbl.index(x_)}" for x_ in self.nbrs(node)]
            W = Operand.contiguous(("fixed", self.W[node]), wl + [f"t{side}", f"s{side}"],
                                   list(self.W[node].shape))
            kl = [f"b{side}{k}" for k in range(half)] + [f"s{side}"] + (["bw"] if side == "v" else [])
            ops.append((W, kl))
            for k in range(half, len(nbl)):
                ops.append((envs[k], [f"a{side}{k}", f"b{side}{k}"]))
        T = x
        for i, (op, kl) in enumerate(ops):
            if i == len(ops) - 1:
                cb.contract(T, op, kl, out=y)
            else:
                T = cb.contract(T, op, kl)
        p = self._finish(cb)
        self.plans[key] = p
        return p

    def _permute(self, src_ptr, dst_ptr, dims, s_src, s_dst, conj=False, scale_ptr=0, scale_mode=0):
        d = _lib.PermuteDesc()
        if len(dims) > MAX_MODES:
            raise ValueError(f"permute needs {len(dims)} modes (max {MAX_MODES})")
        d.src, d.dst, d.n, d.conj = src_ptr, dst_ptr, len(dims), int(conj)
        for i, (n_, a, b) in enumerate(zip(dims, s_src, s_dst)):
            d.dim[i], d.stride_src[i], d.stride_dst[i] = n_, a, b
        d.scale = scale_ptr or None
        d.scale_mode = scale_mode
        check(_lib.load().ptn_zpermute(ctypes.byref(d), _stream_ptr()), "ptn_zpermute")

    @staticmethod
    def _cstrides(dims):
        out, s = [], 1
        for d in reversed(dims):
            out.append(s)
            s *= d
        return list(reversed(out))

    def _ensure_qr_buffers(self, m, k):
        """Grow the QR R/work buffers (bond dimensions change in two-site
        updates); captured QR graphs point at the old buffers and are dropped."""
        lib = _lib.load()
        need_w = (int(lib.ptn_zqr_work_bytes(m, k)) + 15) // 16
        if k * k > self.qr_R.numel() or need_w > self.qr_work.numel():
            self.qr_R = torch.zeros((max(k * k, self.qr_R.numel()),), dtype=CDT, device=self.device)
            self.qr_work = torch.zeros((max(need_w, self.qr_work.numel()),), dtype=CDT, device=self.device)
            self.qr_graphs.clear()
            self.qr_seen.clear()

    def _forget_node(self, nid):
        """Drop every cached plan, QR graph and environment that depends on the
        shape or storage of ``nid``'s tensor."""
        for key in [k for k in self.plans if any(x == nid for x in k[1:3])]:
            del self.plans[key]
        for key in [k for k in self.qr_graphs if k[0] == nid]:
            del self.qr_graphs[key]
        self.qr_seen = {k for k in self.qr_seen if k[0] != nid}
        self.cholqr_fails = {k for k in self.cholqr_fails if k[0] != nid}

    def _set_node_tensor(self, nid, t: torch.Tensor):
        self._touch(nid)
        self.t[nid] = t
        self.state._phys[nid] = t
        self.state.nodes[nid].shape = tuple(t.shape)

    # Jacobi runs on the q x q core when q is at most this, or when the kept
    # rank could exceed half of q; otherwise a subspace iteration reduces T to
    # max_bond_dim + SUBSPACE_OVERSAMPLE columns first. Up to 64 columns the
    # Jacobi sweeps run in one CTA (shared memory, CTA barriers); above, every
    # round of a sweep is a grid-wide barrier (~4 ms for a 128 x 128 core). The
    # subspace iteration costs two QRs and a host round trip per iteration, so
    # below SVD_DIRECT_MAX it is taken only for kept ranks up to
    # SUBSPACE_SMALL_L columns and cores at least four times wider (measured on
    # the 31-site binary tree: max_bond_dim 8 gains 40 % per step, 32 loses).
    SVD_DIRECT_MAX = 384
    SUBSPACE_SMALL_L = 24
    SUBSPACE_OVERSAMPLE = 16
    SUBSPACE_MAX_ITERS = 8

    def _qr_inplace(self, buf: torch.Tensor, p: int, k: int, rname: str) -> torch.Tensor:
        """Householder QR of the p x k column-major matrix in ``buf`` (Q in place);
        returns R (k x k, row-major) in a workspace slot."""
        lib = _lib.load()
        key = ("rowoff_lin", p)
        if key not in self.rowoff:
            self.rowoff[key] = torch.arange(p, dtype=torch.int64, device=self.device)
        R = self.ws.get(rname, k * k)
        qw = self.ws.get("svd_qrwork", (int(lib.ptn_zqr_work_bytes(p, k)) + 15) // 16)
        check(lib.ptn_zqr_keep(buf.data_ptr(), self.rowoff[key].data_ptr(), p, k, p, R.data_ptr(),
                               qw.data_ptr(), _stream_ptr()), "ptn_zqr_keep")
        self.flops += 8 * 2 * p * k * k
        return R

    def _jacobi(self, src: torch.Tensor, m: int, n: int, rs: int, cs: int):
        """Jacobi SVD of an m x n (m >= n) matrix; returns (U slot, V slot, S on host)."""
        lib = _lib.load()
        Uj = self.ws.get("svd_U", m * n)
        Vj = self.ws.get("svd_V", n * n)
        Sb = self.ws.get("svd_S", n + 2, torch.float64)
        Sb.zero_()
        sw = self.ws.get("svd_work", (int(lib.ptn_zsvd_work_bytes(m, n)) + 15) // 16)
        d = _lib.SvdDesc()
        d.A, d.m, d.n, d.row_stride, d.col_stride = src.data_ptr(), m, n, rs, cs
        d.U, d.ldu, d.S, d.V, d.ldv = Uj.data_ptr(), m, Sb.data_ptr(), Vj.data_ptr(), n
        d.work = sw.data_ptr()
        d.status = Sb[n:].data_ptr()
        check(lib.ptn_zsvd_jacobi(ctypes.byref(d), _stream_ptr()), "ptn_zsvd_jacobi")
        host = Sb.cpu()
        code = int(host[n:n + 1].view(torch.int32)[0])
        if code != 0:
            raise _lib.PtnError(code, "Jacobi SVD")
        s = host[:n].numpy().copy()
        if not np.all(np.isfinite(s)):
            raise _lib.PtnError(3, "Jacobi SVD: non-finite singular values")
        return Uj, Vj, s

    def _mat(self, t: torch.Tensor, rows: int, cols: int, row_label: str, col_label: str, ld=None) -> Operand:
        """A column-major rows x cols matrix held in ``t`` as a labelled operand."""
        return Operand(("fixed", t), [row_label, col_label], [rows, cols], [1, rows if ld is None else ld])

    def _subspace_factor(self, x2: torch.Tensor, p: int, q: int, l: int):
        """Range finder with subspace (power) iteration and Rayleigh-Ritz on the
        tall p x q matrix T in ``x2``: T ~= Q1 Vj diag(S) (Qz Uj)^H with
        Q1 (p x l) and Qz (q x l) orthonormal. Iterates until the leading
        l - oversample singular values agree to 1e-14 relative between two
        iterations. The reference computes the full SVD (LAPACK gesdd) and
        keeps at most max_bond_dim values; the kept triplets agree to that
        accuracy when the spectrum has left the subspace by then."""
        key = ("omega", q, l)
        if key not in self.rowoff:
            rng = np.random.default_rng(12345)
            om = (rng.standard_normal((q, l)) + 1j * rng.standard_normal((q, l))) / np.sqrt(2)
            self.rowoff[key] = torch.from_numpy(np.asfortranarray(om).T.copy()).to(self.device).view(-1)
        omega = self.rowoff[key]
        Y = self.ws.get("sub_Y", p * l)
        Z = self.ws.get("sub_Z", q * l)
        T = self._mat(x2, p, q, "i", "k")
        Th = Operand(T.ref, ["i", "k"], [p, q], [1, p])
        # the range-finding products may run on the tensor cores (the FP64
        # Rayleigh-Ritz step below fixes the accuracy); T^H Q1 is always FP64
        cb = ChainBuilder(self.ws)
        cb.contract(T, self._mat(omega, q, l, "k", "c"), ["k"], out=self._mat(Y, p, l, "i", "c"))
        first = self._finish(cb)
        cb = ChainBuilder(self.ws)
        cb.contract(Th, self._mat(Y, p, l, "i", "c"), ["i"], out=self._mat(Z, q, l, "k", "c"), conj_a=True)
        back = cb.plan()
        cb = ChainBuilder(self.ws)
        cb.contract(T, self._mat(Z, q, l, "k", "c"), ["k"], out=self._mat(Y, p, l, "i", "c"))
        fwd = self._finish(cb)
        first.run()
        self.flops += first.flops
        prev = None
        keep = max(1, l - self.SUBSPACE_OVERSAMPLE)
        for it in range(self.SUBSPACE_MAX_ITERS):
            if it > 0:
                fwd.run()                      # Y = T Qz
                self.flops += fwd.flops
            self._qr_inplace(Y, p, l, "sub_RY")   # Y <- Q1
            back.run()                         # Z = T^H Q1
            self.flops += back.flops
            Rz = self._qr_inplace(Z, q, l, "sub_RZ")   # Z <- Qz, Rz
            Uj, Vj, s = self._jacobi(Rz, l, l, l, 1)
            if prev is not None and np.max(np.abs(s[:keep] - prev[:keep])) <= 1e-14 * max(s[0], 1e-300):
                break
            prev = s
        return Y, Z, Uj, Vj, s

    def _write_factor(self, dst: torch.Tensor, ax_side, ax_bond, side_dims, side_labels, Q, q_ld, small,
                      small_ld, k, r, conj=False, scale=None):
        """dst[side legs, bond c] = op(Q @ small)[row, c] * scale[c] for c < r,
        where Q (rows x k, column-major, ld q_ld) may be None (identity), small
        is k x (>= r) column-major with leading dimension small_ld, rows run
        over the side legs in C order, and op = conj when ``conj``."""
        shp = list(dst.shape)
        dstr = self._cstrides(shp)
        srow = self._cstrides(side_dims)
        if Q is None:
            self._permute(small.data_ptr(), dst.data_ptr(), side_dims + [r], srow + [small_ld],
                          [dstr[a] for a in ax_side] + [dstr[ax_bond]], conj=conj,
                          scale_ptr=scale.data_ptr() if scale is not None else 0, scale_mode=len(side_dims))
            return
        conj_b = conj
        if scale is not None:
            tmp = self.ws.get("svd_small_scaled", k * r)
            self._permute(small.data_ptr(), tmp.data_ptr(), [r, k], [small_ld, 1], [k, 1], conj=conj,
                          scale_ptr=scale.data_ptr(), scale_mode=0)
            small, small_ld, conj_b = tmp, k, False
        lab = [None] * len(shp)
        for l_, a in zip(side_labels, ax_side):
            lab[a] = l_
        lab[ax_bond] = "c"
        cb = ChainBuilder(self.ws)
        A = Operand(("fixed", Q), ["k"] + side_labels, [k] + side_dims, [q_ld] + srow)
        B = Operand(("fixed", small), ["k", "c"], [k, r], [1, small_ld])
        cb.contract(A, B, ["k"], out=Operand(("fixed", dst), lab, shp, dstr), conj_a=conj, conj_b=conj_b)
        pl = cb.plan()
        pl.run()
        self.flops += pl.flops

    def svd_split(self, u, v, x2: torch.Tensor, svd) -> np.ndarray:
        """Truncated SVD of the merged pair with the singular values moved into
        v (``split_node_svd`` -> ``contr_truncated_svd_splitting`` (VCONTR),
        ``core/ttn.py:1476-1497``, ``util/tensor_splitting.py:488-572``).
        T (p x q, column-major in ``x2``; T = M or M^T, p >= q) is factored as
        T = Ut diag(S) Vt^H by one of: Jacobi directly (p == q), Householder QR
        then Jacobi on the q x q R (p > q, q small), or subspace iteration to
        max_bond_dim + oversample columns then Jacobi (q large). The kept rank
        comes from ``truncate_singular_values`` (``:448-486``) on the host; the
        factors go straight into u's and v's leg layouts. Returns the kept
        singular values."""
        from .truncation import truncate_singular_values
        info = self._two_site_info(u, v)
        st = self.state
        m, n, vfirst = info["m"], info["n"], info["vfirst"]
        p, q = (m, n) if vfirst else (n, m)
        mbd = svd.max_bond_dim
        l = q if mbd == float("inf") else min(q, int(mbd) + self.SUBSPACE_OVERSAMPLE)
        if (q > self.SVD_DIRECT_MAX and 2 * l <= q) or (q > 64 and l <= self.SUBSPACE_SMALL_L and 4 * l <= q):
            Y, Z, Uj, Vj, s = self._subspace_factor(x2, p, q, l)
            left = (Y, p, Vj, l, l)        # Ut = Q1 Vj
            right = (Z, q, Uj, l, l)       # Vt = Qz Uj
        elif p > q:
            R = self._qr_inplace(x2, p, q, "svd_R")
            Uj, Vj, s = self._jacobi(R, q, q, q, 1)
            left = (x2, p, Uj, q, q)       # Ut = Q Uj
            right = (None, 0, Vj, q, q)    # Vt = Vj
        else:
            Uj, Vj, s = self._jacobi(x2, p, q, 1, p)
            left = (None, 0, Uj, p, q)
            right = (None, 0, Vj, q, q)
        new_s, _ = truncate_singular_values(s, svd)
        r = len(new_s)
        scale = self.ws.get("svd_scale", r, torch.float64)
        scale.copy_(torch.from_numpy(np.ascontiguousarray(new_s, dtype=np.float64)))
        bu, bv = st.phys_axis(u, v), st.phys_axis(v, u)
        old_r = self.shape(u)[bu]
        shp_u, shp_v = self.shape(u), self.shape(v)
        shp_u[bu] = r
        shp_v[bv] = r
        if r == old_r:
            tu, tv = self.t[u], self.t[v]
        else:
            tu = torch.empty(shp_u, dtype=CDT, device=self.device)
            tv = torch.empty(shp_v, dtype=CDT, device=self.device)
        ax_u = [st.phys_axis(u, x) for x in info["nu"]] + [len(shp_u) - 1]
        ax_v = [st.phys_axis(v, x) for x in info["nv"]] + [len(shp_v) - 1]
        U_side = (tu, ax_u, bu, info["du"], info["lu"])
        V_side = (tv, ax_v, bv, info["dv"], info["lv"])
        if vfirst:
            # M = Ut S Vt^H: u <- Ut[:, :r], v[c, j] = S_c conj(Vt[j, c])
            self._write_factor(*U_side, *left[:4], left[4], r)
            self._write_factor(*V_side, *right[:4], right[4], r, conj=True, scale=scale)
        else:
            # M = conj(Vt) S Ut^T: u <- conj(Vt[:, :r]), v[c, j] = S_c Ut[j, c]
            self._write_factor(*U_side, *right[:4], right[4], r, conj=True)
            self._write_factor(*V_side, *left[:4], left[4], r, scale=scale)
        if r != old_r:
            self._forget_node(u)
            self._forget_node(v)
            self.env.pop((u, v), None)
            self.env.pop((v, u), None)
            self._set_node_tensor(u, tu)
            self._set_node_tensor(v, tv)
        self._touch(u, v)
        # logical order: the node that gains the new child lists it first (core/ttn.py:1400-1448)
        if st.nodes[v].parent == u:
            nu_ = st.nodes[u]
            nu_.children = [v] + [c for c in nu_.children if c != v]
        else:
            nv_ = st.nodes[v]
            nv_.children = [u] + [c for c in nv_.children if c != u]
        return new_s

    def evolve_two_site(self, u, v, dt, exp_factor, tol, maxdim, svd, hermitian: bool = True) -> np.ndarray:
        """Two-site update of (u, v) with u the orthogonality centre: merge,
        Krylov exponential of the pair's H_eff, truncated SVD split, centre to
        v, environment E(u -> v) (``TwoSiteTDVP._update_two_site_nodes``,
        ``tdvp_algorithms/twositetdvp.py:89-125``). Returns the kept singular values."""
        info = self._two_site_info(u, v)
        x2 = self.ws.get("two_site", info["m"] * info["n"])
        mp = self.merge_plan(u, v)
        mp.run(0, x2.data_ptr())
        self.flops += mp.flops
        hp = self.heff2_plan(u, v)

        def apply(xp, yp):
            hp.run(xp, yp)
            self.flops += hp.flops
        self.local_exp(x2, apply, dt, exp_factor, tol, maxdim, hermitian, out=x2)
        self.check_device_status()
        s = self.svd_split(u, v, x2, svd)
        self.state.orthogonality_center_id = v
        self.update_env(u, v)
        return s

    # -- TEBD gates -------------------------------------------------------------------
    def apply_single_site_gate(self, nid, op: torch.Tensor):
        """t[nid][..., s'] = sum_s op[s', s] t[nid][..., s] (``absorb_into_open_legs``,
        ``core/ttn.py:929-964``)."""
        shape = self.shape(nid)
        n = len(shape) - 1
        cb = ChainBuilder(self.ws)
        T = Operand.contiguous(("fixed", self.t[nid]), [f"a{k}" for k in range(n)] + ["s"], shape)
        G = Operand.contiguous(("fixed", op), ["t", "s"], list(op.shape))
        out = Operand.contiguous(("ws", "gate_out"), [f"a{k}" for k in range(n)] + ["t"], shape)
        cb.sizes["gate_out"] = out.numel()
        cb.contract(T, G, ["s"], out=out)
        p = cb.plan()
        p.run()
        self.flops += p.flops
        self.t[nid].view(-1).copy_(self.ws.bufs["gate_out"][:self.t[nid].numel()])
        self._touch(nid)

    def apply_two_site_gate(self, u, v, op: torch.Tensor, svd) -> np.ndarray:
        """A two-site gate (legs out_u, out_v, in_u, in_v) on neighbours u, v:
        merge, apply, truncated SVD split with the singular values moved into v
        (``TEBD._apply_one_trotter_step_two_site``, ``time_evolution/tebd.py:103-125``).
        FP64 throughout (one contraction per gate). Returns the kept singular values."""
        info = self._two_site_info(u, v)
        x2 = self.ws.get("two_site", info["m"] * info["n"])
        mp = self.merge_plan(u, v)
        mp.run(0, x2.data_ptr())
        self.flops += mp.flops
        y = self.ws.get("two_site_gate", info["m"] * info["n"])
        cb = ChainBuilder(self.ws)
        X = Operand.contiguous(("fixed", x2), info["labels"], info["dims"])
        G = Operand.contiguous(("fixed", op), ["tu", "tv", "su", "sv"], list(op.shape))
        out_labels = [{"su": "tu", "sv": "tv"}.get(l, l) for l in info["labels"]]
        cb.contract(X, G, ["su", "sv"], out=Operand.contiguous(("fixed", y), out_labels, info["dims"]))
        p = cb.plan()
        p.run()
        self.flops += p.flops
        return self.svd_split(u, v, y, svd)

    def normalise_center(self) -> float:
        """Divide the orthogonality centre by its norm (``TTNS.normalise``,
        ``ttns/ttns.py:105-125``); returns the old norm."""
        c = self.state.orthogonality_center_id
        lib = _lib.load()
        t = self.t[c]
        part = self.ws.get("kry_part", int(lib.ptn_krylov_partials(t.numel())) + 8)
        scal = self.ws.get("kry_scal", 8, torch.float64)
        check(lib.ptn_dznrm2(t.data_ptr(), t.numel(), scal.data_ptr(), part.data_ptr(), _stream_ptr()), "dznrm2")
        check(lib.ptn_zscal_inv(t.data_ptr(), scal.data_ptr(), t.data_ptr(), t.numel(), _stream_ptr()), "zscal")
        self._touch(c)
        return float(scal[0].item())

    def canonical_form(self, center):
        """``canonical_form`` (``core/canonical_form.py:162-208``)."""
        st = self.state
        dist = st.distance_to_node(center)
        maxd = max(dist.values()) if dist else 0
        for d in range(maxd, 0, -1):
            for nid in [x for x in dist if dist[x] == d]:
                target = min(st.nodes[nid].neighbouring_nodes(), key=lambda x: dist[x])
                # complex128 here: before normalisation the state's norm can be far
                # outside the BF16/FP32 range (1e-55 for 61 unit-norm random tensors)
                self.move_orth_one_hop(nid, target, precise=True)
        st.orthogonality_center_id = center

    # -- observables ------------------------------------------------------------------
    def center_energy(self) -> float:
        """<psi|H|psi> / <psi|psi> from the orthogonality centre and the cached
        environments pointing to it (valid whenever those are current, as after
        every one-site TDVP time step): one complex128 H_eff application and
        two dot products, instead of a contraction of the whole network."""
        c = self.state.orthogonality_center_id
        x = self.t[c]
        y = self.ws.get("energy_y", x.numel())
        self.heff_plan(c, fp64=True).run(x.data_ptr(), y.data_ptr())
        lib = _lib.load()
        n = x.numel()
        part = self.ws.get("kry_part", int(lib.ptn_krylov_partials(n)) * 2 + 8)
        h = self.ws.get("energy_h", 2)
        check(lib.ptn_zdot_multi(x.data_ptr(), n, 1, y.data_ptr(), n, h[0:].data_ptr(), 0, part.data_ptr(),
                                 _stream_ptr()), "zdot_multi")
        check(lib.ptn_zdot_multi(x.data_ptr(), n, 1, x.data_ptr(), n, h[1:].data_ptr(), 0, part.data_ptr(),
                                 _stream_ptr()), "zdot_multi")
        v = h.cpu().numpy()
        return float(v[0].real / v[1].real)

    def overlap(self, other: "DeviceNetwork") -> complex:
        """<self|other> for two states on the same tree, bond dimensions free to
        differ (``contract_two_ttns``, ``contractions/state_state_contraction.py:29-66``).
        Each environment has legs (other's bond, self's bond)."""
        st = self.state
        if other.nbrs(st.root_id) != self.nbrs(st.root_id):
            raise ValueError("the two states must share the tree and its leg layout")

        def rec(nid, toward):
            ks, bs = other.shape(nid), self.shape(nid)
            if ks[-1] != bs[-1]:
                raise ValueError(f"physical dimensions of {nid} differ")
            n = len(bs) - 1
            nb = self.nbrs(nid)
            cb = ChainBuilder(self.ws)
            T = Operand.contiguous(("fixed", other.t[nid]), [f"a{k}" for k in range(n)] + ["s"], ks)
            for k, x in enumerate(nb):
                if x == toward:
                    continue
                sub = rec(x, nid)
                T = cb.contract(T, Operand.contiguous(("fixed", sub), [f"a{k}", f"c{k}"], list(sub.shape)),
                                [f"a{k}"])
            B = Operand.contiguous(("fixed", self.t[nid]),
                                   [f"c{k}" if nb[k] != toward else "z" for k in range(n)] + ["s"], bs)
            if toward is None:
                res = torch.zeros((1,), dtype=CDT, device=self.device)
                cb.contract(T, B, [f"c{k}" for k in range(n)] + ["s"], out=Operand(("fixed", res), [], [], []),
                            conj_b=True)
            else:
                k0 = nb.index(toward)
                res = torch.zeros((ks[k0], bs[k0]), dtype=CDT, device=self.device)
                cb.contract(T, B, [f"c{k}" for k in range(n) if k != k0] + ["s"],
                            out=Operand.contiguous(("fixed", res), [f"a{k0}", "z"], [ks[k0], bs[k0]]), conj_b=True)
            cb.plan().run()
            return res
        return complex(rec(st.root_id, None).cpu().numpy()[0])


    def expect_ttno(self, ttno) -> complex:
        """<psi| O |psi> for a TTNO on the same tree (``TTNS.operator_expectation_value``,
        ``ttns/ttns.py:278-297`` -> ``expectation_value``,
        ``contractions/state_operator_contraction.py:26-74``): a second network
        over the same device tensors (no copies) holds O and its own
        environments; all of them point to the root, whose H_eff applied to the
        root tensor is contracted with its conjugate. That network (its plans and
        environment buffers) is kept per operator while the site tensors keep
        their shapes and storage; each call copies the operator's tensors in and
        recomputes the environments."""
        sig = tuple((nid, tuple(t.shape), t.data_ptr()) for nid, t in self.t.items())
        ent = self._ttno_nets.get(id(ttno))
        if ent is not None and ent[0] is ttno and ent[1] == sig:
            other = ent[2]
            other.refresh_hamiltonian(ttno)
        else:
            if len(self._ttno_nets) >= 8:
                self._ttno_nets.pop(next(iter(self._ttno_nets)))
            other = DeviceNetwork(self.state, ttno, device=self.device, precision="plain")
            self._ttno_nets[id(ttno)] = (ttno, sig, other)
        root = self.state.root_id
        other.init_cache_but_one(root)
        x = self.t[root]
        y = torch.empty_like(x)
        other.heff_plan(root).run(x.data_ptr(), y.data_ptr())
        lib = _lib.load()
        n = x.numel()
        part = self.ws.get("kry_part", int(lib.ptn_krylov_partials(n)) * 2 + 8)
        h = self.ws.get("expect_h", 1)
        check(lib.ptn_zdot_multi(x.data_ptr(), n, 1, y.data_ptr(), n, h.data_ptr(), 0, part.data_ptr(),
                                 _stream_ptr()), "zdot_multi")
        return complex(h.cpu().numpy()[0])

    def expect_local(self, ops: dict) -> complex:
        """<psi| prod_i O_i |psi> for single-site operators
        (``TTNS.tensor_product_expectation_value``, ``ttns/ttns.py:240-264``);
        ``{}`` gives <psi|psi>. One entry of ``expect_many``."""
        return complex(self.expect_many([ops])[0])

    OBS_PLANS_KEPT = 16           # observable plans cached per network (operator layouts)

    def expect_many(self, ops_list) -> np.ndarray:
        """<psi| prod_i O_i |psi> for a list of products of one-site operators
        (each a dict node -> d x d matrix acting on the physical leg; ``{}`` is
        <psi|psi>), in one pass over the tree: one launch sequence, one copy of
        the operator matrices to the device and one copy of the values back.

        The reference evaluates each product separately as a deep copy, an
        operator application and a contraction of the whole network
        (``ttns/ttns.py:240-264``, ``contractions/state_state_contraction.py:29-66``,
        called per operator by ``time_evolution/ttn_time_evolution.py:181-197``).
        Here the pass computes norm environments N(u -> v) (the part of the
        tree on u's side of the edge contracted with its conjugate; legs
        (ket, bra)) toward the root for every edge and away from it on the
        paths to the operators' nodes. A one-site product then needs only the
        reduced density matrix of its node, rho[s, t] = psi[.., s] conj(psi[.., t])
        with every neighbour's environment, and Tr(O rho); rho is computed once
        per node however many operators act there. A product on several nodes
        contracts only the subtrees that hold its factors and takes the
        environments for the rest. The values are the reference's up to the
        order of the floating-point sums.

        The plan is cached per operator layout (the nodes of each product) and
        kept while no site tensor changes shape or storage, so repeated
        measurements (the ``run`` loop) reuse it and only copy the matrices."""
        ops_list = [dict(op) for op in ops_list]
        if not ops_list:
            return np.zeros((0,), dtype=np.complex128)
        mats = []
        for op in ops_list:
            for nid, m in op.items():
                if nid not in self.t:
                    raise KeyError(f"no node {nid!r} in the state")
                m = np.asarray(m.detach().cpu().numpy() if isinstance(m, torch.Tensor) else m,
                               dtype=np.complex128)
                d = self.t[nid].shape[-1]
                if m.shape != (d, d):
                    raise ValueError(f"operator on {nid} has shape {m.shape}, the node's physical "
                                     f"dimension is {d}")
                mats.append(m.reshape(-1))
        key = tuple(tuple(op) for op in ops_list)
        sig = tuple((nid, tuple(t.shape), t.data_ptr()) for nid, t in self.t.items())
        if self._obs_sig != sig:
            self._obs_sig = sig
            self._obs_plans = {}
        rec = self._obs_plans.get(key)
        if rec is None:
            if len(self._obs_plans) >= self.OBS_PLANS_KEPT:
                # each plan holds its own norm environments (chi^2 per edge)
                self._obs_plans.pop(next(iter(self._obs_plans)))
            rec = self._obs_plans[key] = self._observable_plan(key)
        plan, opbuf, vals = rec
        if mats:
            opbuf.copy_(torch.from_numpy(np.concatenate(mats)))
        plan.run()
        return vals.cpu().numpy().copy()      # the values buffer is the plan's

    def _observable_plan(self, layout):
        """(plan, operator buffer, values) for ``expect_many`` on products
        acting on the nodes ``layout[i]``."""
        st = self.state
        root = st.root_id
        cb = ChainBuilder(self.ws)
        hold = []
        nenv = {}
        dev = self.device

        def buf(shape):
            t = torch.zeros(shape, dtype=CDT, device=dev)
            hold.append(t)
            return t

        def parent(nid):
            return st.nodes[nid].parent

        def node_step(nid, toward, envs, op=None, rdm=None, out=None):
            """psi[nid] (times ``op`` on the physical leg) with the environments
            ``envs`` (neighbour index -> (chi, chi) tensor, legs (ket, bra)) and
            conj(psi[nid]); the open leg is the bond to ``toward``, or the
            physical pair into ``rdm``, or none (a scalar into ``out``)."""
            shape = self.shape(nid)
            n = len(shape) - 1
            nb = self.nbrs(nid)
            T = Operand.contiguous(("fixed", self.t[nid]), [f"a{k}" for k in range(n)] + ["s"], shape)
            if op is not None:
                T = cb.contract(T, Operand.contiguous(("fixed", op), ["t", "s"], list(op.shape)), ["s"])
                T = Operand(T.ref, ["s" if l == "t" else l for l in T.labels], T.dims, T.strides)
            for k in sorted(envs):
                E = envs[k]
                T = cb.contract(T, Operand.contiguous(("fixed", E), [f"a{k}", f"c{k}"], list(E.shape)),
                                [f"a{k}"])
            phys = "t" if rdm is not None else "s"
            B = Operand.contiguous(("fixed", self.t[nid]),
                                   [f"c{k}" if nb[k] != toward else "z" for k in range(n)] + [phys], shape)
            closed = [f"c{k}" for k in range(n) if nb[k] != toward]
            if rdm is not None:
                d = shape[-1]
                cb.contract(T, B, closed, out=Operand.contiguous(("fixed", rdm), ["s", "t"], [d, d]),
                            conj_b=True)
            elif toward is None:
                cb.contract(T, B, closed + ["s"], out=Operand(("fixed", out), [], [], []), conj_b=True)
            else:
                k0 = nb.index(toward)
                chi = shape[k0]
                cb.contract(T, B, closed + ["s"], out=Operand.contiguous(("fixed", out), [f"a{k0}", "z"],
                                                                          [chi, chi]), conj_b=True)

        def env(u, v):
            """N(u -> v), built on first use (toward the root from the
            children's, away from it from the parent's and the siblings')."""
            if (u, v) in nenv:
                return nenv[(u, v)]
            nb = self.nbrs(u)
            envs = {k: env(x, u) for k, x in enumerate(nb) if x != v}
            E = buf((self.shape(u)[nb.index(v)],) * 2)
            node_step(u, v, envs, out=E)
            nenv[(u, v)] = E
            return E

        # every environment toward the root, leaves first
        post = []

        def walk(nid):
            for c in st.nodes[nid].phys_children:
                walk(c)
            post.append(nid)
        walk(root)
        for nid in post:
            if nid != root:
                env(nid, parent(nid))

        below = {}             # node -> the nodes of its subtree
        for nid in post:
            s = {nid}
            for c in st.nodes[nid].phys_children:
                s |= below[c]
            below[nid] = s

        total = sum(self.t[nid].shape[-1] ** 2 for op in layout for nid in op)
        opbuf = buf((max(total, 1),))
        vals = buf((len(layout),))
        rdms = {}
        off = 0
        for i, nodes in enumerate(layout):
            mats = {}
            for nid in nodes:
                d = self.t[nid].shape[-1]
                mats[nid] = opbuf[off:off + d * d].view(d, d)
                off += d * d
            out = vals[i:i + 1]
            hold.append(out)
            if len(nodes) == 0:
                nb = self.nbrs(root)
                node_step(root, None, {k: env(x, root) for k, x in enumerate(nb)}, out=out)
            elif len(nodes) == 1:
                nid = nodes[0]
                if nid not in rdms:
                    d = self.t[nid].shape[-1]
                    rdms[nid] = buf((d, d))
                    nb = self.nbrs(nid)
                    node_step(nid, None, {k: env(x, nid) for k, x in enumerate(nb)}, rdm=rdms[nid])
                d = self.t[nid].shape[-1]
                cb.contract(Operand.contiguous(("fixed", rdms[nid]), ["s", "t"], [d, d]),
                            Operand.contiguous(("fixed", mats[nid]), ["t", "s"], [d, d]), ["s", "t"],
                            out=Operand(("fixed", out), [], [], []))
            else:
                sites = set(nodes)

                def rec(nid, toward, dst):
                    nb = self.nbrs(nid)
                    envs = {}
                    for k, x in enumerate(nb):
                        if x == toward:
                            continue
                        if below[x] & sites:
                            sub = buf((self.shape(x)[self.nbrs(x).index(nid)],) * 2)
                            rec(x, nid, sub)
                            envs[k] = sub
                        else:
                            envs[k] = env(x, nid)
                    node_step(nid, toward, envs, op=mats.get(nid), out=dst)
                rec(root, None, out)
        plan = cb.plan()
        plan._hold = hold
        return plan, opbuf, vals
