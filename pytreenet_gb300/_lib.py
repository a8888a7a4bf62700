"""ctypes binding of libptn_gb300.so (the C ABI declared in include/ptn_gb300.h).

The library is loaded on first use. There is no CPU fallback: if the library
is missing or CUDA is unavailable, every engine call raises.
"""
from __future__ import annotations

import ctypes
import os

from .build import LIB

MAX_MODES = 8

PTN_OK = 0
_STATUS = {
    1: "invalid argument (shape, stride or null pointer)",
    2: "CUDA launch/runtime error",
    3: "non-finite value in input",
    4: "Krylov breakdown",
    5: "decomposition did not converge",
    6: "configuration outside the kernel's limits",
    7: "a bounded device-side wait ran out",
}


class PtnError(RuntimeError):
    """Error status returned by libptn_gb300."""

    def __init__(self, status: int, what: str):
        super().__init__(f"{what}: ptn status {status} ({_STATUS.get(status, 'unknown')})")
        self.status = status


class PtnArgumentError(PtnError, ValueError):
    pass


class Modes(ctypes.Structure):
    _fields_ = [("n", ctypes.c_int32), ("pad_", ctypes.c_int32),
                ("dim", ctypes.c_int64 * MAX_MODES),
                ("stride_a", ctypes.c_int64 * MAX_MODES),
                ("stride_b", ctypes.c_int64 * MAX_MODES),
                ("stride_c", ctypes.c_int64 * MAX_MODES)]


class ContractDesc(ctypes.Structure):
    _fields_ = [("A", ctypes.c_void_p), ("B", ctypes.c_void_p), ("C", ctypes.c_void_p),
                ("alpha_re", ctypes.c_double), ("alpha_im", ctypes.c_double),
                ("beta_re", ctypes.c_double), ("beta_im", ctypes.c_double),
                ("conj_a", ctypes.c_int32), ("conj_b", ctypes.c_int32),
                ("m", Modes), ("n", Modes), ("k", Modes)]


class CgemmDesc(ctypes.Structure):
    _fields_ = [("A", ctypes.c_void_p), ("lda", ctypes.c_int64), ("a_plane", ctypes.c_int64),
                ("M", ctypes.c_int64), ("K", ctypes.c_int64), ("Bx", ctypes.c_void_p),
                ("ldb", ctypes.c_int64), ("N", ctypes.c_int64), ("out_kind", ctypes.c_int32),
                ("levels", ctypes.c_int32), ("C", ctypes.c_void_p), ("c_plane", ctypes.c_int64),
                ("m_out", Modes), ("n_out", Modes), ("status", ctypes.c_void_p),
                ("partial", ctypes.c_void_p), ("partial_bytes", ctypes.c_int64)]


class ConvertDesc(ctypes.Structure):
    _fields_ = [("src", ctypes.c_void_p), ("dst", ctypes.c_void_p), ("ld", ctypes.c_int64),
                ("plane", ctypes.c_int64), ("conj", ctypes.c_int32), ("levels", ctypes.c_int32),
                ("rows", Modes), ("cols", Modes)]


class SvdDesc(ctypes.Structure):
    _fields_ = [("A", ctypes.c_void_p), ("m", ctypes.c_int64), ("n", ctypes.c_int64),
                ("row_stride", ctypes.c_int64), ("col_stride", ctypes.c_int64),
                ("U", ctypes.c_void_p), ("ldu", ctypes.c_int64), ("S", ctypes.c_void_p),
                ("V", ctypes.c_void_p), ("ldv", ctypes.c_int64), ("work", ctypes.c_void_p),
                ("status", ctypes.c_void_p)]


class PermuteDesc(ctypes.Structure):
    _fields_ = [("src", ctypes.c_void_p), ("dst", ctypes.c_void_p), ("n", ctypes.c_int32),
                ("conj", ctypes.c_int32), ("dim", ctypes.c_int64 * MAX_MODES),
                ("stride_src", ctypes.c_int64 * MAX_MODES), ("stride_dst", ctypes.c_int64 * MAX_MODES),
                ("scale", ctypes.c_void_p), ("scale_mode", ctypes.c_int32), ("pad_", ctypes.c_int32)]


class ExecOp(ctypes.Structure):
    _fields_ = [("kind", ctypes.c_int32), ("a", ctypes.c_int32), ("b", ctypes.c_int32),
                ("c", ctypes.c_int32), ("d", ctypes.c_int32), ("pad_", ctypes.c_int32),
                ("desc", ctypes.c_void_p)]


OP_ZCONTRACT, OP_CGEMM, OP_TO_PLANES, OP_EXPAND_B = 0, 1, 2, 3

_P = ctypes.c_void_p
_I64 = ctypes.c_int64
_I32 = ctypes.c_int32
SIGNATURES = {
    "ptn_zcontract": (ctypes.c_int, [ctypes.POINTER(ContractDesc), _P]),
    "ptn_zcontract_splits": (_I64, [_I64, _I64, ctypes.POINTER(ctypes.c_int64)]),
    "ptn_krylov_partials": (_I64, [_I64]),
    "ptn_zdot_multi": (ctypes.c_int, [_P, _I64, _I32, _P, _I64, _P, _I32, _P, _P]),
    "ptn_zaxpy_multi": (ctypes.c_int, [_P, _I64, _I32, _P, _P, _I64, _P]),
    "ptn_dznrm2": (ctypes.c_int, [_P, _I64, _P, _P, _P]),
    "ptn_zscal_inv": (ctypes.c_int, [_P, _P, _P, _I64, _P]),
    "ptn_zcombine": (ctypes.c_int, [_P, _I64, _I32, _P, _P, _I64, _P]),
    "ptn_zscal_ratio": (ctypes.c_int, [_P, _P, _P, _P, _I64, _P]),
    "ptn_zqr_work_bytes": (_I64, [_I64, _I64]),
    "ptn_zqr_keep": (ctypes.c_int, [_P, _P, _I64, _I64, _I64, _P, _P, _P]),
    "ptn_zqr_path": (ctypes.c_int, [_I64, _I64]),
    "ptn_zqr_keep_steps": (ctypes.c_int, [_P, _P, _I64, _I64, _I64, _P, _P, _P]),
    "ptn_check_finite": (ctypes.c_int, [_P, _I64, _P, _P]),
    "ptn_launch_counter": (ctypes.c_ulonglong, []),
    "ptn_stream_synchronize": (ctypes.c_int, [ctypes.c_void_p]),
    "ptn_zqr_noalloc_max_bytes": (_I64, []),
    "ptn_zqr_keep_noalloc": (ctypes.c_int, [_P, _P, _I64, _I64, _I64, _P, _P]),
    "ptn_zqr_keep_rows": (ctypes.c_int, [_P, _P, _I64, _I64, _I64, _I64, _P, _P, _P]),
    "ptn_znonzero_rows": (ctypes.c_int, [_P, _P, _I64, _I64, _I64, _P, _P]),
    "ptn_zchol_work_bytes": (_I64, [_I64]),
    "ptn_zchol_max_k": (_I64, []),
    "ptn_zchol_upper": (ctypes.c_int, [_P, _I64, _I64, _P, _P, ctypes.c_double, _I32, ctypes.c_double, _P, _P,
                                       _P]),
    "ptn_ztri_mul_upper": (ctypes.c_int, [_P, _P, _P, _I64, _P]),
    "ptn_ztri_inv_newton": (ctypes.c_int, [_P, _P, _P, _P, _I64, _P]),
    "ptn_cgemm_bf16x3": (ctypes.c_int, [ctypes.POINTER(CgemmDesc), _P]),
    "ptn_cgemm_smem_bytes": (ctypes.c_int, [_I32]),
    "ptn_cgemm_partial_bytes": (_I64, [_I64, _I64, _I64]),
    "ptn_to_planes": (ctypes.c_int, [ctypes.POINTER(ConvertDesc), _P]),
    "ptn_expand_b": (ctypes.c_int, [ctypes.POINTER(ConvertDesc), _P]),
    "ptn_zsvd_work_bytes": (_I64, [_I64, _I64]),
    "ptn_zsvd_jacobi": (ctypes.c_int, [ctypes.POINTER(SvdDesc), _P]),
    "ptn_zpermute": (ctypes.c_int, [ctypes.POINTER(PermuteDesc), _P]),
    "ptn_exec_ops": (ctypes.c_int, [ctypes.POINTER(ExecOp), _I32, ctypes.POINTER(ctypes.c_void_p), _I32, _P]),
    "ptn_krylov_gs_step": (ctypes.c_int, [_P, _I64, _I32, _P, _I64, _P, _P, _P, _P, _P]),
}

_lib = None


def library_path() -> str:
    return LIB


def load():
    """Load the CUDA library (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB):
        raise RuntimeError(
            f"{LIB} is missing: build it with `python -m pytreenet_gb300.build` "
            "(the engine has no CPU fallback)")
    lib = ctypes.CDLL(LIB)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def check(status: int, what: str):
    if status != PTN_OK:
        if status == 1:
            raise PtnArgumentError(status, what)
        raise PtnError(status, what)
