"""ctypes binding of include/lgt_ed.h (liblgted.so).

The library is built in-tree by ``lgt_gb300.build``.  There is no fallback:
if the shared library is missing or fails to load, importing this module
raises, and so does every entry point of the package.
"""
from __future__ import annotations

import ctypes
import os

from . import build as _build

LGT_OK = 0
LGT_ERR_ARG = 1
LGT_ERR_SECTOR = 2
LGT_ERR_KEYWIDTH = 3
LGT_ERR_MEMORY = 4
LGT_ERR_CUDA = 5
LGT_ERR_NOCONV = 6
LGT_ERR_DEVICE = 7
LGT_ERR_NOTFOUND = 8
LGT_ERR_UNSUPPORTED = 9

LGT_MODEL_REF = 0
LGT_MODEL_JW = 1
LGT_MODEL_PLAQ = 2
LGT_MODEL_PJW = 3

LGT_FP64 = 0
LGT_FP32 = 1
LGT_FP32_MIXED = 2

LGT_SOLVER_AUTO = 0
LGT_SOLVER_PANEL = 1
LGT_SOLVER_CTA = 2

LGT_DEVICE_PTRS = 1
LGT_ASYNC = 2
LGT_GENERIC_KERNELS = 4
LGT_ROW_ORDER = 8

# every symbol include/lgt_ed.h declares
EXPORTS = (
    "lgt_krylov_defaults", "lgt_last_error", "lgt_version",
    "lgt_basis_create", "lgt_basis_dim", "lgt_basis_keys", "lgt_basis_states",
    "lgt_basis_lookup", "lgt_basis_rank", "lgt_basis_destroy", "lgt_basis_set_stream",
    "lgt_launch_count",
    "lgt_ham_create", "lgt_ham_set_couplings", "lgt_ham_nnz", "lgt_ham_export_csr",
    "lgt_ham_row_order",
    "lgt_matvec", "lgt_ground_state", "lgt_ground_state_observe", "lgt_ground_state_batch",
    "lgt_expm_steps",
    "lgt_expm_steps_grids", "lgt_observe",
    "lgt_observe_noalloc", "lgt_energy", "lgt_autotune", "lgt_ham_destroy",
)


class Tuning(ctypes.Structure):
    _fields_ = [
        ("hpsi_kernel", ctypes.c_int32),
        ("reduce_blocks", ctypes.c_int32),
        ("hpsi_ms", ctypes.c_double),
        ("reduce_ms", ctypes.c_double),
        ("measured", ctypes.c_int32),
    ]


class KrylovOpts(ctypes.Structure):
    _fields_ = [
        ("krylovdim", ctypes.c_int32),
        ("maxiter", ctypes.c_int32),
        ("tol", ctypes.c_double),
        ("precision", ctypes.c_int32),
        ("reorth_passes", ctypes.c_int32),
        ("check_every", ctypes.c_int32),
        ("refine_steps", ctypes.c_int32),
        ("seed", ctypes.c_uint64),
        ("use_graph", ctypes.c_int32),
        ("start_given", ctypes.c_int32),
        ("solver", ctypes.c_int32),
    ]


class Info(ctypes.Structure):
    _fields_ = [
        ("matvecs", ctypes.c_int64),
        ("restarts", ctypes.c_int32),
        ("converged", ctypes.c_int32),
        ("max_residual", ctypes.c_double),
        ("seconds", ctypes.c_double),
    ]


class Obs(ctypes.Structure):
    _fields_ = [
        ("t", ctypes.c_double),
        ("nf_mean", ctypes.c_double),
        ("nf_even", ctypes.c_double),
        ("nf_odd", ctypes.c_double),
        ("E2_mean", ctypes.c_double),
        ("plaq_mean", ctypes.c_double),
        ("n_stag", ctypes.c_double),
        ("norm2", ctypes.c_double),
    ]


class LgtError(RuntimeError):
    """A non-zero lgt_status; ``code`` holds it."""

    def __init__(self, code, msg):
        super().__init__("lgt error %d: %s" % (code, msg))
        self.code = code


class NotConverged(LgtError):
    pass


_lib = None


def library_path() -> str:
    return _build.LIB


def load(build_if_missing: bool = True):
    """Load liblgted.so (building it first if it is missing or stale and a
    CUDA toolkit is available)."""
    global _lib
    if _lib is not None:
        return _lib
    path = _build.LIB
    if build_if_missing and not _build.up_to_date():
        _build.build()
    if not os.path.exists(path):
        raise OSError("liblgted.so not found at %s; run lgt_gb300.build.build()" % path)
    L = ctypes.CDLL(path)
    vp, i32, i64, u32, dbl = (ctypes.c_void_p, ctypes.c_int32, ctypes.c_int64, ctypes.c_uint32,
                              ctypes.c_double)
    pvp = ctypes.POINTER(ctypes.c_void_p)
    sig = {
        "lgt_krylov_defaults": (None, [ctypes.POINTER(KrylovOpts), ctypes.c_int]),
        "lgt_last_error": (ctypes.c_char_p, []),
        "lgt_version": (ctypes.c_char_p, []),
        "lgt_basis_create": (i32, [i32, i32, i32, vp, i32, pvp]),
        "lgt_basis_dim": (i32, [vp, ctypes.POINTER(ctypes.c_int64)]),
        "lgt_basis_keys": (i32, [vp, i64, i64, vp, vp]),
        "lgt_basis_states": (i32, [vp, i64, i64, vp, vp, vp]),
        "lgt_basis_lookup": (i32, [vp, vp, i64, vp]),
        "lgt_basis_rank": (i32, [vp, vp, i64, vp]),
        "lgt_basis_destroy": (None, [vp]),
        "lgt_basis_set_stream": (i32, [vp, vp]),
        "lgt_launch_count": (i32, [ctypes.POINTER(ctypes.c_uint64)]),
        "lgt_ham_create": (i32, [vp, i32, vp, vp, vp, u32, pvp]),
        "lgt_ham_set_couplings": (i32, [vp, vp, vp, vp]),
        "lgt_ham_nnz": (i32, [vp, ctypes.POINTER(ctypes.c_int64)]),
        "lgt_ham_export_csr": (i32, [vp, i32, vp, vp, vp]),
        "lgt_ham_row_order": (i32, [vp, vp]),
        "lgt_matvec": (i32, [vp, vp, vp, i32, i32, u32]),
        "lgt_ground_state": (i32, [vp, ctypes.POINTER(KrylovOpts), vp, vp, vp, u32,
                                   ctypes.POINTER(Info)]),
        "lgt_ground_state_observe": (i32, [vp, ctypes.POINTER(KrylovOpts), vp, vp, vp, u32,
                                           ctypes.POINTER(Info), vp, vp, vp, vp]),
        "lgt_ground_state_batch": (i32, [i32, vp, ctypes.POINTER(KrylovOpts), vp, vp, vp, u32,
                                         ctypes.POINTER(Info)]),
        "lgt_expm_steps": (i32, [vp, ctypes.POINTER(KrylovOpts), dbl, i32, vp, vp, vp, u32,
                                 ctypes.POINTER(Info)]),
        "lgt_expm_steps_grids": (i32, [vp, ctypes.POINTER(KrylovOpts), dbl, i32, vp, vp, vp, vp,
                                       vp, vp, u32, ctypes.POINTER(Info)]),
        "lgt_observe": (i32, [vp, vp, i32, i32, u32, dbl, vp, vp, vp, vp]),
        "lgt_observe_noalloc": (i32, [vp, vp, i32, i32, dbl, vp, vp, vp, vp]),
        "lgt_energy": (i32, [vp, vp, i32, u32, vp]),
        "lgt_autotune": (i32, [vp, i32, i32, ctypes.POINTER(Tuning)]),
        "lgt_ham_destroy": (None, [vp]),
    }
    for name in EXPORTS:
        fn = getattr(L, name)
        fn.restype, fn.argtypes = sig[name]
    _lib = L
    return L


def check(code: int):
    """Raise the matching exception for a non-zero lgt_status."""
    if code == LGT_OK:
        return
    msg = (_lib.lgt_last_error() or b"").decode(errors="replace")
    if code == LGT_ERR_NOCONV:
        raise NotConverged(code, msg)
    if code in (LGT_ERR_SECTOR, LGT_ERR_ARG, LGT_ERR_KEYWIDTH, LGT_ERR_UNSUPPORTED):
        raise ValueError("lgt error %d: %s" % (code, msg))
    raise LgtError(code, msg)


def launch_count() -> int:
    """Kernels launched by the library in this process so far."""
    n = ctypes.c_uint64()
    check(load().lgt_launch_count(ctypes.byref(n)))
    return int(n.value)


def defaults(for_exponentiate: bool = False) -> KrylovOpts:
    o = KrylovOpts()
    load().lgt_krylov_defaults(ctypes.byref(o), 1 if for_exponentiate else 0)
    return o
