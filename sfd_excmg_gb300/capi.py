"""ctypes binding of the C ABI declared in include/sfdx.h.

This is the same boundary a Fortran host binds through ISO_C_BINDING: plain
pointers and sizes, complex arrays as interleaved doubles.  Loading fails
loudly when the native library is missing -- there is no Python fallback.
"""
from __future__ import annotations

import ctypes
import os
import threading

import numpy as np

from . import _build

_LIB = None
_LOCK = threading.Lock()

c_double_p = ctypes.POINTER(ctypes.c_double)
c_int_p = ctypes.POINTER(ctypes.c_int)

SFDX_OK = 0
ERRORS = {
    1: "SFDX_ERR_ARG", 2: "SFDX_ERR_MESH", 3: "SFDX_ERR_CUDA", 4: "SFDX_ERR_NOCONV", 5: "SFDX_ERR_NAN",
    6: "SFDX_ERR_RECEIVER", 7: "SFDX_ERR_IO", 8: "SFDX_ERR_UNSUPPORTED", 9: "SFDX_ERR_TIMEOUT", 10: "SFDX_ERR_NOMEM",
}
QUIRK_COARSEN_SHIFT = 1
QUIRK_EXCMG_MIDPOINT = 2
QUIRK_RX_TRANSPOSE = 4
QUIRK_TOPO_PLANE = 8
QUIRKS_REFERENCE = 15
FP64 = 0
MIXED = 1


class SfdxError(RuntimeError):
    def __init__(self, code: int, where: str):
        self.code = code
        msg = lib().sfdx_strerror(code).decode() if _LIB is not None else ERRORS.get(code, "?")
        super().__init__(f"{where}: {ERRORS.get(code, code)} ({msg})")


class Opts(ctypes.Structure):
    """Mirror of ``struct sfdx_opts`` (include/sfdx.h)."""
    _fields_ = [
        ("level", ctypes.c_int), ("eps", ctypes.c_double), ("solver", ctypes.c_int), ("excmg", ctypes.c_int),
        ("precond", ctypes.c_int), ("div_cor", ctypes.c_int), ("corr_intv", ctypes.c_int),
        ("corr_tol", ctypes.c_double), ("ssor_omega", ctypes.c_double), ("sigma_air", ctypes.c_double),
        ("maxit_plain", ctypes.c_int), ("maxit_level", ctypes.c_int), ("precision", ctypes.c_int),
        ("quirks", ctypes.c_int), ("coarse_tol", ctypes.c_double), ("coarse_maxit", ctypes.c_int),
        ("reliable_every", ctypes.c_int),
        ("batch", ctypes.c_int), ("verbose", ctypes.c_int), ("use_graphs", ctypes.c_int),
    ]

    @classmethod
    def defaults(cls, **kw) -> "Opts":
        o = cls()
        lib().sfdx_default_opts(ctypes.byref(o))
        for k, v in kw.items():
            if k == "precond" and isinstance(v, str):
                v = ord(v)
            if not hasattr(o, k):
                raise AttributeError(f"unknown sfdx option {k!r}")
            setattr(o, k, v)
        return o


# name -> (restype, argtypes)
_PROTO = {
    "sfdx_default_opts": (None, [ctypes.c_void_p]),
    "sfdx_strerror": (ctypes.c_char_p, [ctypes.c_int]),
    "sfdx_version": (ctypes.c_int, []),
    "sfdx_launch_count": (ctypes.c_longlong, []),
    "sfdx_fwd_solve": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                      c_double_p, c_double_p, c_double_p, c_double_p, ctypes.c_int, c_double_p,
                                      c_double_p, c_int_p, c_double_p]),
    "sfdx_plan_create": (ctypes.c_int, [ctypes.POINTER(ctypes.c_void_p), ctypes.c_void_p, ctypes.c_int,
                                        ctypes.c_int, ctypes.c_int, ctypes.c_int, c_double_p, c_double_p,
                                        c_double_p, ctypes.c_int, c_double_p]),
    "sfdx_plan_solve": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p,
                                       ctypes.c_int, c_int_p, c_double_p]),
    "sfdx_plan_impedance": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, c_double_p, ctypes.c_int, c_double_p,
                                           c_double_p]),
    "sfdx_plan_misfit_grad": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, c_double_p, c_double_p, c_double_p,
                                             ctypes.c_double, c_double_p, c_double_p, c_double_p, ctypes.c_int,
                                             c_int_p, c_double_p]),
    "sfdx_plan_fields": (ctypes.c_void_p, [ctypes.c_void_p]),
    "sfdx_plan_solve_batch": (ctypes.c_int, [ctypes.c_int, ctypes.POINTER(ctypes.c_void_p),
                                             ctypes.POINTER(ctypes.c_void_p), ctypes.c_int,
                                             ctypes.POINTER(ctypes.c_void_p), ctypes.c_int,
                                             ctypes.POINTER(ctypes.c_void_p), ctypes.POINTER(ctypes.c_void_p), c_int_p]),
    "sfdx_plan_resolve": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_double, c_int_p,
                                         c_double_p]),
    "sfdx_plan_load": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int]),
    "sfdx_plan_device_bytes": (ctypes.c_longlong, [ctypes.c_void_p]),
    "sfdx_plan_destroy": (None, [ctypes.c_void_p]),
    "sfdx_plan_level_times": (ctypes.c_int, [ctypes.c_void_p, c_double_p, ctypes.c_int]),
    "sfdx_plan_level_fields": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, c_double_p]),
    "sfdx_plan_history": (ctypes.c_int, [ctypes.c_void_p, c_double_p, ctypes.c_int]),
    "sfdx_plan_set_stream": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p]),
    "sfdx_plan_kernel_time": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, c_double_p, c_double_p]),
    "sfdx_impedance": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, c_double_p,
                                      c_double_p, c_double_p, ctypes.c_int, c_double_p, c_double_p, ctypes.c_int,
                                      c_double_p, ctypes.c_int, ctypes.c_int, c_double_p, c_double_p]),
    "sfdx_impedance_topo": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, c_double_p,
                                           c_double_p, c_double_p, ctypes.c_int, c_double_p, c_double_p,
                                           ctypes.c_int, c_double_p, ctypes.c_int, ctypes.c_int, c_int_p,
                                           c_double_p, c_double_p, c_double_p]),
    "sfdx_impedance_misfit": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, c_double_p,
                                             c_double_p, c_double_p, ctypes.c_int, c_double_p, c_double_p,
                                             ctypes.c_int, c_double_p, ctypes.c_int, c_double_p, c_double_p,
                                             c_double_p, c_double_p]),
    "sfdx_mt1d": (ctypes.c_int, [ctypes.c_double, ctypes.c_int, c_double_p, c_double_p, c_double_p, c_double_p,
                                 c_double_p]),
    "sfdx_apply_operator": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, ctypes.c_int, c_double_p, c_double_p,
                                           c_double_p, c_double_p, ctypes.c_int, c_double_p, ctypes.c_int,
                                           c_double_p, c_double_p]),
    "sfdx_build_rhs": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, ctypes.c_int, c_double_p, c_double_p, c_double_p,
                                      c_double_p, ctypes.c_double, c_double_p, c_double_p, c_double_p]),
    "sfdx_vcycle_apply": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, c_double_p,
                                         c_double_p, c_double_p, c_double_p, ctypes.c_int, c_double_p, ctypes.c_int,
                                         ctypes.c_int, c_double_p, c_double_p]),
    "sfdx_precond_apply": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, ctypes.c_int, c_double_p, c_double_p,
                                          c_double_p, c_double_p, ctypes.c_int, c_double_p, ctypes.c_int,
                                          ctypes.c_int, c_double_p, c_double_p]),
    "sfdx_mesh_coarsen": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, ctypes.c_int, c_double_p, c_double_p,
                                         c_double_p, c_double_p, ctypes.c_int, ctypes.c_int, c_double_p, c_double_p,
                                         c_double_p, c_double_p]),
    "sfdx_prolongate": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, ctypes.c_int, c_double_p, c_double_p,
                                       c_double_p, ctypes.c_int, ctypes.c_int, c_double_p, c_double_p, c_double_p,
                                       ctypes.c_int]),
    "sfdx_krylov_solve": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int, c_double_p,
                                         c_double_p, c_double_p, c_double_p, ctypes.c_int, c_double_p, c_double_p,
                                         c_double_p, ctypes.c_double, ctypes.c_int, c_int_p, c_double_p, c_double_p]),
    "sfdx_div_correct": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, ctypes.c_int, c_double_p, c_double_p,
                                        c_double_p, c_double_p, ctypes.c_int, c_double_p, ctypes.c_double, c_int_p]),
    "sfdx_plan_autotune": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, c_int_p, c_int_p]),
    "sfdx_grad_correct": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, ctypes.c_int, c_double_p, c_double_p,
                                         c_double_p, c_double_p, ctypes.c_int, c_double_p, c_double_p, c_double_p,
                                         ctypes.c_double, ctypes.c_int, c_int_p]),
    "sfdx_residual_noalloc": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, ctypes.c_int, c_double_p, c_double_p,
                                             c_double_p, ctypes.c_void_p, ctypes.c_int, c_double_p, ctypes.c_void_p,
                                             ctypes.c_void_p, ctypes.c_void_p, c_double_p, ctypes.c_void_p]),
    "sfdx_read_sizes": (ctypes.c_int, [ctypes.c_char_p, c_int_p, c_int_p, c_int_p, c_int_p, c_int_p, c_int_p]),
    "sfdx_read_model": (ctypes.c_int, [ctypes.c_char_p, ctypes.c_void_p, c_int_p, c_double_p, c_int_p, c_int_p,
                                       c_double_p, c_double_p, c_double_p, c_double_p, c_double_p, c_double_p,
                                       c_int_p]),
    "sfdx_write_ccv": (ctypes.c_int, [ctypes.c_char_p, ctypes.c_double, ctypes.c_char_p, ctypes.c_char_p, ctypes.c_int,
                                      c_double_p, ctypes.c_int]),
    "sfdx_write_res": (ctypes.c_int, [ctypes.c_char_p, ctypes.c_int, c_double_p, ctypes.c_int, c_double_p,
                                      c_double_p]),
    "sfdx_receiver_fields": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, c_double_p,
                                            c_double_p, c_double_p, ctypes.c_int, c_double_p, c_double_p,
                                            ctypes.c_int, c_double_p, ctypes.c_int, c_double_p]),
    "sfdx_write_res_tipper": (ctypes.c_int, [ctypes.c_char_p, ctypes.c_int, c_double_p, ctypes.c_int, c_double_p,
                                             c_double_p, c_double_p]),
}


def library_path() -> str:
    return _build.LIB


def lib(build_if_missing: bool = True):
    """Load libsfdx.so (building it first if absent).  Raises if it cannot be built/loaded."""
    global _LIB
    with _LOCK:
        if _LIB is None:
            path = _build.LIB
            if not os.path.exists(path):
                if not build_if_missing:
                    raise RuntimeError(f"native library {path} is missing; run sfd_excmg_gb300._build.build()")
                _build.build()
            L = ctypes.CDLL(path)
            for name, (res, args) in _PROTO.items():
                fn = getattr(L, name)
                fn.restype = res
                fn.argtypes = args
            _LIB = L
    return _LIB


def check(code: int, where: str) -> None:
    if code != SFDX_OK:
        raise SfdxError(code, where)


def dptr(a: np.ndarray):
    if a.dtype != np.float64 or not a.flags.c_contiguous:
        raise TypeError(f"expected a C-contiguous float64 array, got {a.dtype}")
    return a.ctypes.data_as(c_double_p)


def zptr(a: np.ndarray):
    """Interleaved (re, im) view of a complex128 array as double*."""
    if a.dtype != np.complex128 or not a.flags.c_contiguous:
        raise TypeError(f"expected a C-contiguous complex128 array, got {a.dtype}")
    return a.ctypes.data_as(c_double_p)


def iptr(a: np.ndarray):
    if a.dtype != np.int32 or not a.flags.c_contiguous:
        raise TypeError(f"expected a C-contiguous int32 array, got {a.dtype}")
    return a.ctypes.data_as(c_int_p)
