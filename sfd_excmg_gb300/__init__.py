"""sfd_excmg_gb300 -- GB300-native forward solver for SFD_EXCMG-style 3-D MT modelling.

The compute path is the native library ``_lib/libsfdx.so`` (hand-written
CUDA for sm_103a behind the C ABI in ``include/sfdx.h``); this package is a
thin ctypes face over it plus model I/O and synthetic-model generators.
"""
from . import capi
from .capi import FP64, MIXED, QUIRKS_REFERENCE, Opts, SfdxError
from .model import Model
from .solver import (Plan, apply_operator, build_rhs, fwd_solve, grad_correct, impedance, impedance_topo, krylov_solve,
                     mesh_coarsen,
                     mt1d, precond_apply, vcycle_apply, prolongate, receiver_fields, solve_batch, write_ccv, write_res,
                     impedance_misfit)

__all__ = [
    "capi", "Opts", "SfdxError", "FP64", "MIXED", "QUIRKS_REFERENCE", "Model", "Plan", "fwd_solve", "impedance",
    "impedance_topo",
    "receiver_fields",
    "mt1d", "apply_operator", "build_rhs", "precond_apply", "vcycle_apply", "mesh_coarsen", "prolongate", "krylov_solve",
    "grad_correct", "solve_batch", "write_res", "write_ccv", "impedance_misfit", "sigma_misfit", "log_sigma_misfit",
]


def __getattr__(name):
    # the autograd functions import torch; load them on first use
    if name in ("sigma_misfit", "log_sigma_misfit"):
        from . import adjoint
        return getattr(adjoint, name)
    raise AttributeError(name)


def build(verbose: bool = False) -> str:
    """Compile the native library in-tree (sm_103a) and return its path."""
    from . import _build
    return _build.build(verbose=verbose)
