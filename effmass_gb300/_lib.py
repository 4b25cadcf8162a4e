"""Loader of libhpsi_gb300.so (the CUDA library behind the C ABI).

There is no fallback: if the library is missing or cannot be loaded, every
entry point raises.  ``effmass_gb300.build.build()`` (or
``__graft_entry__.build()``) compiles it in-tree.
"""
from __future__ import annotations

import ctypes as C
import os

from . import abi

LIB_PATH = os.path.join(os.path.dirname(os.path.abspath(__file__)), "libhpsi_gb300.so")

# every entry point declared in include/hpsi_gb300.h
EXPORTS = ["hpsi_abi_version", "hpsi_ctx_create", "hpsi_ctx_destroy", "hpsi_set_kpoint", "hpsi_dim",
           "hpsi_apply", "hpsi_apply_energies", "hpsi_density", "hpsi_sternheimer", "hpsi_kp_sums", "hpsi_beta_table_length", "hpsi_beta_tables", "hpsi_gsphere", "hpsi_hessian_tables",
           "hpsi_set_hessian_tables", "hpsi_hess_apply", "hpsi_grad_apply", "hpsi_velocity_matrix", "hpsi_profile", "hpsi_profile_read",
           "hpsi_apply_noalloc", "hpsi_server_create", "hpsi_server_submit", "hpsi_server_wait",
           "hpsi_server_stats", "hpsi_server_destroy", "hpsi_server_last_error", "hpsi_batch_create",
           "hpsi_batch_buffers", "hpsi_batch_offset", "hpsi_batch_run", "hpsi_batch_apply", "hpsi_batch_info",
           "hpsi_batch_destroy", "hpsi_batch_last_error", "hpsi_selftest_convert", "hpsi_selftest_wait_limit",
           "hpsi_selftest_fft3d", "hpsi_selftest_kpoint_tables",
           "hpsi_last_error"]

_lib = None


class HpsiError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"{abi.STATUS_NAMES.get(status, status)}: {message}")
        self.status = status


def load():
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise RuntimeError(f"{LIB_PATH} is missing: build it with `python -m effmass_gb300.build` "
                           "(the H|psi> path has no CPU fallback)")
    L = C.CDLL(LIB_PATH)
    dp = C.POINTER(C.c_double)
    ctxp = C.c_void_p
    L.hpsi_abi_version.argtypes = []
    L.hpsi_abi_version.restype = C.c_int
    L.hpsi_ctx_create.argtypes = [C.POINTER(abi.HpsiSystem), C.POINTER(ctxp)]
    L.hpsi_ctx_destroy.argtypes = [ctxp]
    L.hpsi_set_kpoint.argtypes = [ctxp, C.c_int, C.POINTER(abi.HpsiKpoint)]
    L.hpsi_dim.argtypes = [ctxp, C.c_int]
    L.hpsi_apply.argtypes = [ctxp, C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_int, C.c_void_p]
    L.hpsi_apply_energies.argtypes = [ctxp, C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int,
                                      C.c_void_p]
    L.hpsi_density.argtypes = [ctxp, C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_void_p]
    L.hpsi_sternheimer.argtypes = [ctxp, C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_int, C.c_double, C.c_int,
                                   C.c_void_p, C.POINTER(C.c_int), dp, C.c_int, C.c_void_p]
    L.hpsi_beta_table_length.argtypes = [C.c_double, C.c_double]
    L.hpsi_beta_tables.argtypes = [C.c_int, C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_void_p, C.c_void_p,
                                   C.c_double, C.c_double, C.c_void_p, C.c_void_p, C.c_int, C.c_void_p]
    L.hpsi_gsphere.argtypes = [dp, dp, C.c_double, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.POINTER(C.c_int),
                               C.c_int, C.c_void_p]
    L.hpsi_hessian_tables.argtypes = [C.c_int, C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_void_p, C.c_void_p,
                                      C.c_double, C.c_double, C.c_void_p, C.c_int, C.c_void_p]
    L.hpsi_set_hessian_tables.argtypes = [ctxp, C.c_int, C.c_int, C.c_double, dp]
    L.hpsi_hess_apply.argtypes = [ctxp, C.c_int, C.c_int, C.c_void_p] + [C.c_void_p] * 6 + [C.c_int, C.c_void_p]
    L.hpsi_kp_sums.argtypes = [C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_double, C.c_void_p, C.c_void_p,
                               C.c_int, C.c_void_p]
    L.hpsi_grad_apply.argtypes = [ctxp, C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                  C.c_int, C.c_void_p]
    L.hpsi_velocity_matrix.argtypes = [ctxp, C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_int, C.c_void_p]
    L.hpsi_apply_noalloc.argtypes = [ctxp, C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_int, C.c_void_p]
    L.hpsi_profile.argtypes = [ctxp, C.c_int]
    L.hpsi_profile_read.argtypes = [ctxp, dp, C.POINTER(C.c_longlong)]
    L.hpsi_selftest_convert.argtypes = [dp, C.c_long] + [C.c_void_p] * 4
    L.hpsi_selftest_wait_limit.argtypes = [C.c_long]
    L.hpsi_selftest_fft3d.argtypes = [C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_int, C.c_int]
    L.hpsi_selftest_kpoint_tables.argtypes = [ctxp, C.c_int, C.c_void_p, C.c_void_p]
    L.hpsi_last_error.argtypes = [ctxp]
    L.hpsi_last_error.restype = C.c_char_p
    for name in EXPORTS:
        if not name.endswith("last_error"):
            getattr(L, name).restype = C.c_int
    if L.hpsi_abi_version() != 1:
        raise RuntimeError("libhpsi_gb300.so ABI version mismatch")
    _lib = L
    return L


def check(status: int, ctx=None):
    if status != 0:
        msg = load().hpsi_last_error(ctx)
        raise HpsiError(status, msg.decode() if msg else "")
    return status
