"""ctypes view of the C ABI declared in include/hpsi_gb300.h.

The structs here mirror ``hpsi_species`` / ``hpsi_system`` / ``hpsi_kpoint``
field for field.  ``pack_system`` / ``pack_kpoint`` turn the numpy objects of
``effmass_gb300.system`` into those structs and keep the backing arrays alive
for as long as the returned holder lives.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HPSI_OK = 0
HPSI_ERR_BAD_ARG = -1
HPSI_ERR_OOM = -2
HPSI_ERR_RANGE = -3
HPSI_ERR_TIMEOUT = -4
HPSI_ERR_CUDA = -5
HPSI_ERR_STATE = -6

HPSI_PREC_FP64 = 0
HPSI_PREC_FP32 = 1
HPSI_PREC_TC = 2
HPSI_PREC_TC_BF16 = 3
HPSI_DEVICE_PTRS = 0x10
HPSI_SYNC = 0x20
HPSI_ONE_STREAM = 0x40
HPSI_BATCH_NO_GRAPH = 0x100
HPSI_BATCH_NO_TUNE = 0x200
HPSI_NOALLOC_SCRATCH_BYTES = 32 * 1024 * 1024

PRECISIONS = {"fp64": HPSI_PREC_FP64, "fp32": HPSI_PREC_FP32, "tc": HPSI_PREC_TC, "tc_bf16": HPSI_PREC_TC_BF16}

STATUS_NAMES = {0: "OK", -1: "BAD_ARG", -2: "OOM", -3: "RANGE", -4: "TIMEOUT", -5: "CUDA", -6: "STATE"}

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)


class HpsiSpecies(C.Structure):
    _fields_ = [("n_proj", C.c_int), ("proj_l", _ip), ("lambda_", _dp), ("nq", C.c_int),
                ("dq", C.c_double), ("q_max", C.c_double), ("beta_q", _dp), ("dbeta_q", _dp)]


class HpsiSystem(C.Structure):
    _fields_ = [("n1", C.c_int), ("n2", C.c_int), ("n3", C.c_int), ("lattice", C.c_double * 9),
                ("omega", C.c_double), ("v_loc", _dp), ("n_species", C.c_int),
                ("species", C.POINTER(HpsiSpecies)), ("n_atoms", C.c_int), ("atom_species", _ip),
                ("atom_tau", _dp)]


class HpsiKpoint(C.Structure):
    _fields_ = [("npw", C.c_int), ("k_frac", C.c_double * 3), ("g_idx", _ip), ("kvec", _dp),
                ("kinetic", _dp)]


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def _i32(a):
    return np.ascontiguousarray(a, dtype=np.int32)


class Packed:
    """A ctypes struct plus the numpy arrays it points into."""

    def __init__(self, struct, keep):
        self.struct = struct
        self._keep = keep

    def ref(self):
        return C.byref(self.struct)


def pack_system(sysm) -> Packed:
    keep = []
    sps = (HpsiSpecies * len(sysm.species))()
    for i, sp in enumerate(sysm.species):
        pl, lam, bq = _i32(sp.proj_l), _f64(sp.lam), _f64(sp.beta_q)
        dbq = _f64(sp.dbeta_q) if sp.dbeta_q is not None else None
        keep += [pl, lam, bq, dbq]
        sps[i].n_proj = sp.n_proj
        sps[i].proj_l = pl.ctypes.data_as(_ip)
        sps[i].lambda_ = lam.ctypes.data_as(_dp)
        sps[i].nq = sp.nq
        sps[i].dq = float(sp.dq)
        sps[i].q_max = float(sp.q_max)
        sps[i].beta_q = bq.ctypes.data_as(_dp)
        sps[i].dbeta_q = dbq.ctypes.data_as(_dp) if dbq is not None else _dp()
    v = _f64(sysm.v_loc)
    asp = _i32(sysm.atom_species)
    tau = _f64(sysm.atom_tau)
    keep += [v, asp, tau, sps]
    s = HpsiSystem()
    s.n1, s.n2, s.n3 = sysm.n1, sysm.n2, sysm.n3
    for i, x in enumerate(np.asarray(sysm.lattice, dtype=np.float64).reshape(9)):
        s.lattice[i] = float(x)
    s.omega = float(sysm.omega)
    s.v_loc = v.ctypes.data_as(_dp)
    s.n_species = len(sysm.species)
    s.species = C.cast(sps, C.POINTER(HpsiSpecies))
    s.n_atoms = int(tau.shape[0])
    s.atom_species = asp.ctypes.data_as(_ip)
    s.atom_tau = tau.ctypes.data_as(_dp)
    return Packed(s, keep)


def pack_kpoint(kp) -> Packed:
    g, K, kin = _i32(kp.g_idx), _f64(kp.kvec), _f64(kp.kinetic)
    s = HpsiKpoint()
    s.npw = int(kp.npw)
    for i in range(3):
        s.k_frac[i] = float(kp.k_frac[i])
    s.g_idx = g.ctypes.data_as(_ip)
    s.kvec = K.ctypes.data_as(_dp)
    s.kinetic = kin.ctypes.data_as(_dp)
    return Packed(s, [g, K, kin])


def cptr(a: np.ndarray):
    """double* to the first element of a complex128/float64 numpy array (or None)."""
    if a is None:
        return None
    assert a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(_dp)


def package_dir() -> str:
    return os.path.dirname(os.path.abspath(__file__))


def repo_root() -> str:
    return os.path.dirname(package_dir())


class HpsiBatchItem(C.Structure):
    _fields_ = [("ctx", C.c_void_p), ("kid", C.c_int), ("nb", C.c_int)]
