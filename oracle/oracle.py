"""ctypes wrapper of oracle/_build/libhpsi_oracle.so — TEST INFRASTRUCTURE.

The CPU restatement of the reference's H|psi> path (oracle/hpsi_oracle.c).
Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline legs use it,
as the checker or as the timed CPU baseline.  The product never imports it.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

from effmass_gb300 import abi

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libhpsi_oracle.so")
REF_DRIVER = os.path.join(HERE, "_ref", "ref_driver")
# the same reference sources at -O3 (default FP contraction): the timed CPU baseline
REF_BENCH = os.path.join(HERE, "_ref", "ref_bench")

_lib = None


def build(quiet: bool = True):
    subprocess.run(["make", "-s", "-C", HERE, "all"], check=True,
                   stdout=subprocess.DEVNULL if quiet else None)


def build_ref(quiet: bool = True) -> bool:
    """Build the reference driver if its generated sources can be had here."""
    r = subprocess.run(["make", "-s", "-C", HERE, "ref"],
                       stdout=subprocess.DEVNULL if quiet else None,
                       stderr=subprocess.DEVNULL if quiet else None)
    return r.returncode == 0 and os.path.exists(REF_DRIVER) and os.path.exists(REF_BENCH)


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = C.CDLL(LIB_PATH)
        dp, ip = C.POINTER(C.c_double), C.POINTER(C.c_int)
        sysp, kpp = C.POINTER(abi.HpsiSystem), C.POINTER(abi.HpsiKpoint)
        L.oracle_hpsi.argtypes = [sysp, kpp, C.c_int, dp, dp, C.c_int]
        L.oracle_grad.argtypes = [sysp, kpp, C.c_int, dp, dp, dp, dp]
        L.oracle_velocity.argtypes = [sysp, kpp, C.c_int, dp, dp]
        L.oracle_density.argtypes = [sysp, kpp, C.c_int, dp, dp, dp]
        L.oracle_beta_tables.argtypes = [C.c_int, dp, dp, C.c_int, C.c_int, ip, dp, C.c_double, C.c_double, dp, dp]
        L.oracle_ylm.argtypes = [C.c_int, C.c_int, dp, dp, dp, dp, dp]
        L.oracle_ylm.restype = None
        L.oracle_beta_interp.argtypes = [dp, C.c_int, C.c_double, C.c_double, C.c_double, C.c_double, dp]
        L.oracle_structure_factor.argtypes = [C.c_int, ip, dp, dp, C.c_int, C.c_int, C.c_int, dp]
        L.oracle_fft3d.argtypes = [dp, C.c_int, C.c_int, C.c_int, C.c_int]
        L.oracle_fft3d.restype = None
        L.oracle_fft1d.argtypes = [dp, C.c_int, C.c_int, C.c_double]
        L.oracle_spherical.argtypes = [C.c_int, dp, dp, dp, dp]
        L.oracle_spherical.restype = None
        L.oracle_d2beta_tables.argtypes = [C.c_int, dp, dp, C.c_int, C.c_int, ip, dp, C.c_double, C.c_double, dp]
        L.oracle_hess.argtypes = [sysp, kpp, C.c_int, dp, C.POINTER(dp), C.c_int, C.c_double, dp]
        L.oracle_hess_tables.argtypes = [C.c_int, dp, dp, C.c_int, C.c_int, ip, dp, C.c_double, C.c_double, dp]
        _lib = L
    return _lib


def _check(rc):
    if rc != 0:
        raise RuntimeError(f"oracle status {abi.STATUS_NAMES.get(rc, rc)}")


def hpsi(sysm, kp, psi: np.ndarray, hpsi_out: np.ndarray = None, threads: int = 1) -> np.ndarray:
    psi = np.ascontiguousarray(psi, dtype=np.complex128).reshape(-1, kp.npw)
    out = np.zeros_like(psi) if hpsi_out is None else hpsi_out
    S, K = abi.pack_system(sysm), abi.pack_kpoint(kp)
    _check(lib().oracle_hpsi(S.ref(), K.ref(), psi.shape[0], abi.cptr(psi), abi.cptr(out), threads))
    return out


def grad(sysm, kp, psi: np.ndarray):
    psi = np.ascontiguousarray(psi, dtype=np.complex128).reshape(-1, kp.npw)
    out = np.zeros((3,) + psi.shape, dtype=np.complex128)
    S, K = abi.pack_system(sysm), abi.pack_kpoint(kp)
    _check(lib().oracle_grad(S.ref(), K.ref(), psi.shape[0], abi.cptr(psi), abi.cptr(out[0]),
                             abi.cptr(out[1]), abi.cptr(out[2])))
    return out


def velocity(sysm, kp, psi: np.ndarray):
    psi = np.ascontiguousarray(psi, dtype=np.complex128).reshape(-1, kp.npw)
    nb = psi.shape[0]
    out = np.zeros((3, nb, nb), dtype=np.complex128)
    S, K = abi.pack_system(sysm), abi.pack_kpoint(kp)
    _check(lib().oracle_velocity(S.ref(), K.ref(), nb, abi.cptr(psi), abi.cptr(out)))
    return out


def density(sysm, kp, psi: np.ndarray, occ, rho: np.ndarray = None) -> np.ndarray:
    """rho[i][j][k] += sum_b occ_b |psi_b(r)|^2 (the reference's buildDensity for one k-point)."""
    psi = np.ascontiguousarray(psi, dtype=np.complex128).reshape(-1, kp.npw)
    occ = np.ascontiguousarray(occ, dtype=np.float64)
    out = np.zeros(sysm.n1 * sysm.n2 * sysm.n3) if rho is None else rho
    S, K = abi.pack_system(sysm), abi.pack_kpoint(kp)
    _check(lib().oracle_density(S.ref(), K.ref(), psi.shape[0], abi.cptr(psi), abi.cptr(occ), abi.cptr(out)))
    return out


def beta_tables(r, rab, uniform: bool, l, beta, dq: float = 0.01, q_max: float = 20.0):
    """(beta_q, dbeta_q) [n_proj][nq] as the reference's BetaqTables / DBetaqTables build them."""
    r = np.ascontiguousarray(r, dtype=np.float64)
    rab = np.ascontiguousarray(rab, dtype=np.float64)
    l = np.ascontiguousarray(l, dtype=np.int32)
    beta = np.ascontiguousarray(beta, dtype=np.float64)
    nq = int(np.ceil(q_max / dq)) + 4
    bq = np.zeros((beta.shape[0], nq))
    dbq = np.zeros_like(bq)
    _check(lib().oracle_beta_tables(r.size, abi.cptr(r), abi.cptr(rab), int(uniform), beta.shape[0],
                                    l.ctypes.data_as(C.POINTER(C.c_int)), abi.cptr(beta), dq, q_max,
                                    abi.cptr(bq), abi.cptr(dbq)))
    return bq, dbq


def d2beta_tables(r, rab, uniform: bool, l, beta, dq: float = 0.01, q_max: float = 20.0):
    """d2beta/dq2 [n_proj][nq] as the reference's D2BetaqTables builds it (raw)."""
    r = np.ascontiguousarray(r, dtype=np.float64)
    rab = np.ascontiguousarray(rab, dtype=np.float64)
    l = np.ascontiguousarray(l, dtype=np.int32)
    beta = np.ascontiguousarray(beta, dtype=np.float64)
    nq = int(np.ceil(q_max / dq)) + 4
    d2 = np.zeros((beta.shape[0], nq))
    _check(lib().oracle_d2beta_tables(r.size, abi.cptr(r), abi.cptr(rab), int(uniform), beta.shape[0],
                                      l.ctypes.data_as(C.POINTER(C.c_int)), abi.cptr(beta), dq, q_max,
                                      abi.cptr(d2)))
    return d2


def hess_tables(r, rab, uniform: bool, l, beta, dq: float = 0.01, q_max: float = 20.0):
    """[3][n_proj][nq] radial tables F0 = beta/q^l, F1 = F0'/q, F3 = (F0'' - F0'/q)/q^2 (raw)."""
    r = np.ascontiguousarray(r, dtype=np.float64)
    rab = np.ascontiguousarray(rab, dtype=np.float64)
    l = np.ascontiguousarray(l, dtype=np.int32)
    beta = np.ascontiguousarray(beta, dtype=np.float64)
    nq = int(np.ceil(q_max / dq)) + 4
    f = np.zeros((3, beta.shape[0], nq))
    _check(lib().oracle_hess_tables(r.size, abi.cptr(r), abi.cptr(rab), int(uniform), beta.shape[0],
                                    l.ctypes.data_as(C.POINTER(C.c_int)), abi.cptr(beta), dq, q_max, abi.cptr(f)))
    return f


def hess(sysm, kp, psi: np.ndarray, ftabs, dq: float) -> np.ndarray:
    """d2H/dk_a dk_b |psi> [6][nb][npw] (xx, yy, zz, xy, xz, yz); ftabs[s] are the
    species' radial tables [3][n_proj][nq] (F0, F1, F3, raw) on q_i = i dq."""
    psi = np.ascontiguousarray(psi, dtype=np.complex128).reshape(-1, kp.npw)
    ft = [np.ascontiguousarray(f, dtype=np.float64) for f in ftabs]
    nq = ft[0].shape[-1]
    arr = (C.POINTER(C.c_double) * len(ft))(*[abi.cptr(f) for f in ft])
    out = np.zeros((6,) + psi.shape, dtype=np.complex128)
    S, K = abi.pack_system(sysm), abi.pack_kpoint(kp)
    _check(lib().oracle_hess(S.ref(), K.ref(), psi.shape[0], abi.cptr(psi), arr, nq, dq, abi.cptr(out)))
    return out


def ylm(lmax: int, theta, phi):
    theta = np.ascontiguousarray(theta, dtype=np.float64)
    phi = np.ascontiguousarray(phi, dtype=np.float64)
    ng = theta.shape[0]
    nlm = (lmax + 1) ** 2
    y = np.zeros((nlm, ng))
    dth = np.zeros((nlm, ng))
    dph = np.zeros((nlm, ng))
    lib().oracle_ylm(lmax, ng, abi.cptr(theta), abi.cptr(phi), abi.cptr(y), abi.cptr(dth), abi.cptr(dph))
    return y, dth, dph


def beta_interp(table, dq, q_max, norm, q):
    t = np.ascontiguousarray(table, dtype=np.float64)
    out = C.c_double()
    rc = lib().oracle_beta_interp(abi.cptr(t), t.shape[0], dq, q_max, norm, q, C.byref(out))
    return rc, out.value


def structure_factor(g_idx, k_frac, tau, n):
    g = np.ascontiguousarray(g_idx, dtype=np.int32).reshape(-1, 3)
    kf = np.ascontiguousarray(k_frac, dtype=np.float64)
    t = np.ascontiguousarray(tau, dtype=np.float64)
    out = np.zeros(g.shape[0], dtype=np.complex128)
    rc = lib().oracle_structure_factor(g.shape[0], g.ctypes.data_as(C.POINTER(C.c_int)), abi.cptr(kf),
                                       abi.cptr(t), n[0], n[1], n[2], abi.cptr(out))
    return rc, out


def fft3d(grid: np.ndarray, direction: str) -> np.ndarray:
    g = np.ascontiguousarray(grid, dtype=np.complex128).copy()
    n1, n2, n3 = g.shape
    lib().oracle_fft3d(abi.cptr(g), n1, n2, n3, +1 if direction == "G2R" else -1)
    return g


def fft1d(x: np.ndarray, sign: int, fct: float) -> np.ndarray:
    c = np.ascontiguousarray(x, dtype=np.complex128).copy()
    _check(lib().oracle_fft1d(abi.cptr(c), c.shape[0], sign, fct))
    return c


def spherical(kvec):
    K = np.ascontiguousarray(kvec, dtype=np.float64)
    ng = K.shape[0]
    q, th, ph = np.zeros(ng), np.zeros(ng), np.zeros(ng)
    lib().oracle_spherical(ng, abi.cptr(K), abi.cptr(q), abi.cptr(th), abi.cptr(ph))
    return q, th, ph
