"""Python mirror of the reference's H_psi operator API over libhpsi_gb300.so.

Reference interface (bzzlfd/effmass, src/H_psi/hamiltonian.cppm):

    Hamiltonian H(...); H.load...(); H.finalize(...)      -> Hamiltonian(system)
    auto op = H.at_k(ik);                                 -> op = H.at_k(ik, kpoint)
    op(psi, hpsi)            // hpsi += H psi, one band    -> op(psi, hpsi)
    op(n_bands, psi, hpsi)   // declared, never defined    -> op(n_bands, psi, hpsi)
    op.dim(); op.set_ikpt(j)                              -> op.dim(); op.set_ikpt(j)
    H.gradient().at_k(ik)(psi, GradHPsi{x, y, z})         -> H.gradient().at_k(ik)(psi, GradHPsi(x, y, z))

Outputs accumulate, as in the reference (the caller zeroes them).  Arrays
may be numpy complex128 (host memory: copied in and out inside the call) or
CUDA torch complex128 tensors (device memory: used in place, launched on the
current torch stream).  Errors raise ``HpsiError`` with the library's status
(BAD_ARG / RANGE / STATE ... for the reference's invalid_argument /
domain_error / runtime_error).
"""
from __future__ import annotations

import ctypes as C
import dataclasses
from typing import Optional

import numpy as np

from . import abi
from ._lib import HpsiError, check, load


def _is_torch(x) -> bool:
    return type(x).__module__.startswith("torch")


def _ptr(x, npw: int, nb: int, name: str):
    """(pointer, is_device) of a complex128 block of nb*npw values."""
    if x is None:
        return None, None
    if _is_torch(x):
        import torch
        if x.dtype != torch.complex128 or not x.is_contiguous():
            raise HpsiError(abi.HPSI_ERR_BAD_ARG, f"{name}: need a contiguous complex128 tensor")
        if x.numel() < nb * npw:
            raise HpsiError(abi.HPSI_ERR_BAD_ARG, f"{name}: {x.numel()} values < {nb}*{npw}")
        return C.c_void_p(x.data_ptr()), bool(x.is_cuda)
    if not isinstance(x, np.ndarray) or x.dtype != np.complex128 or not x.flags["C_CONTIGUOUS"]:
        raise HpsiError(abi.HPSI_ERR_BAD_ARG, f"{name}: need a C-contiguous complex128 array")
    if x.size < nb * npw:
        raise HpsiError(abi.HPSI_ERR_BAD_ARG, f"{name}: {x.size} values < {nb}*{npw}")
    return C.c_void_p(x.ctypes.data), False


def _stream_for(device: bool):
    if not device:
        return None
    import torch
    return C.c_void_p(torch.cuda.current_stream().cuda_stream)


@dataclasses.dataclass
class GradHPsi:
    """Outputs of dH/dk_{x,y,z}|psi>; None skips a direction (the reference's empty span)."""
    x: Optional[object] = None
    y: Optional[object] = None
    z: Optional[object] = None


class Hamiltonian:
    """Device-resident system (V_loc, tables, atoms) — the reference's finalized Hamiltonian."""

    def __init__(self, system, precision: str = "fp64"):
        self._lib = load()
        self.system = system
        self.precision = precision
        self._packed = abi.pack_system(system)
        h = C.c_void_p()
        st = self._lib.hpsi_ctx_create(C.byref(self._packed.struct), C.byref(h))
        check(st, None)
        self._ctx = h
        self._kpoints = {}

    # -- lifetime --
    def close(self):
        if getattr(self, "_ctx", None):
            self._lib.hpsi_ctx_destroy(self._ctx)
            self._ctx = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    @property
    def ctx(self):
        return self._ctx

    def flags(self, precision: Optional[str] = None, device: bool = False) -> int:
        f = abi.PRECISIONS[precision or self.precision]
        if device:
            f |= abi.HPSI_DEVICE_PTRS
        return f

    # -- k-points --
    def set_kpoint(self, kid: int, kpoint):
        packed = abi.pack_kpoint(kpoint)
        check(self._lib.hpsi_set_kpoint(self._ctx, kid, C.byref(packed.struct)), self._ctx)
        self._kpoints[kid] = kpoint

    def dim(self, kid: int) -> int:
        n = self._lib.hpsi_dim(self._ctx, kid)
        if n < 0:
            check(n, self._ctx)
        return n

    def at_k(self, kid: int, kpoint=None, precision: Optional[str] = None) -> "Callable":
        if kpoint is not None:
            self.set_kpoint(kid, kpoint)
        return Callable(self, kid, precision)

    def gradient(self) -> "Gradient":
        return Gradient(self)

    # -- instrumentation --
    PHASES = ["build", "g2r_planes", "x_pass", "r2g_planes", "proj_gemm", "reduce", "expand_gemm", "other"]

    def profile(self, on: bool = True):
        """Reset and switch the per-phase CUDA-event profile of later calls."""
        check(self._lib.hpsi_profile(self._ctx, 1 if on else 0), self._ctx)

    def profile_read(self):
        """{phase: (milliseconds, launches)} summed over the calls since profile(True)."""
        ms = (C.c_double * 8)()
        n = (C.c_longlong * 8)()
        check(self._lib.hpsi_profile_read(self._ctx, ms, n), self._ctx)
        return {name: (ms[i], int(n[i])) for i, name in enumerate(self.PHASES)}

    # -- raw calls --
    def apply(self, kid: int, nb: int, psi, hpsi, precision: Optional[str] = None, one_stream: bool = False):
        """hpsi += H psi.  one_stream: keep the tensor-core projection chain on the
        caller's stream (HPSI_ONE_STREAM) instead of the side stream."""
        npw = self.dim(kid)
        p, dev_p = _ptr(psi, npw, nb, "psi")
        h, dev_h = _ptr(hpsi, npw, nb, "hpsi")
        if dev_p != dev_h:
            raise HpsiError(abi.HPSI_ERR_BAD_ARG, "psi and hpsi must both be host or both be device arrays")
        f = self.flags(precision, dev_p) | (abi.HPSI_ONE_STREAM if one_stream else 0)
        check(self._lib.hpsi_apply(self._ctx, kid, nb, p, h, f, _stream_for(dev_p)), self._ctx)

    def apply_energies(self, kid: int, nb: int, psi, hpsi, precision: Optional[str] = None, e=None):
        """hpsi += H psi and return e[b] = <psi_b|H|psi_b> (FP64 reductions on the device)."""
        npw = self.dim(kid)
        p, dev_p = _ptr(psi, npw, nb, "psi")
        h, dev_h = _ptr(hpsi, npw, nb, "hpsi")
        if dev_p != dev_h:
            raise HpsiError(abi.HPSI_ERR_BAD_ARG, "psi and hpsi must both be host or both be device arrays")
        if e is None:
            if dev_p:
                import torch
                e = torch.zeros(nb, dtype=torch.float64, device=psi.device)
            else:
                e = np.zeros(nb, dtype=np.float64)
        ep = e.data_ptr() if dev_p else e.ctypes.data
        check(self._lib.hpsi_apply_energies(self._ctx, kid, nb, p, h, ep, self.flags(precision, dev_p),
                                            _stream_for(dev_p)), self._ctx)
        return e

    def sternheimer(self, kid: int, psi, eps, direction: int, tol: float = 1e-10, max_iter: int = 500,
                    precision: Optional[str] = None):
        """Solve P_c (H - eps_n) P_c x_n = -P_c dH/dk_a psi_n for the occupied eigenstates psi
        (numpy [nv, npw]); returns (x [nv, npw], iterations, relative residuals [nv])."""
        npw = self.dim(kid)
        psi = np.ascontiguousarray(psi, dtype=np.complex128)
        nv = psi.shape[0]
        eps = np.ascontiguousarray(eps, dtype=np.float64)
        x = np.zeros_like(psi)
        its = C.c_int()
        res = np.zeros(nv)
        st = self._lib.hpsi_sternheimer(self._ctx, kid, nv, psi.ctypes.data, eps.ctypes.data, direction, tol,
                                        max_iter, x.ctypes.data, C.byref(its),
                                        res.ctypes.data_as(C.POINTER(C.c_double)), self.flags(precision, False),
                                        None)
        check(st, self._ctx)
        return x, its.value, res

    def set_hessian_tables(self, species: int, f, dq: float):
        """Attach the [3][n_proj][nq] Hessian radial tables (hessian_tables) to a species."""
        f = np.ascontiguousarray(f, dtype=np.float64)
        check(self._lib.hpsi_set_hessian_tables(self._ctx, species, f.shape[-1], dq,
                                                f.ctypes.data_as(C.POINTER(C.c_double))), self._ctx)

    def hess_apply(self, kid: int, nb: int, psi, out: dict, precision: Optional[str] = None):
        """out[ab] += d2H/dk_a dk_b psi for ab in xx, yy, zz, xy, xz, yz (missing keys skipped)."""
        npw = self.dim(kid)
        p, dev = _ptr(psi, npw, nb, "psi")
        ptrs = []
        for name in ("xx", "yy", "zz", "xy", "xz", "yz"):
            o = out.get(name)
            q, d = _ptr(o, npw, nb, name)
            if o is not None and d != dev:
                raise HpsiError(abi.HPSI_ERR_BAD_ARG, "psi and outputs must live in the same memory")
            ptrs.append(q)
        check(self._lib.hpsi_hess_apply(self._ctx, kid, nb, p, *ptrs, self.flags(precision, dev), _stream_for(dev)),
              self._ctx)
        return out

    def density(self, kid: int, nb: int, psi, occ, rho=None, precision: Optional[str] = None):
        """rho += sum_b occ_b |psi_b(r)|^2 (the reference's buildDensity for one k-point), [n1, n2, n3]."""
        npw = self.dim(kid)
        p, dev = _ptr(psi, npw, nb, "psi")
        s = self.system
        if rho is None:
            if dev:
                import torch
                rho = torch.zeros((s.n1, s.n2, s.n3), dtype=torch.float64, device=psi.device)
            else:
                rho = np.zeros((s.n1, s.n2, s.n3), dtype=np.float64)
        if dev:
            op, rp = occ.data_ptr(), rho.data_ptr()
        else:
            occ = np.ascontiguousarray(occ, dtype=np.float64)
            if rho.dtype != np.float64 or not rho.flags["C_CONTIGUOUS"] or rho.size != s.n1 * s.n2 * s.n3:
                raise HpsiError(abi.HPSI_ERR_BAD_ARG, "rho must be a C-contiguous float64 grid")
            op, rp = occ.ctypes.data, rho.ctypes.data
        check(self._lib.hpsi_density(self._ctx, kid, nb, p, op, rp, self.flags(precision, dev), _stream_for(dev)),
              self._ctx)
        return rho

    def grad_apply(self, kid: int, nb: int, psi, out: GradHPsi, precision: Optional[str] = None):
        npw = self.dim(kid)
        p, dev = _ptr(psi, npw, nb, "psi")
        ptrs = []
        for name in ("x", "y", "z"):
            o = getattr(out, name)
            q, d = _ptr(o, npw, nb, name)
            if o is not None and d != dev:
                raise HpsiError(abi.HPSI_ERR_BAD_ARG, "psi and outputs must live in the same memory")
            ptrs.append(q)
        check(self._lib.hpsi_grad_apply(self._ctx, kid, nb, p, ptrs[0], ptrs[1], ptrs[2],
                                        self.flags(precision, dev), _stream_for(dev)), self._ctx)

    def velocity_matrix(self, kid: int, nb: int, psi, out=None, precision: Optional[str] = None):
        """M[a][m][n] = <psi_m|dH/dk_a|psi_n> (complex128 [3, nb, nb], overwritten)."""
        npw = self.dim(kid)
        p, dev = _ptr(psi, npw, nb, "psi")
        if out is None:
            if dev:
                import torch
                out = torch.zeros((3, nb, nb), dtype=torch.complex128, device=psi.device)
            else:
                out = np.zeros((3, nb, nb), dtype=np.complex128)
        m, dm = _ptr(out, nb, 3 * nb, "m")
        if dm != dev:
            raise HpsiError(abi.HPSI_ERR_BAD_ARG, "psi and m must live in the same memory")
        check(self._lib.hpsi_velocity_matrix(self._ctx, kid, nb, p, m, self.flags(precision, dev),
                                             _stream_for(dev)), self._ctx)
        return out


class Callable:
    """H|psi> at a fixed k-point (the reference's Hamiltonian::Callable)."""

    def __init__(self, parent: Hamiltonian, kid: int, precision: Optional[str] = None):
        self._h = parent
        self._kid = kid
        self._prec = precision
        parent.dim(kid)  # raises STATE if the slot is unbound

    def dim(self) -> int:
        return self._h.dim(self._kid)

    def set_ikpt(self, kid: int, kpoint=None):
        if kpoint is not None:
            self._h.set_kpoint(kid, kpoint)
        self._h.dim(kid)
        self._kid = kid

    def __call__(self, *args):
        if len(args) == 2:
            psi, hpsi = args
            nb = 1
        elif len(args) == 3:
            nb, psi, hpsi = args
        else:
            raise TypeError("call as op(psi, hpsi) or op(n_bands, psi, hpsi)")
        self._h.apply(self._kid, int(nb), psi, hpsi, self._prec)


class Gradient:
    def __init__(self, parent: Hamiltonian):
        self._h = parent

    def at_k(self, kid: int, kpoint=None, precision: Optional[str] = None) -> "GradientCallable":
        if kpoint is not None:
            self._h.set_kpoint(kid, kpoint)
        return GradientCallable(self._h, kid, precision)


class GradientCallable:
    """dH/dk_alpha|psi> at a fixed k-point (the reference's Gradient::Callable)."""

    def __init__(self, parent: Hamiltonian, kid: int, precision: Optional[str] = None):
        self._h = parent
        self._kid = kid
        self._prec = precision
        parent.dim(kid)

    def dim(self) -> int:
        return self._h.dim(self._kid)

    def __call__(self, psi, out: GradHPsi, n_bands: int = 1):
        self._h.grad_apply(self._kid, int(n_bands), psi, out, self._prec)


def kp_sums(m, e, n_low: int, deg_tol: float = 1e-8):
    """FP64 k·p sums s[n][a][b] = sum_{m != n, |e_n - e_m| > deg_tol} Re(M_a[n][m] M_b[m][n]) / (e_n - e_m)
    for the lowest n_low bands, from a velocity matrix m [3, nb, nb] and energies e [nb] (numpy host
    arrays or CUDA torch tensors).  Returns (s [n_low, 3, 3], skipped [n_low])."""
    L = load()
    nb = int(e.shape[0])
    if _is_torch(m):
        import torch
        s = torch.zeros((n_low, 3, 3), dtype=torch.float64, device=m.device)
        k = torch.zeros(n_low, dtype=torch.int32, device=m.device)
        check(L.hpsi_kp_sums(nb, n_low, m.data_ptr(), e.data_ptr(), deg_tol, s.data_ptr(), k.data_ptr(),
                             abi.HPSI_DEVICE_PTRS | abi.HPSI_SYNC, None))
        return s, k
    m = np.ascontiguousarray(m, dtype=np.complex128)
    e = np.ascontiguousarray(e, dtype=np.float64)
    s = np.zeros((n_low, 3, 3), dtype=np.float64)
    k = np.zeros(n_low, dtype=np.int32)
    check(L.hpsi_kp_sums(nb, n_low, m.ctypes.data, e.ctypes.data, deg_tol, s.ctypes.data, k.ctypes.data, 0, None))
    return s, k


def beta_tables(r, rab, uniform: bool, l, beta, dq: float = 0.01, q_max: float = 20.0, derivative: bool = True):
    """beta(q) (and dbeta/dq) tables [n_proj][nq] of radial projectors, built on the device."""
    L = load()
    r = np.ascontiguousarray(r, dtype=np.float64)
    rab = np.ascontiguousarray(rab, dtype=np.float64)
    l = np.ascontiguousarray(l, dtype=np.int32)
    beta = np.ascontiguousarray(beta, dtype=np.float64)
    nq = L.hpsi_beta_table_length(dq, q_max)
    if nq < 0:
        check(nq)
    bq = np.zeros((beta.shape[0], nq))
    dbq = np.zeros_like(bq) if derivative else None
    check(L.hpsi_beta_tables(r.size, r.ctypes.data, rab.ctypes.data, int(uniform), beta.shape[0], l.ctypes.data,
                             beta.ctypes.data, dq, q_max, bq.ctypes.data,
                             dbq.ctypes.data if dbq is not None else None, 0, None))
    return bq, dbq


def gsphere(lattice, k_frac, ecut: float):
    """The k-point's G-sphere generated on the device, (g1, g2, g3) order: a system.KPoint."""
    from .system import KPoint
    L = load()
    A = np.ascontiguousarray(lattice, dtype=np.float64).reshape(9)
    kf = np.ascontiguousarray(k_frac, dtype=np.float64).reshape(3)
    dp = C.POINTER(C.c_double)
    n = C.c_int()
    check(L.hpsi_gsphere(A.ctypes.data_as(dp), kf.ctypes.data_as(dp), ecut, 0, None, None, None, C.byref(n), 0, None))
    g = np.zeros((n.value, 3), dtype=np.int32)
    K = np.zeros((n.value, 3))
    kin = np.zeros(n.value)
    check(L.hpsi_gsphere(A.ctypes.data_as(dp), kf.ctypes.data_as(dp), ecut, n.value, g.ctypes.data, K.ctypes.data,
                         kin.ctypes.data, C.byref(n), 0, None))
    return KPoint(npw=n.value, k_frac=kf.copy(), g_idx=g, kvec=K, kinetic=kin)


def hessian_tables(r, rab, uniform: bool, l, beta, dq: float = 0.01, q_max: float = 20.0):
    """Hessian radial tables [3][n_proj][nq] (F0, F1, F3) of radial projectors, built on the device."""
    L = load()
    r = np.ascontiguousarray(r, dtype=np.float64)
    rab = np.ascontiguousarray(rab, dtype=np.float64)
    l = np.ascontiguousarray(l, dtype=np.int32)
    beta = np.ascontiguousarray(beta, dtype=np.float64)
    nq = L.hpsi_beta_table_length(dq, q_max)
    f = np.zeros((3, beta.shape[0], nq))
    check(L.hpsi_hessian_tables(r.size, r.ctypes.data, rab.ctypes.data, int(uniform), beta.shape[0], l.ctypes.data,
                                beta.ctypes.data, dq, q_max, f.ctypes.data, 0, None))
    return f
