"""Synthetic plane-wave systems for the H|psi> path (host-side set-up, numpy).

The reference reads its inputs from PWmat files (OUT.GKK, OUT.VR,
atom.config, UPF).  This module builds the same quantities directly:

* lattice and atoms of diamond-structure cells (2-atom fcc, 8- and 64-atom
  simple-cubic supercells);
* the G-sphere of one k-point: integer g, K = k+G (Cartesian, bohr^-1) and
  kinetic |k+G|^2/2 — the data ``GKK::loadKPoint`` provides
  (src/io/GKK.cppm:511-593);
* the local potential V_loc(r) on the FFT grid, layout [i][j][k] with k
  fastest (src/io/RHO.cppm:51-61);
* Kleinman-Bylander projectors beta_l(q) = q^l exp(-q^2 rc^2/4) with a
  symmetric D per l, diagonalised per l exactly as the reference's
  ``diagonalizeNonlocal`` (src/pseudo/ncpp_advance.cppm:65-153) leaves it:
  eigenvalues lambda_i and the rotated radial functions;
* seeded, orthonormalised band coefficients psi(G).

Everything here runs once per system, off the per-band hot path.
"""
from __future__ import annotations

import dataclasses
import math
import struct
from typing import List, Optional

import numpy as np

BOHR_ANGSTROM = 0.52917721067


@dataclasses.dataclass
class Species:
    """One pseudopotential species after per-l diagonalisation of D."""
    z: int
    proj_l: np.ndarray          # [n_proj] int32
    lam: np.ndarray             # [n_proj] Ha
    dq: float
    q_max: float
    beta_q: np.ndarray          # [n_proj, nq] raw beta(q_i) (no 1/sqrt(Omega))
    dbeta_q: np.ndarray         # [n_proj, nq] raw dbeta/dq(q_i)
    # radial description (for writing a reference spec); optional
    rc: Optional[np.ndarray] = None       # [n_raw] rc per raw projector
    raw_l: Optional[np.ndarray] = None    # [n_raw]
    d_ha: Optional[np.ndarray] = None     # [n_raw, n_raw] undiagonalised D (Ha)

    @property
    def n_proj(self) -> int:
        return int(self.proj_l.shape[0])

    @property
    def nq(self) -> int:
        return int(self.beta_q.shape[1])


@dataclasses.dataclass
class KPoint:
    npw: int
    k_frac: np.ndarray          # [3]
    g_idx: np.ndarray           # [npw, 3] int32
    kvec: np.ndarray            # [npw, 3] K = k+G, Cartesian bohr^-1
    kinetic: np.ndarray         # [npw] |K|^2/2


@dataclasses.dataclass
class System:
    name: str
    lattice: np.ndarray         # [3, 3] bohr, row n = a_n
    omega: float
    n1: int
    n2: int
    n3: int
    v_loc: np.ndarray           # [n1*n2*n3] Ha
    species: List[Species]
    atom_species: np.ndarray    # [n_atoms] index into species
    atom_z: np.ndarray          # [n_atoms]
    atom_tau: np.ndarray        # [n_atoms, 3] fractional
    ecut: float                 # Ha

    @property
    def n_atoms(self) -> int:
        return int(self.atom_tau.shape[0])

    @property
    def n_proj_total(self) -> int:
        """Projectors summed over atoms and m (skipping |lambda| < 1e-15 as the reference does)."""
        tot = 0
        for a in range(self.n_atoms):
            sp = self.species[self.atom_species[a]]
            for i in range(sp.n_proj):
                if abs(sp.lam[i]) >= 1e-15:
                    tot += 2 * int(sp.proj_l[i]) + 1
        return tot

    def reciprocal(self) -> np.ndarray:
        """Rows b_n with a_m . b_n = 2 pi delta_mn (bohr^-1)."""
        return 2.0 * np.pi * np.linalg.inv(self.lattice).T


# --------------------------------------------------------------------------
# geometry
# --------------------------------------------------------------------------

def diamond_fcc(a: float = 10.26):
    lat = 0.5 * a * np.array([[0.0, 1.0, 1.0], [1.0, 0.0, 1.0], [1.0, 1.0, 0.0]])
    tau = np.array([[0.0, 0.0, 0.0], [0.25, 0.25, 0.25]])
    return lat, tau


def diamond_sc(a_conv: float = 10.26, rep: int = 1):
    """Simple-cubic supercell of rep^3 conventional diamond cells (8 atoms each)."""
    fcc = np.array([[0, 0, 0], [0, 0.5, 0.5], [0.5, 0, 0.5], [0.5, 0.5, 0]])
    basis = np.concatenate([fcc, fcc + 0.25])
    taus = []
    for i in range(rep):
        for j in range(rep):
            for k in range(rep):
                for b in basis:
                    taus.append((b + np.array([i, j, k])) / rep)
    lat = a_conv * rep * np.eye(3)
    return lat, np.array(taus)


def g_sphere(lattice: np.ndarray, k_frac, ecut: float, n=(None, None, None)) -> KPoint:
    """All G with |k+G|^2/2 < ecut, ordered by kinetic energy then (g1,g2,g3)."""
    B = 2.0 * np.pi * np.linalg.inv(lattice).T
    k_frac = np.asarray(k_frac, dtype=np.float64)
    gmax = int(math.ceil(math.sqrt(2.0 * ecut) / min(np.linalg.norm(B, axis=1)) * 2)) + 2
    r = np.arange(-gmax, gmax + 1)
    g = np.stack(np.meshgrid(r, r, r, indexing="ij"), axis=-1).reshape(-1, 3)
    K = (g + k_frac) @ B
    kin = 0.5 * np.einsum("ij,ij->i", K, K)
    sel = kin < ecut
    g, K, kin = g[sel], K[sel], kin[sel]
    order = np.lexsort((g[:, 2], g[:, 1], g[:, 0], kin))
    g, K, kin = g[order], K[order], kin[order]
    return KPoint(npw=int(g.shape[0]), k_frac=k_frac.copy(), g_idx=g.astype(np.int32),
                  kvec=np.ascontiguousarray(K), kinetic=np.ascontiguousarray(kin))


def local_potential(lattice, tau, n1, n2, n3, depth=3.0, width=1.2) -> np.ndarray:
    """V(r) = sum over atoms and periodic images of -depth*exp(-|r-tau|^2/width^2) (Ha),
    on the grid r = (i/n1, j/n2, k/n3) in fractional coordinates, layout [i][j][k].

    Evaluated as its Fourier series: V(G) = (1/Omega) sum_a exp(-i G.tau_a) *
    (-depth pi^(3/2) width^3 exp(-|G|^2 width^2/4)), summed over the grid's G
    with numpy's FFT.  The Gaussian's transform at the grid's largest |G| is
    below 1e-18 for the named systems, so this equals the real-space image sum
    to rounding."""
    lattice = np.asarray(lattice, dtype=np.float64)
    omega = abs(np.linalg.det(lattice))
    B = 2.0 * np.pi * np.linalg.inv(lattice).T
    f = [np.fft.fftfreq(n, 1.0 / n) for n in (n1, n2, n3)]
    g = np.stack(np.meshgrid(*f, indexing="ij"), axis=-1)
    G = g @ B
    G2 = np.einsum("...i,...i->...", G, G)
    ft = -depth * np.pi ** 1.5 * width ** 3 * np.exp(-G2 * width * width / 4.0)
    S = np.zeros((n1, n2, n3), dtype=np.complex128)
    for t in np.asarray(tau, dtype=np.float64):
        S += np.exp(-2j * np.pi * (g @ t))
    coeff = ft * S / omega
    v = np.fft.ifftn(coeff) * (n1 * n2 * n3)
    return np.ascontiguousarray(v.real.reshape(-1))


def local_potential_direct(lattice, tau, points_frac, depth=3.0, width=1.2, nimg=2) -> np.ndarray:
    """Real-space image sum of the same potential at given fractional points (for checks)."""
    lattice = np.asarray(lattice, dtype=np.float64)
    F = np.asarray(points_frac, dtype=np.float64).reshape(-1, 3)
    shifts = np.stack(np.meshgrid(*[np.arange(-nimg, nimg + 1)] * 3, indexing="ij"), -1).reshape(-1, 3)
    v = np.zeros(F.shape[0])
    for t in np.asarray(tau, dtype=np.float64):
        d = F - t
        d -= np.round(d)
        for s in shifts:
            rc = (d + s) @ lattice
            v += -depth * np.exp(-np.einsum("ij,ij->i", rc, rc) / (width * width))
    return v


# --------------------------------------------------------------------------
# pseudopotential tables
# --------------------------------------------------------------------------

def beta_analytic(l: int, rc: float, q: np.ndarray):
    e = np.exp(-q * q * rc * rc / 4.0)
    b = q ** l * e
    if l == 0:
        db = -0.5 * rc * rc * q * e
    else:
        db = (l * q ** (l - 1) - 0.5 * rc * rc * q ** (l + 1)) * e
    return b, db


def make_species(z: int, l_max: int, rcs=(1.0, 1.4), seed: int = 7, dq: float = 0.01,
                 q_max: float = 30.0) -> Species:
    """KB species with len(rcs) projectors per l; D_l symmetric U[-2,2] Ha, diagonalised per l."""
    rng = np.random.default_rng(seed)
    nq = int(math.ceil(q_max / dq)) + 1 + 3
    q = np.arange(nq) * dq
    raw_l, raw_rc = [], []
    for l in range(l_max + 1):
        for rc in rcs:
            raw_l.append(l)
            raw_rc.append(rc)
    nraw = len(raw_l)
    D = np.zeros((nraw, nraw))
    proj_l, lam, bq, dbq = [], [], [], []
    for l in range(l_max + 1):
        idx = [i for i in range(nraw) if raw_l[i] == l]
        m = len(idx)
        blk = rng.uniform(-2.0, 2.0, size=(m, m))
        blk = 0.5 * (blk + blk.T)
        D[np.ix_(idx, idx)] = blk
        w, U = np.linalg.eigh(blk)
        raw = [beta_analytic(l, raw_rc[i], q) for i in idx]
        for kk in range(m):
            b = sum(U[ii, kk] * raw[ii][0] for ii in range(m))
            db = sum(U[ii, kk] * raw[ii][1] for ii in range(m))
            proj_l.append(l)
            lam.append(w[kk])
            bq.append(b)
            dbq.append(db)
    return Species(z=z, proj_l=np.array(proj_l, dtype=np.int32), lam=np.array(lam), dq=dq,
                   q_max=q_max, beta_q=np.ascontiguousarray(np.array(bq)),
                   dbeta_q=np.ascontiguousarray(np.array(dbq)), rc=np.array(raw_rc),
                   raw_l=np.array(raw_l, dtype=np.int32), d_ha=D)


# --------------------------------------------------------------------------
# named workloads
# --------------------------------------------------------------------------

def make_system(name: str, seed: int = 7) -> System:
    """Named systems: 'fcc2' (24^3, Ecut 15 Ha, s+p), 'sc8' (36^3, 17.5 Ha, s+p),
    'sc64' (72^3, 20 Ha, s+p+d), 'tiny' (12^3, 4 Ha, s+p, for fast tests)."""
    if name == "fcc2":
        lat, tau = diamond_fcc(10.26)
        n, ecut, lmax = (24, 24, 24), 15.0, 1
    elif name == "sc8":
        lat, tau = diamond_sc(10.26, 1)
        n, ecut, lmax = (36, 36, 36), 17.5, 1
    elif name == "sc64":
        lat, tau = diamond_sc(10.26, 2)
        n, ecut, lmax = (72, 72, 72), 20.0, 2
    elif name == "tiny":
        lat, tau = diamond_fcc(10.26)
        n, ecut, lmax = (12, 12, 12), 4.0, 1
    elif name == "tinyd":
        lat, tau = diamond_fcc(10.26)
        n, ecut, lmax = (15, 16, 18), 5.0, 2
    else:
        raise ValueError(f"unknown system {name!r}")
    sp = make_species(6, lmax, seed=seed)
    v = local_potential(lat, tau, *n)
    return System(name=name, lattice=lat, omega=float(abs(np.linalg.det(lat))), n1=n[0], n2=n[1], n3=n[2],
                  v_loc=np.ascontiguousarray(v), species=[sp],
                  atom_species=np.zeros(tau.shape[0], dtype=np.int32),
                  atom_z=np.full(tau.shape[0], 6, dtype=np.int32),
                  atom_tau=np.ascontiguousarray(tau), ecut=ecut)


def default_kpoint(name: str):
    return {"fcc2": (0.25, 0.25, 0.25), "tiny": (0.25, 0.25, 0.25), "tinyd": (0.1, -0.2, 0.3),
            "sc8": (0.0, 0.0, 0.0), "sc64": (0.0, 0.0, 0.0)}[name]


def mp_grid(m: int):
    """Monkhorst-Pack fractional k-points (unshifted offsets (2i-m-1)/(2m))."""
    v = [(2 * i - m - 1) / (2.0 * m) for i in range(1, m + 1)]
    return [(a, b, c) for a in v for b in v for c in v]


def make_bands(kp: KPoint, nb: int, seed: int = 11) -> np.ndarray:
    """[nb, npw] complex128: Gaussian entries * 1/(1+|k+G|^2)^2, orthonormalised (Cholesky-QR)."""
    rng = np.random.default_rng(seed)
    q2 = 2.0 * kp.kinetic
    w = 1.0 / (1.0 + q2) ** 2
    X = (rng.standard_normal((kp.npw, nb)) + 1j * rng.standard_normal((kp.npw, nb))) * w[:, None]
    for _ in range(2):
        S = X.conj().T @ X
        L = np.linalg.cholesky(S)
        X = np.linalg.solve(L.conj(), X.T).T
    return np.ascontiguousarray(X.T)


# --------------------------------------------------------------------------
# reference spec writer (inputs for oracle/ref_driver.cpp)
# --------------------------------------------------------------------------

def _radial_upf(l: int, rc: float, r: np.ndarray) -> np.ndarray:
    """UPF-convention r*beta(r) whose Fourier-Bessel transform is q^l exp(-q^2 rc^2/4)."""
    C = 4.0 * math.pi * math.sqrt(math.pi) * rc ** (2 * l + 3) / 2 ** (l + 2)
    return r ** (l + 1) * np.exp(-(r / rc) ** 2) / C


def write_spec(path: str, sysm: System, kpts: List[KPoint], psi: List[np.ndarray],
               dr: float = 0.01, r_max: float = 12.0):
    nr = int(round(r_max / dr)) + 1
    r = np.arange(nr) * dr
    rab = np.full(nr, dr)
    with open(path, "wb") as f:
        f.write(b"HPSISPC1")
        f.write(struct.pack("3i", sysm.n1, sysm.n2, sysm.n3))
        f.write(np.ascontiguousarray(sysm.lattice, dtype=np.float64).tobytes())
        f.write(struct.pack("d", sysm.ecut))
        f.write(struct.pack("i", sysm.n_atoms))
        f.write(np.ascontiguousarray(sysm.atom_z, dtype=np.int32).tobytes())
        f.write(np.ascontiguousarray(sysm.atom_tau, dtype=np.float64).tobytes())
        f.write(np.ascontiguousarray(sysm.v_loc, dtype=np.float64).tobytes())
        f.write(struct.pack("i", len(sysm.species)))
        for sp in sysm.species:
            f.write(struct.pack("ii", sp.z, nr))
            f.write(r.tobytes())
            f.write(rab.tobytes())
            nraw = len(sp.raw_l)
            f.write(struct.pack("i", nraw))
            for i in range(nraw):
                f.write(struct.pack("ii", int(sp.raw_l[i]), nr))
                f.write(_radial_upf(int(sp.raw_l[i]), float(sp.rc[i]), r).tobytes())
            f.write(np.ascontiguousarray(2.0 * sp.d_ha, dtype=np.float64).tobytes())  # Ry
        f.write(struct.pack("i", len(kpts)))
        for kp in kpts:
            f.write(struct.pack("i", kp.npw))
            f.write(np.ascontiguousarray(kp.kvec, dtype=np.float64).tobytes())
            f.write(np.ascontiguousarray(kp.kinetic, dtype=np.float64).tobytes())
        nb = psi[0].shape[0] if psi else 0
        f.write(struct.pack("i", nb))
        for p in psi:
            f.write(np.ascontiguousarray(p, dtype=np.complex128).tobytes())


def read_golden(path: str):
    """Parse the fixture written by ``ref_driver golden``."""
    with open(path, "rb") as f:
        buf = f.read()
    off = 0

    def take(fmt):
        nonlocal off
        v = struct.unpack_from(fmt, buf, off)
        off += struct.calcsize(fmt)
        return v

    def arr(dtype, n):
        nonlocal off
        a = np.frombuffer(buf, dtype=dtype, count=n, offset=off).copy()
        off += a.nbytes
        return a

    assert buf[:8] == b"HPSIREF1"
    off = 8
    A = arr(np.float64, 9).reshape(3, 3)
    (omega,) = take("d")
    (nsp,) = take("i")
    species = []
    for _ in range(nsp):
        (z,) = take("i")
        dq, qmax, norm = take("3d")
        nt, nq = take("2i")
        ls, lams, bqs, dbqs = [], [], [], []
        for _ in range(nt):
            l, ib = take("2i")
            (lam,) = take("d")
            ls.append(l)
            lams.append(lam)
            bqs.append(arr(np.float64, nq))
            dbqs.append(arr(np.float64, nq))
        species.append(dict(z=z, dq=dq, q_max=qmax, norm=norm, proj_l=np.array(ls, dtype=np.int32),
                            lam=np.array(lams), beta_q=np.array(bqs), dbeta_q=np.array(dbqs)))
    nk, nb = take("2i")
    kpts = []
    for _ in range(nk):
        (ng,) = take("i")
        kf = arr(np.float64, 3)
        g = arr(np.int32, 3 * ng).reshape(ng, 3)
        K = arr(np.float64, 3 * ng).reshape(ng, 3)
        kin = arr(np.float64, ng)
        q = arr(np.float64, ng)
        th = arr(np.float64, ng)
        ph = arr(np.float64, ng)
        hpsi = arr(np.float64, 2 * ng * nb).view(np.complex128).reshape(nb, ng)
        grads = arr(np.float64, 6 * ng * nb).view(np.complex128).reshape(nb, 3, ng)
        kpts.append(dict(npw=ng, k_frac=kf, g_idx=g, kvec=K, kinetic=kin, q=q, theta=th, phi=ph,
                         hpsi=hpsi, grad=grads))
    assert off == len(buf), (off, len(buf))
    return dict(lattice=A, omega=omega, species=species, kpts=kpts, nband=nb)


def system_from_golden(sysm: System, gold) -> System:
    """The same system with the lattice/volume/tables exactly as the reference used them."""
    sps = []
    for s in gold["species"]:
        sps.append(Species(z=s["z"], proj_l=s["proj_l"], lam=s["lam"], dq=s["dq"], q_max=s["q_max"],
                           beta_q=np.ascontiguousarray(s["beta_q"]),
                           dbeta_q=np.ascontiguousarray(s["dbeta_q"])))
    return dataclasses.replace(sysm, lattice=gold["lattice"], omega=gold["omega"], species=sps)


def kpoint_from_golden(gk) -> KPoint:
    return KPoint(npw=gk["npw"], k_frac=gk["k_frac"], g_idx=np.ascontiguousarray(gk["g_idx"]),
                  kvec=np.ascontiguousarray(gk["kvec"]), kinetic=np.ascontiguousarray(gk["kinetic"]))
