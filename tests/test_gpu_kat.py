"""Known-answer tests of the device FFT, Y_lm and structure-factor kernels,
each on its own (the H|psi> parity tests see them only through the whole
operator).

FFT (hpsi_selftest_fft3d: the line transforms the local-term kernels are built
from, on a full grid): the reference's FFT known answers
(test/math/test_fft.cpp:21-126 — a delta, a cosine and a constant along one
axis of length 8, n = 2, round trips at n = 6, 45 and on a 6x8x5 grid), then
numpy's FFT in the reference's convention (G->r = N * ifftn, r->G = fftn / N)
for the complex64 compile-time plans and register transform (24^3, 36^3,
64^3, 72^3) and a grid that needs the wide radices 7, 11 and 13.

Y_lm (hpsi_selftest_kpoint_tables: the tables the projector build reads): the
reference's closed forms with the Condon-Shortley phase
(test/math/test_sph_harmonics.cpp:37-60, the theta = 0 limits of the
angular gradients :273-292) for l <= 2 on every G of a general k-point, and
the oracle's restatement of the reference's recurrences for l <= 2.

S(g,k) (the same entry point): exp(-2 pi i (k+g).tau) for tau = 0 (S = 1) and
tau = (1/8, 1/4, 3/8) as in test/H_psi/test_structure_factor.cpp:27-60.
"""
import ctypes as C

import numpy as np
import pytest

from conftest import rel_err
from effmass_gb300 import abi

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def lib():
    from effmass_gb300.build import build
    from effmass_gb300._lib import load
    build()
    return load()


def fft3d(lib, grid, direction, prec="fp64"):
    g = np.ascontiguousarray(grid, dtype=np.complex128).copy()
    n1, n2, n3 = g.shape
    st = lib.hpsi_selftest_fft3d(n1, n2, n3, C.c_void_p(g.ctypes.data), +1 if direction == "G2R" else -1,
                                 abi.PRECISIONS[prec])
    assert st == abi.HPSI_OK
    return g


@pytest.mark.parametrize("prec,eps", [("fp64", 1e-12), ("fp32", 1e-6)])
def test_fft_1d_known_answers(lib, prec, eps):
    n = 8
    d = np.zeros((1, 1, n), complex)
    d[0, 0, 0] = 1.0
    r = fft3d(lib, d, "R2G", prec)
    assert np.abs(r - 1.0 / n).max() < eps                     # delta -> 1/n everywhere
    assert np.abs(fft3d(lib, r, "G2R", prec) - d).max() < eps  # and back
    c = np.cos(2 * np.pi * np.arange(n) / n).astype(complex).reshape(1, 1, n)
    rc = fft3d(lib, c, "R2G", prec)[0, 0]
    assert abs(abs(rc[1]) - 0.5) < eps and abs(abs(rc[n - 1]) - 0.5) < eps
    assert np.abs(np.delete(rc, [1, n - 1])).max() < eps
    k = fft3d(lib, np.ones((1, 1, n), complex), "R2G", prec)[0, 0]
    assert abs(abs(k[0]) - 1.0) < eps and np.abs(k[1:]).max() < eps
    two = fft3d(lib, np.array([[[1.0, 0.0]]], complex), "G2R", prec)[0, 0]
    assert np.abs(two - 1.0).max() < eps
    six = np.zeros((1, 1, 6), complex)
    six[0, 0, 0] = 1.0
    assert np.abs(fft3d(lib, fft3d(lib, six, "R2G", prec), "G2R", prec) - six).max() < eps
    i = np.arange(45)
    x45 = (i * 0.1 + 1j * np.sin(0.1 * i)).reshape(1, 1, 45)
    assert np.abs(fft3d(lib, fft3d(lib, x45, "R2G", prec), "G2R", prec) - x45).max() < eps * 10


@pytest.mark.parametrize("prec,eps", [("fp64", 1e-12), ("fp32", 1e-5)])
def test_fft_3d_round_trips(lib, prec, eps):
    n1, n2, n3 = 6, 8, 5
    i = np.arange(n1 * n2 * n3)
    g = ((i % 7) + 1j * ((i * i) % 11)).reshape(n1, n2, n3)
    assert np.abs(fft3d(lib, fft3d(lib, g, "G2R", prec), "R2G", prec) - g).max() < eps
    d = np.zeros((n1, n2, n3), complex)
    d[0, 0, 0] = 1.0
    assert np.abs(fft3d(lib, fft3d(lib, d, "G2R", prec), "R2G", prec) - d).max() < eps


@pytest.mark.parametrize("shape,prec,tol", [
    ((6, 8, 5), "fp64", 1e-13), ((15, 16, 18), "fp64", 1e-13), ((7, 11, 13), "fp64", 1e-13),
    ((24, 24, 24), "fp32", 1e-6), ((36, 36, 36), "fp32", 1e-6), ((64, 64, 64), "fp32", 1e-6),
    ((72, 72, 72), "fp32", 1e-6), ((7, 11, 13), "fp32", 1e-6), ((20, 27, 10), "fp32", 1e-6)])
def test_fft_matches_numpy(lib, shape, prec, tol):
    rng = np.random.default_rng(11)
    g = rng.standard_normal(shape) + 1j * rng.standard_normal(shape)
    N = np.prod(shape)
    assert rel_err(fft3d(lib, g, "G2R", prec), np.fft.ifftn(g) * N) <= tol
    assert rel_err(fft3d(lib, g, "R2G", prec), np.fft.fftn(g) / N) <= tol


def _tables(lib, H, kid, npw, lmax, natom):
    nlm = (lmax + 1) ** 2
    y = np.zeros((3, nlm, npw))
    sf = np.zeros((natom, npw), complex)
    st = lib.hpsi_selftest_kpoint_tables(H.ctx, kid, C.c_void_p(y.ctypes.data), C.c_void_p(sf.ctypes.data))
    assert st == abi.HPSI_OK
    return y, sf


def test_ylm_and_structure_factor_known_answers(lib, oracle_lib):
    from effmass_gb300 import system as S
    from effmass_gb300.hamiltonian import Hamiltonian
    sysm = S.make_system("tinyd")
    assert len(sysm.atom_tau) == 2
    sysm.atom_tau = np.ascontiguousarray([[0.0, 0.0, 0.0], [0.125, 0.25, 0.375]])
    kf = np.array([0.1, 0.2, 0.3])
    kp = S.g_sphere(sysm.lattice, tuple(kf), sysm.ecut)
    lmax = max(int(max(sp.proj_l)) for sp in sysm.species)
    assert lmax == 2
    with Hamiltonian(sysm) as H:
        H.set_kpoint(0, kp)
        y, sf = _tables(lib, H, 0, kp.npw, lmax, len(sysm.atom_tau))
    K = kp.kvec
    q = np.linalg.norm(K, axis=1)
    th = np.where(q > 0, np.arccos(np.clip(K[:, 2] / np.where(q > 0, q, 1), -1, 1)), 0.0)
    ph = np.where(q > 0, np.arctan2(K[:, 1], K[:, 0]), 0.0)
    ct, st_, cp, sp = np.cos(th), np.sin(th), np.cos(ph), np.sin(ph)
    a1, a2 = np.sqrt(3 / (4 * np.pi)), np.sqrt(15 / (4 * np.pi))
    closed = {  # index l*l + l + m, the reference's real Y_lm with the Condon-Shortley phase
        0: np.full_like(q, 0.5 / np.sqrt(np.pi)),
        1: -a1 * st_ * sp, 2: a1 * ct, 3: -a1 * st_ * cp,
        4: 0.5 * a2 * st_ ** 2 * np.sin(2 * ph), 5: -a2 * st_ * ct * sp,
        6: np.sqrt(5 / (16 * np.pi)) * (3 * ct ** 2 - 1), 7: -a2 * st_ * ct * cp,
        8: 0.5 * a2 * st_ ** 2 * np.cos(2 * ph)}
    for lm, v in closed.items():
        assert np.abs(y[0, lm] - v).max() <= 1e-13, lm
    # angular gradients of l = 1: d/dtheta and (1/sin theta) d/dphi
    assert np.abs(y[1, 2] - (-a1 * st_)).max() <= 1e-13
    assert np.abs(y[1, 3] - (-a1 * ct * cp)).max() <= 1e-13
    assert np.abs(y[2, 3] - (a1 * sp)).max() <= 1e-13
    assert np.abs(y[2, 1] - (-a1 * cp)).max() <= 1e-13
    # the oracle's restatement of the reference's recurrences (values and gradients)
    yo, dto, dpo = oracle_lib.ylm(lmax, th, ph)
    assert np.abs(y[0] - yo).max() <= 1e-14 and np.abs(y[1] - dto).max() <= 1e-14
    assert np.abs(y[2] - dpo).max() <= 1e-14
    # structure factors
    for a, tau in enumerate(sysm.atom_tau):
        ref = np.exp(-2j * np.pi * ((kf[None, :] + kp.g_idx) @ tau))
        assert np.abs(sf[a] - ref).max() <= 1e-13, a
    assert np.abs(sf[0] - 1.0).max() <= 1e-15  # tau = 0
