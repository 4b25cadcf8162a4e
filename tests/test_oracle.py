"""The oracle (oracle/hpsi_oracle.c) pinned against the reference.

* end to end: the reference's own H|psi> and dH/dk|psi>, compiled from its
  sources and run on the same inputs (tests/golden/*.npz, made by
  tests/golden/make_golden.py);
* per component: the known-answer tests of the reference's unit tests —
  test/math/test_fft.cpp, test/math/test_sph_harmonics.cpp,
  test/H_psi/test_structure_factor.cpp — restated here, plus the rules of
  BetaqTables::interpolate (src/pseudo/ncpp_advance.cppm:644-674).
"""
import math
import os

import numpy as np
import pytest

from conftest import CASES, load_case, rel_err
from effmass_gb300 import abi


# ---------------------------------------------------------------- end to end
@pytest.mark.parametrize("case", CASES)
def test_oracle_matches_reference_hpsi(oracle_lib, case):
    sysm, kp, psi, href, _ = load_case(case)
    h = oracle_lib.hpsi(sysm, kp, psi)
    # same arithmetic in the same order: agreement to the last bits
    assert rel_err(h, href) <= 1e-14, case


@pytest.mark.parametrize("case", CASES)
def test_oracle_matches_reference_grad(oracle_lib, case):
    sysm, kp, psi, _, gref = load_case(case)
    g = oracle_lib.grad(sysm, kp, psi)
    assert rel_err(g, gref) <= 1e-14, case


@pytest.mark.parametrize("case", CASES)
def test_oracle_matches_reference_density(oracle_lib, case):
    """rho from the reference's buildDensity (src/support/density.cppm:41-94),
    occupations with one empty band, aliasing included (the 4^3 case)."""
    import numpy as np
    sysm, kp, psi, _, _ = load_case(case)
    z = np.load(os.path.join(os.path.dirname(__file__), "golden", f"{case}.npz"))
    rho = oracle_lib.density(sysm, kp, psi, z["occ"])
    assert rel_err(rho, z["rho"]) <= 1e-14, rel_err(rho, z["rho"])


@pytest.mark.parametrize("case", ["tiny", "tinyd"])
def test_oracle_beta_tables_match_reference(oracle_lib, case):
    """beta(q) and dbeta/dq tables built from the radial projectors the reference
    integrated (after its sortByL / diagonalizeNonlocal), against its own tables."""
    z = np.load(os.path.join(os.path.dirname(__file__), "golden", f"{case}.npz"))
    bq, dbq = oracle_lib.beta_tables(z["rad_r"], z["rad_rab"], bool(z["rad_uniform"]), z["rad_l"], z["rad_beta"],
                                     float(z["sp_dq"]), float(z["sp_q_max"]))
    assert bq.shape == z["sp_beta_q"].shape
    # the same operations in the same order: bit for bit
    assert np.array_equal(bq, z["sp_beta_q"]) and np.array_equal(dbq, z["sp_dbeta_q"])


@pytest.mark.parametrize("case", ["tiny", "tinyd", "fcc2"])
def test_oracle_spherical_coordinates_match_reference(oracle_lib, case):
    import os
    z = np.load(os.path.join(os.path.dirname(__file__), "golden", f"{case}.npz"))
    q, th, ph = oracle_lib.spherical(z["kvec"])
    assert np.array_equal(q, z["q"]) and np.array_equal(th, z["theta"]) and np.array_equal(ph, z["phi"])


def test_oracle_threads_agree(oracle_lib):
    sysm, kp, psi, href, _ = load_case("fcc2")
    h4 = oracle_lib.hpsi(sysm, kp, psi, threads=4)
    assert rel_err(h4, href) <= 1e-14


def test_oracle_hermitian(oracle_lib):
    sysm, kp, psi, _, _ = load_case("tinyd")
    h = oracle_lib.hpsi(sysm, kp, psi)
    M = psi.conj() @ h.T  # <psi_m|H|psi_n>
    assert np.abs(M - M.conj().T).max() <= 1e-12 * np.abs(M).max()


def test_oracle_velocity_is_hermitian_and_consistent(oracle_lib):
    sysm, kp, psi, _, gref = load_case("tiny")
    V = oracle_lib.velocity(sysm, kp, psi)
    for a in range(3):
        assert np.abs(V[a] - V[a].conj().T).max() <= 1e-12 * np.abs(V[a]).max()
        assert np.allclose(V[a], psi.conj() @ gref[a].T, rtol=0, atol=1e-13 * np.abs(V[a]).max())


# ------------------------------------------------- FFT (test/math/test_fft.cpp)
def _fft3(oracle_lib, x, shape, direction):
    return oracle_lib.fft3d(np.asarray(x, dtype=np.complex128).reshape(shape), direction).ravel()


def test_fft_delta_n8(oracle_lib):
    x = np.zeros(8, complex)
    x[0] = 1
    y = _fft3(oracle_lib, x, (1, 1, 8), "R2G")
    assert np.allclose(y, 1.0 / 8, rtol=0, atol=1e-12)
    z = _fft3(oracle_lib, y, (1, 1, 8), "G2R")
    assert np.abs(z - x).max() < 1e-14


def test_fft_cosine_and_constant(oracle_lib):
    n = 8
    x = np.cos(2 * np.pi * np.arange(n) / n).astype(complex)
    y = _fft3(oracle_lib, x, (1, 1, n), "R2G")
    assert abs(abs(y[1]) - 0.5) < 1e-12 and abs(abs(y[n - 1]) - 0.5) < 1e-12
    c = _fft3(oracle_lib, np.ones(n), (1, 1, n), "R2G")
    assert abs(abs(c[0]) - 1) < 1e-12 and np.abs(c[1:]).max() < 1e-12


def test_fft_small_lengths(oracle_lib):
    y = _fft3(oracle_lib, [1, 0], (1, 1, 2), "G2R")
    assert np.abs(y - 1).max() < 1e-15
    x6 = np.zeros(6, complex)
    x6[0] = 1
    assert np.abs(_fft3(oracle_lib, _fft3(oracle_lib, x6, (1, 1, 6), "R2G"), (1, 1, 6), "G2R") - x6).max() < 1e-14
    i = np.arange(45)
    x45 = i * 0.1 + 1j * np.sin(0.1 * i)
    r = _fft3(oracle_lib, _fft3(oracle_lib, x45, (1, 1, 45), "R2G"), (1, 1, 45), "G2R")
    assert np.abs(r - x45).max() < 1e-12


def test_fft3d_roundtrip_6x8x5(oracle_lib):
    i = np.arange(240)
    g = (i % 7) + 1j * ((i * i) % 11)
    r = _fft3(oracle_lib, _fft3(oracle_lib, g, (6, 8, 5), "G2R"), (6, 8, 5), "R2G")
    assert np.abs(r - g).max() < 1e-12
    d = np.zeros(240, complex)
    d[0] = 1
    r = _fft3(oracle_lib, _fft3(oracle_lib, d, (6, 8, 5), "G2R"), (6, 8, 5), "R2G")
    assert np.abs(r - d).max() < 1e-14


@pytest.mark.parametrize("shape", [(24, 24, 24), (15, 16, 18), (1, 7, 13)])
def test_fft3d_conventions_vs_numpy(oracle_lib, shape):
    rng = np.random.default_rng(3)
    g = rng.standard_normal(shape) + 1j * rng.standard_normal(shape)
    # G2R = unnormalised backward (exp(+iGr)); R2G = forward with 1/n per axis
    b = oracle_lib.fft3d(g, "G2R")
    assert rel_err(b, np.fft.ifftn(g) * g.size) < 1e-14
    f = oracle_lib.fft3d(g, "R2G")
    assert rel_err(f, np.fft.fftn(g) / g.size) < 1e-14


# ------------------------------- Y_lm (test/math/test_sph_harmonics.cpp)
C1 = math.sqrt(3 / (4 * math.pi))


def _ylm(oracle_lib, lmax, th, ph):
    y, dth, dph = oracle_lib.ylm(lmax, np.array([th]), np.array([ph]))
    idx = lambda l, m: l * l + l + m  # noqa: E731
    return (lambda l, m: y[idx(l, m), 0]), (lambda l, m: dth[idx(l, m), 0]), (lambda l, m: dph[idx(l, m), 0])


def test_ylm_closed_forms(oracle_lib):
    Y, _, _ = _ylm(oracle_lib, 3, 0.0, 0.0)
    assert abs(Y(0, 0) - 1 / (2 * math.sqrt(math.pi))) < 1e-12
    Y, _, _ = _ylm(oracle_lib, 3, 0.5, 0.0)
    assert abs(Y(1, 0) - C1 * math.cos(0.5)) < 1e-12
    Y, _, _ = _ylm(oracle_lib, 3, 0.5, 0.3)
    assert abs(Y(1, 1) + C1 * math.sin(0.5) * math.cos(0.3)) < 1e-12  # Condon-Shortley
    assert abs(Y(1, -1) + C1 * math.sin(0.5) * math.sin(0.3)) < 1e-12


def test_ylm_theta_zero_limits(oracle_lib):
    Y, DT, DP = _ylm(oracle_lib, 5, 0.0, 0.3)
    assert abs(Y(5, 0) - math.sqrt(11 / (4 * math.pi))) < 1e-12
    assert abs(Y(5, 3)) < 1e-12
    assert abs(DT(1, 1) + C1 * math.cos(0.3)) < 1e-12
    assert abs(DT(1, -1) + C1 * math.sin(0.3)) < 1e-12
    for l in range(2, 5):
        for m in range(2, l + 1):
            assert abs(DT(l, m)) < 1e-14 and abs(DT(l, -m)) < 1e-14


def test_ylm_angular_gradients(oracle_lib):
    th, ph = 0.7, 0.3
    Y, DT, DP = _ylm(oracle_lib, 4, th, ph)
    st = math.sin(th)
    assert abs(DT(0, 0)) < 1e-12
    assert abs(DT(1, 0) + C1 * st) < 1e-12
    for l in range(5):
        assert abs(DP(l, 0)) < 1e-12
        for m in range(1, l + 1):
            assert abs(DP(l, m) - (-m / st) * Y(l, -m)) < 1e-12
            assert abs(DP(l, -m) - (m / st) * Y(l, m)) < 1e-12
    # finite differences (1e-6)
    h = 1e-6
    Yp, _, _ = _ylm(oracle_lib, 4, th + h, ph)
    Ym, _, _ = _ylm(oracle_lib, 4, th - h, ph)
    Yq, _, _ = _ylm(oracle_lib, 4, th, ph + h)
    Yr, _, _ = _ylm(oracle_lib, 4, th, ph - h)
    for l in range(5):
        for m in range(-l, l + 1):
            assert abs((Yp(l, m) - Ym(l, m)) / (2 * h) - DT(l, m)) < 1e-6
            assert abs((Yq(l, m) - Yr(l, m)) / (2 * h) - st * DP(l, m)) < 1e-6


# ----------------- structure factor (test/H_psi/test_structure_factor.cpp)
def test_structure_factor_known_answers(oracle_lib):
    rc, s = oracle_lib.structure_factor([[5, -3, 2]], [0.1, 0.2, 0.3], [0, 0, 0], (20, 20, 32))
    assert rc == 0 and abs(s[0] - 1) < 1e-12
    g, k, tau = np.array([2, -1, 3]), np.array([0.1, 0.2, 0.3]), np.array([0.125, 0.25, 0.375])
    rc, s = oracle_lib.structure_factor([g], k, tau, (20, 20, 32))
    arg = -2 * math.pi * float(np.dot(k + g, tau))
    assert abs(s[0] - complex(math.cos(arg), math.sin(arg))) < 1e-12
    gs = np.stack(np.meshgrid(*[np.arange(-5, 5)] * 3, indexing="ij"), -1).reshape(-1, 3)
    rc, s = oracle_lib.structure_factor(gs, [0.125, 0.25, 0.375], tau, (20, 20, 32))
    assert np.abs(np.abs(s) - 1).max() < 1e-12
    direct = np.exp(-2j * np.pi * ((gs + [0.125, 0.25, 0.375]) @ tau))
    assert np.abs(s - direct).max() < 1e-12


def test_structure_factor_cache_range(oracle_lib):
    # cache index g + n/2 + 4 must lie in [0, n+8) (src/H_psi/structure_factor.cppm:66-72)
    assert oracle_lib.structure_factor([[-10, 0, 0]], [0, 0, 0], [0.1, 0, 0], (12, 12, 12))[0] == 0
    assert oracle_lib.structure_factor([[-11, 0, 0]], [0, 0, 0], [0.1, 0, 0], (12, 12, 12))[0] == abi.HPSI_ERR_RANGE
    assert oracle_lib.structure_factor([[9, 0, 0]], [0, 0, 0], [0.1, 0, 0], (12, 12, 12))[0] == 0
    assert oracle_lib.structure_factor([[10, 0, 0]], [0, 0, 0], [0.1, 0, 0], (12, 12, 12))[0] == abi.HPSI_ERR_RANGE


# -------------- beta(q) interpolation (src/pseudo/ncpp_advance.cppm:644-674)
def test_beta_interp_rules(oracle_lib):
    dq, qmax = 0.01, 20.0
    nq = int(math.ceil(qmax / dq)) + 1 + 3
    q = np.arange(nq) * dq
    cubic = 0.3 - 1.2 * q + 0.7 * q ** 2 - 0.05 * q ** 3
    norm = 0.5
    # exact on cubic tables (4-point Lagrange), including the i0 < 0 clamp region
    for qq in [0.0, 0.004, 0.01, 0.0137, 1.2345, 19.999, 20.0]:
        rc, v = oracle_lib.beta_interp(cubic, dq, qmax, norm, qq)
        assert rc == 0
        exact = (0.3 - 1.2 * qq + 0.7 * qq ** 2 - 0.05 * qq ** 3) * norm
        assert abs(v - exact) < 1e-9, qq
    rc, v = oracle_lib.beta_interp(cubic, dq, qmax, norm, 0.0)
    assert v == cubic[0] * norm
    assert oracle_lib.beta_interp(cubic, dq, qmax, norm, 20.0000001)[0] == abi.HPSI_ERR_RANGE
    assert oracle_lib.beta_interp(cubic, dq, qmax, norm, -1e-9)[0] == abi.HPSI_ERR_RANGE


def test_solid_harmonics_table_matches_reference_ylm(oracle_lib):
    """effmass_gb300/csrc/solid_harmonics.inc (R_lm = |K|^l Y_lm, used by the
    Hessian's projector derivatives) against the oracle's Y_lm, which is pinned to
    the reference's RealSphericalHarmonicsEngine."""
    import re
    txt = open(os.path.join(os.path.dirname(__file__), "..", "effmass_gb300", "csrc", "solid_harmonics.inc")).read()
    rows = re.findall(r"\{(\{.*?\})\},\s*// l=(\d+) m=(-?\d+)", txt)
    assert len(rows) == 25
    rng = np.random.default_rng(0)
    K = rng.standard_normal((64, 3)) * rng.uniform(0.2, 3.0, (64, 1))
    q = np.linalg.norm(K, axis=1)
    Y = oracle_lib.ylm(4, np.arccos(K[:, 2] / q), np.arctan2(K[:, 1], K[:, 0]))[0]
    for idx, (body, l, m) in enumerate(rows):
        l = int(l)
        assert idx == l * l + l + int(m)
        R = np.zeros(len(q))
        for c, a, b, cz in re.findall(r"\{([-0-9.e]+), (\d+), (\d+), (\d+)\}", body):
            R += float(c) * K[:, 0] ** int(a) * K[:, 1] ** int(b) * K[:, 2] ** int(cz)
        assert np.abs(R / q ** l - Y[idx]).max() <= 1e-14 * max(1.0, np.abs(Y[idx]).max()), (l, m)
