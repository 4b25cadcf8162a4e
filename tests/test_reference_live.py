"""The oracle against the reference itself on inputs the fixtures do not
hold: the reference, compiled from its own sources (oracle/Makefile `ref`),
runs here on freshly seeded systems, k-points and bands, and the oracle must
reproduce its H|psi> and dH/dk|psi> to the last bits.  Skipped where that
build is absent: it needs the reference's sources, which only the build host
has."""
import os
import subprocess
import tempfile

import numpy as np
import pytest

from conftest import as_used, reference_golden, rel_err
from effmass_gb300 import system as S
from oracle import oracle as O

pytestmark = pytest.mark.skipif(not os.path.exists(O.REF_DRIVER), reason="reference build (oracle/_ref) absent")


def _reference(sysm, kp, psi):
    """The reference's golden record for one k-point and its bands."""
    return reference_golden(sysm, [kp], [psi])


def _reference_density(sysm, kp, psi, occ):
    """The reference's buildDensity of the bands with occupations occ."""
    with tempfile.TemporaryDirectory() as td:
        spec, occ_txt, rho_bin = (os.path.join(td, f) for f in ("spec.bin", "occ.txt", "rho.bin"))
        S.write_spec(spec, sysm, [kp], [psi])
        np.savetxt(occ_txt, occ, fmt="%.17g")
        subprocess.run([O.REF_DRIVER, "density", spec, occ_txt, rho_bin, os.path.join(td, "wd")], check=True,
                       stderr=subprocess.DEVNULL, timeout=600)
        raw = open(rho_bin, "rb").read()
    assert raw[:8] == b"RHOREF01"
    dims = tuple(np.frombuffer(raw[8:20], dtype=np.int32))
    assert dims == (sysm.n1, sysm.n2, sysm.n3)
    return np.frombuffer(raw[20:], dtype=np.float64).copy()


@pytest.mark.parametrize("name,k_frac,grid,seed", [
    ("tinyd", (0.37, -0.11, 0.05), None, 101),       # s+p+d, non-cubic 15x16x18, general k
    ("tiny", (-0.2, 0.3, 0.45), (5, 6, 7), 202),     # prime grid lengths 5 and 7
    ("tiny", (0.0, 0.0, 0.0), (4, 4, 4), 303),       # Gamma on a grid the sphere aliases on
])
def test_oracle_matches_live_reference(name, k_frac, grid, seed):
    sysm = S.make_system(name)
    if grid is not None:
        sysm.n1, sysm.n2, sysm.n3 = grid
        sysm.v_loc = S.local_potential(sysm.lattice, sysm.atom_tau, *grid)
    kp = S.g_sphere(sysm.lattice, k_frac, sysm.ecut)
    psi = S.make_bands(kp, 3, seed=seed)
    used, kp_used, gk = as_used(sysm, _reference(sysm, kp, psi))
    assert np.array_equal(kp_used.g_idx, kp.g_idx)  # the reference read the G-sphere in the order written
    h = O.hpsi(used, kp_used, psi)
    assert rel_err(h, gk["hpsi"]) <= 1e-14
    grad = O.grad(used, kp_used, psi)
    assert rel_err(grad, np.transpose(gk["grad"], (1, 0, 2))) <= 1e-14
    # charge density with one empty band (the reference skips it)
    occ = np.array([2.0, 0.0, 0.7])
    rho = O.density(used, kp_used, psi, occ)
    assert rel_err(rho.ravel(), _reference_density(sysm, kp, psi, occ)) <= 1e-14


@pytest.mark.parametrize("name,dr,r_max", [("tinyd", 0.02, 10.0), ("sc8", 0.005, 14.0)])
def test_oracle_beta_tables_match_live_reference(name, dr, r_max):
    """beta(q) and dbeta/dq tables: the reference integrates radial projectors
    written on a mesh the fixtures do not use; the oracle, given the radial
    inputs the reference reports, builds the same tables bit for bit."""
    import sys
    sys.path.insert(0, os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden"))
    from make_golden import read_tables
    sysm = S.make_system(name)
    kp = S.g_sphere(sysm.lattice, (0.1, 0.2, 0.3), sysm.ecut)
    psi = S.make_bands(kp, 1, seed=7)
    with tempfile.TemporaryDirectory() as td:
        spec, tab = os.path.join(td, "spec.bin"), os.path.join(td, "tab.bin")
        S.write_spec(spec, sysm, [kp], [psi], dr=dr, r_max=r_max)
        subprocess.run([O.REF_DRIVER, "tables", spec, tab, os.path.join(td, "wd")], check=True,
                       stderr=subprocess.DEVNULL, timeout=600)
        rad = read_tables(tab)
    # the reference's finalize builds its tables at its defaults dq = 0.01,
    # q_max = 20 (src/H_psi/hamiltonian.cpp:307-309): 2004 points
    bq, dbq = O.beta_tables(rad["r"], rad["rab"], bool(rad["uniform"]), rad["l"], rad["beta"], 0.01, 20.0)
    assert bq.shape == rad["beta_q"].shape
    assert np.array_equal(bq, rad["beta_q"]) and np.array_equal(dbq, rad["dbeta_q"])
    # D2BetaqTables (src/pseudo/ncpp_advance.cppm:908-1085), which the Hessian
    # needs: bit for bit, and rebuilt from the Hessian's F0, F1, F3 tables
    d2 = O.d2beta_tables(rad["r"], rad["rab"], bool(rad["uniform"]), rad["l"], rad["beta"], 0.01, 20.0)
    assert np.array_equal(d2, rad["d2beta_q"])
    from test_oracle_hessian import beta_from_f
    f = O.hess_tables(rad["r"], rad["rab"], bool(rad["uniform"]), rad["l"], rad["beta"], 0.01, 20.0)
    q = np.arange(f.shape[-1]) * 0.01
    for p, l in enumerate(rad["l"]):
        b2 = beta_from_f(f[:, p], int(l), q)[2]
        sel = q > 0 if l >= 2 else np.ones_like(q, dtype=bool)
        assert np.abs(b2[sel] - d2[p][sel]).max() <= 1e-12 * np.abs(d2[p]).max(), (p, l)
