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

from conftest import rel_err
from effmass_gb300 import system as S
from oracle import oracle as O

pytestmark = pytest.mark.skipif(not os.path.exists(O.REF_DRIVER), reason="reference build (oracle/_ref) absent")


def _reference(sysm, kp, psi):
    """The reference's golden record for one k-point and its bands."""
    with tempfile.TemporaryDirectory() as td:
        spec, gold = os.path.join(td, "spec.bin"), os.path.join(td, "gold.bin")
        S.write_spec(spec, sysm, [kp], [psi])
        subprocess.run([O.REF_DRIVER, "golden", spec, gold, os.path.join(td, "wd")], check=True,
                       stderr=subprocess.DEVNULL, timeout=600)
        return S.read_golden(gold)


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


def _as_used(sysm, g):
    """System and k-point as the reference used them: its own beta/dbeta tables
    and lambda (after its per-l diagonalisation), its G-sphere views."""
    sp, gk = g["species"][0], g["kpts"][0]
    species = S.Species(z=6, proj_l=sp["proj_l"], lam=sp["lam"], dq=float(sp["dq"]), q_max=float(sp["q_max"]),
                        beta_q=np.ascontiguousarray(sp["beta_q"]), dbeta_q=np.ascontiguousarray(sp["dbeta_q"]))
    used = S.System(name=sysm.name, lattice=g["lattice"], omega=float(g["omega"]), n1=sysm.n1, n2=sysm.n2,
                    n3=sysm.n3, v_loc=np.ascontiguousarray(sysm.v_loc), species=[species],
                    atom_species=np.ascontiguousarray(sysm.atom_species),
                    atom_z=np.full(len(sysm.atom_tau), 6, dtype=np.int32),
                    atom_tau=np.ascontiguousarray(sysm.atom_tau), ecut=0.0)
    kp = S.KPoint(npw=int(gk["g_idx"].shape[0]), k_frac=gk["k_frac"], g_idx=np.ascontiguousarray(gk["g_idx"]),
                  kvec=np.ascontiguousarray(gk["kvec"]), kinetic=np.ascontiguousarray(gk["kinetic"]))
    return used, kp, gk


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
    used, kp_used, gk = _as_used(sysm, _reference(sysm, kp, psi))
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
