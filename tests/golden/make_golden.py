#!/usr/bin/env python3
"""Regenerate the golden fixtures in tests/golden/ from the reference itself.

Each fixture is produced by running the reference's own H|psi> and dH/dk|psi>
(compiled from its sources by oracle/Makefile `ref`, driven by
oracle/ref_driver.cpp) on a synthetic system from effmass_gb300.system.  The
fixture stores everything the reference used — lattice, volume, raw beta and
dbeta tables with lambda after its per-l diagonalisation, the G-sphere views
(g_idx, K, kinetic, q, theta, phi, inferred k), V_loc, atoms, psi — and its
outputs hpsi and grad, and the reference's charge density (buildDensity) of the
same bands with seeded occupations.

Run in a checkout where the reference sources are available:
    python tests/golden/make_golden.py
"""
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from effmass_gb300 import system as S  # noqa: E402
from oracle import oracle as O  # noqa: E402

# name -> (system, k_frac, n_bands, grid override, species override)
CASES = {
    # 12^3 grid, s+p, k=(1/4,1/4,1/4): the smallest complete case
    "tiny": ("tiny", (0.25, 0.25, 0.25), 3, None),
    # non-cubic 15x16x18 grid (radices 3,5 / 2,4 / 2,3), s+p+d, general k
    "tinyd": ("tinyd", (0.1, -0.2, 0.3), 3, None),
    # 4^3 grid too small for the sphere: 40 of its 104 G-vectors share a grid
    # point with another (the reference's scatter keeps the last one, its
    # gather reads it for all)
    "alias": ("tiny", (0.25, 0.25, 0.25), 2, (4, 4, 4)),
    # the 2-atom fcc cell at Ecut 15 Ha, 24^3, 8 bands (the plain FP64 configuration)
    "fcc2": ("fcc2", (0.25, 0.25, 0.25), 8, None),
    # 8-atom simple-cubic cell, 36^3, off-Gamma k
    "sc8": ("sc8", (0.125, 0.375, -0.375), 2, None),
}


def read_tables(path):
    """The first species of a TABREF01 file: mesh, rotated beta(r) and the
    reference's beta(q), dbeta/dq and d2beta/dq2 tables."""
    raw = open(path, "rb").read()
    assert raw[:8] == b"TABREF01"
    o = 8

    def ints(n):
        nonlocal o
        v = np.frombuffer(raw, dtype=np.int32, count=n, offset=o)
        o += 4 * n
        return v

    def dbl(n):
        nonlocal o
        v = np.frombuffer(raw, dtype=np.float64, count=n, offset=o).copy()
        o += 8 * n
        return v

    ints(1)  # species count
    _z, mtype, nr = ints(3)
    r, rab = dbl(nr), dbl(nr)
    (np_,) = ints(1)
    ls, betas = [], np.zeros((np_, nr))
    for i in range(np_):
        l, ln = ints(2)
        ls.append(l)
        betas[i, :ln] = dbl(ln)
    nt, nq = ints(2)
    bq = dbl(nt * nq).reshape(nt, nq)
    dbq = dbl(nt * nq).reshape(nt, nq)
    # D2BetaqTables (files written before the driver exported them end here)
    d2bq = dbl(nt * nq).reshape(nt, nq) if len(raw) >= o + 8 * nt * nq else None
    return dict(uniform=int(mtype == 0), r=r, rab=rab, l=np.array(ls, dtype=np.int32), beta=betas,
                beta_q=bq, dbeta_q=dbq, d2beta_q=d2bq)


def make_case(name, sysname, kf, nb, grid):
    sysm = S.make_system(sysname)
    if grid is not None:
        sysm.n1, sysm.n2, sysm.n3 = grid
        sysm.v_loc = S.local_potential(sysm.lattice, sysm.atom_tau, *grid)
    kp = S.g_sphere(sysm.lattice, kf, sysm.ecut)
    psi = S.make_bands(kp, nb, seed=17)
    # occupations in [0, 2] with one empty band (the reference skips those)
    occ = np.random.default_rng(23).uniform(0.0, 2.0, nb)
    occ[nb // 2] = 0.0
    with tempfile.TemporaryDirectory() as td:
        spec = os.path.join(td, "spec.bin")
        gold = os.path.join(td, "gold.bin")
        S.write_spec(spec, sysm, [kp], [psi])
        subprocess.run([O.REF_DRIVER, "golden", spec, gold, os.path.join(td, "wd")], check=True,
                       stderr=subprocess.DEVNULL)
        g = S.read_golden(gold)
        # the reference's buildDensity on the same k-point and bands
        occ_txt, rho_bin = os.path.join(td, "occ.txt"), os.path.join(td, "rho.bin")
        np.savetxt(occ_txt, occ, fmt="%.17g")
        subprocess.run([O.REF_DRIVER, "density", spec, occ_txt, rho_bin, os.path.join(td, "wd2")], check=True,
                       stderr=subprocess.DEVNULL)
        # the radial inputs the reference integrated into its beta / dbeta tables
        tab_bin = os.path.join(td, "tab.bin")
        subprocess.run([O.REF_DRIVER, "tables", spec, tab_bin, os.path.join(td, "wd3")], check=True,
                       stderr=subprocess.DEVNULL)
        rad = read_tables(tab_bin)
        raw = open(rho_bin, "rb").read()
        assert raw[:8] == b"RHOREF01"
        dims = np.frombuffer(raw[8:20], dtype=np.int32)
        rho = np.frombuffer(raw[20:], dtype=np.float64).copy()
        assert tuple(dims) == (sysm.n1, sysm.n2, sysm.n3) and rho.size == int(np.prod(dims))
    sp = g["species"][0]
    gk = g["kpts"][0]
    out = dict(
        n=np.array([sysm.n1, sysm.n2, sysm.n3], dtype=np.int32),
        lattice=g["lattice"], omega=np.array(g["omega"]), v_loc=sysm.v_loc,
        atom_tau=sysm.atom_tau, atom_species=sysm.atom_species,
        sp_proj_l=sp["proj_l"], sp_lam=sp["lam"], sp_dq=np.array(sp["dq"]), sp_q_max=np.array(sp["q_max"]),
        sp_beta_q=sp["beta_q"], sp_dbeta_q=sp["dbeta_q"],
        k_frac=gk["k_frac"], g_idx=gk["g_idx"], kvec=gk["kvec"], kinetic=gk["kinetic"],
        q=gk["q"], theta=gk["theta"], phi=gk["phi"],
        psi=psi, hpsi=gk["hpsi"], grad=gk["grad"], occ=occ, rho=rho,
        rad_uniform=np.array(rad["uniform"]), rad_r=rad["r"], rad_rab=rad["rab"], rad_l=rad["l"],
        rad_beta=rad["beta"])
    # the tables of the tables mode are the same the golden mode exported
    assert np.array_equal(rad["beta_q"], sp["beta_q"]) and np.array_equal(rad["dbeta_q"], sp["dbeta_q"])
    np.savez_compressed(os.path.join(HERE, f"{name}.npz"), **out)
    return kp.npw


def main():
    if not O.build_ref(quiet=False):
        raise SystemExit("reference driver unavailable (needs the reference sources)")
    for name, (sysname, kf, nb, grid) in CASES.items():
        npw = make_case(name, sysname, kf, nb, grid)
        print(f"{name}: npw={npw} nb={nb}")


if __name__ == "__main__":
    main()
