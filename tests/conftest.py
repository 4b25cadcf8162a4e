import os
import subprocess
import sys
import tempfile

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

from effmass_gb300 import system as S  # noqa: E402

GOLDEN = os.path.join(ROOT, "tests", "golden")
CASES = ["tiny", "tinyd", "alias", "fcc2", "sc8"]


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built libhpsi_gb300.so")


def load_case(name):
    """(System, KPoint, psi[nb,npw], hpsi_ref[nb,npw], grad_ref[3,nb,npw]) of a golden fixture."""
    z = np.load(os.path.join(GOLDEN, f"{name}.npz"))
    n = z["n"]
    sp = S.Species(z=6, proj_l=z["sp_proj_l"], lam=z["sp_lam"], dq=float(z["sp_dq"]), q_max=float(z["sp_q_max"]),
                   beta_q=np.ascontiguousarray(z["sp_beta_q"]), dbeta_q=np.ascontiguousarray(z["sp_dbeta_q"]))
    sysm = S.System(name=name, lattice=z["lattice"], omega=float(z["omega"]), n1=int(n[0]), n2=int(n[1]),
                    n3=int(n[2]), v_loc=np.ascontiguousarray(z["v_loc"]), species=[sp],
                    atom_species=np.ascontiguousarray(z["atom_species"]),
                    atom_z=np.full(z["atom_tau"].shape[0], 6, dtype=np.int32),
                    atom_tau=np.ascontiguousarray(z["atom_tau"]), ecut=0.0)
    kp = S.KPoint(npw=int(z["g_idx"].shape[0]), k_frac=z["k_frac"], g_idx=np.ascontiguousarray(z["g_idx"]),
                  kvec=np.ascontiguousarray(z["kvec"]), kinetic=np.ascontiguousarray(z["kinetic"]))
    grad = np.ascontiguousarray(np.transpose(z["grad"], (1, 0, 2)))
    return sysm, kp, np.ascontiguousarray(z["psi"]), np.ascontiguousarray(z["hpsi"]), grad


def rel_err(a, b):
    a = np.asarray(a)
    b = np.asarray(b)
    return float(np.linalg.norm((a - b).ravel()) / max(np.linalg.norm(b.ravel()), 1e-300))


@pytest.fixture(scope="session")
def oracle_lib():
    from oracle import oracle as O
    O.build()
    return O


def reference_golden(sysm, kps, psis):
    """The reference's own golden record (oracle/_ref/ref_driver `golden` mode)
    for the k-points kps with bands psis[i]: H|psi>, dH/dk|psi> and everything
    the reference used.  Needs the reference build (oracle.build_ref())."""
    from oracle import oracle as O
    with tempfile.TemporaryDirectory() as td:
        spec, gold = os.path.join(td, "spec.bin"), os.path.join(td, "gold.bin")
        S.write_spec(spec, sysm, list(kps), list(psis))
        subprocess.run([O.REF_DRIVER, "golden", spec, gold, os.path.join(td, "wd")], check=True,
                       stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL, timeout=1200)
        return S.read_golden(gold)


def as_used(sysm, g, ik=0):
    """System and k-point ik as the reference used them: its own beta/dbeta
    tables and lambda (after its per-l diagonalisation), its G-sphere views.
    Returns (System, KPoint, golden k-point record)."""
    sp, gk = g["species"][0], g["kpts"][ik]
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
