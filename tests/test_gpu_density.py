"""Charge density (hpsi_density) against the reference's own buildDensity
(src/support/density.cppm:41-94, golden fixtures made by running it):
FP64 within 1e-12 relative, complex64 transforms within 1e-6; at the full
64-atom size through Parseval (sum_r rho = N sum_b occ_b |psi_b|^2)."""
import os

import numpy as np
import pytest

from conftest import CASES, load_case, rel_err

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


@pytest.fixture(scope="module")
def built():
    from effmass_gb300 import build
    build.build()


@pytest.mark.parametrize("case", CASES)
def test_density_matches_reference(built, case):
    from effmass_gb300.hamiltonian import Hamiltonian
    sysm, kp, psi, _, _ = load_case(case)
    z = np.load(os.path.join(GOLDEN, f"{case}.npz"))
    with Hamiltonian(sysm) as H:
        H.set_kpoint(0, kp)
        for prec, tol in (("fp64", 1e-12), ("fp32", 1e-6), ("tc", 1e-6)):
            rho = H.density(0, psi.shape[0], psi, z["occ"], precision=prec)
            assert rel_err(rho.ravel(), z["rho"]) <= tol, (case, prec, rel_err(rho.ravel(), z["rho"]))


def test_density_accumulates_over_kpoints_and_device_pointers(built):
    torch = pytest.importorskip("torch")
    from effmass_gb300 import system as S
    from effmass_gb300.hamiltonian import Hamiltonian
    from oracle import oracle as O
    sysm = S.make_system("fcc2")
    kps = [S.g_sphere(sysm.lattice, k, sysm.ecut) for k in S.mp_grid(2)[:3]]
    occ = np.array([2.0, 2.0, 1.5, 0.0, 0.5])
    ref = np.zeros(sysm.n1 * sysm.n2 * sysm.n3)
    with Hamiltonian(sysm) as H:
        rho = torch.zeros((sysm.n1, sysm.n2, sysm.n3), dtype=torch.float64, device="cuda")
        o = torch.from_numpy(occ).cuda()
        for i, kp in enumerate(kps):
            H.set_kpoint(i, kp)
            psi = S.make_bands(kp, occ.size, seed=i)
            H.density(i, occ.size, torch.from_numpy(psi).cuda(), o, rho=rho, precision="fp64")
            O.density(sysm, kp, psi, occ, ref)
        assert rel_err(rho.cpu().numpy().ravel(), ref) <= 1e-12


def test_full_size_parseval(built):
    from effmass_gb300 import system as S
    from effmass_gb300.hamiltonian import Hamiltonian
    sysm = S.make_system("sc64")
    kp = S.g_sphere(sysm.lattice, (0, 0, 0), sysm.ecut)
    psi = S.make_bands(kp, 48, seed=2)
    occ = np.random.default_rng(0).uniform(0, 2, 48)
    N = sysm.n1 * sysm.n2 * sysm.n3
    expect = N * float(np.sum(occ * np.sum(np.abs(psi) ** 2, axis=1)))
    with Hamiltonian(sysm) as H:
        H.set_kpoint(0, kp)
        for prec, tol in (("fp64", 1e-12), ("fp32", 1e-6)):
            rho = H.density(0, 48, psi, occ, precision=prec)
            assert abs(rho.sum() - expect) <= tol * expect, (prec, rho.sum(), expect)
            assert rho.min() >= 0.0
