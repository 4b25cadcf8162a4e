"""Sternheimer solve for dpsi/dk (hpsi_sternheimer) against the exact
sum over states of a dense diagonalisation.

The occupied states are the lowest eigenvectors of the k-point's FP64
Hamiltonian matrix (built column by column with the FP64 GPU path, itself
pinned to the reference) so that P_c (H - e_n) P_c is positive definite on
the conduction space; the exact answer is
  x_n = -sum_{m unoccupied} |m><m| dH/dk_a |n> / (E_m - E_n)."""
import numpy as np
import pytest

from conftest import rel_err

pytestmark = pytest.mark.gpu


def _dense(H, kid, npw, nv):
    eye = np.eye(npw, dtype=np.complex128)
    out = np.zeros_like(eye)
    H.apply(kid, npw, eye, out, "fp64")
    Hm = out.T.copy()                       # column j = H e_j
    Hm = 0.5 * (Hm + Hm.conj().T)
    E, V = np.linalg.eigh(Hm)
    assert E[nv] - E[nv - 1] > 1e-3          # a gap above the occupied bands
    return E, V


def _exact(H, kid, E, V, nv, direction):
    from effmass_gb300.hamiltonian import GradHPsi
    psi = np.ascontiguousarray(V[:, :nv].T)
    g = [None, None, None]
    g[direction] = np.zeros_like(psi)
    H.grad_apply(kid, nv, psi, GradHPsi(*g))
    d = g[direction]
    Vc = V[:, nv:]
    coef = Vc.conj().T @ d.T                 # <m|dH|n>, m unoccupied
    x = -(Vc @ (coef / (E[nv:, None] - E[None, :nv]))).T
    return psi, x


@pytest.mark.parametrize("case,nv", [("tiny", 4), ("fcc2", 4)])
def test_sternheimer_matches_sum_over_states(case, nv):
    from effmass_gb300 import build, system as S
    from effmass_gb300.hamiltonian import Hamiltonian
    build.build()
    sysm = S.make_system(case)
    kp = S.g_sphere(sysm.lattice, (0.1, 0.2, 0.3), sysm.ecut)
    with Hamiltonian(sysm) as H:
        H.set_kpoint(0, kp)
        E, V = _dense(H, 0, kp.npw, nv)
        for direction in (0, 2):
            psi, x_ref = _exact(H, 0, E, V, nv, direction)
            x, its, res = H.sternheimer(0, psi, E[:nv], direction, tol=1e-11, precision="fp64")
            assert res.max() <= 1e-11 and its > 0
            assert rel_err(x, x_ref) <= 1e-8, (case, direction, rel_err(x, x_ref), its)
            # mixed-precision H inside the solve: limited by the H|psi> error
            x32, its32, _ = H.sternheimer(0, psi, E[:nv], direction, tol=1e-6, precision="tc")
            assert rel_err(x32, x_ref) <= 1e-5, (case, direction, rel_err(x32, x_ref))
