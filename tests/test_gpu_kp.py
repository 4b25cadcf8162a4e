"""Velocity matrices on the tensor cores and the FP64 k·p sums
(hpsi_velocity_matrix with HPSI_PREC_TC / TC_BF16, hpsi_kp_sums).

The k·p sums have no counterpart in the reference; they are checked against
the same sum written out in numpy (FP64).  The tensor-core velocity matrices
are checked against the FP64 path (itself pinned to the oracle in
test_gpu_parity.py) at 1e-6 relative."""
import numpy as np
import pytest

from conftest import load_case, rel_err

pytestmark = pytest.mark.gpu


def kp_numpy(M, E, n_low, tol):
    nb = E.shape[0]
    S = np.zeros((n_low, 3, 3))
    K = np.zeros(n_low, dtype=int)
    for n in range(n_low):
        for m in range(nb):
            if m == n:
                continue
            d = E[n] - E[m]
            if abs(d) <= tol:
                K[n] += 1
                continue
            for a in range(3):
                for b in range(3):
                    S[n, a, b] += (M[a, n, m] * M[b, m, n]).real / d
    return S, K


@pytest.fixture(scope="module")
def built():
    from effmass_gb300 import build
    build.build()


def test_kp_sums_match_numpy(built):
    from effmass_gb300.hamiltonian import kp_sums
    rng = np.random.default_rng(0)
    nb, n_low = 40, 8
    A = rng.standard_normal((3, nb, nb)) + 1j * rng.standard_normal((3, nb, nb))
    M = A + np.conj(np.transpose(A, (0, 2, 1)))  # Hermitian per direction, like <m|dH|n>
    E = np.sort(rng.uniform(-0.5, 0.8, nb))
    E[5] = E[4] + 1e-12  # a degenerate pair inside the lowest bands
    S, K = kp_sums(M, E, n_low, 1e-9)
    Sr, Kr = kp_numpy(M, E, n_low, 1e-9)
    assert np.array_equal(K, Kr) and K[4] == 1 and K[5] == 1
    assert np.abs(S - Sr).max() <= 1e-12 * np.abs(Sr).max()
    # symmetric in (a, b) for Hermitian M
    assert np.abs(S - np.transpose(S, (0, 2, 1))).max() <= 1e-12 * np.abs(S).max()


def test_kp_sums_device_tensors(built):
    torch = pytest.importorskip("torch")
    from effmass_gb300.hamiltonian import kp_sums
    rng = np.random.default_rng(1)
    nb = 24
    M = rng.standard_normal((3, nb, nb)) + 1j * rng.standard_normal((3, nb, nb))
    E = np.sort(rng.uniform(-0.5, 0.8, nb))
    S, K = kp_sums(torch.from_numpy(M).cuda(), torch.from_numpy(E).cuda(), 8, 0.0)
    Sr, _ = kp_numpy(M, E, 8, 0.0)
    assert np.abs(S.cpu().numpy() - Sr).max() <= 1e-12 * np.abs(Sr).max()


@pytest.mark.parametrize("prec,tol", [("tc", 1e-6), ("tc_bf16", 2e-6), ("fp32", 1e-6)])
def test_velocity_mixed_vs_fp64(built, prec, tol):
    from effmass_gb300.hamiltonian import Hamiltonian
    sysm, kp, psi, _, _ = load_case("sc8")
    with Hamiltonian(sysm) as H:
        H.set_kpoint(0, kp)
        V64 = H.velocity_matrix(0, psi.shape[0], psi, precision="fp64")
        V = H.velocity_matrix(0, psi.shape[0], psi, precision=prec)
    assert rel_err(V, V64) <= tol, (prec, rel_err(V, V64))
    # Hermitian per direction: <m|dH|n> = conj(<n|dH|m>)
    assert np.abs(V - np.conj(np.transpose(V, (0, 2, 1)))).max() <= 10 * tol * np.abs(V64).max()


def test_full_size_velocity_and_kp(built):
    """64-atom cell, 64 bands: tensor-core velocity within 1e-6 of FP64, and the
    k·p sums of the lowest 8 bands from both within 5e-6 relative: each term
    divides |M|^2 by a band gap (~0.02 Ha here), which amplifies the velocity
    error, so the derived sums carry a few times its relative error."""
    from effmass_gb300 import system as S
    from effmass_gb300.hamiltonian import Hamiltonian, kp_sums
    sysm = S.make_system("sc64")
    kp = S.g_sphere(sysm.lattice, (0.01, 0.0, 0.0), sysm.ecut)
    psi = S.make_bands(kp, 64, seed=5)
    E = np.sort(np.random.default_rng(5).uniform(-0.5, 0.8, 64))
    with Hamiltonian(sysm) as H:
        H.set_kpoint(0, kp)
        V64 = H.velocity_matrix(0, 64, psi, precision="fp64")
        Vtc = H.velocity_matrix(0, 64, psi, precision="tc")
    assert rel_err(Vtc, V64) <= 1e-6
    s64, _ = kp_sums(V64, E, 8)
    stc, _ = kp_sums(Vtc, E, 8)
    assert np.abs(stc - s64).max() <= 5e-6 * np.abs(s64).max()
