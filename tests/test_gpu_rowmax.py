"""The tensor-core band operand scales each band by its largest coefficient,
which the G->r pass takes while it scatters psi.  A G-vector that shares its
grid point with a later one is not scattered (the later write wins); its
coefficient must still count.  Here a k-point gets such a pair, and the
unscattered coefficient is made the largest of its band by far: an FP16
operand scaled without it would overflow."""
import numpy as np
import pytest

from conftest import load_case, rel_err

pytestmark = pytest.mark.gpu


def _with_twin(sysm, kp):
    """kp plus G' = G + (n1, 0, 0) for the first G with g1 <= 0: both land on
    one grid point, and G (the earlier) is the one not scattered."""
    from effmass_gb300 import system as S
    g = np.asarray(kp.g_idx).reshape(-1, 3)
    i0 = int(np.nonzero(g[:, 0] <= 0)[0][0])
    g2 = np.vstack([g, g[i0] + np.array([sysm.n1, 0, 0])]).astype(np.int32)
    B = 2.0 * np.pi * np.linalg.inv(np.asarray(sysm.lattice)).T
    K = (g2 + np.asarray(kp.k_frac)) @ B
    kin = 0.5 * np.einsum("ij,ij->i", K, K)
    return S.KPoint(npw=int(g2.shape[0]), k_frac=np.asarray(kp.k_frac).copy(), g_idx=np.ascontiguousarray(g2),
                    kvec=np.ascontiguousarray(K), kinetic=np.ascontiguousarray(kin)), i0


@pytest.mark.parametrize("prec", ["tc", "tc_bf16"])
def test_unscattered_coefficient_sets_the_scale(prec):
    from effmass_gb300 import build
    from effmass_gb300 import system as S
    from effmass_gb300.hamiltonian import Hamiltonian
    build.build()
    sysm, kp0, _, _, _ = load_case("alias")
    kp, hidden = _with_twin(sysm, kp0)
    psi = S.make_bands(kp, 3, seed=11)
    psi[0, hidden] = 1e3 * np.abs(psi[0]).max() * (1 + 1j)
    with Hamiltonian(sysm) as H:
        H.set_kpoint(0, kp)
        ref = np.zeros_like(psi)
        H.apply(0, psi.shape[0], psi, ref, "fp64")
        got = np.zeros_like(psi)
        H.apply(0, psi.shape[0], psi, got, prec)
    assert np.isfinite(got).all()
    assert rel_err(got, ref) <= {"tc": 1e-6, "tc_bf16": 2e-6}[prec]
