"""beta(q) / dbeta(q)/dq tables built on the device (hpsi_beta_tables) from
the radial projectors the reference integrated, against the reference's own
tables (golden fixtures): within 1e-13 of their largest value (the device sums
the Simpson terms in another order; sin/cos may differ in the last bit)."""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


@pytest.mark.parametrize("case", ["tiny", "tinyd", "fcc2", "sc8"])
def test_device_tables_match_reference(case):
    from effmass_gb300 import build
    from effmass_gb300.hamiltonian import beta_tables
    build.build()
    z = np.load(os.path.join(GOLDEN, f"{case}.npz"))
    bq, dbq = beta_tables(z["rad_r"], z["rad_rab"], bool(z["rad_uniform"]), z["rad_l"], z["rad_beta"],
                          float(z["sp_dq"]), float(z["sp_q_max"]))
    assert bq.shape == z["sp_beta_q"].shape
    assert np.abs(bq - z["sp_beta_q"]).max() <= 1e-13 * np.abs(z["sp_beta_q"]).max()
    assert np.abs(dbq - z["sp_dbeta_q"]).max() <= 1e-13 * np.abs(z["sp_dbeta_q"]).max()


def test_uniform_mesh_and_short_projectors_match_oracle():
    """A uniform mesh and projectors of 1, 2, 4 and 5 points (every Simpson branch).
    Up to l = 4 at 0.5 <= q r < l the upward Bessel recurrence (the reference's
    method) amplifies last-bit differences of sin/cos between host and device,
    so this case is held to 1e-11 of the largest value."""
    from oracle import oracle as O
    from effmass_gb300.hamiltonian import beta_tables
    nr = 40
    r = np.arange(nr) * 0.05
    rab = np.full(nr, 0.05)
    beta = np.zeros((5, nr))
    lens = [1, 2, 4, 5, 33]
    for p, n in enumerate(lens):
        beta[p, :n] = np.exp(-r[:n]) * (1 + p) * r[:n] ** 2 + (p + 1) * 1e-3
    l = np.array([0, 1, 2, 1, 3], dtype=np.int32)
    bq, dbq = beta_tables(r, rab, True, l, beta, 0.05, 5.0)
    obq, odbq = O.beta_tables(r, rab, True, l, beta, 0.05, 5.0)
    assert np.abs(bq - obq).max() <= 1e-11 * np.abs(obq).max()
    assert np.abs(dbq - odbq).max() <= 1e-11 * np.abs(odbq).max()


@pytest.mark.parametrize("name,k", [("fcc2", (0.25, 0.25, 0.25)), ("sc8", (0.1, -0.2, 0.3)), ("sc64", (0, 0, 0))])
def test_device_gsphere_matches_host_and_H_is_invariant(name, k):
    """The device G-sphere is the host helper's set of G (there in kinetic
    order, here in (g1, g2, g3) order) with the same K and kinetic energies,
    and H|psi> on it is the host-ordered result permuted."""
    from effmass_gb300 import system as S
    from effmass_gb300.hamiltonian import Hamiltonian, gsphere
    from conftest import rel_err
    sysm = S.make_system(name)
    host = S.g_sphere(sysm.lattice, k, sysm.ecut)
    dev = gsphere(sysm.lattice, k, sysm.ecut)
    assert dev.npw == host.npw
    key = lambda g: np.lexsort((g[:, 2], g[:, 1], g[:, 0]))
    ih, idv = key(host.g_idx), key(dev.g_idx)
    assert np.array_equal(host.g_idx[ih], dev.g_idx[idv])
    assert np.array_equal(idv, np.arange(dev.npw))          # already in (g1, g2, g3) order
    assert np.abs(host.kvec[ih] - dev.kvec).max() <= 1e-13 * np.abs(host.kvec).max()
    assert np.abs(host.kinetic[ih] - dev.kinetic).max() <= 1e-13 * host.kinetic.max()
    if name != "sc64":
        psi = S.make_bands(host, 3, seed=4)
        with Hamiltonian(sysm) as H:
            H.set_kpoint(0, host)
            H.set_kpoint(1, dev)
            a, b = np.zeros_like(psi), np.zeros_like(psi)
            H.apply(0, 3, psi, a, "fp64")
            H.apply(1, 3, np.ascontiguousarray(psi[:, ih]), b, "fp64")
        assert rel_err(b, a[:, ih]) <= 1e-12
