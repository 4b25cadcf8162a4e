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
