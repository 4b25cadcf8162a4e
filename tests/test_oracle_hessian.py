"""The oracle's d2H/dk_a dk_b |psi> and its radial tables, on the CPU.

The reference declares the Hessian operator (src/H_psi/hamiltonian.cppm:84-91)
but leaves it empty (src/H_psi/hamiltonian_hessian.cpp:48-50), so the oracle's
restatement (oracle_hess) is pinned to what the reference does define:

* its radial tables: F0 = beta/q^l, F1 = F0'/q, F3 = (F0'' - F0'/q)/q^2
  (oracle_hess_tables) give back the reference's beta(q) and dbeta/dq tables
  stored in the golden fixtures (beta = F0 q^l, beta' = F1 q^(l+1) +
  l F0 q^(l-1)) and the reference's D2BetaqTables (beta'' = F3 q^(l+2) +
  (2l+1) F1 q^l + l(l-1) F0 q^(l-2); oracle_d2beta_tables is bit-identical to
  D2BetaqTables in test_reference_live.py);
* its gradient: central differences of the oracle's dH/dk_a|psi> (pinned to
  the reference's Gradient::Callable to 1e-14) at K +- h e_b, within 1e-6;
* the kinetic part alone (all lambda = 0) is delta_ab psi exactly, and
  <psi_m| d2H/dk_a dk_b |psi_n> is Hermitian.
"""
import copy
import os

import numpy as np
import pytest

from conftest import GOLDEN, load_case, rel_err
from effmass_gb300 import system as S

NAMES = ("xx", "yy", "zz", "xy", "xz", "yz")
PAIRS = ((0, 0), (1, 1), (2, 2), (0, 1), (0, 2), (1, 2))


def _ftables(oracle_lib, z):
    return oracle_lib.hess_tables(z["rad_r"], z["rad_rab"], bool(z["rad_uniform"]), z["rad_l"], z["rad_beta"],
                                  float(z["sp_dq"]), float(z["sp_q_max"]))


def beta_from_f(f, l, q):
    """beta, beta' and beta'' of one projector from its F0, F1, F3 rows."""
    with np.errstate(divide="ignore", invalid="ignore"):
        b0 = f[0] * q ** l
        b1 = f[1] * q ** (l + 1) + (l * f[0] * q ** (l - 1) if l >= 1 else 0.0)
        b2 = f[2] * q ** (l + 2) + (2 * l + 1) * f[1] * q ** l + (l * (l - 1) * f[0] * q ** (l - 2) if l >= 2 else 0.0)
    return b0, b1, b2


@pytest.mark.parametrize("case", ["tinyd", "sc8"])
def test_f_tables_give_back_reference_tables(oracle_lib, case):
    z = np.load(os.path.join(GOLDEN, f"{case}.npz"))
    f = _ftables(oracle_lib, z)
    dq, qm = float(z["sp_dq"]), float(z["sp_q_max"])
    d2 = oracle_lib.d2beta_tables(z["rad_r"], z["rad_rab"], bool(z["rad_uniform"]), z["rad_l"], z["rad_beta"], dq, qm)
    q = np.arange(f.shape[-1]) * dq
    for p, l in enumerate(z["rad_l"]):
        b0, b1, b2 = beta_from_f(f[:, p], int(l), q)
        ref0, ref1 = z["sp_beta_q"][p], z["sp_dbeta_q"][p]
        assert np.abs(b0 - ref0).max() <= 1e-13 * np.abs(ref0).max(), (p, l)
        sel = q > 0
        assert np.abs(b1[sel] - ref1[sel]).max() <= 1e-12 * np.abs(ref1).max(), (p, l)
        sel2 = q > 0 if l >= 2 else np.ones_like(q, dtype=bool)
        assert np.abs(b2[sel2] - d2[p][sel2]).max() <= 1e-12 * np.abs(d2[p]).max(), (p, l)


def _shifted(kp, lattice, dK):
    K = kp.kvec + dK
    kf = kp.k_frac + np.asarray(dK) @ np.asarray(lattice).T / (2 * np.pi)
    return S.KPoint(npw=kp.npw, k_frac=kf, g_idx=kp.g_idx.copy(), kvec=np.ascontiguousarray(K),
                    kinetic=0.5 * np.einsum("ij,ij->i", K, K))


@pytest.mark.parametrize("case", ["tinyd", "sc8"])
def test_oracle_hessian_is_the_derivative_of_the_reference_gradient(oracle_lib, case):
    sysm, kp, psi, _, _ = load_case(case)
    z = np.load(os.path.join(GOLDEN, f"{case}.npz"))
    f = _ftables(oracle_lib, z)
    H = oracle_lib.hess(sysm, kp, psi, [f], float(z["sp_dq"]))
    h = 1e-4
    for k, (a, b) in enumerate(PAIRS):
        e = np.zeros(3)
        e[b] = h
        gp = oracle_lib.grad(sysm, _shifted(kp, sysm.lattice, e), psi)[a]
        gm = oracle_lib.grad(sysm, _shifted(kp, sysm.lattice, -e), psi)[a]
        assert rel_err(H[k], (gp - gm) / (2 * h)) <= 1e-6, (case, NAMES[k])


def test_oracle_hessian_kinetic_only_and_hermitian(oracle_lib):
    sysm, kp, psi, _, _ = load_case("tinyd")
    z = np.load(os.path.join(GOLDEN, "tinyd.npz"))
    f = _ftables(oracle_lib, z)
    free = copy.deepcopy(sysm)
    for sp in free.species:
        sp.lam = np.zeros_like(sp.lam)
    H0 = oracle_lib.hess(free, kp, psi, [f], float(z["sp_dq"]))
    for k, (a, b) in enumerate(PAIRS):
        assert np.array_equal(H0[k], psi if a == b else np.zeros_like(psi)), NAMES[k]
    H = oracle_lib.hess(sysm, kp, psi, [f], float(z["sp_dq"]))
    for k in range(6):
        M = psi.conj() @ H[k].T
        assert np.abs(M - M.conj().T).max() <= 1e-12 * np.abs(M).max(), NAMES[k]
