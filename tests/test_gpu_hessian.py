"""Hessian d2H/dk_a dk_b |psi> (hpsi_hess_apply).  The reference's operator is
an empty stub, so it is checked against the oracle's restatement (oracle_hess,
itself pinned in test_oracle_hessian.py) to 1e-12 in FP64, and against what the
reference does define:

* its radial tables: the Hessian tables F0 = beta/q^l and F1 = F0'/q, built on
  the device from the radial projectors the reference integrated, give back
  the reference's beta(q) and dbeta/dq tables (beta = F0 q^l,
  beta' = F1 q^(l+1) + l F0 q^(l-1)) and its D2BetaqTables
  (beta'' = F3 q^(l+2) + (2l+1) F1 q^l + l(l-1) F0 q^(l-2), against the
  oracle's restatement that is bit-identical to the reference's);
* its gradient (pinned in test_gpu_parity.py): central differences of
  dH/dk_a |psi> at K +- h e_b (same G set) within 1e-6 relative;
* the kinetic part alone (all lambda = 0): out_ab = delta_ab psi exactly;
* Hermiticity of <psi_m| d2H/dk_a dk_b |psi_n>."""
import copy
import os

import numpy as np
import pytest

from conftest import load_case, rel_err

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(__file__), "golden")
NAMES = ("xx", "yy", "zz", "xy", "xz", "yz")
PAIRS = ((0, 0), (1, 1), (2, 2), (0, 1), (0, 2), (1, 2))


def _tables(z):
    from effmass_gb300.hamiltonian import hessian_tables
    return hessian_tables(z["rad_r"], z["rad_rab"], bool(z["rad_uniform"]), z["rad_l"], z["rad_beta"],
                          float(z["sp_dq"]), float(z["sp_q_max"]))


@pytest.fixture(scope="module")
def built():
    from effmass_gb300 import build
    build.build()


@pytest.mark.parametrize("case", ["tiny", "tinyd"])
def test_hessian_tables_reproduce_reference_beta_tables(built, case):
    z = np.load(os.path.join(GOLDEN, f"{case}.npz"))
    f = _tables(z)
    q = np.arange(f.shape[-1]) * float(z["sp_dq"])
    for p, l in enumerate(z["rad_l"]):
        beta = f[0, p] * q ** l
        dbeta = f[1, p] * q ** (l + 1) + (l * f[0, p] * q ** (l - 1) if l > 0 else 0.0)
        assert np.abs(beta - z["sp_beta_q"][p]).max() <= 1e-12 * np.abs(z["sp_beta_q"][p]).max(), (p, l)
        sel = q > 0
        assert np.abs(dbeta[sel] - z["sp_dbeta_q"][p][sel]).max() <= 1e-11 * np.abs(z["sp_dbeta_q"][p]).max(), (p, l)


@pytest.mark.parametrize("case", ["tinyd", "sc8"])
def test_device_hessian_tables_match_oracle_and_reference_d2beta(built, oracle_lib, case):
    from test_oracle_hessian import beta_from_f
    z = np.load(os.path.join(GOLDEN, f"{case}.npz"))
    f = _tables(z)
    fo = oracle_lib.hess_tables(z["rad_r"], z["rad_rab"], bool(z["rad_uniform"]), z["rad_l"], z["rad_beta"],
                                float(z["sp_dq"]), float(z["sp_q_max"]))
    d2 = oracle_lib.d2beta_tables(z["rad_r"], z["rad_rab"], bool(z["rad_uniform"]), z["rad_l"], z["rad_beta"],
                                  float(z["sp_dq"]), float(z["sp_q_max"]))
    q = np.arange(f.shape[-1]) * float(z["sp_dq"])
    for p, l in enumerate(z["rad_l"]):
        for t in range(3):
            assert np.abs(f[t, p] - fo[t, p]).max() <= 1e-13 * np.abs(fo[t, p]).max(), (p, t)
        b2 = beta_from_f(f[:, p], int(l), q)[2]
        sel = q > 0 if l >= 2 else np.ones_like(q, dtype=bool)
        assert np.abs(b2[sel] - d2[p][sel]).max() <= 1e-12 * np.abs(d2[p]).max(), (p, l)


@pytest.mark.parametrize("case,prec,tol", [("tinyd", "fp64", 1e-12), ("sc8", "fp64", 1e-12),
                                           ("tinyd", "fp32", 1e-5), ("sc8", "fp32", 1e-5)])
def test_hessian_matches_oracle(built, oracle_lib, case, prec, tol):
    from effmass_gb300.hamiltonian import Hamiltonian
    sysm, kp, psi, _, _ = load_case(case)
    z = np.load(os.path.join(GOLDEN, f"{case}.npz"))
    f = _tables(z)
    ref = oracle_lib.hess(sysm, kp, psi, [f], float(z["sp_dq"]))
    with Hamiltonian(sysm) as H:
        H.set_hessian_tables(0, f, float(z["sp_dq"]))
        H.set_kpoint(0, kp)
        out = {n: np.zeros_like(psi) for n in NAMES}
        H.hess_apply(0, psi.shape[0], psi, out, prec)
    errs = {n: rel_err(out[n], ref[k]) for k, n in enumerate(NAMES)}
    assert max(errs.values()) <= tol, (case, prec, errs)


def _shifted(kp, lattice, dK):
    from effmass_gb300 import system as S
    K = kp.kvec + dK
    kf = kp.k_frac + np.asarray(dK) @ np.asarray(lattice).T / (2 * np.pi)
    return S.KPoint(npw=kp.npw, k_frac=kf, g_idx=kp.g_idx.copy(), kvec=np.ascontiguousarray(K),
                    kinetic=0.5 * np.einsum("ij,ij->i", K, K))


@pytest.mark.parametrize("case,prec,tol", [("tinyd", "fp64", 1e-6), ("fcc2", "fp64", 1e-6), ("tinyd", "fp32", 1e-4)])
def test_hessian_matches_central_differences_of_the_gradient(built, case, prec, tol):
    from effmass_gb300.hamiltonian import GradHPsi, Hamiltonian
    sysm, kp, psi, _, _ = load_case(case)
    z = np.load(os.path.join(GOLDEN, f"{case}.npz"))
    f = _tables(z)
    h = 1e-4
    with Hamiltonian(sysm) as H:
        H.set_hessian_tables(0, f, float(z["sp_dq"]))
        H.set_kpoint(0, kp)
        for b in range(3):
            e = np.zeros(3)
            e[b] = h
            H.set_kpoint(1 + 2 * b, _shifted(kp, sysm.lattice, e))
            H.set_kpoint(2 + 2 * b, _shifted(kp, sysm.lattice, -e))
        out = {n: np.zeros_like(psi) for n in NAMES}
        H.hess_apply(0, psi.shape[0], psi, out, prec)
        for n, (a, b) in zip(NAMES, PAIRS):
            gp = [None, None, None]
            gm = [None, None, None]
            gp[a] = np.zeros_like(psi)
            gm[a] = np.zeros_like(psi)
            H.gradient().at_k(1 + 2 * b, precision="fp64")(psi, GradHPsi(*gp), n_bands=psi.shape[0])
            H.gradient().at_k(2 + 2 * b, precision="fp64")(psi, GradHPsi(*gm), n_bands=psi.shape[0])
            fd = (gp[a] - gm[a]) / (2 * h)
            assert rel_err(out[n], fd) <= tol, (case, prec, n, rel_err(out[n], fd))


def test_kinetic_only_and_hermitian(built):
    from effmass_gb300.hamiltonian import Hamiltonian
    sysm, kp, psi, _, _ = load_case("tinyd")
    z = np.load(os.path.join(GOLDEN, "tinyd.npz"))
    f = _tables(z)
    free = copy.deepcopy(sysm)
    for sp in free.species:
        sp.lam = np.zeros_like(sp.lam)
    with Hamiltonian(free) as H:
        H.set_hessian_tables(0, f, float(z["sp_dq"]))
        H.set_kpoint(0, kp)
        out = {n: np.zeros_like(psi) for n in NAMES}
        H.hess_apply(0, psi.shape[0], psi, out, "fp64")
        for n, (a, b) in zip(NAMES, PAIRS):
            assert np.array_equal(out[n], psi if a == b else np.zeros_like(psi)), n
    with Hamiltonian(sysm) as H:
        H.set_hessian_tables(0, f, float(z["sp_dq"]))
        H.set_kpoint(0, kp)
        out = {"xy": np.zeros_like(psi), "zz": np.zeros_like(psi)}
        H.hess_apply(0, psi.shape[0], psi, out, "fp64")
        for n in out:
            M = psi.conj() @ out[n].T
            assert np.abs(M - M.conj().T).max() <= 1e-12 * np.abs(M).max(), n


def test_missing_tables_is_state_error(built):
    from effmass_gb300.hamiltonian import Hamiltonian
    from effmass_gb300._lib import HpsiError
    from effmass_gb300 import abi
    sysm, kp, psi, _, _ = load_case("tiny")
    with Hamiltonian(sysm) as H:
        H.set_kpoint(0, kp)
        with pytest.raises(HpsiError) as ei:
            H.hess_apply(0, psi.shape[0], psi, {"xx": np.zeros_like(psi)}, "fp64")
        assert ei.value.status == abi.HPSI_ERR_STATE
