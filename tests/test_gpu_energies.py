"""Band energies beside H|psi> (hpsi_apply_energies): FP64 reductions on the
device, with the complex64 transform's gain error removed by its own Parseval
norm.

Bar: the FP64 path reproduces the Rayleigh quotients of the reference's own
H|psi> outputs (golden fixtures) to 1e-12 Ha; the FP32 and split-FP16
tensor-core paths give band energies within 1e-8 Ha of the FP64 values, also
at the full 64-atom size.  Split BF16 (8-bit pieces: hi + lo holds a value to
~2^-17) is held to 3e-8 Ha.  hpsi itself is hpsi_apply's: bit for bit in FP64
and FP32; the tensor-core paths use shorter accumulation chains for the
energies, so their hpsi agrees within the path's tolerance."""
import numpy as np
import pytest

from conftest import CASES, load_case, rel_err

pytestmark = pytest.mark.gpu

E_TOL = {"fp32": 1e-8, "tc": 1e-8, "tc_bf16": 3e-8}  # Ha


def _rq(psi, h):
    return np.einsum("bg,bg->b", psi.conj(), h).real


@pytest.fixture(scope="module")
def built():
    from effmass_gb300 import build
    build.build()


@pytest.mark.parametrize("case", CASES)
def test_energies_match_reference_rayleigh_quotients(built, case):
    from effmass_gb300.hamiltonian import Hamiltonian
    sysm, kp, psi, href, _ = load_case(case)
    e_ref = _rq(psi, href)
    errs = {}
    with Hamiltonian(sysm) as H:
        H.set_kpoint(0, kp)
        for prec in ("fp64", "fp32", "tc", "tc_bf16"):
            h = np.zeros_like(psi)
            e = H.apply_energies(0, psi.shape[0], psi, h, prec)
            errs[prec] = float(np.abs(e - e_ref).max())
            h2 = np.zeros_like(psi)
            H.apply(0, psi.shape[0], psi, h2, prec)
            if prec in ("fp64", "fp32"):
                assert np.array_equal(h, h2), (case, prec)
            else:
                assert rel_err(h, h2) <= 2e-6, (case, prec)
    assert errs["fp64"] <= 1e-12, errs
    # On the aliasing grid (two G-vectors on one grid point) the call returns the
    # Rayleigh quotient of the computed hpsi (no Parseval normalisation), which
    # keeps the complex64 transform's gain error: held to 3e-8 Ha there.
    tol = {p: max(E_TOL[p], 3e-8) for p in E_TOL} if case == "alias" else E_TOL
    assert all(errs[p] <= tol[p] for p in tol), (case, errs)


def test_full_size_energies_within_1e_8(built):
    from effmass_gb300 import system as S
    from effmass_gb300.hamiltonian import Hamiltonian
    sysm = S.make_system("sc64")
    kp = S.g_sphere(sysm.lattice, (0, 0, 0), sysm.ecut)
    psi = S.make_bands(kp, 32, seed=11)
    with Hamiltonian(sysm) as H:
        H.set_kpoint(0, kp)
        h64 = np.zeros_like(psi)
        e64 = H.apply_energies(0, psi.shape[0], psi, h64, "fp64")
        assert np.abs(e64 - _rq(psi, h64)).max() <= 1e-12
        errs = {}
        for prec in ("fp32", "tc", "tc_bf16"):
            h = np.zeros_like(psi)
            e = H.apply_energies(0, psi.shape[0], psi, h, prec)
            errs[prec] = float(np.abs(e - e64).max())
            assert rel_err(h, h64) <= 2e-6
        assert all(errs[p] <= E_TOL[p] for p in E_TOL), errs


def test_device_pointers_and_accumulation(built):
    torch = pytest.importorskip("torch")
    from effmass_gb300.hamiltonian import Hamiltonian
    sysm, kp, psi, href, _ = load_case("sc8")
    with Hamiltonian(sysm) as H:
        H.set_kpoint(0, kp)
        p = torch.from_numpy(psi).cuda()
        base = torch.full_like(p, 0.5 - 0.25j)
        h = base.clone()
        e = H.apply_energies(0, psi.shape[0], p, h, "fp32")
        assert rel_err((h - base).cpu().numpy(), href) <= 1e-6
        assert np.abs(e.cpu().numpy() - _rq(psi, href)).max() <= E_TOL["fp32"]
