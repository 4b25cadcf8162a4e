"""GPU parity of libhpsi_gb300.so, called through the C ABI.

Tolerances (relative, in the 2-norm over all bands and G):
  FP64 path  vs the reference's own outputs (golden fixtures):  1e-12
  FP32 path  vs the reference's own outputs:                   1e-6
The 64-atom cell itself is pinned to the reference in
test_gpu_reference_c1.py (4 bands per k-point).  Here, at 64-atom sizes that
need many bands (band chunks, 320 bands), the FP32 path is checked against
the FP64 GPU path (1e-6) and size-independent properties are checked
(Hermiticity of <psi_m|H|psi_n>, linearity).
"""
import ctypes as C

import numpy as np
import pytest

from conftest import CASES, load_case, rel_err
from effmass_gb300 import abi

pytestmark = pytest.mark.gpu

TOL = {"fp64": 1e-12, "fp32": 1e-6, "tc": 1e-6, "tc_bf16": 2e-6}


@pytest.fixture(scope="module")
def H_of():
    from effmass_gb300.build import build
    build()
    from effmass_gb300.hamiltonian import Hamiltonian
    made = {}

    def get(case):
        if case not in made:
            sysm, kp, psi, href, gref = load_case(case)
            H = Hamiltonian(sysm)
            H.set_kpoint(0, kp)
            made[case] = (H, sysm, kp, psi, href, gref)
        return made[case]

    yield get
    for v in made.values():
        v[0].close()


@pytest.mark.parametrize("prec", ["fp64", "fp32", "tc", "tc_bf16"])
@pytest.mark.parametrize("case", CASES)
def test_hpsi_matches_reference(H_of, case, prec):
    H, sysm, kp, psi, href, _ = H_of(case)
    out = np.zeros_like(psi)
    op = H.at_k(0, precision=prec)
    op(psi.shape[0], psi, out)
    assert rel_err(out, href) <= TOL[prec], (case, prec, rel_err(out, href))


@pytest.mark.parametrize("prec", ["fp64", "fp32", "tc", "tc_bf16"])
@pytest.mark.parametrize("case", CASES)
def test_grad_matches_reference(H_of, case, prec):
    from effmass_gb300.hamiltonian import GradHPsi
    H, sysm, kp, psi, _, gref = H_of(case)
    out = np.zeros((3,) + psi.shape, dtype=np.complex128)
    H.gradient().at_k(0, precision=prec)(psi, GradHPsi(out[0], out[1], out[2]), n_bands=psi.shape[0])
    assert rel_err(out, gref) <= TOL[prec], (case, prec, rel_err(out, gref))


def test_single_band_call_and_accumulate(H_of):
    H, sysm, kp, psi, href, _ = H_of("fcc2")
    op = H.at_k(0)
    assert op.dim() == kp.npw
    base = np.full(kp.npw, 0.25 - 0.5j)
    out = base.copy()
    op(np.ascontiguousarray(psi[3]), out)  # hpsi += H psi (reference semantics)
    assert rel_err(out - base, href[3]) <= 1e-12


def test_grad_skips_missing_directions(H_of):
    from effmass_gb300.hamiltonian import GradHPsi
    H, sysm, kp, psi, _, gref = H_of("tinyd")
    y = np.zeros_like(psi)
    H.gradient().at_k(0)(psi, GradHPsi(None, y, None), n_bands=psi.shape[0])
    assert rel_err(y, gref[1]) <= 1e-12


def test_device_pointers_and_stream(H_of):
    torch = pytest.importorskip("torch")
    H, sysm, kp, psi, href, _ = H_of("sc8")
    p = torch.from_numpy(psi).cuda()
    h = torch.zeros_like(p)
    s = torch.cuda.Stream()
    with torch.cuda.stream(s):
        H.apply(0, psi.shape[0], p, h, "fp64")
    s.synchronize()
    assert rel_err(h.cpu().numpy(), href) <= 1e-12


def test_velocity_matrix_matches_oracle(H_of, oracle_lib):
    H, sysm, kp, psi, _, gref = H_of("tinyd")
    V = H.velocity_matrix(0, psi.shape[0], psi)
    Vo = oracle_lib.velocity(sysm, kp, psi)
    assert rel_err(V, Vo) <= 1e-12
    V32 = H.velocity_matrix(0, psi.shape[0], psi, precision="fp32")
    assert rel_err(V32, Vo) <= 1e-6


def test_zero_bands_is_noop(H_of):
    H, sysm, kp, psi, _, _ = H_of("tiny")
    out = np.zeros((1, kp.npw), dtype=np.complex128)
    H.apply(0, 0, psi, out)
    assert not out.any()


def test_unbound_slot_and_bad_precision(H_of):
    from effmass_gb300._lib import HpsiError, load
    H, sysm, kp, psi, _, _ = H_of("tiny")
    with pytest.raises(HpsiError) as ei:
        H.dim(7)
    assert ei.value.status == abi.HPSI_ERR_STATE
    lib = load()
    out = np.zeros_like(psi)
    st = lib.hpsi_apply(H.ctx, 0, 1, C.c_void_p(psi.ctypes.data), C.c_void_p(out.ctypes.data), 9, None)
    assert st == abi.HPSI_ERR_BAD_ARG


def test_q_beyond_table_is_range_error():
    from effmass_gb300.hamiltonian import Hamiltonian
    from effmass_gb300._lib import HpsiError
    sysm, kp, psi, _, _ = load_case("tiny")
    sp = sysm.species[0]
    sp.q_max = float(np.sqrt(2 * kp.kinetic.max())) * 0.5  # the reference's domain_error case
    with Hamiltonian(sysm) as H:
        with pytest.raises(HpsiError) as ei:
            H.set_kpoint(0, kp)
        assert ei.value.status == abi.HPSI_ERR_RANGE


def test_several_slots_and_rebinding():
    from effmass_gb300 import system as S
    from effmass_gb300.hamiltonian import Hamiltonian
    from oracle import oracle as O
    sysm = S.make_system("tinyd")
    kps = [S.g_sphere(sysm.lattice, k, sysm.ecut) for k in [(0, 0, 0), (0.5, 0.5, 0.5), (0.1, 0.2, -0.3)]]
    with Hamiltonian(sysm) as H:
        for i, kp in enumerate(kps):
            H.set_kpoint(i, kp)
        for i, kp in enumerate(kps):
            psi = S.make_bands(kp, 2, seed=i)
            out = np.zeros_like(psi)
            H.at_k(i)(2, psi, out)
            assert rel_err(out, O.hpsi(sysm, kp, psi)) <= 1e-12
        H.set_kpoint(1, kps[2])  # rebinding replaces the slot
        psi = S.make_bands(kps[2], 2, seed=5)
        out = np.zeros_like(psi)
        H.at_k(1)(2, psi, out)
        assert rel_err(out, O.hpsi(sysm, kps[2], psi)) <= 1e-12


def test_lambda_zero_projectors_are_skipped():
    from effmass_gb300 import system as S
    from effmass_gb300.hamiltonian import Hamiltonian
    from oracle import oracle as O
    sysm = S.make_system("tiny")
    sysm.species[0].lam = sysm.species[0].lam.copy()
    sysm.species[0].lam[1] = 0.0
    kp = S.g_sphere(sysm.lattice, (0.25, 0.25, 0.25), sysm.ecut)
    psi = S.make_bands(kp, 2)
    with Hamiltonian(sysm) as H:
        H.set_kpoint(0, kp)
        out = np.zeros_like(psi)
        H.at_k(0)(2, psi, out)
    assert rel_err(out, O.hpsi(sysm, kp, psi)) <= 1e-12


def test_single_plane_wave():
    from effmass_gb300 import system as S
    from effmass_gb300.hamiltonian import Hamiltonian
    from oracle import oracle as O
    sysm = S.make_system("tiny")
    kp = S.g_sphere(sysm.lattice, (0.0, 0.0, 0.0), 0.05)  # only G = 0 (q = 0: theta = phi = 0 branch)
    assert kp.npw == 1
    psi = np.array([[0.6 - 0.8j]])
    with Hamiltonian(sysm) as H:
        H.set_kpoint(0, kp)
        out = np.zeros_like(psi)
        H.at_k(0)(1, psi, out)
        from effmass_gb300.hamiltonian import GradHPsi
        g = np.zeros((3, 1, 1), dtype=np.complex128)
        H.gradient().at_k(0)(psi, GradHPsi(g[0], g[1], g[2]))
    assert rel_err(out, O.hpsi(sysm, kp, psi)) <= 1e-12
    assert rel_err(g, O.grad(sysm, kp, psi)) <= 1e-12


# ------------------------------------------------------------ full size
@pytest.fixture(scope="module")
def sc64():
    from effmass_gb300 import system as S
    from effmass_gb300.hamiltonian import Hamiltonian
    sysm = S.make_system("sc64")
    kp = S.g_sphere(sysm.lattice, (0, 0, 0), sysm.ecut)
    assert kp.npw == 37073
    psi = S.make_bands(kp, 16, seed=3)
    H = Hamiltonian(sysm)
    H.set_kpoint(0, kp)
    yield H, kp, psi
    H.close()


def test_full_size_mixed_vs_fp64_and_hermitian(sc64):
    H, kp, psi = sc64
    h64 = np.zeros_like(psi)
    H.apply(0, psi.shape[0], psi, h64, "fp64")
    for prec in ("fp32", "tc", "tc_bf16"):
        hm = np.zeros_like(psi)
        H.apply(0, psi.shape[0], psi, hm, prec)
        assert rel_err(hm, h64) <= TOL[prec], (prec, rel_err(hm, h64))
    M = psi.conj() @ h64.T
    assert np.abs(M - M.conj().T).max() <= 1e-11 * np.abs(M).max()


def test_full_size_grad_mixed_vs_fp64(sc64):
    from effmass_gb300.hamiltonian import GradHPsi
    H, kp, psi = sc64
    g64 = np.zeros((3,) + psi.shape, dtype=np.complex128)
    H.gradient().at_k(0, precision="fp64")(psi, GradHPsi(g64[0], g64[1], g64[2]), n_bands=psi.shape[0])
    for prec in ("fp32", "tc"):
        g = np.zeros_like(g64)
        H.gradient().at_k(0, precision=prec)(psi, GradHPsi(g[0], g[1], g[2]), n_bands=psi.shape[0])
        assert rel_err(g, g64) <= TOL[prec], (prec, rel_err(g, g64))


def test_full_size_band_chunks(sc64):
    """320 bands of the 64-atom cell: their sphere planes (519 MB) exceed the
    512 MB band chunk, so the local term runs in two chunks and the tensor-core
    band operand takes its row maxima in a separate pass.  The first and last
    bands agree with separate FP64 calls."""
    import torch
    from effmass_gb300 import system as S
    H, kp, _ = sc64
    nb = 320
    psi = S.make_bands(kp, nb, seed=5)
    p = torch.from_numpy(psi).cuda()
    for prec in ("tc", "fp32"):
        h = torch.zeros_like(p)
        H.apply(0, nb, p, h, prec)
        torch.cuda.synchronize()
        out = h.cpu().numpy()
        for lo in (0, nb - 8):
            ref = np.zeros((8, kp.npw), dtype=np.complex128)
            H.apply(0, 8, np.ascontiguousarray(psi[lo:lo + 8]), ref, "fp64")
            assert rel_err(out[lo:lo + 8], ref) <= TOL[prec], (prec, lo, rel_err(out[lo:lo + 8], ref))


def test_full_size_linearity(sc64):
    H, kp, psi = sc64
    a, b = 0.3 - 1.1j, -0.7 + 0.2j
    mix = np.ascontiguousarray(a * psi[0:4] + b * psi[4:8])
    hm = np.zeros_like(mix)
    h = np.zeros_like(psi)
    H.apply(0, 4, mix, hm, "fp64")
    H.apply(0, psi.shape[0], psi, h, "fp64")
    assert rel_err(hm, a * h[0:4] + b * h[4:8]) <= 1e-12


def test_wide_radix_grid_matches_oracle():
    """A 14 x 21 x 13 grid needs the radix-7 and radix-13 stages (the wide kernel set)."""
    from effmass_gb300 import system as S
    from effmass_gb300.hamiltonian import Hamiltonian
    from oracle import oracle as O
    sysm = S.make_system("tiny")
    sysm.n1, sysm.n2, sysm.n3 = 14, 21, 13
    sysm.v_loc = S.local_potential(sysm.lattice, sysm.atom_tau, 14, 21, 13)
    kp = S.g_sphere(sysm.lattice, (0.1, 0.2, 0.3), sysm.ecut)
    psi = S.make_bands(kp, 3)
    ref = O.hpsi(sysm, kp, psi)
    with Hamiltonian(sysm) as H:
        H.set_kpoint(0, kp)
        for prec, tol in (("fp64", 1e-12), ("fp32", 1e-6), ("tc", 1e-6)):
            out = np.zeros_like(psi)
            H.at_k(0, precision=prec)(3, psi, out)
            assert rel_err(out, ref) <= tol, (prec, rel_err(out, ref))
