"""hpsi_apply_noalloc: H|psi> for callers that cannot allocate device memory
during the call (a fixed device-memory budget, a runtime whose allocator owns
the device, or code that must not add an allocation's implicit device
synchronisation).

Its scratch is a 32 MiB static device array instead of the context's
workspace.  This test calls it through the C ABI, twice in a row (the array
keeps the previous call's contents), and compares each result with the
existing entry point hpsi_apply on the same inputs: within 1e-12 (FP64) and
1e-6 (FP32) relative, the tolerances of the other parity tests.  One case
(1001 bands of the 64-atom cell in FP64, on a stream of its own) needs more
partial sums than the scratch holds, so its nonlocal term runs in chunks of
251 bands with a last chunk of 248.  It also checks the refusals: the
tensor-core precisions, host pointers, projector matrices not yet built, and
a band whose FFT planes do not fit the scratch, which is refused before any
launch with hpsi left as it was.  (A refusal on the partial sums alone would
need more than a million projectors per band; the same up-front check covers
it.)

This file is collected last so that a run stopping at the first failure has
already run every other test.
"""
import ctypes as C

import numpy as np
import pytest

from effmass_gb300 import abi

pytestmark = pytest.mark.gpu

TOL = {"fp64": 1e-12, "fp32": 1e-6}


def _noalloc(H, kid, nb, psi_d, hpsi_d, prec, sync=True, stream=None):
    import torch
    from effmass_gb300._lib import load
    lib = load()
    fn = lib.hpsi_apply_noalloc
    fn.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_int, C.c_void_p]
    fn.restype = C.c_int
    flags = abi.PRECISIONS[prec] | abi.HPSI_DEVICE_PTRS | (abi.HPSI_SYNC if sync else 0)
    st = stream if stream is not None else torch.cuda.current_stream()
    return fn(H.ctx, kid, nb, C.c_void_p(psi_d.data_ptr()), C.c_void_p(hpsi_d.data_ptr()), flags,
              C.c_void_p(st.cuda_stream))


def _rel(a, b):
    import torch
    return float(torch.linalg.norm(a - b) / torch.linalg.norm(b))


@pytest.mark.parametrize("name,nb", [("fcc2", 8), ("sc64", 40)])
def test_noalloc_matches_hpsi_apply_twice(name, nb):
    torch = pytest.importorskip("torch")
    from effmass_gb300 import build, system as S
    from effmass_gb300.hamiltonian import Hamiltonian
    build.build()
    sysm = S.make_system(name)
    kp = S.g_sphere(sysm.lattice, S.default_kpoint(name), sysm.ecut)
    psi = torch.from_numpy(S.make_bands(kp, nb, seed=23)).cuda()
    with Hamiltonian(sysm) as H:
        H.set_kpoint(0, kp)
        for prec in ("fp64", "fp32"):
            ref = torch.zeros_like(psi)
            H.apply(0, nb, psi, ref, prec)  # existing entry point (also builds the projector matrices)
            torch.cuda.synchronize()
            for call in range(2):
                out = torch.zeros_like(psi)
                st = _noalloc(H, 0, nb, psi, out, prec)
                assert st == 0, (name, prec, call, st)
                err = _rel(out, ref)
                assert err <= TOL[prec], (name, prec, call, err)


def test_noalloc_chunked_partial_sums_on_own_stream():
    """1001 bands of the 64-atom cell (1152 projectors) in FP64: the partial
    sums of all bands exceed the scratch, so the nonlocal term runs in chunks
    of 251 bands and a last chunk of 248, on a non-default stream."""
    torch = pytest.importorskip("torch")
    from effmass_gb300 import build, system as S
    from effmass_gb300.hamiltonian import Hamiltonian
    build.build()
    sysm = S.make_system("sc64")
    kp = S.g_sphere(sysm.lattice, S.default_kpoint("sc64"), sysm.ecut)
    nb = 1001
    psi = torch.from_numpy(S.make_bands(kp, 8, seed=29)).cuda().repeat(126, 1)[:nb].contiguous()
    psi *= torch.linspace(0.5, 1.5, nb, dtype=torch.float64, device="cuda")[:, None]
    with Hamiltonian(sysm) as H:
        H.set_kpoint(0, kp)
        ref = torch.zeros_like(psi)
        H.apply(0, nb, psi, ref, "fp64")
        torch.cuda.synchronize()
        side = torch.cuda.Stream()
        for call in range(2):
            out = torch.zeros_like(psi)
            torch.cuda.synchronize()
            st = _noalloc(H, 0, nb, psi, out, "fp64", stream=side)
            assert st == 0, (call, st)
            err = _rel(out, ref)
            assert err <= TOL["fp64"], (call, err)


def test_noalloc_refusals():
    torch = pytest.importorskip("torch")
    from effmass_gb300 import build, system as S
    from effmass_gb300.hamiltonian import Hamiltonian
    build.build()
    sysm = S.make_system("tiny")
    kp = S.g_sphere(sysm.lattice, (0.25, 0.25, 0.25), sysm.ecut)
    psi = torch.from_numpy(S.make_bands(kp, 2)).cuda()
    out = torch.zeros_like(psi)
    with Hamiltonian(sysm) as H:
        H.set_kpoint(0, kp)
        # projector matrices of fp32 not built yet on this k-point
        assert _noalloc(H, 0, 2, psi, out, "fp32") == abi.HPSI_ERR_STATE
        # the tensor-core precisions are not offered
        for prec in ("tc", "tc_bf16"):
            assert _noalloc(H, 0, 2, psi, out, prec) == abi.HPSI_ERR_BAD_ARG
        # host pointers are refused
        from effmass_gb300._lib import load
        lib = load()
        h = np.zeros((2, kp.npw), dtype=np.complex128)
        p = np.ascontiguousarray(psi.cpu().numpy())
        st = lib.hpsi_apply_noalloc(H.ctx, 0, 2, C.c_void_p(p.ctypes.data), C.c_void_p(h.ctypes.data),
                                    abi.HPSI_PREC_FP64, None)
        assert st == abi.HPSI_ERR_BAD_ARG


def test_noalloc_rejects_planes_beyond_scratch():
    torch = pytest.importorskip("torch")
    from effmass_gb300 import build, system as S
    from effmass_gb300.hamiltonian import Hamiltonian
    build.build()
    # a long cell: 361 of 400 x-planes hold sphere points; one band's complex128
    # planes (361 * 80 * 80 * 16 bytes = 37 MB) exceed the 32 MiB scratch
    lat = np.diag([400.0, 10.0, 10.0])
    sysm = S.System(name="long", lattice=lat, omega=4e4, n1=400, n2=80, n3=80, v_loc=np.zeros(400 * 80 * 80),
                    species=[], atom_species=np.zeros(0, np.int32), atom_z=np.zeros(0, np.int32),
                    atom_tau=np.zeros((0, 3)), ecut=4.0)
    B = 2 * np.pi * np.linalg.inv(lat).T
    r1, r2 = np.arange(-200, 200), np.arange(-6, 7)
    g = np.stack(np.meshgrid(r1, r2, r2, indexing="ij"), -1).reshape(-1, 3)
    K = g @ B
    kin = 0.5 * (K * K).sum(1)
    sel = kin < sysm.ecut
    kp = S.KPoint(npw=int(sel.sum()), k_frac=np.zeros(3), g_idx=np.ascontiguousarray(g[sel], dtype=np.int32),
                  kvec=np.ascontiguousarray(K[sel]), kinetic=np.ascontiguousarray(kin[sel]))
    assert len(np.unique(kp.g_idx[:, 0])) * 80 * 80 * 16 > abi.HPSI_NOALLOC_SCRATCH_BYTES
    psi = torch.ones((1, kp.npw), dtype=torch.complex128, device="cuda")
    before = torch.arange(kp.npw, dtype=torch.float64, device="cuda").to(torch.complex128)[None, :]
    out = before.clone()
    with Hamiltonian(sysm) as H:
        H.set_kpoint(0, kp)
        assert _noalloc(H, 0, 1, psi, out, "fp64") == abi.HPSI_ERR_BAD_ARG
        from effmass_gb300._lib import load
        assert b"scratch" in load().hpsi_last_error(H.ctx)
        torch.cuda.synchronize()
        assert torch.equal(out, before)  # refused before any launch
