"""Batched k-point plans (hpsi_batch_*): one graph launch over many k-points
of several cells with ragged npw and band counts.

Pinned to the reference through the golden fixtures (an item of the batch is
a fixture's k-point and bands): FP64 within 1e-12, FP32 and the tensor-core
plans (ragged tcgen05 GEMMs, split FP16) within 1e-6, split BF16 within 2e-6.
Every other item is compared with the per-k hpsi_apply of the same precision
(itself pinned by test_gpu_parity.py)."""
import numpy as np
import pytest

from conftest import load_case, rel_err
from effmass_gb300 import abi

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def cells():
    from effmass_gb300 import build, system as S
    from effmass_gb300.hamiltonian import Hamiltonian
    build.build()
    out = {}
    # the golden fcc2 and tinyd k-points in slot 0, Monkhorst-Pack points after them
    for name, mp in (("fcc2", 2), ("tinyd", 2), ("sc8", 1)):
        sysm, kp0, psi0, href0, _ = load_case(name)
        ecut = S.make_system(name).ecut
        H = Hamiltonian(sysm)
        H.set_kpoint(0, kp0)
        kps = [kp0]
        for i, k in enumerate(S.mp_grid(mp)[:5]):
            kp = S.g_sphere(sysm.lattice, k, ecut)
            H.set_kpoint(i + 1, kp)
            kps.append(kp)
        out[name] = (H, kps, psi0, href0)
    yield out
    for H, *_ in out.values():
        H.close()


def _items(cells, seed=0):
    """Ragged items: (H, kid, psi) with 0..12 bands; slot 0 carries the golden bands."""
    from effmass_gb300 import system as S
    rng = np.random.default_rng(seed)
    items = []
    for name, (H, kps, psi0, _) in cells.items():
        items.append((H, 0, psi0))
        for kid in range(1, len(kps)):
            nb = int(rng.integers(0, 13)) if kid != 1 else 0  # one empty item per cell
            psi = S.make_bands(kps[kid], max(nb, 1), seed=int(rng.integers(0, 1 << 30)))[:nb]
            items.append((H, kid, np.ascontiguousarray(psi)))
    return items


def _plan(items, precision, **kw):
    from effmass_gb300.batch import Batch
    return Batch([(H, kid, psi.shape[0]) for H, kid, psi in items], precision=precision, **kw)


TOL = {"fp64": 1e-12, "fp32": 1e-6, "tc": 1e-6, "tc_bf16": 2e-6}


@pytest.mark.parametrize("precision", ["fp64", "fp32", "tc", "tc_bf16"])
def test_batch_matches_reference_and_per_k(cells, precision):
    tol = TOL[precision]
    items = _items(cells)
    with _plan(items, precision) as plan:
        psi = plan.pack([p for _, _, p in items])
        hpsi = plan.empty()
        plan.apply(psi, hpsi)
        outs = plan.split(hpsi)
        info = plan.info()
    assert info["graph"] and info["tuned"] and len(info["cells"]) == 3
    for (H, kid, p), got in zip(items, outs):
        if p.shape[0] == 0:
            assert got.size == 0
            continue
        ref = np.zeros_like(p)
        H.apply(kid, p.shape[0], p, ref, precision)
        assert rel_err(got, ref) <= tol, (kid, precision, rel_err(got, ref))
    # the golden items against the reference's own outputs
    golden = {id(H): href for H, _, _, href in cells.values()}
    for (H, kid, p), got in zip(items, outs):
        if kid == 0:
            assert rel_err(got, golden[id(H)]) <= tol


def test_graph_equals_eager_bitwise(cells):
    items = _items(cells, seed=1)
    res = []
    for graph in (True, False):
        with _plan(items, "fp32", graph=graph, tune=False) as plan:
            psi = plan.pack([p for _, _, p in items])
            hpsi = plan.empty()
            plan.apply(psi, hpsi)
            assert plan.info()["graph"] is graph
            res.append(hpsi)
    assert np.array_equal(res[0], res[1])


def test_tuned_and_default_tiles_agree(cells):
    items = _items(cells, seed=2)
    res = []
    for tune in (True, False):
        with _plan(items, "fp64", tune=tune) as plan:
            psi = plan.pack([p for _, _, p in items])
            hpsi = plan.empty()
            plan.apply(psi, hpsi)
            res.append(hpsi)
    assert rel_err(res[0], res[1]) <= 1e-13


def test_accumulates_and_runs_on_resident_buffers(cells):
    torch = pytest.importorskip("torch")
    items = _items(cells, seed=3)
    with _plan(items, "fp32") as plan:
        psi = plan.pack([p for _, _, p in items])
        base = np.random.default_rng(0).standard_normal(plan.n_complex) * (1 + 1j)
        hpsi = base.copy()
        plan.apply(psi, hpsi)  # host buffers: hpsi += H psi
        # device tensors, then twice on the resident buffers
        tp = torch.from_numpy(psi).cuda()
        th = torch.zeros_like(tp)
        plan.apply(tp, th, device=True)
        assert rel_err(th.cpu().numpy(), hpsi - base) <= 1e-12
        plan.run()
        plan.run()
        torch.cuda.synchronize()
        p_dev, h_dev, n = plan.device_buffers()
        assert n == plan.n_complex and p_dev and h_dev
        # the resident hpsi now holds 3 x H psi (apply left H psi there, the two runs added 2 x)
        out = _device_view(h_dev, 2 * n).cpu().numpy().view(np.complex128)
        assert rel_err(out, 3 * (hpsi - base)) <= 1e-6


def _device_view(ptr, n_doubles):
    """A torch tensor aliasing n_doubles float64 at device pointer ptr."""
    import torch

    class _Cuda:
        __cuda_array_interface__ = {"shape": (n_doubles,), "typestr": "<f8", "data": (ptr, False), "version": 3}

    return torch.as_tensor(_Cuda(), device="cuda")


def test_rebinding_a_slot_invalidates_the_plan(cells):
    from effmass_gb300._lib import HpsiError
    from effmass_gb300 import system as S
    H, kps, psi0, _ = cells["tinyd"]
    kp = S.g_sphere(H.system.lattice, (0.3, 0.1, 0.2), S.make_system("tinyd").ecut)
    H.set_kpoint(7, kps[2])
    psi = S.make_bands(kps[2], 3, seed=9)
    with _plan([(H, 7, psi)], "fp32") as plan:
        plan.apply(psi.reshape(-1).copy(), plan.empty())
        H.set_kpoint(7, kp)
        with pytest.raises(HpsiError) as ei:
            plan.run()
        assert ei.value.status == abi.HPSI_ERR_STATE


def test_unbound_slot_and_precision_refused(cells):
    import ctypes as C
    from effmass_gb300._lib import HpsiError, load
    from effmass_gb300.batch import Batch
    H, *_ = cells["tinyd"]
    with pytest.raises(HpsiError) as ei:
        Batch([(H, 99, 4)], precision="fp32")
    assert ei.value.status == abi.HPSI_ERR_STATE
    lib = load()
    Batch([(H, 0, 1)], precision="fp32").close()  # binds the batch entry points
    arr = (abi.HpsiBatchItem * 1)(abi.HpsiBatchItem(H.ctx.value, 0, 4))
    out = C.c_void_p()
    assert lib.hpsi_batch_create(arr, 1, 7, C.byref(out)) == abi.HPSI_ERR_BAD_ARG  # no such precision
    assert not out.value


@pytest.mark.parametrize("precision", ["tc", "tc_bf16"])
def test_tensor_core_plan_blocks_of_bands(cells, precision):
    """Items of more than 128 bands (split into 128-band blocks of the ragged
    GEMMs, the last one with N = 2 nbp > 128 rows), items of one band, and the
    graph against eager launches: all equal the per-k tensor-core hpsi_apply."""
    from effmass_gb300 import system as S
    H, kps, _, _ = cells["fcc2"]
    items = [(H, 1, S.make_bands(kps[1], 200, seed=5)), (H, 2, S.make_bands(kps[2], 1, seed=6)),
             (H, 3, S.make_bands(kps[3], 17, seed=7))]
    res = []
    for graph in (True, False):
        with _plan(items, precision, graph=graph, tune=False) as plan:
            psi = plan.pack([p for _, _, p in items])
            hpsi = plan.empty()
            plan.apply(psi, hpsi)
            assert plan.info()["precision"] == precision
            res.append(plan.split(hpsi))
    for (H_, kid, p), got, got_eager in zip(items, res[0], res[1]):
        ref = np.zeros_like(p)
        H_.apply(kid, p.shape[0], p, ref, precision)
        assert rel_err(got, ref) <= TOL[precision], (kid, rel_err(got, ref))
        assert np.array_equal(got, got_eager)


def test_tensor_core_plan_survives_per_k_format_switch(cells):
    """A tensor-core plan reads the k-points' generator tables; per-k calls in
    the other split format build that format's tables beside them (nothing the
    plan points to is freed), so the plan's next run gives the same result."""
    from effmass_gb300 import system as S
    H, kps, _, _ = cells["tinyd"]
    items = [(H, 2, S.make_bands(kps[2], 5, seed=21)), (H, 3, S.make_bands(kps[3], 3, seed=22))]
    with _plan(items, "tc", tune=False) as plan:
        psi = plan.pack([p for _, _, p in items])
        first = plan.empty()
        plan.apply(psi, first)
        for H_, kid, p in items:
            H_.apply(kid, p.shape[0], p, np.zeros_like(p), "tc_bf16")  # the other format's tables
        again = plan.empty()
        plan.apply(psi, again)
    assert np.array_equal(first, again)
