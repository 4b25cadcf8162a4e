"""The serving loop (hpsi_server_*): results of a request are the same alone and
in a mixed, concurrently running stream — where jobs overtake one another and
small cells' jobs are merged into one ragged launch set — within the
tensor-core tolerance (1e-6 relative), agree with direct hpsi_apply /
hpsi_velocity_matrix calls, and admission respects the device budget."""
import numpy as np
import pytest

from conftest import rel_err
from effmass_gb300 import abi

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def systems():
    from effmass_gb300 import build, system as S
    from effmass_gb300.hamiltonian import Hamiltonian
    build.build()
    out = []
    for name, kpts in (("tiny", [(0.25, 0.25, 0.25), (0.0, 0.0, 0.0)]), ("fcc2", [(0.25, 0.25, 0.25), (0.1, 0.2, 0.3)]),
                       ("sc8", [(0.0, 0.0, 0.0)])):
        sysm = S.make_system(name)
        H = Hamiltonian(sysm)
        kps = []
        for i, k in enumerate(kpts):
            kp = S.g_sphere(sysm.lattice, k, sysm.ecut)
            H.set_kpoint(i, kp)
            kps.append(kp)
        out.append((H, kps))
    yield out
    for H, _ in out:
        H.close()


def _requests(systems, seed=0):
    """A mixed list of requests: (system, k, nb, with velocity) with seeded psi."""
    from effmass_gb300 import system as S
    rng = np.random.default_rng(seed)
    reqs = []
    for r in range(12):
        si = int(rng.integers(0, len(systems)))
        H, kps = systems[si]
        jobs = []
        for _ in range(int(rng.integers(1, 3))):
            ki = int(rng.integers(0, len(kps)))
            nb = int(rng.integers(1, 20))
            psi = S.make_bands(kps[ki], nb, seed=int(rng.integers(0, 10 ** 6)))
            jobs.append(dict(system=si, kid=ki, psi=psi, vel=bool(rng.integers(0, 2))))
        reqs.append(jobs)
    return reqs


def _run(srv_factory, reqs, concurrent):
    from effmass_gb300.serving import Job
    outs = []
    with srv_factory() as srv:
        tickets = []
        for jobs in reqs:
            js = [Job(j["system"], j["kid"], j["psi"], np.zeros_like(j["psi"]),
                      np.zeros((3, j["psi"].shape[0], j["psi"].shape[0]), dtype=np.complex128) if j["vel"] else None)
                  for j in jobs]
            outs.append(js)
            t = srv.submit(js)
            if concurrent:
                tickets.append(t)
            else:
                srv.wait(t)
        for t in tickets:
            srv.wait(t)
        stats = srv.stats()
    return outs, stats


def test_same_alone_and_in_the_mix(systems):
    from effmass_gb300.serving import Server
    reqs = _requests(systems)
    hams = [h for h, _ in systems]
    alone, _ = _run(lambda: Server(hams, lanes=1, budget_gb=2, precision="tc"), reqs, concurrent=False)
    mixed, stats = _run(lambda: Server(hams, lanes=4, budget_gb=2, precision="tc", merge_max_bands=256,
                                       bypass_ms=5.0), reqs, concurrent=True)
    assert stats["completed"] == len(reqs)
    for a_jobs, m_jobs, jobs in zip(alone, mixed, reqs):
        for a, m, j in zip(a_jobs, m_jobs, jobs):
            assert rel_err(m.hpsi, a.hpsi) <= 1e-6
            if a.vel is not None:
                assert rel_err(m.vel, a.vel) <= 1e-6
            # and against a direct FP64 call of the library
            H, kps = systems[j["system"]]
            ref = np.zeros_like(j["psi"])
            H.apply(j["kid"], j["psi"].shape[0], j["psi"], ref, "fp64")
            assert rel_err(m.hpsi, ref) <= 1e-6
            if a.vel is not None:
                vref = H.velocity_matrix(j["kid"], j["psi"].shape[0], j["psi"], precision="fp64")
                assert rel_err(m.vel, vref) <= 1e-6


def test_merged_units_match_direct_calls(systems):
    """One lane kept busy by a first job while many small requests queue: the
    scheduler merges the queued jobs of each small cell into ragged units."""
    from effmass_gb300 import system as S
    from effmass_gb300.serving import Job, Server
    hams = [h for h, _ in systems]
    rng = np.random.default_rng(5)
    reqs = []
    for r in range(40):
        si = int(rng.integers(0, len(systems)))
        H, kps = systems[si]
        ki = int(rng.integers(0, len(kps)))
        nb = int(rng.integers(1, 24))
        psi = S.make_bands(kps[ki], nb, seed=int(rng.integers(0, 10 ** 6)))
        vel = bool(rng.integers(0, 2))
        reqs.append((si, ki, psi, vel))
    with Server(hams, lanes=1, budget_gb=2, precision="tc", merge_max_bands=512, bypass_ms=50.0) as srv:
        H, kps = systems[2]
        big = S.make_bands(kps[0], 96, seed=3)
        t0 = srv.submit([Job(2, 0, big, np.zeros_like(big))])
        jobs = [Job(si, ki, psi, np.zeros_like(psi),
                    np.zeros((3, psi.shape[0], psi.shape[0]), dtype=np.complex128) if vel else None)
                for si, ki, psi, vel in reqs]
        ts = [srv.submit([j]) for j in jobs]
        srv.wait(t0)
        for t in ts:
            srv.wait(t)
        st = srv.stats()
    assert st["completed"] == len(reqs) + 1
    assert st["merged_units"] >= 1 and st["merged_jobs"] >= 2, st
    for (si, ki, psi, vel), j in zip(reqs, jobs):
        H, kps = systems[si]
        ref = np.zeros_like(psi)
        H.apply(ki, psi.shape[0], psi, ref, "fp64")
        assert rel_err(j.hpsi, ref) <= 1e-6
        if vel:
            vref = H.velocity_matrix(ki, psi.shape[0], psi, precision="fp64")
            assert rel_err(j.vel, vref) <= 1e-6


def test_budget_admission_and_refusals(systems):
    from effmass_gb300 import system as S
    from effmass_gb300.serving import Job, Server
    from effmass_gb300._lib import HpsiError
    hams = [h for h, _ in systems]
    H, kps = systems[2]
    psi = S.make_bands(kps[0], 24, seed=1)
    # a budget that holds about one such request at a time: all still complete
    with Server(hams, lanes=4, budget_gb=0.05, precision="fp32") as srv:
        ts = [srv.submit([Job(2, 0, psi, np.zeros_like(psi))]) for _ in range(6)]
        times = [srv.wait(t) for t in ts]
        st = srv.stats()
        assert st["completed"] == 6 and st["peak_bytes"] <= st["budget_bytes"]
        assert max(t["queue_ms"] for t in times) >= 0.0
        # larger than the whole budget: refused at submit
        big = S.make_bands(kps[0], 400, seed=2)
        with pytest.raises(HpsiError) as ei:
            srv.submit([Job(2, 0, big, np.zeros_like(big))])
        assert ei.value.status == abi.HPSI_ERR_OOM
        # unbound k-point slot
        with pytest.raises(HpsiError) as ei:
            srv.submit([Job(2, 5, psi, np.zeros_like(psi))])
        assert ei.value.status == abi.HPSI_ERR_STATE
