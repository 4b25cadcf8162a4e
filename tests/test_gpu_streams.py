"""The tensor-core H|psi> runs its projection chain on a side stream beside
the FFT passes (default) or on the caller's stream (HPSI_ONE_STREAM): the
kernels and their inputs are the same, so the results are bit-identical."""
import numpy as np
import pytest

from conftest import load_case

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name", ["tinyd", "sc8"])
def test_side_stream_equals_one_stream(name):
    torch = pytest.importorskip("torch")
    from effmass_gb300 import build
    from effmass_gb300.hamiltonian import Hamiltonian
    build.build()
    sysm, kp, psi, _, _ = load_case(name)
    with Hamiltonian(sysm) as H:
        H.set_kpoint(0, kp)
        p = torch.from_numpy(np.ascontiguousarray(psi)).cuda()
        outs = []
        for one in (False, True):
            h = torch.zeros_like(p)
            H.apply(0, p.shape[0], p, h, "tc", one_stream=one)
            H.apply(0, p.shape[0], p, h, "tc", one_stream=one)  # accumulates: 2 H psi
            torch.cuda.synchronize()
            outs.append(h.cpu().numpy())
        assert np.array_equal(outs[0], outs[1])
        assert np.abs(outs[0]).max() > 0
