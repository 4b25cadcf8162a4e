"""A bounded device-side wait that runs out, without any fault.

Every mbarrier wait of the tensor-core GEMMs is bounded.  A test-only entry
point (hpsi_selftest_wait_limit) lowers the poll limit of the MMA issuer's wait
for a loaded stage to zero, so that this wait gives up at once in every CTA:
the CTA sets the context's error flag, raises its abort flag (the bulk-copy
producer stops issuing), waits — with the full bound — for the copies already
in flight to land, and frees its TMEM.  Nothing is faulted or trapped; the
copies still complete.  The synchronising hpsi_apply must then return
HPSI_ERR_TIMEOUT, and with the limit restored the next hpsi_apply on the same
context must be correct again (1e-6 against the reference's own output).
"""
import numpy as np
import pytest

from conftest import load_case, rel_err
from effmass_gb300 import abi

pytestmark = pytest.mark.gpu


def test_issuer_wait_runs_out_then_context_recovers():
    from effmass_gb300.build import build
    from effmass_gb300._lib import HpsiError, load
    from effmass_gb300.hamiltonian import Hamiltonian
    build()
    lib = load()
    sysm, kp, psi, href, _ = load_case("sc8")
    with Hamiltonian(sysm) as H:
        H.set_kpoint(0, kp)
        out = np.zeros_like(psi)
        H.apply(0, psi.shape[0], psi, out, "tc")  # builds the operands at the default limit
        assert rel_err(out, href) <= 1e-6
        try:
            assert lib.hpsi_selftest_wait_limit(0) == abi.HPSI_OK
            out = np.zeros_like(psi)
            with pytest.raises(HpsiError) as ei:
                H.apply(0, psi.shape[0], psi, out, "tc")  # host buffers: synchronising
            assert ei.value.status == abi.HPSI_ERR_TIMEOUT
            assert b"gave up" in lib.hpsi_last_error(H.ctx)
        finally:
            assert lib.hpsi_selftest_wait_limit(-1) == abi.HPSI_OK
        for prec in ("tc", "tc_bf16"):
            out = np.zeros_like(psi)
            H.apply(0, psi.shape[0], psi, out, prec)
            assert rel_err(out, href) <= 2e-6, prec
