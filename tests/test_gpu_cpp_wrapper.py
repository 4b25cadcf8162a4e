"""The header-only C++ mirror (include/hpsi_gb300.hpp) in behaviour, not only
in syntax: tests/cpp/hpsi_wrapper_check.cpp is compiled as a C++20 program,
linked to libhpsi_gb300.so, and run on the reference's golden record of the
s+p+d case at a general k-point.  It checks the reference-style
Hamiltonian::Callable (both call forms, accumulation), Gradient::Callable (an
empty span skips a direction), set_ikpt, device spans on a stream, and the
exception mapping (std::invalid_argument, std::domain_error,
std::runtime_error); see the program's header for the list."""
import os
import shutil
import subprocess
import tempfile

import numpy as np
import pytest

from conftest import ROOT, load_case

pytestmark = pytest.mark.gpu


def _write_case(path, sysm, kp, psi, href, gref):
    sp = sysm.species[0]
    with open(path, "wb") as f:
        w = lambda a, dt: f.write(np.ascontiguousarray(a, dtype=dt).tobytes())  # noqa: E731
        w([sysm.n1, sysm.n2, sysm.n3], np.int32)
        w(np.asarray(sysm.lattice).reshape(9), np.float64)
        w([sysm.omega], np.float64)
        w([len(sysm.atom_tau)], np.int32)
        w(sysm.atom_species, np.int32)
        w(sysm.atom_tau, np.float64)
        w([len(sp.proj_l)], np.int32)
        w(sp.proj_l, np.int32)
        w(sp.lam, np.float64)
        w([sp.beta_q.shape[1]], np.int32)
        w([sp.dq, sp.q_max], np.float64)
        w(sp.beta_q, np.float64)
        w(sp.dbeta_q, np.float64)
        w(sysm.v_loc, np.float64)
        w([kp.npw], np.int32)
        w(kp.k_frac, np.float64)
        w(kp.g_idx, np.int32)
        w(kp.kvec, np.float64)
        w(kp.kinetic, np.float64)
        w([psi.shape[0]], np.int32)
        w(psi, np.complex128)
        w(href, np.complex128)
        w(gref, np.complex128)


def test_cpp_callable_against_reference_golden():
    from effmass_gb300 import build
    lib = build.build()
    cuda = os.path.dirname(os.path.dirname(shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"))
    sysm, kp, psi, href, gref = load_case("tinyd")
    with tempfile.TemporaryDirectory() as td:
        exe = os.path.join(td, "check")
        subprocess.run(["g++", "-std=c++20", "-O1", "-I", os.path.join(ROOT, "include"), "-I",
                        os.path.join(cuda, "include"), os.path.join(ROOT, "tests", "cpp", "hpsi_wrapper_check.cpp"),
                        "-o", exe, "-L", os.path.dirname(lib), "-lhpsi_gb300", "-Wl,-rpath," + os.path.dirname(lib),
                        "-L", os.path.join(cuda, "lib64"), "-lcudart", "-Wl,-rpath," + os.path.join(cuda, "lib64")],
                       check=True, capture_output=True, text=True)
        case = os.path.join(td, "case.bin")
        _write_case(case, sysm, kp, psi, href, gref)
        r = subprocess.run([exe, case], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert r.stdout.count("ok  ") >= 11, r.stdout
