"""CPU checks of the C ABI boundary: the library builds, loads and exports
every entry point include/hpsi_gb300.h declares; the ctypes structs match the
C layout; without a GPU the library fails loudly instead of computing on the
host."""
import ctypes as C
import os
import re
import subprocess
import tempfile

import pytest

from conftest import ROOT
from effmass_gb300 import abi

HEADER = os.path.join(ROOT, "include", "hpsi_gb300.h")


def declared_functions():
    txt = open(HEADER).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(hpsi_[a-z_0-9]+)\s*\(", txt)))


@pytest.fixture(scope="module")
def lib():
    from effmass_gb300 import build, _lib
    build.build()
    return _lib.load()


def test_header_declares_the_api():
    names = declared_functions()
    for n in ["hpsi_ctx_create", "hpsi_ctx_destroy", "hpsi_set_kpoint", "hpsi_apply", "hpsi_grad_apply",
              "hpsi_velocity_matrix", "hpsi_last_error", "hpsi_dim", "hpsi_abi_version"]:
        assert n in names


def test_library_exports_every_declared_symbol(lib):
    from effmass_gb300 import _lib
    out = subprocess.run(["nm", "-D", "--defined-only", _lib.LIB_PATH], capture_output=True, text=True, check=True).stdout
    exported = set(l.split()[-1] for l in out.splitlines() if l.strip())
    missing = [n for n in declared_functions() if n not in exported]
    assert not missing, missing
    assert lib.hpsi_abi_version() == 1


def test_struct_layout_matches_c():
    src = r"""
    #include <stdio.h>
    #include <stddef.h>
    #include "hpsi_gb300.h"
    int main(void){
      printf("%zu %zu %zu %zu\n", sizeof(hpsi_species), offsetof(hpsi_species,dq), offsetof(hpsi_species,beta_q), offsetof(hpsi_species,dbeta_q));
      printf("%zu %zu %zu %zu %zu\n", sizeof(hpsi_system), offsetof(hpsi_system,lattice), offsetof(hpsi_system,omega), offsetof(hpsi_system,species), offsetof(hpsi_system,atom_tau));
      printf("%zu %zu %zu %zu\n", sizeof(hpsi_kpoint), offsetof(hpsi_kpoint,k_frac), offsetof(hpsi_kpoint,g_idx), offsetof(hpsi_kpoint,kinetic));
      printf("%zu %zu %zu\n", sizeof(hpsi_batch_item), offsetof(hpsi_batch_item,kid), offsetof(hpsi_batch_item,nb));
      printf("%zu %zu %zu\n", sizeof(hpsi_job), offsetof(hpsi_job,psi), offsetof(hpsi_job,vel));
      printf("%zu %zu %zu %zu %zu\n", sizeof(hpsi_server_config), offsetof(hpsi_server_config,device_budget_bytes), offsetof(hpsi_server_config,precision), offsetof(hpsi_server_config,merge_max_bands), offsetof(hpsi_server_config,bypass_ms));
      printf("%zu %zu %zu\n", sizeof(hpsi_server_statistics), offsetof(hpsi_server_statistics,peak_bytes), offsetof(hpsi_server_statistics,merged_jobs));
      return 0; }
    """
    with tempfile.TemporaryDirectory() as td:
        cfile = os.path.join(td, "l.c")
        exe = os.path.join(td, "l")
        open(cfile, "w").write(src)
        subprocess.run(["gcc", "-I", os.path.dirname(HEADER), cfile, "-o", exe], check=True)
        got = [list(map(int, l.split())) for l in subprocess.run([exe], capture_output=True, text=True).stdout.splitlines()]
    S, Y, K = abi.HpsiSpecies, abi.HpsiSystem, abi.HpsiKpoint
    assert got[0] == [C.sizeof(S), S.dq.offset, S.beta_q.offset, S.dbeta_q.offset]
    assert got[1] == [C.sizeof(Y), Y.lattice.offset, Y.omega.offset, Y.species.offset, Y.atom_tau.offset]
    assert got[2] == [C.sizeof(K), K.k_frac.offset, K.g_idx.offset, K.kinetic.offset]
    from effmass_gb300.serving import HpsiJob, HpsiServerConfig, HpsiServerStatistics
    B = abi.HpsiBatchItem
    assert got[3] == [C.sizeof(B), B.kid.offset, B.nb.offset]
    assert got[4] == [C.sizeof(HpsiJob), HpsiJob.psi.offset, HpsiJob.vel.offset]
    assert got[5] == [C.sizeof(HpsiServerConfig), HpsiServerConfig.device_budget_bytes.offset,
                      HpsiServerConfig.precision.offset, HpsiServerConfig.merge_max_bands.offset,
                      HpsiServerConfig.bypass_ms.offset]
    T = HpsiServerStatistics
    assert got[6] == [C.sizeof(T), T.peak_bytes.offset, T.merged_jobs.offset]


def test_cpp_wrapper_header_compiles():
    """include/hpsi_gb300.hpp (the Callable-style C++ mirror) is valid C++20 against the C header."""
    src = r"""
    #include "hpsi_gb300.hpp"
    #include <complex>
    #include <span>
    void use(hpsi::Hamiltonian& H, std::span<const std::complex<double>> psi, std::span<std::complex<double>> out) {
        auto op = H.at_k(0);
        op(psi, out);
        (void)op.dim();
    }
    int main() { return 0; }
    """
    with tempfile.TemporaryDirectory() as td:
        cfile = os.path.join(td, "w.cpp")
        open(cfile, "w").write(src)
        r = subprocess.run(["g++", "-std=c++20", "-fsyntax-only", "-I", os.path.dirname(HEADER), cfile],
                           capture_output=True, text=True)
        assert r.returncode == 0, r.stderr[-2000:]


def test_batch_rejects_bad_arguments_before_device_use(lib):
    h = C.c_void_p()
    lib.hpsi_batch_create.argtypes = [C.c_void_p, C.c_int, C.c_int, C.POINTER(C.c_void_p)]
    assert lib.hpsi_batch_create(None, 0, 0, C.byref(h)) == abi.HPSI_ERR_BAD_ARG
    assert not h.value
    items = (abi.HpsiBatchItem * 1)(abi.HpsiBatchItem(None, 0, 4))
    assert lib.hpsi_batch_create(C.cast(items, C.c_void_p), 1, abi.HPSI_PREC_TC, C.byref(h)) == abi.HPSI_ERR_BAD_ARG
    assert lib.hpsi_batch_create(C.cast(items, C.c_void_p), 1, 0, C.byref(h)) == abi.HPSI_ERR_BAD_ARG


def _has_gpu():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.mark.skipif(_has_gpu(), reason="checks the no-GPU failure path")
def test_no_gpu_fails_loudly(lib):
    from effmass_gb300 import system as S
    from effmass_gb300.hamiltonian import Hamiltonian
    from effmass_gb300._lib import HpsiError
    sysm = S.make_system("tiny")
    with pytest.raises(HpsiError) as ei:
        Hamiltonian(sysm)
    assert ei.value.status in (abi.HPSI_ERR_CUDA, abi.HPSI_ERR_OOM)


def test_invalid_system_rejected_before_device_use(lib):
    from effmass_gb300 import system as S
    from effmass_gb300.hamiltonian import Hamiltonian
    from effmass_gb300._lib import HpsiError
    sysm = S.make_system("tiny")
    sysm.n1 = 17 * 19  # prime factors beyond the FFT radices
    with pytest.raises(HpsiError) as ei:
        Hamiltonian(sysm)
    assert ei.value.status == abi.HPSI_ERR_BAD_ARG
    assert "FFT length" in str(ei.value)


def test_header_constants_match_abi():
    """Every numeric #define of include/hpsi_gb300.h that abi.py mirrors has the same value."""
    import re
    hdr = open(os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include",
                            "hpsi_gb300.h")).read()
    found = 0
    for name, val in re.findall(r"#define\s+(HPSI_\w+)\s+(0x[0-9A-Fa-f]+|-?\d+)", hdr):
        if hasattr(abi, name):
            assert getattr(abi, name) == int(val, 0), name
            found += 1
    assert found >= 10
