"""Python view of the serving loop of libhpsi_gb300.so (hpsi_server_*).

    srv = Server([H_fcc2, H_sc8, H_sc64], lanes=4, budget_gb=24, precision="tc")
    t = srv.submit([Job(system=0, kid=3, psi=psi, hpsi=out, vel=v), ...])
    times = srv.wait(t)          # {'queue_ms', 'run_ms', 'total_ms'}

Jobs run on the GPU concurrently (one CUDA stream per lane); a job is admitted,
in arrival order (later jobs that fit may overtake for up to ``bypass_ms``), as
soon as a lane is free and its buffers fit in the device budget; with
``merge_max_bands`` > 0 jobs of small cells are merged into one ragged launch
set.  A request completes when its last job does.  Arrays are host numpy complex128 (pinned memory, e.g. from
``pinned_empty``, gives asynchronous copies) and must stay alive until wait().
"""
from __future__ import annotations

import ctypes as C
import dataclasses
from typing import List, Optional

import numpy as np

from . import abi
from ._lib import HpsiError, load


class HpsiJob(C.Structure):
    _fields_ = [("system", C.c_int), ("kid", C.c_int), ("nb", C.c_int), ("psi", C.c_void_p),
                ("hpsi", C.c_void_p), ("vel", C.c_void_p)]


class HpsiServerConfig(C.Structure):
    _fields_ = [("lanes", C.c_int), ("device_budget_bytes", C.c_double), ("precision", C.c_int),
                ("merge_max_bands", C.c_int), ("bypass_ms", C.c_double)]


class HpsiRequestTimes(C.Structure):
    _fields_ = [("queue_ms", C.c_double), ("run_ms", C.c_double), ("total_ms", C.c_double)]


class HpsiServerStatistics(C.Structure):
    _fields_ = [("completed", C.c_longlong), ("queued", C.c_longlong), ("running", C.c_longlong),
                ("budget_bytes", C.c_double), ("peak_bytes", C.c_double), ("units", C.c_longlong),
                ("merged_units", C.c_longlong), ("merged_jobs", C.c_longlong)]


def _bind(L):
    if getattr(L, "_srv_bound", False):
        return
    L.hpsi_server_create.argtypes = [C.POINTER(C.c_void_p), C.c_int, C.POINTER(HpsiServerConfig),
                                     C.POINTER(C.c_void_p)]
    L.hpsi_server_submit.argtypes = [C.c_void_p, C.POINTER(HpsiJob), C.c_int, C.POINTER(C.c_longlong)]
    L.hpsi_server_wait.argtypes = [C.c_void_p, C.c_longlong, C.c_double, C.POINTER(HpsiRequestTimes)]
    L.hpsi_server_stats.argtypes = [C.c_void_p, C.POINTER(HpsiServerStatistics)]
    L.hpsi_server_destroy.argtypes = [C.c_void_p]
    L.hpsi_server_last_error.argtypes = [C.c_void_p]
    L.hpsi_server_last_error.restype = C.c_char_p
    for n in ("hpsi_server_create", "hpsi_server_submit", "hpsi_server_wait", "hpsi_server_stats",
              "hpsi_server_destroy"):
        getattr(L, n).restype = C.c_int
    L._srv_bound = True


class _PinnedArray(np.ndarray):
    """ndarray view of page-locked memory that keeps its owning tensor alive."""


def pinned_empty(shape, dtype=np.complex128):
    """A page-locked host array (through torch) for asynchronous copies."""
    import torch
    tdt = {np.complex128: torch.complex128, np.float64: torch.float64}[np.dtype(dtype).type]
    t = torch.empty(tuple(shape), dtype=tdt).pin_memory()
    arr = t.numpy().view(_PinnedArray)
    arr._owner = t
    return arr


@dataclasses.dataclass
class Job:
    system: int
    kid: int
    psi: np.ndarray                 # [nb, npw] complex128
    hpsi: np.ndarray                # [nb, npw] complex128, accumulated
    vel: Optional[np.ndarray] = None  # [3, nb, nb] complex128 or None

    @property
    def nb(self) -> int:
        return int(self.psi.shape[0]) if self.psi.ndim == 2 else 1


class Server:
    def __init__(self, hamiltonians: List, lanes: int = 4, budget_gb: float = 16.0, precision: str = "tc",
                 merge_max_bands: int = 0, bypass_ms: float = 0.0):
        self._lib = load()
        _bind(self._lib)
        self._hams = list(hamiltonians)
        arr = (C.c_void_p * len(self._hams))(*[h.ctx.value for h in self._hams])
        cfg = HpsiServerConfig(lanes, budget_gb * (1 << 30), abi.PRECISIONS[precision], merge_max_bands, bypass_ms)
        h = C.c_void_p()
        st = self._lib.hpsi_server_create(arr, len(self._hams), C.byref(cfg), C.byref(h))
        if st:
            raise HpsiError(st, (self._lib.hpsi_server_last_error(None) or b"").decode())
        self._srv = h
        self._keep = {}

    def _check(self, st):
        if st:
            raise HpsiError(st, (self._lib.hpsi_server_last_error(self._srv) or b"").decode())

    def submit(self, jobs: List[Job]) -> int:
        arr = (HpsiJob * len(jobs))()
        for i, j in enumerate(jobs):
            for a in (j.psi, j.hpsi) + ((j.vel,) if j.vel is not None else ()):
                if a.dtype != np.complex128 or not a.flags["C_CONTIGUOUS"]:
                    raise HpsiError(abi.HPSI_ERR_BAD_ARG, "jobs need C-contiguous complex128 arrays")
            arr[i] = HpsiJob(j.system, j.kid, j.nb, j.psi.ctypes.data, j.hpsi.ctypes.data,
                             j.vel.ctypes.data if j.vel is not None else None)
        t = C.c_longlong()
        self._check(self._lib.hpsi_server_submit(self._srv, arr, len(jobs), C.byref(t)))
        self._keep[t.value] = jobs
        return t.value

    def wait(self, ticket: int, timeout_s: float = 600.0):
        tm = HpsiRequestTimes()
        st = self._lib.hpsi_server_wait(self._srv, ticket, timeout_s, C.byref(tm))
        self._keep.pop(ticket, None)
        self._check(st)
        return {"queue_ms": tm.queue_ms, "run_ms": tm.run_ms, "total_ms": tm.total_ms}

    def stats(self):
        s = HpsiServerStatistics()
        self._check(self._lib.hpsi_server_stats(self._srv, C.byref(s)))
        return {"completed": s.completed, "queued": s.queued, "running": s.running,
                "budget_bytes": s.budget_bytes, "peak_bytes": s.peak_bytes, "units": s.units,
                "merged_units": s.merged_units, "merged_jobs": s.merged_jobs}

    def close(self):
        if getattr(self, "_srv", None):
            self._lib.hpsi_server_destroy(self._srv)
            self._srv = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
