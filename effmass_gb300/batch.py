"""Python view of the batched k-point plans of libhpsi_gb300.so (hpsi_batch_*).

    plan = Batch([(H_fcc2, kid, 32) for kid in range(216)] + [(H_sc8, kid, 48) for kid in range(64)],
                 precision="fp32")
    hpsi = plan.apply(psi_packed, hpsi_packed)       # hpsi += H psi for every item
    plan.info()                                      # tuned tiles per cell

psi/hpsi are packed item after item, each item [nb][npw] band-major complex128
(``plan.split(x)`` gives per-item views).  ``plan.run()`` applies H to the
plan's own device buffers (``plan.device_buffers()``) with one graph launch.
"""
from __future__ import annotations

import ctypes as C
import json
from typing import List, Sequence, Tuple

import numpy as np

from . import abi
from ._lib import HpsiError, load


def _bind(L):
    if getattr(L, "_batch_bound", False):
        return
    L.hpsi_batch_create.argtypes = [C.POINTER(abi.HpsiBatchItem), C.c_int, C.c_int, C.POINTER(C.c_void_p)]
    L.hpsi_batch_buffers.argtypes = [C.c_void_p, C.POINTER(C.c_void_p), C.POINTER(C.c_void_p),
                                     C.POINTER(C.c_size_t)]
    L.hpsi_batch_offset.argtypes = [C.c_void_p, C.c_int, C.POINTER(C.c_size_t)]
    L.hpsi_batch_run.argtypes = [C.c_void_p, C.c_void_p]
    L.hpsi_batch_apply.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_void_p]
    L.hpsi_batch_info.argtypes = [C.c_void_p, C.c_char_p, C.c_size_t]
    L.hpsi_batch_destroy.argtypes = [C.c_void_p]
    L.hpsi_batch_last_error.argtypes = [C.c_void_p]
    L.hpsi_batch_last_error.restype = C.c_char_p
    L._batch_bound = True


class Batch:
    """A plan over items (hamiltonian, kid, nb); precision "fp32", "fp64", or
    "tc" / "tc_bf16" (the nonlocal term as ragged tensor-core GEMMs)."""

    def __init__(self, items: Sequence[Tuple[object, int, int]], precision: str = "fp32", graph: bool = True,
                 tune: bool = True):
        self._lib = load()
        _bind(self._lib)
        self._items = [(h, int(k), int(nb)) for h, k, nb in items]
        arr = (abi.HpsiBatchItem * len(self._items))()
        for i, (h, k, nb) in enumerate(self._items):
            arr[i] = abi.HpsiBatchItem(h.ctx.value, k, nb)
        flags = abi.PRECISIONS[precision]
        if not graph:
            flags |= abi.HPSI_BATCH_NO_GRAPH
        if not tune:
            flags |= abi.HPSI_BATCH_NO_TUNE
        h = C.c_void_p()
        st = self._lib.hpsi_batch_create(arr, len(self._items), flags, C.byref(h))
        if st:
            raise HpsiError(st, (self._lib.hpsi_batch_last_error(None) or b"").decode())
        self._b = h
        self.npw = [hm.dim(k) for hm, k, _ in self._items]
        self.nb = [nb for _, _, nb in self._items]
        self.offsets = []
        for i in range(len(self._items)):
            o = C.c_size_t()
            self._check(self._lib.hpsi_batch_offset(self._b, i, C.byref(o)))
            self.offsets.append(o.value)
        self.n_complex = int(sum(n * b for n, b in zip(self.npw, self.nb)))

    def _check(self, st):
        if st:
            raise HpsiError(st, (self._lib.hpsi_batch_last_error(self._b) or b"").decode())

    def empty(self) -> np.ndarray:
        return np.zeros(self.n_complex, dtype=np.complex128)

    def split(self, x: np.ndarray) -> List[np.ndarray]:
        """Per-item [nb][npw] views of a packed array."""
        return [x[o:o + b * n].reshape(b, n) for o, b, n in zip(self.offsets, self.nb, self.npw)]

    def pack(self, arrays: Sequence[np.ndarray], out=None) -> np.ndarray:
        out = self.empty() if out is None else out
        for v, a in zip(self.split(out), arrays):
            v[...] = a
        return out

    def device_buffers(self):
        """(psi, hpsi, n_complex): device pointers of the plan's resident buffers."""
        p, h, n = C.c_void_p(), C.c_void_p(), C.c_size_t()
        self._check(self._lib.hpsi_batch_buffers(self._b, C.byref(p), C.byref(h), C.byref(n)))
        return p.value, h.value, n.value

    def run(self, stream=None):
        """hpsi_buffer += H psi_buffer on the device (one graph launch)."""
        s = stream.cuda_stream if stream is not None and hasattr(stream, "cuda_stream") else stream
        self._check(self._lib.hpsi_batch_run(self._b, s))

    def apply(self, psi, hpsi, stream=None, device: bool = False):
        """hpsi += H psi for packed host (numpy) or device (torch) arrays."""
        if device:
            pp, hp, flags = psi.data_ptr(), hpsi.data_ptr(), abi.HPSI_DEVICE_PTRS | abi.HPSI_SYNC
        else:
            for a in (psi, hpsi):
                if a.dtype != np.complex128 or not a.flags["C_CONTIGUOUS"] or a.size != self.n_complex:
                    raise HpsiError(abi.HPSI_ERR_BAD_ARG, "packed C-contiguous complex128 arrays of n_complex")
            pp, hp, flags = psi.ctypes.data, hpsi.ctypes.data, 0
        s = stream.cuda_stream if stream is not None and hasattr(stream, "cuda_stream") else stream
        self._check(self._lib.hpsi_batch_apply(self._b, pp, hp, flags, s))
        return hpsi

    def info(self) -> dict:
        n = self._lib.hpsi_batch_info(self._b, None, 0)
        buf = C.create_string_buffer(max(n, 1))
        self._lib.hpsi_batch_info(self._b, buf, n)
        return json.loads(buf.value.decode())

    def close(self):
        if getattr(self, "_b", None):
            self._lib.hpsi_batch_destroy(self._b)
            self._b = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
