"""The batching form: many Hamiltonians in one graph launch (qpe_batch_*).

Batch(programs, precision, dtype) keeps one register per program. run() evolves
every register from its block 0, applies the QIFT and records each phase
histogram: one launch of one CUDA graph holding, per class of structurally
identical programs, a device-side loop over the controlled powers.
"""
from __future__ import annotations

import ctypes as C
import math

import numpy as np

from . import _native as N


class BatchInfo(C.Structure):
    _fields_ = [("instances", C.c_uint32), ("classes", C.c_uint32), ("touches_per_run", C.c_uint64),
                ("amplitudes", C.c_uint64), ("launches_per_run", C.c_uint32), ("reserved", C.c_uint32)]


class BatchClass(C.Structure):
    _fields_ = [("num_orbitals", C.c_uint32), ("n_alpha", C.c_uint32), ("n_beta", C.c_uint32),
                ("members", C.c_uint32), ("touches_per_power", C.c_uint64), ("ms_per_power", C.c_float),
                ("tile_lines", C.c_uint32), ("warps_per_cta", C.c_uint32)]


_PROTOS = {
    "qpe_batch_create": (C.c_int, [C.c_void_p, C.c_uint32, C.POINTER(C.c_void_p), C.c_uint32, C.c_int,
                                   C.POINTER(C.c_void_p)]),
    "qpe_batch_destroy": (C.c_int, [C.c_void_p]),
    "qpe_batch_upload": (C.c_int, [C.c_void_p, C.c_uint32, C.c_void_p, C.c_uint64, C.c_uint64]),
    "qpe_batch_download": (C.c_int, [C.c_void_p, C.c_uint32, C.c_void_p, C.c_uint64, C.c_uint64]),
    "qpe_batch_tune": (C.c_int, [C.c_void_p]),
    "qpe_batch_run": (C.c_int, [C.c_void_p, C.c_int]),
    "qpe_batch_phase_probs": (C.c_int, [C.c_void_p, C.c_uint32, C.POINTER(C.c_double)]),
    "qpe_batch_get_info": (C.c_int, [C.c_void_p, C.POINTER(BatchInfo)]),
    "qpe_batch_class_info": (C.c_int, [C.c_void_p, C.c_uint32, C.POINTER(BatchClass)]),
}


def _lib():
    L = N.lib()
    if not getattr(L, "_batch_protos", False):
        for name, (res, args) in _PROTOS.items():
            fn = getattr(L, name)
            fn.restype, fn.argtypes = res, args
        L._batch_protos = True
    return L


class Batch:
    def __init__(self, programs, precision: int, dtype=np.complex64, device: int = 0):
        self.dtype = np.dtype(dtype)
        code = {np.dtype(np.complex128): N.QPE_C128, np.dtype(np.complex64): N.QPE_C64}[self.dtype]
        self.programs = list(programs)  # keeps the programs alive
        self.precision = precision
        self.shapes = [(p.num_orbitals, p.n_alpha, p.n_beta) for p in self.programs]
        self.ld = [math.comb(m, a) * math.comb(m, b) for m, a, b in self.shapes]
        self._lib = _lib()
        arr = (C.c_void_p * len(self.programs))(*[p._h.value for p in self.programs])
        h = C.c_void_p()
        N.check(self._lib.qpe_batch_create(N.context(device), len(self.programs), arr, precision, code, C.byref(h)))
        self._h = h

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            self._lib.qpe_batch_destroy(h)
            self._h = None

    def __len__(self):
        return len(self.programs)

    @property
    def info(self) -> dict:
        i = BatchInfo()
        N.check(self._lib.qpe_batch_get_info(self._h, C.byref(i)))
        return {f: getattr(i, f) for f, _ in BatchInfo._fields_}

    def classes(self) -> list:
        """Per class: orbitals, electrons per spin, members, touches per power
        (all members) and the tuned time of one power of the class alone."""
        out = []
        for i in range(self.info["classes"]):
            c = BatchClass()
            N.check(self._lib.qpe_batch_class_info(self._h, i, C.byref(c)))
            out.append({f: getattr(c, f) for f, _ in BatchClass._fields_})
        return out

    def upload(self, i: int, host: np.ndarray, first: int = 0) -> None:
        a = np.ascontiguousarray(host, self.dtype)
        N.check(self._lib.qpe_batch_upload(self._h, i, a.ctypes.data_as(C.c_void_p), first, a.size))

    def download(self, i: int, first: int = 0, count: int | None = None, out=None) -> np.ndarray:
        size = (1 << self.precision) * self.ld[i]
        count = size - first if count is None else count
        out = np.empty(count, self.dtype) if out is None else out
        N.check(self._lib.qpe_batch_download(self._h, i, out.ctypes.data_as(C.c_void_p), first, count))
        return out

    def tune(self) -> None:
        N.check(self._lib.qpe_batch_tune(self._h))

    def run(self, synchronize: bool = True) -> None:
        N.check(self._lib.qpe_batch_run(self._h, 1 if synchronize else 0))

    def phase_probs(self, i: int) -> np.ndarray:
        p = np.zeros(1 << self.precision)
        N.check(self._lib.qpe_batch_phase_probs(self._h, i, p.ctypes.data_as(C.POINTER(C.c_double))))
        return p
