"""OffsetComputer: combinatorial ranks of fixed-weight bit strings
(cpp/offset_computer.hpp:14-252), computed by the device kernels.

rank() batches OffsetComputer::rank; an instance built from one bit vector answers
rank_with_swap / rank_with_double_swap from device-built prefix tables.
"""
from __future__ import annotations

import ctypes as C
import math

import numpy as np

from . import _native as N

_NO = 0xFFFFFFFF


class OffsetComputer:
    def __init__(self, n: int, bv: int, bv_rank: int | None = None, device: int = 0):
        self.n, self.bv, self.device = int(n), int(bv), device
        self._rank = OffsetComputer.rank(bv, device=device)
        if bv_rank is not None and bv_rank != self._rank:
            raise ValueError("bv_rank does not match rank(bv)")

    @staticmethod
    def ranks(bvs, device: int = 0) -> np.ndarray:
        a = np.ascontiguousarray(bvs, np.uint64)
        out = np.zeros(len(a), np.int64)
        N.check(N.lib().qpe_rank(N.context(device), a.ctypes.data_as(C.POINTER(C.c_uint64)),
                                 out.ctypes.data_as(C.POINTER(C.c_int64)), len(a)))
        return out

    @staticmethod
    def rank(bv, device: int = 0):
        """OffsetComputer::rank (:16-27). Scalar in, scalar out; arrays batch."""
        if np.ndim(bv):
            return OffsetComputer.ranks(bv, device)
        return int(OffsetComputer.ranks([bv], device)[0])

    @staticmethod
    def unrank(nbits: int, weight: int, ranks, device: int = 0) -> np.ndarray:
        r = np.ascontiguousarray(np.atleast_1d(ranks), np.int64)
        out = np.zeros(len(r), np.uint64)
        N.check(N.lib().qpe_unrank(N.context(device), nbits, weight, r.ctypes.data_as(C.POINTER(C.c_int64)),
                                   out.ctypes.data_as(C.POINTER(C.c_uint64)), len(r)))
        return out

    def _query(self, rows) -> np.ndarray:
        q = np.ascontiguousarray(rows, np.uint32).reshape(-1, 4)
        out = np.zeros(len(q), np.int64)
        N.check(N.lib().qpe_rank_with_swaps(N.context(self.device), self.n, self.bv,
                                            q.ctypes.data_as(C.POINTER(C.c_uint32)),
                                            out.ctypes.data_as(C.POINTER(C.c_int64)), len(q)))
        return out

    def rank_with_swap(self, i: int, j: int) -> int:
        return int(self._query([(i, j, _NO, _NO)])[0])

    def rank_with_double_swap(self, i: int, j: int, k: int, l: int) -> int:
        return int(self._query([(i, j, k, l)])[0])

    def rank_with_swaps(self, rows) -> np.ndarray:
        """Batch: rows of (i, j, k, l); k = l = 0xFFFFFFFF marks a single swap."""
        return self._query(rows)

    def rank_self(self) -> int:
        return self._rank


TABLE_KINDS = {"N": 0, "NN": 1, "CA": 2, "CNA": 3, "CCAA": 4}


def axis_table(kind, nbits: int, weight: int, orbitals, device: int = 0):
    """Device-built index table of one discover*_BVs routine with the runs
    expanded: (i01, i10, parity) arrays (i10 / parity zero for N and NN)."""
    k = TABLE_KINDS[kind] if isinstance(kind, str) else int(kind)
    orb = np.zeros(4, np.uint32)
    orb[:len(orbitals)] = orbitals
    cnt = C.c_size_t()
    nfix, nocc = (1, 2, 2, 3, 4)[k], (1, 2, 1, 2, 2)[k]
    cap = math.comb(nbits - nfix, weight - nocc) if weight >= nocc else 0
    i01 = np.zeros(max(cap, 1), np.uint32)
    i10 = np.zeros(max(cap, 1), np.uint32)
    par = np.zeros(max(cap, 1), np.uint8)
    N.check(N.lib().qpe_axis_table(N.context(device), k, nbits, weight, orb.ctypes.data_as(C.POINTER(C.c_uint32)),
                                   i01.ctypes.data_as(C.POINTER(C.c_uint32)), i10.ctypes.data_as(C.POINTER(C.c_uint32)),
                                   par.ctypes.data_as(C.POINTER(C.c_uint8)), max(cap, 1), C.byref(cnt)))
    n = cnt.value
    return i01[:n], i10[:n], par[:n]
