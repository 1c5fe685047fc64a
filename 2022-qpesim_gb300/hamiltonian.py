"""Hamiltonian: the reference's term-compiler interface (cpp/hamiltonian.hpp:24-184)
over the native host compiler (include/qpe_gb300_hamiltonian.h).

Method names, argument meaning and conventions follow the reference:
1-based spatial orbitals for AddOneBodyTerm / AddTwoBodyTerm, 0-based HalfUp
spin-orbital indices (alpha o -> o, beta o -> M + o) for the coefficient getters.
"""
from __future__ import annotations

import ctypes as C
import enum

import numpy as np

from . import _native as N
from .synthetic import Integrals


class SpinIndex(enum.IntEnum):
    """cpp/types.hpp:15-19. Only HalfUp is used by the hot path."""
    HalfUp = 0
    UpDown = 1


class Hamiltonian:
    def __init__(self):
        h = C.c_void_p()
        N.check(N.lib().qpe_ham_create(C.byref(h)))
        self._h = h
        self._lib = N.lib()

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            self._lib.qpe_ham_destroy(h)
            self._h = None

    # ---- compiler methods (cpp/hamiltonian.cc:301-398) ----
    def AddOneBodyTerm(self, targets, coeff: float) -> None:
        p, q = targets
        N.check(self._lib.qpe_ham_add_one_body(self._h, int(p), int(q), float(coeff)))

    def AddTwoBodyTerm(self, targets, coeff: float) -> None:
        p, q, r, s = targets
        N.check(self._lib.qpe_ham_add_two_body(self._h, int(p), int(q), int(r), int(s), float(coeff)))

    def IndexTerms(self, convention: SpinIndex = SpinIndex.HalfUp) -> None:
        if convention != SpinIndex.HalfUp:
            raise ValueError("only SpinIndex.HalfUp is supported (the hot path's convention)")
        N.check(self._lib.qpe_ham_index_terms(self._h))

    def IngestBroombridge(self, filepath, precision: int = 5):
        """Reads a Broombridge file (cpp/hamiltonian.cc:8-144) with the native
        reader; returns the StateVector with the first initial-state suggestion
        (Jordan-Wigner signs applied) in block 0."""
        from .state_vector import StateVector
        path = str(filepath).encode()
        m, e = C.c_uint32(), C.c_uint32()
        probe = Hamiltonian()
        N.check(self._lib.qpe_ham_ingest_broombridge(probe._h, path, C.byref(m), C.byref(e), None, 0))
        sv = StateVector(precision, m.value, e.value)
        blk = np.zeros(sv.ld, np.complex128)
        N.check(self._lib.qpe_ham_ingest_broombridge(self._h, path, None, None,
                                                     blk.view(np.float64).ctypes.data_as(C.POINTER(C.c_double)),
                                                     sv.ld))
        sv[:sv.ld] = blk
        return sv

    # ---- fields the reference sets while ingesting (cpp/hamiltonian.hpp:144-150) ----
    def SetNumOrbitals(self, m: int) -> None:
        N.check(self._lib.qpe_ham_set_num_orbitals(self._h, int(m)))

    def SetIdentity(self, v: float) -> None:
        N.check(self._lib.qpe_ham_set_identity(self._h, float(v)))

    def SetNumOccupied(self, e: int) -> None:
        N.check(self._lib.qpe_ham_set_num_occupied(self._h, int(e)))

    def SetTimestep(self, t: float) -> None:
        N.check(self._lib.qpe_ham_set_timestep(self._h, float(t)))

    def num_orbitals(self) -> int:
        v = C.c_uint32()
        N.check(self._lib.qpe_ham_get_num_orbitals(self._h, C.byref(v)))
        return v.value

    def num_occupied(self) -> int:
        v = C.c_uint32()
        N.check(self._lib.qpe_ham_get_num_occupied(self._h, C.byref(v)))
        return v.value

    def GetIdentityTerm(self) -> float:
        v = C.c_double()
        N.check(self._lib.qpe_ham_get_identity(self._h, C.byref(v)))
        return v.value

    # ---- segmented terms (cpp/hamiltonian.cc:253-299) ----
    def segment_counts(self) -> dict:
        c = (C.c_size_t * 5)()
        N.check(self._lib.qpe_ham_segment_counts(self._h, c))
        return {k: int(c[i]) for i, k in enumerate(N.TERM_KINDS)}

    def segmented_terms(self) -> dict:
        """kind -> TERM_DTYPE array: indices plus the coefficient getters at the
        current timestep (the arrays the C ABI consumes)."""
        counts = self.segment_counts()
        out = {}
        for i, k in enumerate(N.TERM_KINDS):
            a = np.zeros(counts[k], N.TERM_DTYPE)
            if counts[k]:
                N.check(self._lib.qpe_ham_segment_terms(self._h, i, a.ctypes.data_as(C.POINTER(N.QpeTerm)), None,
                                                        counts[k]))
            out[k] = a
        return out

    def PrintIndexedSegmentedHamiltonianTerms(self):
        """(pp, pq, pqqp, pqqr, pqrs) lists of ((indices), coefficient), map order."""
        counts = self.segment_counts()
        res = []
        for i, k in enumerate(N.TERM_KINDS):
            a = np.zeros(counts[k], N.TERM_DTYPE)
            raw = np.zeros(counts[k])
            if counts[k]:
                N.check(self._lib.qpe_ham_segment_terms(self._h, i, a.ctypes.data_as(C.POINTER(N.QpeTerm)),
                                                        raw.ctypes.data_as(C.POINTER(C.c_double)), counts[k]))
            if i < 2:
                res.append([((int(t["p"]), int(t["q"])), float(v)) for t, v in zip(a, raw)])
            else:
                res.append([((int(t["p"]), int(t["q"]), int(t["r"]), int(t["s"])), float(v)) for t, v in zip(a, raw)])
        return tuple(res)

    # ---- coefficient getters (cpp/hamiltonian.cc:661-783) ----
    def pp_term(self, p: int) -> complex:
        o = (C.c_double * 2)()
        N.check(self._lib.qpe_ham_pp_term(self._h, p, o))
        return complex(o[0], o[1])

    def _quad(self, fn, *args):
        o = (C.c_double * 8)()
        N.check(fn(self._h, *args, o))
        return [complex(o[2 * i], o[2 * i + 1]) for i in range(4)]

    def pq_term(self, p: int, q: int, parity: int):
        return self._quad(self._lib.qpe_ham_pq_term, p, q, parity)

    def pqqp_term(self, p: int, q: int) -> complex:
        o = (C.c_double * 2)()
        N.check(self._lib.qpe_ham_pqqp_term(self._h, p, q, o))
        return complex(o[0], o[1])

    def pqqr_term(self, p: int, q: int, r: int, parity: int):
        return self._quad(self._lib.qpe_ham_pqqr_term, p, q, r, parity)

    def pqrs_term(self, p: int, q: int, r: int, s: int, parity: int):
        return self._quad(self._lib.qpe_ham_pqrs_term, p, q, r, s, parity)

    # ---- convenience ----
    @classmethod
    def from_integrals(cls, ints: Integrals, num_occupied: int, timestep: float) -> "Hamiltonian":
        """AddOneBodyTerm / AddTwoBodyTerm for every integral, then IndexTerms and
        SetTimestep, the way IngestBroombridge + main set a Hamiltonian up."""
        h = cls()
        h.SetNumOrbitals(ints.n_orbitals)
        h.SetIdentity(ints.identity)
        h.SetNumOccupied(num_occupied)
        for p, q, v in ints.one_body:
            h.AddOneBodyTerm((p, q), v)
        for p, q, r, s, v in ints.two_body:
            h.AddTwoBodyTerm((p, q, r, s), v)
        h.IndexTerms()
        h.SetTimestep(timestep)
        return h
