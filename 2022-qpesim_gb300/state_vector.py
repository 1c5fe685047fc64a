"""StateVector: the reference's QPE register (cpp/state_vector.hpp:16-379).

A complex128 numpy array of 2^precision blocks, each C(M, Na) * C(M, Nb)
amplitudes (block k = ancilla value k; inside a block, alpha rank major, beta rank
minor). qift() and IdentifyPhaseAmplitudes() run on the GPU through the C ABI.
"""
from __future__ import annotations

import ctypes as C
import math

import numpy as np

from . import _native as N


class StateVector(np.ndarray):
    def __new__(cls, precision: int, num_orbitals: int, num_occupied: int, num_occupied_beta: int | None = None):
        nb = num_occupied if num_occupied_beta is None else num_occupied_beta
        if not (0 < precision) or num_occupied > num_orbitals or nb > num_orbitals:
            raise ValueError("invalid StateVector shape")
        ca, cb = math.comb(num_orbitals, num_occupied), math.comb(num_orbitals, nb)
        obj = np.zeros((1 << precision) * ca * cb, np.complex128).view(cls)
        obj.precision = precision
        obj.num_orbitals = num_orbitals
        obj.num_occupied = num_occupied
        obj.num_occupied_beta = nb
        obj.c_alpha, obj.c_beta = ca, cb
        return obj

    def __array_finalize__(self, obj):
        if obj is None:
            return
        for k in ("precision", "num_orbitals", "num_occupied", "num_occupied_beta", "c_alpha", "c_beta"):
            setattr(self, k, getattr(obj, k, None))

    @property
    def ld(self) -> int:
        """Amplitudes per ancilla block."""
        return self.c_alpha * self.c_beta

    def block(self, k: int) -> np.ndarray:
        return np.asarray(self)[k * self.ld:(k + 1) * self.ld]

    def _dptr(self):
        a = np.asarray(self)
        assert a.flags.c_contiguous
        return a.view(np.float64).ctypes.data_as(C.POINTER(C.c_double))

    def qift(self, device: int = 0) -> None:
        """In-place QIFT (cpp/state_vector.hpp:115-179) on the GPU."""
        N.check(N.lib().qpe_qift(N.context(device), self.precision, self.ld, self._dptr()))

    def IdentifyPhaseAmplitudes(self, device: int = 0) -> np.ndarray:
        """Per-ancilla-value probability (cpp/state_vector.hpp:341-372) on the GPU."""
        probs = np.zeros(1 << self.precision)
        N.check(N.lib().qpe_identify_phase_amplitudes(N.context(device), self.precision, self.ld, self._dptr(),
                                                      probs.ctypes.data_as(C.POINTER(C.c_double))))
        return probs
