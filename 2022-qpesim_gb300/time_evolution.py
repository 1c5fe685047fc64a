"""Controlled Trotterized evolution on the GPU.

time_evolve_over_terms(state_vector, hamiltonian, precision) is the reference's
call (cpp/time_evolution_over_terms.hpp:92-139) with the same arguments and
effect: block k of the register becomes U^k applied to block 0, U one
first-order Trotter step in the term order of applyUnitary_reordered.

Program and DeviceState are the device-resident form: a Program holds one
Hamiltonian's compiled term passes and index tables, a DeviceState a
2^P x Ca x Cb register (complex128 or complex64) that stays in HBM between
evolve(), qift() and phase_probs().
"""
from __future__ import annotations

import ctypes as C
import math

import numpy as np

from . import _native as N
from .hamiltonian import Hamiltonian


def time_evolve_over_terms(state_vector, hamiltonian: Hamiltonian, precision: int, device: int = 0) -> complex:
    """Evolves every block of `state_vector` from its block 0 (host buffers; the
    library copies block 0 to the device and the whole register back)."""
    M, e = hamiltonian.num_orbitals(), hamiltonian.num_occupied()
    ld = math.comb(M, e) ** 2
    a = np.asarray(state_vector)
    if a.dtype != np.complex128 or not a.flags.c_contiguous or a.size != (1 << precision) * ld:
        raise ValueError("state_vector must be a contiguous complex128 array of 2^precision * C(M, e)^2")
    args, keep = N.seg_args(hamiltonian.segmented_terms())
    N.check(N.lib().qpe_time_evolve_over_terms(N.context(device), M, e, precision, *args,
                                               a.view(np.float64).ctypes.data_as(C.POINTER(C.c_double))))
    return complex(0.0)  # the reference returns an unset std::complex (:98, :138)


def time_evolve_iqpe(state_vector, hamiltonian: Hamiltonian, num_of_applications: int, device: int = 0) -> None:
    """The reference's time_evolve_iqpe (cpp/time_evolution_over_terms.hpp:141-155):
    block 1 of `state_vector` receives num_of_applications sweeps of U in the term
    order of applyUnitary (:174-372), in place; no block is copied."""
    M, e = hamiltonian.num_orbitals(), hamiltonian.num_occupied()
    ld = math.comb(M, e) ** 2
    a = np.asarray(state_vector)
    if a.dtype != np.complex128 or not a.flags.c_contiguous or a.size % ld or a.size < 2 * ld:
        raise ValueError("state_vector must be a contiguous complex128 array of 2^precision * C(M, e)^2, precision >= 1")
    precision = (a.size // ld).bit_length() - 1
    args, keep = N.seg_args(hamiltonian.segmented_terms())
    N.check(N.lib().qpe_time_evolve_iqpe(N.context(device), M, e, precision, *args, int(num_of_applications),
                                         a.view(np.float64).ctypes.data_as(C.POINTER(C.c_double))))


def plan_program(seg: dict, num_orbitals: int, n_alpha: int, n_beta: int, trotter_order: int = 1,
                 steps: int = 1) -> dict:
    """Host-only planning of a Program (qpe_program_plan): op, pass and update counts."""
    args, keep = N.seg_args(seg)
    info = N.ProgramInfo()
    N.check(N.lib().qpe_program_plan(num_orbitals, n_alpha, n_beta, *args, trotter_order, steps, C.byref(info)))
    return {f: getattr(info, f) for f, _ in N.ProgramInfo._fields_}


class Program:
    """Compiled term program of one Hamiltonian (qpe_program_create).

    trotter_order 2 applies a forward and a reversed sweep per step; pass
    coefficients computed at half the step for a symmetric product. steps is the
    number of Trotter steps per controlled power. (1, 1) is the reference.
    apply_unitary_order builds the sweep in applyUnitary's term order (the
    iterative variant) instead of applyUnitary_reordered's."""

    def __init__(self, hamiltonian_or_terms, num_orbitals=None, n_alpha=None, n_beta=None, trotter_order=1,
                 steps=1, device=0, apply_unitary_order=False):
        if isinstance(hamiltonian_or_terms, Hamiltonian):
            h = hamiltonian_or_terms
            seg = h.segmented_terms()
            num_orbitals = h.num_orbitals()
            n_alpha = n_alpha or h.num_occupied()
            n_beta = n_beta or n_alpha
        else:
            seg = hamiltonian_or_terms
        self.num_orbitals, self.n_alpha, self.n_beta = int(num_orbitals), int(n_alpha), int(n_beta)
        self.device = device
        self._lib = N.lib()
        args, keep = N.seg_args(seg)
        h = C.c_void_p()
        N.check(self._lib.qpe_program_create(N.context(device), self.num_orbitals, self.n_alpha, self.n_beta, *args,
                                             int(trotter_order) | (N.QPE_PROGRAM_APPLY_UNITARY_ORDER
                                                                   if apply_unitary_order else 0),
                                             int(steps), C.byref(h)))
        self._h = h
        info = N.ProgramInfo()
        N.check(self._lib.qpe_program_get_info(h, C.byref(info)))
        self.info = {f: getattr(info, f) for f, _ in N.ProgramInfo._fields_}

    @property
    def touches_per_power(self) -> int:
        return int(self.info["touches_per_power"])

    def unit_schedule(self) -> tuple:
        """(cluster size, column-pair passes scheduled) of the update-unit schedule
        the program last built for strategy 7 (qpe_program_unit_schedule)."""
        k, n = C.c_uint32(), C.c_uint32()
        N.check(self._lib.qpe_program_unit_schedule(self._h, C.byref(k), C.byref(n)))
        return int(k.value), int(n.value)

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            self._lib.qpe_program_destroy(h)
            self._h = None


class DeviceState:
    """Device-resident QPE register (qpe_state_create)."""

    def __init__(self, num_orbitals, n_alpha, n_beta, precision, dtype=np.complex128, device=0):
        self.dtype = np.dtype(dtype)
        code = {np.dtype(np.complex128): N.QPE_C128, np.dtype(np.complex64): N.QPE_C64}[self.dtype]
        self.num_orbitals, self.n_alpha, self.n_beta, self.precision = num_orbitals, n_alpha, n_beta, precision
        self.c_alpha, self.c_beta = math.comb(num_orbitals, n_alpha), math.comb(num_orbitals, n_beta)
        self.ld = self.c_alpha * self.c_beta
        self.size = (1 << precision) * self.ld
        self._lib = N.lib()
        h = C.c_void_p()
        N.check(self._lib.qpe_state_create(N.context(device), num_orbitals, n_alpha, n_beta, precision, code,
                                           C.byref(h)))
        self._h = h

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            self._lib.qpe_state_destroy(h)
            self._h = None

    def upload(self, host: np.ndarray, first: int = 0) -> None:
        a = np.ascontiguousarray(host, self.dtype)
        N.check(self._lib.qpe_state_upload(self._h, a.ctypes.data_as(C.c_void_p), first, a.size))

    def download(self, first: int = 0, count: int | None = None, out: np.ndarray | None = None) -> np.ndarray:
        count = self.size - first if count is None else count
        out = np.empty(count, self.dtype) if out is None else out
        N.check(self._lib.qpe_state_download(self._h, out.ctypes.data_as(C.c_void_p), first, count))
        return out

    def zero(self) -> None:
        N.check(self._lib.qpe_state_zero(self._h))

    def evolve(self, program: Program, first_power: int = 0, last_power: int = 0, strategy: int = 0,
               cluster_size: int = 0, fp64_contract: bool = False, replicas: int = 0) -> None:
        """strategy: 0 auto (autotuned per program), 1 one CTA resident in shared
        memory, 2 a cluster of cluster_size CTAs (0: smallest that fits), 3
        global-memory tile passes, 4 a cluster whose tiles are processed by
        four-warp groups with every update split over four lanes, 5 a cluster
        whose column-pair tiles are processed as in 4 and row and column tiles
        as in 2, 6 a cluster whose rows, columns and column pairs are each
        processed by a three-warp group (pair updates over four lanes, diagonal
        updates over two), 7 as 6 with the column-pair passes as windows of
        independent update units; with 7, `replicas` clusters (up to 8) each hold
        the block and split the row and column passes. fp64_contract allows FMAs
        in complex128 (within 1e-12 of the reference instead of bit-identical)."""
        opts = N.EvolveOpts(strategy, first_power, last_power, cluster_size,
                            N.QPE_EVOLVE_FP64_CONTRACT if fp64_contract else 0, 0, replicas)
        N.check(self._lib.qpe_evolve(self._h, program._h, C.byref(opts)))

    def evolve_in_place(self, program: Program, block: int = 1, repeats: int = 1, strategy: int = 0,
                        cluster_size: int = 0, fp64_contract: bool = False, replicas: int = 0) -> None:
        """Applies the program's power `repeats` times to block `block` in place
        (time_evolve_iqpe's evolution with block = 1)."""
        flags = N.QPE_EVOLVE_IN_PLACE | (N.QPE_EVOLVE_FP64_CONTRACT if fp64_contract else 0)
        opts = N.EvolveOpts(strategy, block, 0, cluster_size, flags, repeats, replicas)
        N.check(self._lib.qpe_evolve(self._h, program._h, C.byref(opts)))

    def qift(self) -> None:
        N.check(self._lib.qpe_state_qift(self._h))

    def phase_probs(self) -> np.ndarray:
        p = np.zeros(1 << self.precision)
        N.check(self._lib.qpe_state_phase_probs(self._h, p.ctypes.data_as(C.POINTER(C.c_double))))
        return p

    def last_replicas(self) -> int:
        """Replica clusters of the last evolve (1 unless strategy 7 ran with replicas)."""
        r = C.c_uint32()
        N.check(self._lib.qpe_state_last_replicas(self._h, C.byref(r)))
        return r.value

    def last_strategy(self) -> tuple:
        """(strategy, cluster size) of the last evolve: 1 resident, 2 cluster, 3 tiled, 4 grouped cluster,
        5 cluster with grouped column-pair tiles, 6 cluster of three-warp groups."""
        s, k = C.c_uint32(), C.c_uint32()
        N.check(self._lib.qpe_state_last_strategy(self._h, C.byref(s), C.byref(k)))
        return s.value, k.value

    def block_norms(self) -> np.ndarray:
        p = np.zeros(1 << self.precision)
        N.check(self._lib.qpe_state_block_norms(self._h, p.ctypes.data_as(C.POINTER(C.c_double))))
        return p
