"""ctypes bindings of lib/libqpe_gb300.so (include/qpe_gb300.h,
include/qpe_gb300_hamiltonian.h).

The library is the only compute path: if it is missing or fails to load, every
entry point raises instead of falling back to anything else.
"""
from __future__ import annotations

import ctypes as C
import threading
from pathlib import Path

import numpy as np

PKG = Path(__file__).resolve().parent
LIB_PATH = PKG / "lib" / "libqpe_gb300.so"

QPE_OK = 0
QPE_ERR_INVALID, QPE_ERR_UNSUPPORTED, QPE_ERR_NOMEM, QPE_ERR_CUDA, QPE_ERR_TIMEOUT, QPE_ERR_NO_DEVICE = 1, 2, 3, 4, 5, 6
ERRORS = {1: "invalid argument", 2: "unsupported", 3: "out of memory", 4: "CUDA error", 5: "timeout",
          6: "no CUDA device"}
QPE_C128, QPE_C64 = 0, 1
TERM_KINDS = ("pp", "pq", "pqqp", "pqqr", "pqrs")


class QpeError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"[{ERRORS.get(code, code)}] {msg}")
        self.code = code


class QpeTerm(C.Structure):
    _fields_ = [("p", C.c_uint32), ("q", C.c_uint32), ("r", C.c_uint32), ("s", C.c_uint32),
                ("even", C.c_double * 4), ("odd", C.c_double * 4)]


class ProgramInfo(C.Structure):
    _fields_ = [("num_orbitals", C.c_uint32), ("n_alpha", C.c_uint32), ("n_beta", C.c_uint32),
                ("c_alpha", C.c_uint32), ("c_beta", C.c_uint32), ("num_ops", C.c_uint32),
                ("num_ops_per_power", C.c_uint32), ("touches_per_sweep", C.c_uint64),
                ("touches_per_power", C.c_uint64), ("table_entries", C.c_uint64),
                ("num_passes_per_power", C.c_uint32), ("reserved", C.c_uint32)]


class EvolveOpts(C.Structure):
    _fields_ = [("strategy", C.c_uint32), ("first_power", C.c_uint32), ("last_power", C.c_uint32),
                ("cluster_size", C.c_uint32), ("flags", C.c_uint32), ("repeats", C.c_uint32),
                ("replicas", C.c_uint32)]


QPE_EVOLVE_FP64_CONTRACT, QPE_EVOLVE_IN_PLACE = 1, 2
QPE_PROGRAM_APPLY_UNITARY_ORDER = 0x100


TERM_DTYPE = np.dtype([("p", "<u4"), ("q", "<u4"), ("r", "<u4"), ("s", "<u4"),
                       ("even", "<f8", (4,)), ("odd", "<f8", (4,))])
assert TERM_DTYPE.itemsize == C.sizeof(QpeTerm)

_vp = C.c_void_p
_P_TERM = C.POINTER(QpeTerm)
_PD = C.POINTER(C.c_double)

# name: (restype, argtypes)
PROTOTYPES = {
    "qpe_version": (C.c_int, []),
    "qpe_last_error": (C.c_char_p, []),
    "qpe_device_count": (C.c_int, [C.POINTER(C.c_int)]),
    "qpe_context_create": (C.c_int, [C.c_int, C.POINTER(_vp)]),
    "qpe_context_destroy": (C.c_int, [_vp]),
    "qpe_synchronize": (C.c_int, [_vp]),
    "qpe_timer_record": (C.c_int, [_vp, C.c_uint32]),
    "qpe_timer_elapsed_ms": (C.c_int, [_vp, C.c_uint32, C.c_uint32, C.POINTER(C.c_float)]),
    "qpe_host_alloc": (C.c_int, [C.c_size_t, C.POINTER(_vp)]),
    "qpe_host_free": (C.c_int, [_vp]),
    "qpe_flush_l2": (C.c_int, [_vp]),
    "qpe_measure_fp64_peak": (C.c_int, [_vp, C.POINTER(C.c_double)]),
    "qpe_selftest_bounded_wait": (C.c_int, [_vp, C.c_uint32, C.c_int]),
    "qpe_rank": (C.c_int, [_vp, C.POINTER(C.c_uint64), C.POINTER(C.c_int64), C.c_size_t]),
    "qpe_unrank": (C.c_int, [_vp, C.c_uint32, C.c_uint32, C.POINTER(C.c_int64), C.POINTER(C.c_uint64), C.c_size_t]),
    "qpe_rank_with_swaps": (C.c_int, [_vp, C.c_uint32, C.c_uint64, C.POINTER(C.c_uint32), C.POINTER(C.c_int64),
                                      C.c_size_t]),
    "qpe_axis_table": (C.c_int, [_vp, C.c_int, C.c_uint32, C.c_uint32, C.POINTER(C.c_uint32), C.POINTER(C.c_uint32),
                                 C.POINTER(C.c_uint32), C.POINTER(C.c_uint8), C.c_size_t, C.POINTER(C.c_size_t)]),
    "qpe_time_evolve_over_terms": (C.c_int, [_vp, C.c_uint32, C.c_uint32, C.c_uint32] + [_P_TERM, C.c_size_t] * 5
                                   + [_PD]),
    "qpe_time_evolve_iqpe": (C.c_int, [_vp, C.c_uint32, C.c_uint32, C.c_uint32] + [_P_TERM, C.c_size_t] * 5
                             + [C.c_uint32, _PD]),
    "qpe_qift": (C.c_int, [_vp, C.c_uint32, C.c_uint64, _PD]),
    "qpe_identify_phase_amplitudes": (C.c_int, [_vp, C.c_uint32, C.c_uint64, _PD, _PD]),
    "qpe_program_create": (C.c_int, [_vp, C.c_uint32, C.c_uint32, C.c_uint32] + [_P_TERM, C.c_size_t] * 5
                           + [C.c_uint32, C.c_uint32, C.POINTER(_vp)]),
    "qpe_program_destroy": (C.c_int, [_vp]),
    "qpe_program_plan": (C.c_int, [C.c_uint32, C.c_uint32, C.c_uint32] + [_P_TERM, C.c_size_t] * 5
                         + [C.c_uint32, C.c_uint32, C.POINTER(ProgramInfo)]),
    "qpe_program_get_info": (C.c_int, [_vp, C.POINTER(ProgramInfo)]),
    "qpe_program_unit_schedule": (C.c_int, [_vp, C.POINTER(C.c_uint32), C.POINTER(C.c_uint32)]),
    "qpe_state_create": (C.c_int, [_vp, C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint32, C.c_int, C.POINTER(_vp)]),
    "qpe_state_destroy": (C.c_int, [_vp]),
    "qpe_state_upload": (C.c_int, [_vp, _vp, C.c_uint64, C.c_uint64]),
    "qpe_state_download": (C.c_int, [_vp, _vp, C.c_uint64, C.c_uint64]),
    "qpe_state_zero": (C.c_int, [_vp]),
    "qpe_evolve": (C.c_int, [_vp, _vp, C.POINTER(EvolveOpts)]),
    "qpe_state_qift": (C.c_int, [_vp]),
    "qpe_state_phase_probs": (C.c_int, [_vp, _PD]),
    "qpe_state_block_norms": (C.c_int, [_vp, _PD]),
    "qpe_state_last_strategy": (C.c_int, [_vp, C.POINTER(C.c_uint32), C.POINTER(C.c_uint32)]),
    "qpe_state_last_replicas": (C.c_int, [_vp, C.POINTER(C.c_uint32)]),
    # host-side term compiler
    # learned initial-state model
    "qpe_mlp_create": (C.c_int, [_vp, C.c_uint32, C.c_uint32, C.c_uint64, C.POINTER(_vp)]),
    "qpe_mlp_destroy": (C.c_int, [_vp]),
    "qpe_mlp_num_params": (C.c_int, [_vp, C.POINTER(C.c_uint64)]),
    "qpe_mlp_get_params": (C.c_int, [_vp, C.POINTER(C.c_float)]),
    "qpe_mlp_set_params": (C.c_int, [_vp, C.POINTER(C.c_float)]),
    "qpe_mlp_set_data": (C.c_int, [_vp, C.POINTER(C.c_uint64), C.POINTER(C.c_float), C.POINTER(C.c_float),
                                   C.POINTER(C.c_float), C.c_uint64]),
    "qpe_mlp_train": (C.c_int, [_vp, C.c_uint32, C.c_float, C.c_uint64, C.POINTER(C.c_float)]),
    "qpe_mlp_forward": (C.c_int, [_vp, C.POINTER(C.c_uint64), C.c_uint64, C.POINTER(C.c_float)]),
    "qpe_mlp_gradients": (C.c_int, [_vp, C.POINTER(C.c_uint64), C.POINTER(C.c_float), C.POINTER(C.c_float),
                                    C.POINTER(C.c_float), C.c_uint32, C.POINTER(C.c_float), C.POINTER(C.c_float)]),
    "qpe_mlp_tensor_flops_per_step": (C.c_int, [_vp, C.POINTER(C.c_double)]),
    "qpe_mlp_create2": (C.c_int, [_vp, C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint64, C.POINTER(_vp)]),
    "qpe_mlp_set_data2": (C.c_int, [_vp, C.POINTER(C.c_uint64), C.POINTER(C.c_float), C.POINTER(C.c_float),
                                    C.POINTER(C.c_float), C.POINTER(C.c_float), C.c_uint64]),
    "qpe_mlp_forward2": (C.c_int, [_vp, C.POINTER(C.c_uint64), C.POINTER(C.c_float), C.c_uint64,
                                   C.POINTER(C.c_float)]),
    "qpe_mlp_gradients2": (C.c_int, [_vp, C.POINTER(C.c_uint64), C.POINTER(C.c_float), C.POINTER(C.c_float),
                                     C.POINTER(C.c_float), C.POINTER(C.c_float), C.c_uint32, C.POINTER(C.c_float),
                                     C.POINTER(C.c_float)]),
    "qpe_gemm_bf16": (C.c_int, [_vp, C.c_uint32, C.c_uint32, C.c_uint32, C.POINTER(C.c_uint16),
                                C.POINTER(C.c_uint16), C.POINTER(C.c_float), C.c_uint32]),
    "qpe_ham_create": (C.c_int, [C.POINTER(_vp)]),
    "qpe_ham_destroy": (C.c_int, [_vp]),
    "qpe_ham_add_one_body": (C.c_int, [_vp, C.c_int, C.c_int, C.c_double]),
    "qpe_ham_add_two_body": (C.c_int, [_vp, C.c_int, C.c_int, C.c_int, C.c_int, C.c_double]),
    "qpe_ham_ingest_broombridge": (C.c_int, [_vp, C.c_char_p, C.POINTER(C.c_uint32), C.POINTER(C.c_uint32), _PD,
                                             C.c_size_t]),
    "qpe_ham_set_num_orbitals": (C.c_int, [_vp, C.c_uint32]),
    "qpe_ham_set_num_occupied": (C.c_int, [_vp, C.c_uint32]),
    "qpe_ham_set_identity": (C.c_int, [_vp, C.c_double]),
    "qpe_ham_set_timestep": (C.c_int, [_vp, C.c_double]),
    "qpe_ham_get_num_orbitals": (C.c_int, [_vp, C.POINTER(C.c_uint32)]),
    "qpe_ham_get_num_occupied": (C.c_int, [_vp, C.POINTER(C.c_uint32)]),
    "qpe_ham_get_identity": (C.c_int, [_vp, _PD]),
    "qpe_ham_index_terms": (C.c_int, [_vp]),
    "qpe_ham_segment_counts": (C.c_int, [_vp, C.POINTER(C.c_size_t)]),
    "qpe_ham_segment_terms": (C.c_int, [_vp, C.c_int, _P_TERM, _PD, C.c_size_t]),
    "qpe_ham_pp_term": (C.c_int, [_vp, C.c_uint32, _PD]),
    "qpe_ham_pq_term": (C.c_int, [_vp, C.c_uint32, C.c_uint32, C.c_uint32, _PD]),
    "qpe_ham_pqqp_term": (C.c_int, [_vp, C.c_uint32, C.c_uint32, _PD]),
    "qpe_ham_pqqr_term": (C.c_int, [_vp, C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint32, _PD]),
    "qpe_ham_pqrs_term": (C.c_int, [_vp, C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint32, _PD]),
}

_lib = None
_lock = threading.Lock()


def lib() -> C.CDLL:
    """The loaded native library (loads it on first use; raises if absent)."""
    global _lib
    if _lib is not None:
        return _lib
    with _lock:
        if _lib is None:
            if not LIB_PATH.exists():
                raise QpeError(6, f"native library {LIB_PATH} is missing: run __graft_entry__.build() "
                                  "(the CUDA path is the only implementation)")
            L = C.CDLL(str(LIB_PATH))
            for name, (res, args) in PROTOTYPES.items():
                fn = getattr(L, name)
                fn.restype = res
                fn.argtypes = args
            _lib = L
    return _lib


def check(rc: int) -> None:
    if rc != QPE_OK:
        msg = lib().qpe_last_error()
        raise QpeError(rc, msg.decode() if msg else "")


def terms_arg(arr):
    """(pointer, count) for a TERM_DTYPE array (or None)."""
    if arr is None or len(arr) == 0:
        return None, 0
    if arr.dtype != TERM_DTYPE or not arr.flags.c_contiguous:
        arr = np.ascontiguousarray(arr, dtype=TERM_DTYPE)
    return arr.ctypes.data_as(_P_TERM), len(arr)


def seg_args(seg: dict) -> list:
    out, keep = [], []
    for k in TERM_KINDS:
        a = seg.get(k)
        if a is not None and len(a):
            a = np.ascontiguousarray(a, dtype=TERM_DTYPE)
            keep.append(a)
        out += list(terms_arg(a))
    return out, keep


_contexts: dict = {}


def context(device: int = 0):
    """Per-process default context on `device` (created on first use)."""
    with _lock:
        ctx = _contexts.get(device)
    if ctx is None:
        h = C.c_void_p()
        check(lib().qpe_context_create(device, C.byref(h)))
        with _lock:
            ctx = _contexts.setdefault(device, h)
    return ctx


def device_count() -> int:
    n = C.c_int(0)
    check(lib().qpe_device_count(C.byref(n)))
    return n.value


class Timer:
    """CUDA events on the library's stream: record(slot), elapsed_ms(a, b)."""

    def __init__(self, device: int = 0):
        self.ctx = context(device)

    def record(self, slot: int) -> None:
        check(lib().qpe_timer_record(self.ctx, slot))

    def elapsed_ms(self, a: int, b: int) -> float:
        v = C.c_float()
        check(lib().qpe_timer_elapsed_ms(self.ctx, a, b, C.byref(v)))
        return float(v.value)


class PinnedBuffer:
    """Page-locked host array (cudaMallocHost) viewed as numpy."""

    def __init__(self, count: int, dtype):
        self.dtype = np.dtype(dtype)
        p = C.c_void_p()
        check(lib().qpe_host_alloc(count * self.dtype.itemsize, C.byref(p)))
        self._p = p
        buf = (C.c_char * (count * self.dtype.itemsize)).from_address(p.value)
        self.array = np.frombuffer(buf, self.dtype, count)

    def __del__(self):
        p = getattr(self, "_p", None)
        if p:
            self.array = None
            lib().qpe_host_free(p)
            self._p = None
