"""ctypes bindings of the oracle (TEST INFRASTRUCTURE ONLY).

`Oracle` wraps build/liborc.so, the CPU restatement of the reference's hot path
(oracle/qpe_oracle.cc). `Reference` wraps _ref/libref.so, the reference itself
compiled from its own sources with the shims in ref_shims/ (only present where
the reference sources were available at build time). Only tests/, the smoke test
of __graft_entry__ and bench.py's CPU-baseline leg use this module, as the checker.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ORC_LIB = HERE / "build" / "liborc.so"
ORC_FAST_LIB = HERE / "build" / "liborc_fast.so"
REF_LIB = HERE / "_ref" / "libref.so"
REF_FAST_LIB = HERE / "_ref" / "libref_fast.so"


def reference_cpp() -> Path | None:
    """The reference's cpp/ directory where its sources are present: the
    QPE_REFERENCE_CPP environment variable, else the default of the oracle's
    build recipe (Makefile); None where neither exists (as on a GPU host)."""
    env = os.environ.get("QPE_REFERENCE_CPP")
    if env:
        return Path(env) if Path(env).is_dir() else None
    try:
        out = subprocess.run(["make", "-s", "-C", str(HERE), "print-ref"], capture_output=True, text=True,
                             check=True).stdout.strip()
    except (OSError, subprocess.CalledProcessError):
        return None
    return Path(out) if out and Path(out).is_dir() else None


class QpeTerm(C.Structure):
    """Mirror of `qpe_term` (include/qpe_gb300.h)."""

    _fields_ = [("p", C.c_uint32), ("q", C.c_uint32), ("r", C.c_uint32), ("s", C.c_uint32),
                ("even", C.c_double * 4), ("odd", C.c_double * 4)]


TERM_DTYPE = np.dtype([("p", "<u4"), ("q", "<u4"), ("r", "<u4"), ("s", "<u4"),
                       ("even", "<f8", (4,)), ("odd", "<f8", (4,))])
assert TERM_DTYPE.itemsize == C.sizeof(QpeTerm)


def _elf_matches(path: Path) -> bool:
    import platform
    try:
        head = path.read_bytes()[:20]
    except OSError:
        return False
    want = {"x86_64": 62, "aarch64": 183, "arm64": 183}.get(platform.machine())
    return want is None or int.from_bytes(head[18:20], "little") == want


def build(ref: bool | None = None) -> None:
    """Builds the oracle (and, when the reference sources exist, oracle/_ref)."""
    src = reference_cpp()
    targets = ["all"]
    if ref or (ref is None and src is not None):
        targets.append("ref")
    for t in (ORC_LIB, ORC_FAST_LIB, REF_LIB, REF_FAST_LIB):
        if t.exists() and not _elf_matches(t):
            t.unlink()
    extra = [f"REF={src}"] if src is not None else []
    subprocess.run(["make", "-s", "-C", str(HERE), *extra, *targets], check=True)


def _ptr(a: np.ndarray, ct=C.c_double):
    return a.ctypes.data_as(C.POINTER(ct))


def terms_ptr(t: np.ndarray):
    if t is None or len(t) == 0:
        return None, 0
    assert t.dtype == TERM_DTYPE and t.flags.c_contiguous
    return t.ctypes.data_as(C.POINTER(QpeTerm)), len(t)


class Oracle:
    def __init__(self, fast: bool = False):
        path = ORC_FAST_LIB if fast else ORC_LIB
        if not path.exists():
            build(ref=False)
        self.lib = C.CDLL(str(path))
        L = self.lib
        L.orc_nchoosek.restype = C.c_uint64
        L.orc_nchoosek.argtypes = [C.c_int, C.c_int]
        L.orc_rank.restype = C.c_int64
        L.orc_rank.argtypes = [C.c_uint64]
        L.orc_next_comb.restype = C.c_uint64
        L.orc_next_comb.argtypes = [C.c_uint64]
        L.orc_parity.restype = C.c_uint
        L.orc_parity.argtypes = [C.c_uint64]
        L.orc_discover.restype = C.c_int64
        L.orc_discover.argtypes = [C.c_int, C.c_uint, C.c_uint, C.c_uint, C.c_uint, C.c_uint, C.c_uint,
                                   C.POINTER(C.c_uint64), C.POINTER(C.c_uint64), C.POINTER(C.c_uint64),
                                   C.POINTER(C.c_uint), C.c_size_t]
        P = C.POINTER(QpeTerm)
        L.orc_time_evolve.restype = C.c_int
        L.orc_time_evolve.argtypes = [C.c_uint, C.c_uint, C.c_uint, C.c_uint, P, C.c_size_t, P, C.c_size_t, P,
                                      C.c_size_t, P, C.c_size_t, P, C.c_size_t, C.c_uint, C.c_uint, C.c_uint,
                                      C.c_uint, C.POINTER(C.c_double)]
        L.orc_time_evolve_iqpe.restype = C.c_int
        L.orc_time_evolve_iqpe.argtypes = [C.c_uint, C.c_uint, C.c_uint, C.c_uint, P, C.c_size_t, P, C.c_size_t, P,
                                           C.c_size_t, P, C.c_size_t, P, C.c_size_t, C.c_uint,
                                           C.POINTER(C.c_double)]
        L.orc_qift.restype = C.c_int
        L.orc_qift.argtypes = [C.c_uint, C.c_uint64, C.POINTER(C.c_double)]
        L.orc_identify_phase_amplitudes.restype = C.c_int
        L.orc_identify_phase_amplitudes.argtypes = [C.c_uint, C.c_uint64, C.POINTER(C.c_double),
                                                    C.POINTER(C.c_double)]
        L.orc_rank_with_swaps.restype = C.c_int
        L.orc_rank_with_swaps.argtypes = [C.c_uint, C.c_uint64, C.POINTER(C.c_uint32), C.POINTER(C.c_int64),
                                          C.c_size_t]
        L.orc_num_threads.restype = C.c_int
        L.orc_set_threads.argtypes = [C.c_int]
        L.orc_touches_per_power.restype = C.c_uint64
        L.orc_touches_per_power.argtypes = [C.c_uint, C.c_uint, C.c_uint, P, C.c_size_t, P, C.c_size_t, P,
                                            C.c_size_t, P, C.c_size_t, P, C.c_size_t, C.c_uint, C.c_uint]
        L.orc_terms_create.restype = C.c_void_p
        L.orc_terms_destroy.argtypes = [C.c_void_p]
        L.orc_terms_set.argtypes = [C.c_void_p, C.c_uint, C.c_uint, C.c_double]
        L.orc_terms_add_one_body.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_double]
        L.orc_terms_add_two_body.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_int, C.c_double]
        L.orc_terms_segments.restype = C.c_int
        L.orc_terms_segments.argtypes = [C.c_void_p, C.POINTER(C.c_size_t), C.POINTER(P),
                                         C.POINTER(C.POINTER(C.c_double)), C.POINTER(C.c_size_t)]

    def nchoosek(self, n, k):
        return int(self.lib.orc_nchoosek(n, k))

    def rank(self, bv):
        return int(self.lib.orc_rank(bv))

    def next_comb(self, x):
        return int(self.lib.orc_next_comb(x))

    def parity(self, x):
        return int(self.lib.orc_parity(x))

    def discover(self, kind, M, e, p=0, q=0, r=0, s=0, cap=1 << 20):
        ni = np.zeros(cap, np.uint64)
        o1 = np.zeros(cap, np.uint64)
        o2 = np.zeros(cap, np.uint64)
        pa = np.zeros(cap, np.uint32)
        n = self.lib.orc_discover(kind, M, e, p, q, r, s, _ptr(ni, C.c_uint64), _ptr(o1, C.c_uint64),
                                  _ptr(o2, C.c_uint64), _ptr(pa, C.c_uint), cap)
        assert n >= 0
        return ni[:n].copy(), o1[:n].copy(), o2[:n].copy(), pa[:n].copy()

    def time_evolve(self, M, na, nb, P, seg, state, order=1, steps=1, first=0, last=0):
        """seg: dict kind-name -> TERM_DTYPE array; state: complex128 array (modified)."""
        assert state.dtype == np.complex128 and state.flags.c_contiguous
        args = []
        for k in ("pp", "pq", "pqqp", "pqqr", "pqrs"):
            args += list(terms_ptr(seg.get(k)))
        rc = self.lib.orc_time_evolve(M, na, nb, P, *args, order, steps, first, last,
                                      state.view(np.float64).ctypes.data_as(C.POINTER(C.c_double)))
        if rc:
            raise RuntimeError(f"orc_time_evolve failed: {rc}")
        return state

    def time_evolve_iqpe(self, M, na, nb, P, seg, state, applications):
        """time_evolve_iqpe: block 1 of `state` evolved in place (applyUnitary order)."""
        assert state.dtype == np.complex128 and state.flags.c_contiguous
        args = []
        for k in ("pp", "pq", "pqqp", "pqqr", "pqrs"):
            args += list(terms_ptr(seg.get(k)))
        rc = self.lib.orc_time_evolve_iqpe(M, na, nb, P, *args, applications,
                                           state.view(np.float64).ctypes.data_as(C.POINTER(C.c_double)))
        if rc:
            raise RuntimeError(f"orc_time_evolve_iqpe failed: {rc}")
        return state

    def qift(self, P, ld, state):
        rc = self.lib.orc_qift(P, ld, state.view(np.float64).ctypes.data_as(C.POINTER(C.c_double)))
        if rc:
            raise RuntimeError(f"orc_qift failed: {rc}")
        return state

    def identify_phase_amplitudes(self, P, ld, state):
        probs = np.zeros(1 << P)
        rc = self.lib.orc_identify_phase_amplitudes(P, ld, state.view(np.float64).ctypes.data_as(C.POINTER(C.c_double)),
                                                    _ptr(probs))
        if rc:
            raise RuntimeError(f"orc_identify_phase_amplitudes failed: {rc}")
        return probs

    def rank_with_swaps(self, n, bv, swaps):
        swaps = np.ascontiguousarray(swaps, np.uint32).reshape(-1, 4)
        out = np.zeros(len(swaps), np.int64)
        rc = self.lib.orc_rank_with_swaps(n, bv, _ptr(swaps, C.c_uint32), _ptr(out, C.c_int64), len(swaps))
        if rc:
            raise RuntimeError("orc_rank_with_swaps failed")
        return out

    def segmented_terms(self, num_orbitals, num_occupied, t, one_body, two_body, with_raw=False):
        """The oracle's term compiler (terms_oracle.cc): AddOneBodyTerm(p, q, v) for
        each (p, q, v) of one_body, AddTwoBodyTerm(p, q, r, s, v) for each
        (p, q, r, s, v) of two_body, IndexTerms, then the five segments with the
        getters' coefficients at timestep t. Returns kind -> TERM_DTYPE array (and
        kind -> indexed values with with_raw)."""
        L = self.lib
        h = L.orc_terms_create()
        try:
            L.orc_terms_set(h, num_orbitals, num_occupied, t)
            for p, q, v in one_body:
                L.orc_terms_add_one_body(h, int(p), int(q), float(v))
            for p, q, r, s_, v in two_body:
                L.orc_terms_add_two_body(h, int(p), int(q), int(r), int(s_), float(v))
            counts = (C.c_size_t * 5)()
            if L.orc_terms_segments(h, counts, None, None, None):
                raise RuntimeError("orc_terms_segments: unknown term shape")
            arrs = [np.zeros(int(counts[k]), TERM_DTYPE) for k in range(5)]
            raws = [np.zeros(int(counts[k])) for k in range(5)]
            P = C.POINTER(QpeTerm)
            outs = (P * 5)(*[a.ctypes.data_as(P) for a in arrs])
            rptr = (C.POINTER(C.c_double) * 5)(*[_ptr(r) for r in raws])
            caps = (C.c_size_t * 5)(*[len(a) for a in arrs])
            if L.orc_terms_segments(h, counts, outs, rptr, caps):
                raise RuntimeError("orc_terms_segments failed")
        finally:
            L.orc_terms_destroy(h)
        kinds = ("pp", "pq", "pqqp", "pqqr", "pqrs")
        seg = dict(zip(kinds, arrs))
        return (seg, dict(zip(kinds, raws))) if with_raw else seg

    def touches_per_power(self, M, na, nb, seg, order=1, steps=1):
        """Amplitude updates of one controlled power, counted from the oracle's run
        tables (2 per pair update, 1 per diagonal phase)."""
        args = []
        for k in ("pp", "pq", "pqqp", "pqqr", "pqrs"):
            args += list(terms_ptr(seg.get(k)))
        return int(self.lib.orc_touches_per_power(M, na, nb, *args, order, steps))

    def set_threads(self, n):
        self.lib.orc_set_threads(int(n))

    def num_threads(self):
        return int(self.lib.orc_num_threads())


class Reference:
    """The reference's own code (oracle/_ref/libref.so)."""

    @staticmethod
    def available(fast: bool = False) -> bool:
        p = REF_FAST_LIB if fast else REF_LIB
        return p.exists() and _elf_matches(p)

    def __init__(self, fast: bool = False):
        path = REF_FAST_LIB if fast else REF_LIB
        self.lib = C.CDLL(str(path))
        L = self.lib
        L.ref_ham_create.restype = C.c_void_p
        L.ref_ham_create.argtypes = [C.c_uint, C.c_uint, C.c_double, C.c_size_t, C.POINTER(C.c_int),
                                     C.POINTER(C.c_double), C.c_size_t, C.POINTER(C.c_int), C.POINTER(C.c_double),
                                     C.c_double]
        L.ref_ham_from_broombridge.restype = C.c_void_p
        L.ref_ham_from_broombridge.argtypes = [C.c_char_p, C.c_uint, C.c_double, C.POINTER(C.c_uint),
                                               C.POINTER(C.c_uint), C.POINTER(C.c_double), C.POINTER(C.c_double),
                                               C.c_size_t]
        L.ref_ham_destroy.argtypes = [C.c_void_p]
        L.ref_ham_set_timestep.argtypes = [C.c_void_p, C.c_double]
        L.ref_segment_counts.argtypes = [C.c_void_p, C.POINTER(C.c_size_t)]
        L.ref_segment_terms.restype = C.c_size_t
        L.ref_segment_terms.argtypes = [C.c_void_p, C.c_int, C.POINTER(QpeTerm), C.POINTER(C.c_double), C.c_size_t]
        L.ref_time_evolve.argtypes = [C.c_void_p, C.c_uint, C.POINTER(C.c_double)]
        L.ref_time_evolve_iqpe.argtypes = [C.c_void_p, C.c_uint, C.POINTER(C.c_double), C.c_uint]
        L.ref_time_steps.restype = C.c_double
        L.ref_time_steps.argtypes = [C.c_void_p, C.c_uint, C.POINTER(C.c_double), C.c_uint]
        L.ref_qift.argtypes = [C.c_uint, C.c_uint, C.c_uint, C.POINTER(C.c_double)]
        L.ref_identify_phase_amplitudes.argtypes = [C.c_uint, C.c_uint, C.c_uint, C.POINTER(C.c_double),
                                                    C.POINTER(C.c_double)]
        L.ref_rank.restype = C.c_int64
        L.ref_rank.argtypes = [C.c_uint64]
        L.ref_nchoosek.restype = C.c_uint64
        L.ref_nchoosek.argtypes = [C.c_int, C.c_int]
        L.ref_rank_with_swaps.argtypes = [C.c_uint, C.c_uint64, C.POINTER(C.c_uint32), C.POINTER(C.c_int64),
                                          C.c_size_t]
        L.ref_discover.restype = C.c_int64
        L.ref_discover.argtypes = [C.c_int, C.c_uint, C.c_uint, C.c_uint, C.c_uint, C.c_uint, C.c_uint,
                                   C.POINTER(C.c_uint64), C.POINTER(C.c_uint64), C.POINTER(C.c_uint64),
                                   C.POINTER(C.c_uint), C.c_size_t]
        L.ref_run_doctests.restype = C.c_int
        L.ref_run_doctests.argtypes = [C.c_char_p, C.c_char_p, C.c_size_t, C.POINTER(C.c_long),
                                       C.POINTER(C.c_long), C.c_int]

    def hamiltonian(self, M, e, one_body, two_body, dt, identity=0.0):
        ob = np.asarray([(p, q) for p, q, _ in one_body], np.int32).reshape(-1, 2)
        obv = np.asarray([v for *_, v in one_body], np.float64)
        tb = np.asarray([t[:4] for t in two_body], np.int32).reshape(-1, 4)
        tbv = np.asarray([t[4] for t in two_body], np.float64)
        h = self.lib.ref_ham_create(M, e, identity, len(ob), _ptr(ob, C.c_int), _ptr(obv), len(tb), _ptr(tb, C.c_int),
                                    _ptr(tbv), dt)
        return h

    def broombridge(self, path, precision, dt):
        M, e, ident = C.c_uint(), C.c_uint(), C.c_double()
        h = self.lib.ref_ham_from_broombridge(str(path).encode(), precision, dt, C.byref(M), C.byref(e),
                                              C.byref(ident), None, 0)
        if not h:
            raise RuntimeError(f"reference could not ingest {path}")
        C_ = self.nchoosek(M.value, e.value)
        s0 = np.zeros((1 << precision) * C_ * C_, np.complex128)
        self.lib.ref_ham_destroy(h)
        h = self.lib.ref_ham_from_broombridge(str(path).encode(), precision, dt, C.byref(M), C.byref(e),
                                              C.byref(ident), s0.view(np.float64).ctypes.data_as(C.POINTER(C.c_double)),
                                              len(s0))
        return h, M.value, e.value, ident.value, s0

    def destroy(self, h):
        self.lib.ref_ham_destroy(h)

    def segments(self, h):
        counts = (C.c_size_t * 5)()
        self.lib.ref_segment_counts(h, counts)
        out, raws = {}, {}
        for kind, name in enumerate(("pp", "pq", "pqqp", "pqqr", "pqrs")):
            n = counts[kind]
            arr = np.zeros(n, TERM_DTYPE)
            raw = np.zeros(n)
            if n:
                self.lib.ref_segment_terms(h, kind, arr.ctypes.data_as(C.POINTER(QpeTerm)), _ptr(raw), n)
            out[name], raws[name] = arr, raw
        return out, raws

    def time_evolve(self, h, P, state):
        self.lib.ref_time_evolve(h, P, state.view(np.float64).ctypes.data_as(C.POINTER(C.c_double)))
        return state

    def time_evolve_iqpe(self, h, P, state, applications):
        self.lib.ref_time_evolve_iqpe(h, P, state.view(np.float64).ctypes.data_as(C.POINTER(C.c_double)),
                                      applications)
        return state

    def time_steps(self, h, P, state, nsteps):
        return float(self.lib.ref_time_steps(h, P, state.view(np.float64).ctypes.data_as(C.POINTER(C.c_double)),
                                             nsteps))

    def qift(self, P, M, e, state):
        self.lib.ref_qift(P, M, e, state.view(np.float64).ctypes.data_as(C.POINTER(C.c_double)))
        return state

    def identify_phase_amplitudes(self, P, M, e, state):
        probs = np.zeros(1 << P)
        self.lib.ref_identify_phase_amplitudes(P, M, e, state.view(np.float64).ctypes.data_as(C.POINTER(C.c_double)),
                                               _ptr(probs))
        return probs

    def rank(self, bv):
        return int(self.lib.ref_rank(bv))

    def nchoosek(self, n, k):
        return int(self.lib.ref_nchoosek(n, k))

    def rank_with_swaps(self, n, bv, swaps):
        swaps = np.ascontiguousarray(swaps, np.uint32).reshape(-1, 4)
        out = np.zeros(len(swaps), np.int64)
        self.lib.ref_rank_with_swaps(n, bv, _ptr(swaps, C.c_uint32), _ptr(out, C.c_int64), len(swaps))
        return out

    def discover(self, kind, M, e, p=0, q=0, r=0, s=0, cap=1 << 20):
        ni = np.zeros(cap, np.uint64)
        o1 = np.zeros(cap, np.uint64)
        o2 = np.zeros(cap, np.uint64)
        pa = np.zeros(cap, np.uint32)
        n = self.lib.ref_discover(kind, M, e, p, q, r, s, _ptr(ni, C.c_uint64), _ptr(o1, C.c_uint64),
                                  _ptr(o2, C.c_uint64), _ptr(pa, C.c_uint), cap)
        assert n >= 0
        return ni[:n].copy(), o1[:n].copy(), o2[:n].copy(), pa[:n].copy()

    def run_doctests(self, name_filter=""):
        names = C.create_string_buffer(1 << 16)
        checks = (C.c_long * 64)()
        failed = (C.c_long * 64)()
        n = self.lib.ref_run_doctests(name_filter.encode(), names, len(names), checks, failed, 64)
        labels = names.value.decode().split("\n")
        return {labels[i]: (checks[i], failed[i]) for i in range(max(n, 0))}
