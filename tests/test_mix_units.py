"""The column-pair update-unit scheduler and the row and column passes' per-line
programs (csrc/mix_units.cpp, strategy 7), on the CPU: tests/units/mix_units_check.cc runs every scheduled window of a program both
the tile runner's way and the warp programs' way on a random complex128 block and
counts differences (bit for bit) and broken kernel invariants (team layout,
bounds, one owner per stage index and per amplitude). The GPU parity tests run
the same schedules in k_resident_lean against the oracle."""
import ctypes as C
import math
import subprocess

import numpy as np
import pytest

from conftest import ROOT

CSRC = ROOT / "2022-qpesim_gb300" / "csrc"
KINDS = ("pp", "pq", "pqqp", "pqqr", "pqrs")


@pytest.fixture(scope="module")
def checker(tmp_path_factory):
    out = tmp_path_factory.mktemp("units") / "libmix_units_check.so"
    cmd = ["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-shared", "-fPIC", f"-I{CSRC}", f"-I{ROOT / 'include'}",
           str(ROOT / "tests" / "units" / "mix_units_check.cc"), str(CSRC / "mix_units.cpp"),
           str(CSRC / "program_build.cpp"), "-o", str(out)]
    subprocess.run(cmd, check=True, capture_output=True, text=True)
    lib = C.CDLL(str(out))
    lib.mix_units_check.restype = C.c_int
    lib.mix_units_check.argtypes = [C.c_uint, C.c_uint, C.c_uint, C.c_void_p, C.c_void_p, C.c_uint, C.c_uint,
                                    C.c_uint, C.c_uint, C.c_uint, C.POINTER(C.c_uint)]
    lib.line_units_check.restype = C.c_int
    lib.line_units_check.argtypes = lib.mix_units_check.argtypes
    return lib


def _run(q, lib, n, K, order, wpc, max_window, seed=0):
    M, e = n // 2, n // 4
    h = q.Hamiltonian.from_integrals(q.synthetic_integrals(n, seed), e, 0.05)
    seg = h.segmented_terms()
    arrs = [np.ascontiguousarray(seg[k], dtype=q._native.TERM_DTYPE) for k in KINDS]
    ptrs = (C.c_void_p * 5)(*[a.ctypes.data for a in arrs])
    ns = (C.c_size_t * 5)(*[len(a) for a in arrs])
    stats = (C.c_uint * 4)()
    stage = max(2 * math.comb(M, e), 3 * 64)  # the lean kernel's group stage with units
    bad = lib.mix_units_check(M, e, e, ptrs, ns, order, K, wpc, stage, max_window, stats)
    return bad, dict(scheduled=stats[0], windows=stats[1], wp_words=stats[2], max_quads=stats[3])


def test_headline_schedule(q, checker):
    """n = 16, N = 8, cluster of 16, 15 warps per CTA, windows of up to 8 passes
    (the headline configuration): every one of the 392 column-pair passes is
    scheduled, in fewer windows, and the unit runs equal the tile runs bit for bit."""
    bad, st = _run(q, checker, 16, 16, 2, 15, 8)
    assert bad == 0
    assert st["scheduled"] == 392
    assert st["windows"] < 392 // 2
    assert st["max_quads"] <= 40  # the most update slots one CTA runs at one level


@pytest.mark.parametrize("n,K,order,wpc,max_window", [(16, 16, 1, 15, 1), (16, 8, 1, 15, 4), (16, 8, 2, 9, 2),
                                                      (12, 16, 1, 15, 4), (12, 4, 2, 15, 2), (14, 16, 1, 9, 4),
                                                      (10, 4, 1, 6, 3), (8, 2, 1, 15, 4), (16, 2, 2, 15, 4)])
def test_schedules_equal_tile_runs(q, checker, n, K, order, wpc, max_window):
    bad, st = _run(q, checker, n, K, order, wpc, max_window, seed=n)
    assert bad == 0, st


def test_units_too_large_fall_back(q, checker):
    """n = 20 (70 row pairs per term and column pair): no unit fits a three-warp
    group, so no pass is scheduled and every column-pair pass keeps the tiles."""
    bad, st = _run(q, checker, 20, 16, 1, 15, 4)
    assert bad == 0 and st["scheduled"] == 0 and st["windows"] == 0


@pytest.mark.parametrize("n,K,order,wpc,replicas", [(16, 16, 2, 15, 1), (16, 16, 2, 15, 5), (16, 16, 1, 15, 3),
                                                    (12, 4, 2, 15, 2), (12, 16, 1, 9, 1), (14, 8, 1, 15, 2),
                                                    (8, 2, 1, 15, 2)])
def test_line_programs_equal_line_runs(q, checker, n, K, order, wpc, replicas):
    """The row and column passes' per-line programs (conditions evaluated on the
    host, terms split into levels of at most 24 pair or 48 diagonal updates)
    give the line runner's results bit for bit, each line on the replica that
    exchanges it and rows on the CTA that owns them."""
    M, e = n // 2, n // 4
    h = q.Hamiltonian.from_integrals(q.synthetic_integrals(n, n), e, 0.05)
    seg = h.segmented_terms()
    arrs = [np.ascontiguousarray(seg[k], dtype=q._native.TERM_DTYPE) for k in KINDS]
    ptrs = (C.c_void_p * 5)(*[a.ctypes.data for a in arrs])
    ns = (C.c_size_t * 5)(*[len(a) for a in arrs])
    stats = (C.c_uint * 4)()
    stage = max(2 * math.comb(M, e), 3 * 64)
    bad = checker.line_units_check(M, e, e, ptrs, ns, order, K, wpc, stage, replicas, stats)
    assert bad == 0
    assert stats[0] > 0  # passes with programs


def test_general_matrices_keep_the_runners(q, checker):
    """A pair term whose matrix is not of the inline form (m00 real, m01
    imaginary) keeps its pass on the tile or line runner: the schedules leave
    that pass out and stay exact for the rest."""
    n, K = 12, 4
    M, e = n // 2, n // 4
    seg = {k: np.array(v, copy=True) for k, v in
           q.Hamiltonian.from_integrals(q.synthetic_integrals(n, 3), e, 0.05).segmented_terms().items()}
    pqrs, pq = seg["pqrs"], seg["pq"]
    mixed = np.flatnonzero((pqrs["p"] < M) & (pqrs["s"] < M) & (pqrs["q"] >= M) & (pqrs["r"] >= M))
    pqrs["even"][mixed[0], 1] = 1e-3  # m00 of one column-pair term gets an imaginary part
    pq["odd"][0, 1] = 1e-3            # and m00 of one pq term
    arrs = [np.ascontiguousarray(seg[k], dtype=q._native.TERM_DTYPE) for k in KINDS]
    ptrs = (C.c_void_p * 5)(*[a.ctypes.data for a in arrs])
    ns = (C.c_size_t * 5)(*[len(a) for a in arrs])
    stage = max(2 * math.comb(M, e), 3 * 64)
    s1, s2 = (C.c_uint * 4)(), (C.c_uint * 4)()
    assert checker.mix_units_check(M, e, e, ptrs, ns, 1, K, 15, stage, 8, s1) == 0
    assert checker.line_units_check(M, e, e, ptrs, ns, 1, K, 15, stage, 1, s2) == 0
    clean = [np.ascontiguousarray(v, dtype=q._native.TERM_DTYPE) for v in
             (q.Hamiltonian.from_integrals(q.synthetic_integrals(n, 3), e, 0.05).segmented_terms()[k] for k in KINDS)]
    cp = (C.c_void_p * 5)(*[a.ctypes.data for a in clean])
    c1, c2 = (C.c_uint * 4)(), (C.c_uint * 4)()
    assert checker.mix_units_check(M, e, e, cp, ns, 1, K, 15, stage, 8, c1) == 0
    assert checker.line_units_check(M, e, e, cp, ns, 1, K, 15, stage, 1, c2) == 0
    assert s1[0] < c1[0]  # fewer column-pair passes scheduled
    assert s2[0] < c2[0]  # fewer row / column passes with programs


@pytest.mark.parametrize("n,na,nb,K,replicas", [(14, 4, 3, 8, 2), (12, 2, 4, 4, 1), (16, 3, 4, 16, 3)])
def test_schedules_with_unequal_spins(q, checker, n, na, nb, K, replicas):
    """Both schedules with different alpha and beta electron counts (rows and
    columns of different lengths)."""
    M = n // 2
    seg = q.Hamiltonian.from_integrals(q.synthetic_integrals(n, 40 + n), max(na, nb), 0.05).segmented_terms()
    arrs = [np.ascontiguousarray(seg[k], dtype=q._native.TERM_DTYPE) for k in KINDS]
    ptrs = (C.c_void_p * 5)(*[a.ctypes.data for a in arrs])
    ns = (C.c_size_t * 5)(*[len(a) for a in arrs])
    stage = max(2 * math.comb(M, na), 3 * 64)
    s1, s2 = (C.c_uint * 4)(), (C.c_uint * 4)()
    assert checker.mix_units_check(M, na, nb, ptrs, ns, 2, K, 15, stage, 8, s1) == 0
    assert checker.line_units_check(M, na, nb, ptrs, ns, 2, K, 15, stage, replicas, s2) == 0
