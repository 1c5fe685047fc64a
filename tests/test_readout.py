"""The reference's readout formulas (cpp/main.cc:152-167) and the corrected
estimators, on hand-built histograms (CPU)."""
import math

import numpy as np


def _main_cc_readout(probs, identity, dt, P):
    """cpp/main.cc:152-167 step by step: the weighted mean index accumulated in
    order, divided by 2^P; E = -1 * 2 * 2 * acos(0) * phase + identity (no
    division by dt); margin of error 2 * 2 * acos(0) / (dt * 2^P)."""
    total = 0.0
    for idx, amp in enumerate(probs):
        total += idx * amp
    phase = total / (1 << P)
    energy = -1.0 * 2 * 2 * math.acos(0.0) * phase + identity
    moe = 2 * 2 * math.acos(0.0) / (dt * (1 << P))
    return phase, energy, moe


def test_reference_formulas_on_a_hand_built_histogram(q):
    P = 3
    probs = np.array([0.125, 0.25, 0.0, 0.5, 0.0, 0.0, 0.125, 0.0])
    assert q.reference_phase(probs) == 2.5 / 8
    phase, energy, moe = _main_cc_readout(probs, 0.75, 0.05, P)
    assert q.reference_phase(probs) == phase
    assert q.reference_energy(probs, 0.75) == energy == -2 * math.pi * 0.3125 + 0.75
    assert q.readout.margin_of_error(0.05, P) == moe


def test_reference_formulas_match_main_cc_on_random_histograms(q):
    rng = np.random.default_rng(5)
    for P in (1, 4, 7, 10):
        p = rng.random(1 << P)
        p /= p.sum()
        phase, energy, moe = _main_cc_readout(p, -1.25, 0.1, P)
        assert abs(q.reference_phase(p) - phase) <= 1e-15
        assert abs(q.reference_energy(p, -1.25) - energy) <= 1e-13
        assert q.readout.margin_of_error(0.1, P) == moe


def test_corrected_estimators_on_a_peak(q):
    """A single eigenphase: block k = exp(-i E k t) gives a Fejer peak at
    j / N = -E t / (2 pi) mod 1. The argmax bin, the sub-bin estimate and the
    dt-corrected energy recover E; the reference's weighted mean does not divide
    by t, so it is off unless t = 1."""
    N, t, E = 128, 0.05, -7.3
    k = np.arange(N)
    amps = np.exp(-1j * E * k * t) / math.sqrt(N)
    probs = np.abs(np.fft.fft(amps) / math.sqrt(N)) ** 2
    ph = q.subbin_phase(probs)
    assert abs(q.phase_to_energy(ph, t) - E) < 1e-4  # two-bin amplitude-ratio interpolation
    assert abs(q.phase_to_energy(q.readout.argmax_phase(probs), t) - E) <= q.readout.margin_of_error(t, 7)
    assert abs(q.reference_energy(probs) - E) > 1.0


def test_qpe_cost_model_and_shared_ground_bin(q):
    """The learned-state evaluation's yardsticks: the textbook QPE cost model and
    the ground bin shared by several starts' histograms."""
    L = q.learned_state
    t = 0.05
    # bins of at most 2e-3 Ha at t = 0.05 need 16 ancilla qubits
    secs, runs, bits = L.qpe_time_to_precision(0.5, 1e-6, t)
    assert bits == 16 and runs == 4 and abs(secs - 4 * 65535e-6) < 1e-12
    assert L.qpe_time_to_precision(0.0, 1e-6, t)[0] is None
    assert L.qpe_time_to_precision(0.01, 1e-6, t)[1] > L.qpe_time_to_precision(0.1, 1e-6, t)[1]
    # the ground peak (lowest energy) is strong in one histogram and a small local
    # maximum in the other; both give the same shared bin
    n = 64
    p1 = np.full(n, 1e-6)
    p2 = np.full(n, 1e-6)
    ground = 10
    p1[ground], p1[40] = 0.5, 0.3
    p2[ground], p2[40] = 0.01, 0.9
    assert q.phase_to_energy(ground / n, t) < q.phase_to_energy(40 / n, t)
    assert L.shared_ground_bin([p1, p2], t) == ground
    assert L.shared_ground_bin([p2], t) == ground


def test_learned_candidates_and_truncation(q):
    L = q.learned_state
    rng = np.random.default_rng(3)
    psi = rng.standard_normal(400) + 1j * rng.standard_normal(400)
    psi /= np.linalg.norm(psi)
    c = L.learned_candidates(psi)
    assert len(c) == 1 + len(L.CANDIDATE_TRUNCATIONS)
    assert np.array_equal(c[0], psi)
    for m, x in zip(L.CANDIDATE_TRUNCATIONS, c[1:]):
        assert np.count_nonzero(x) == m and abs(np.linalg.norm(x) - 1) < 1e-12
    top = int(np.argmax(np.abs(psi)))
    assert np.count_nonzero(c[1]) == 1 and abs(abs(c[1][top]) - 1.0) < 1e-15
