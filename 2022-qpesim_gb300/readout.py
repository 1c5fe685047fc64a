"""Phase and energy readout from the QIFT histogram (cpp/main.cc:152-167).

reference_energy() is the reference's formula, kept as it is: the histogram's
weighted mean index / 2^P is the phase and E = -2 pi phase + identity, with no
division by the time step (correct only for dt = 1). The corrected estimators
below divide by the evolution time per controlled power and also report the
argmax bin and a sub-bin estimate.
"""
from __future__ import annotations

import math

import numpy as np


def reference_phase(probs: np.ndarray) -> float:
    """main.cc:152-161: sum_j j * prob_j / 2^P."""
    n = len(probs)
    return float(np.dot(np.arange(n), probs) / n)


def reference_energy(probs: np.ndarray, identity: float = 0.0) -> float:
    """main.cc:165: E = -2 pi phase + identity."""
    return -2.0 * math.pi * reference_phase(probs) + identity


def margin_of_error(dt: float, precision: int) -> float:
    """main.cc:167: 2 pi / (dt * 2^P)."""
    return 2.0 * math.pi / (dt * (1 << precision))


def phase_to_energy(phase: float, t_power: float, identity: float = 0.0) -> float:
    """Block k holds exp(-i E k t) psi, whose forward DFT peaks at
    j / N = -E t / (2 pi) mod 1; this returns E in (-pi/t, pi/t] + identity."""
    e = -2.0 * math.pi * phase / t_power
    period = 2.0 * math.pi / t_power
    e = (e + period / 2.0) % period - period / 2.0
    return e + identity


def argmax_phase(probs: np.ndarray) -> float:
    return float(np.argmax(probs)) / len(probs)


def subbin_phase(probs: np.ndarray) -> float:
    """Peak bin refined by the ratio of its larger neighbour (for a Fejer-kernel
    peak |sin(pi N d)/ (N sin(pi d))|^2 the amplitude ratio a1 / (a0 + a1) gives the
    fractional offset d)."""
    n = len(probs)
    j = int(np.argmax(probs))
    a0 = math.sqrt(max(probs[j], 0.0))
    left, right = math.sqrt(max(probs[(j - 1) % n], 0.0)), math.sqrt(max(probs[(j + 1) % n], 0.0))
    if right >= left:
        d = right / (a0 + right) if a0 + right > 0 else 0.0
    else:
        d = -left / (a0 + left) if a0 + left > 0 else 0.0
    return ((j + d) / n) % 1.0


def success_probability(probs: np.ndarray, e_target: float, t_power: float, tol: float,
                        identity: float = 0.0) -> float:
    """Total probability of the bins whose energy lies within tol of e_target."""
    n = len(probs)
    es = np.array([phase_to_energy(j / n, t_power, identity) for j in range(n)])
    return float(probs[np.abs(es - e_target) <= tol].sum())
