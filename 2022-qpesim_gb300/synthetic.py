"""Seeded synthetic molecular integrals and the Hartree-Fock start.

The reference reads its Hamiltonians from Broombridge files; for benchmarking
this project draws them from a fixed distribution instead:

  h_pq = h_qp ~ N(0, 1) * exp(-|p - q| / 2)                        (p >= q)
  (pq|rs)     ~ N(0, 0.1^2) * exp(-(|p - q| + |r - s|) / 3)         one draw per
              8-fold orbit: p >= q, r >= s, pair(p, q) >= pair(r, s)

with 1-based spatial orbitals, drawn in that order from numpy's PCG64 with one
seed per Hamiltonian. One-body values go to AddOneBodyTerm(p, q) (p >= q). Each
two-body value is the Broombridge row [p, q, r, s, v] in Mulliken order, which
IngestBroombridge passes as AddTwoBodyTerm(p, r, s, q)
(cpp/hamiltonian.cc:40-52). The identity term is 0.

The Hartree-Fock start occupies the lowest n_alpha alpha and n_beta beta
orbitals: block-0 index rank(2^na - 1) * Cb + rank(2^nb - 1) = 0, amplitude
2^(-P/2) (the ancilla preparation of cpp/main.cc:111-115).
"""
from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np


@dataclass
class Integrals:
    n_orbitals: int                 # spatial orbitals M
    one_body: list                  # (p, q, v), 1-based, p >= q
    two_body: list                  # (p, r, s, q, v): AddTwoBodyTerm arguments
    identity: float = 0.0
    seed: int = 0


def synthetic_integrals(n_spin_orbitals: int, seed: int, two_body_sigma: float = 0.1) -> Integrals:
    if n_spin_orbitals % 2 or n_spin_orbitals < 2:
        raise ValueError("n_spin_orbitals must be a positive even number")
    M = n_spin_orbitals // 2
    rng = np.random.Generator(np.random.PCG64(seed))
    one = []
    for p in range(1, M + 1):
        for q in range(1, p + 1):
            one.append((p, q, float(rng.standard_normal() * math.exp(-abs(p - q) / 2.0))))
    pairs = [(p, q) for p in range(1, M + 1) for q in range(1, p + 1)]
    two = []
    for i, (p, q) in enumerate(pairs):
        for r, s in pairs[: i + 1]:
            v = float(rng.normal(0.0, two_body_sigma) * math.exp(-(abs(p - q) + abs(r - s)) / 3.0))
            two.append((p, r, s, q, v))
    return Integrals(M, one, two, 0.0, seed)


def hf_block0(ca: int, cb: int, precision: int, dtype=np.complex128) -> np.ndarray:
    """Block 0 of the QPE register for the Hartree-Fock start."""
    b = np.zeros(ca * cb, dtype)
    b[0] = 2.0 ** (-precision / 2.0)
    return b
