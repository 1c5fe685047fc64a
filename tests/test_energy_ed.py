"""Energies by exact diagonalisation, on CPU with the oracle (small sectors).

The sector Hamiltonian that a Trotter sweep exponentiates is read back from
the sweep itself: every applied term is U_k = exp(-i t G_k), with G_k = h (+-1) X
on each of its amplitude pairs (the sign is the Jordan-Wigner parity of the
pair) or h on the amplitudes a diagonal term acts on. Evolving basis vectors
through one term at a time gives G_k exactly (from its off-diagonal sin(h t) or
its diagonal phase), and H = sum_k G_k over the terms applyUnitary_reordered
applies. Checks: H is Hermitian; one first-order sweep differs from exp(-i H dt)
by O(dt^2); the QPE histogram's sub-bin energy lands on H's spectrum within
the resolution of the register.
"""
import math

import numpy as np
import pytest
from scipy.linalg import expm

KINDS = ("pp", "pq", "pqqp", "pqqr", "pqrs")


def _applied_terms(seg):
    """(kind, index) of every term of the sweep, in applyUnitary_reordered order
    (pqqr nested under its pq term; unmatched pqqr terms are skipped)."""
    out = [("pp", i) for i in range(len(seg["pp"]))] + [("pqqp", i) for i in range(len(seg["pqqp"]))]
    for i, pq in enumerate(seg["pq"]):
        out.append(("pq", i))
        for j, t in enumerate(seg["pqqr"]):
            if t["p"] == pq["q"] and t["s"] == pq["p"]:
                out.append(("pqqr", j))
    return out + [("pqrs", i) for i in range(len(seg["pqrs"]))]


def _sector_hamiltonian(q, orc, M, e, ints, t=0.37):
    h = q.Hamiltonian.from_integrals(ints, e, t)
    seg = h.segmented_terms()
    raw = h.PrintIndexedSegmentedHamiltonianTerms()
    rawv = {k: np.array([v for _, v in raw[i]], float) for i, k in enumerate(KINDS)}
    C = math.comb(M, e)
    d = C * C
    H = np.zeros((d, d))
    for kind, i in _applied_terms(seg):
        one = {k: seg[k][:0] for k in KINDS}
        one[kind] = seg[kind][i:i + 1]
        if kind == "pqqr":
            # a pqqr term is applied only under its pq term (p_ == q, r_ == p):
            # give it that parent with the identity matrix
            t4 = seg["pqqr"][i]
            parent = [j for j, pq in enumerate(seg["pq"]) if pq["q"] == t4["p"] and pq["p"] == t4["s"]][0]
            ident = seg["pq"][parent:parent + 1].copy()
            ident["even"] = [1.0, 0.0, 0.0, 0.0]
            ident["odd"] = [1.0, 0.0, 0.0, 0.0]
            one["pq"] = ident
        hk = rawv[kind][i]
        U = np.zeros((d, d), complex)
        for j in range(d):
            st = np.zeros(2 * d, complex)
            st[j] = 1.0
            orc.time_evolve(M, e, e, 1, one, st)
            U[:, j] = st[d:]
        if kind in ("pp", "pqqp"):
            acted = np.abs(np.diag(U) - 1.0) > 1e-12
            H[acted, acted] += hk
        else:
            s = math.sin(hk * t)
            if abs(s) < 1e-9:
                continue
            off = U - np.diag(np.diag(U))
            H += (-off.imag / s) * hk
    return H, seg


@pytest.mark.parametrize("n,seed", [(8, 0), (8, 5), (10, 2)])
def test_sector_hamiltonian_and_trotter_order(q, orc, n, seed):
    M, e = n // 2, n // 4
    ints = q.synthetic_integrals(n, seed)
    H, _ = _sector_hamiltonian(q, orc, M, e, ints)
    assert np.allclose(H, H.T, atol=1e-12)
    d = H.shape[0]
    rng = np.random.default_rng(seed)
    psi = rng.standard_normal(d) + 1j * rng.standard_normal(d)
    psi /= np.linalg.norm(psi)
    errs = []
    for dt in (0.02, 0.01):
        seg = q.Hamiltonian.from_integrals(ints, e, dt).segmented_terms()
        st = np.zeros(2 * d, complex)
        st[:d] = psi
        orc.time_evolve(M, e, e, 1, seg, st)
        errs.append(np.linalg.norm(st[d:] - expm(-1j * H * dt) @ psi))
    # first-order Trotter: the local error scales as dt^2
    assert 3.0 < errs[0] / errs[1] < 5.0, errs


def _power(q, orc, M, e, ints, psi, dt, order, steps):
    """One controlled power of total time dt in `steps` Trotter steps: order 1
    sweeps at dt / steps, order 2 a forward and a reversed sweep at dt / (2 steps)
    each (the coefficient time the plain-n16 workload uses is dt / 2 per sweep)."""
    t = dt / (2 * steps) if order == 2 else dt / steps
    seg = q.Hamiltonian.from_integrals(ints, e, t).segmented_terms()
    d = len(psi)
    st = np.zeros(2 * d, complex)
    st[:d] = psi
    orc.time_evolve(M, e, e, 1, seg, st, order=order, steps=steps)
    return st[d:]


@pytest.mark.parametrize("n,seed", [(8, 0), (8, 5), (10, 2)])
def test_second_order_trotter_is_second_order(q, orc, n, seed):
    """The order-2 extension (a forward and a reversed sweep per step, the mode
    the plain-n16 workload runs with 4 steps per power; the reference has first
    order only, cpp/time_evolution_over_terms.hpp:116-137) against exp(-i H dt)
    of the sector Hamiltonian read back from the sweep:
    - its one-step error falls about 8x from dt to dt / 2 (local error dt^3),
      where first order falls about 4x (dt^2);
    - four order-2 steps of dt / 4 are about 16x closer than one step of dt;
    - as dt -> 0, four order-2 steps converge to one first-order step, their
      difference falling about 4x per halving (it is first order's dt^2 error)."""
    M, e = n // 2, n // 4
    ints = q.synthetic_integrals(n, seed)
    H, _ = _sector_hamiltonian(q, orc, M, e, ints)
    d = H.shape[0]
    rng = np.random.default_rng(100 + seed)
    psi = rng.standard_normal(d) + 1j * rng.standard_normal(d)
    psi /= np.linalg.norm(psi)
    dts = (0.04, 0.02, 0.01)
    exact = {dt: expm(-1j * H * dt) @ psi for dt in dts}
    e1 = [np.linalg.norm(_power(q, orc, M, e, ints, psi, dt, 1, 1) - exact[dt]) for dt in dts]
    e2 = [np.linalg.norm(_power(q, orc, M, e, ints, psi, dt, 2, 1) - exact[dt]) for dt in dts]
    e24 = [np.linalg.norm(_power(q, orc, M, e, ints, psi, dt, 2, 4) - exact[dt]) for dt in dts]
    diff = [np.linalg.norm(_power(q, orc, M, e, ints, psi, dt, 2, 4) - _power(q, orc, M, e, ints, psi, dt, 1, 1))
            for dt in dts]
    for i in range(2):
        assert 3.0 < e1[i] / e1[i + 1] < 5.0, e1
        assert 6.0 < e2[i] / e2[i + 1] < 10.0, e2
        assert 6.0 < e24[i] / e24[i + 1] < 10.0, e24
        assert 3.0 < diff[i] / diff[i + 1] < 5.0, diff
    for i in range(3):
        assert 10.0 < e2[i] / e24[i] < 22.0, (e2, e24)
        assert e2[i] < e1[i]


def test_qpe_energy_on_the_spectrum(q, orc):
    n, seed, P, dt = 8, 3, 10, 0.05
    M, e = n // 2, n // 4
    ints = q.synthetic_integrals(n, seed)
    H, _ = _sector_hamiltonian(q, orc, M, e, ints)
    evals = np.linalg.eigvalsh(H)
    seg = q.Hamiltonian.from_integrals(ints, e, dt).segmented_terms()
    d = H.shape[0]
    st = np.zeros((1 << P) * d, complex)
    st[0] = 2 ** (-P / 2)
    orc.time_evolve(M, e, e, P, seg, st)
    orc.qift(P, d, st)
    probs = orc.identify_phase_amplitudes(P, d, st)
    est = q.phase_to_energy(q.subbin_phase(probs), dt)
    # the peak estimate is an eigenvalue of H up to the register's resolution
    # and the first-order Trotter shift
    res = 2 * math.pi / (dt * (1 << P))
    assert np.min(np.abs(evals - est)) < 0.5 * res + 0.05


def test_diagonal_energies_match_the_sector_hamiltonian(q, orc):
    """The learned model's diagonal-energy feature <x|H|x> (pp and pqqp terms) is
    the diagonal of the sector Hamiltonian read back from the sweep."""
    M, e = 4, 2
    ints = q.synthetic_integrals(8, 3)
    H, _ = _sector_hamiltonian(q, orc, M, e, ints)
    h = q.Hamiltonian.from_integrals(ints, e, 0.05)
    L = q.learned_state
    strings = L.register_strings(M, e, e)
    assert np.abs(L.diagonal_energies(h, strings) - np.diag(H)).max() < 1e-12
    f = L.diagonal_features(h, strings)
    assert f.shape == (len(strings), L.N_DIAG_FEATURES) and f[:, 0].min() == 0.0 and f[:, 1].max() == 1.0
