"""The learned-state pipeline's data: a ground-state projection post-selected
from a QPE run on the GPU is the ground state of the sector Hamiltonian (read
back from the sweep and diagonalised on the CPU, as in test_energy_ed), and the
model's proposed state is a normalised state over the register's strings."""
import math

import numpy as np
import pytest

from test_energy_ed import _sector_hamiltonian

pytestmark = pytest.mark.gpu


def test_post_selected_projection_is_the_ground_state(gpu, orc):
    q = gpu
    L = q.learned_state
    n, seed, P, dt = 8, 3, 9, 0.05
    M, e = n // 2, n // 4
    ints = q.synthetic_integrals(n, seed)
    H, _ = _sector_hamiltonian(q, orc, M, e, ints)
    evals, evecs = np.linalg.eigh(H)
    prog = q.Program(q.Hamiltonian.from_integrals(ints, e, dt).segmented_terms(), M, e, e)
    st = q.DeviceState(M, e, e, P)
    # a start dominated by the ground state, with a little of every other state
    rng = np.random.default_rng(1)
    b0 = evecs[:, 0] + 0.05 * rng.standard_normal(st.ld)
    b0 = b0 / np.linalg.norm(b0) * 2 ** (-P / 2)
    st.upload(b0.astype(np.complex128))
    st.evolve(prog)
    st.qift()
    probs = st.phase_probs()
    j0 = L.ground_bin(probs, dt)
    est = L.subbin_energy(probs / probs.sum(), j0, 1 << P, dt)
    res = 2 * math.pi / (dt * (1 << P))
    assert abs(est - evals[0]) < 0.5 * res + 0.05
    g = st.download()[j0 * st.ld:(j0 + 1) * st.ld]
    g = g / np.linalg.norm(g)
    assert abs(np.vdot(evecs[:, 0], g)) ** 2 > 0.9


def test_proposed_state_and_targets(gpu):
    q = gpu
    L = q.learned_state
    strings = L.register_strings(5, 2, 2)
    m = L.AmplitudeMLP(10, batch=128, seed=4)
    psi = L.proposed_state(m, strings)
    assert psi.shape == (len(strings),) and abs(np.linalg.norm(psi) - 1) < 1e-12
    la, ph, w = L.state_targets(psi)
    j = int(np.argmax(np.abs(psi)))
    assert abs(ph[j]) < 1e-6 and np.all(w > 0) and abs(w.mean() - 1.05) < 1e-4
    np.testing.assert_allclose(np.exp(la), np.maximum(np.abs(psi), 1e-6), rtol=1e-6)
