"""What the trained network gains over Hartree-Fock, judged by exact ground states.

n = 12, N = 6 (400 amplitudes per block). The model is trained on the tensor
cores on the simulator's own post-selected QPE ground projections (48 seeded
Hamiltonians, 8 ancilla qubits, from each Hamiltonian's lowest-diagonal
determinant). On 8 held-out Hamiltonians the exact Trotterized ground state is
the lowest eigenvector of one controlled power U (built column by column with
the oracle and diagonalised), so neither start is favoured by the yardstick.
The start that is run is chosen without the answer: the model proposes its
state and its cuts to the m largest amplitudes, the lowest variational energy
(one short GPU evolution each, batched) picks one of them, and it is run if that
energy is below Hartree-Fock's, else Hartree-Fock is. Checks: the chosen start's
QPE success (the GPU histogram's mass in the exact ground bin +- 1) is never
below Hartree-Fock's, so with the textbook QPE cost model it is never slower to
1e-3 Ha; and the gain is large: the learned start's median exact overlap is at
least 100x Hartree-Fock's, and its success beats Hartree-Fock's on at least 6
of the 8.
"""
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_learned_start_gain_over_hartree_fock(gpu, orc, record_property):
    q = gpu
    L = q.learned_state
    n, M, na, nb, dt, Pd, P, tau = 12, 6, 3, 3, 0.05, 8, 8, 1e-3
    strings = L.register_strings(M, na, nb)
    d = len(strings)

    def ham(s, t=dt):
        return q.Hamiltonian.from_integrals(q.synthetic_integrals(n, s), na, t)

    train = [ham(1000 + i) for i in range(48)]
    bt = q.Batch([q.Program(h.segmented_terms(), M, na, nb) for h in train], Pd, dtype=np.complex64)
    for i, h in enumerate(train):
        bt.upload(i, (L.lowest_diagonal_state(h, strings) * 2.0 ** (-Pd / 2)).astype(np.complex64))
    bt.run()
    la, ph, wt = [], [], []
    for i in range(len(train)):
        j0 = L.ground_bin(bt.phase_probs(i), dt)
        a, b, c = L.state_targets(bt.download(i, first=j0 * d, count=d))
        la.append(a)
        ph.append(b)
        wt.append(c)
    model = L.AmplitudeMLP(n, batch=8192, seed=1, n_feat=L.N_DIAG_FEATURES)
    model.set_data(np.concatenate([strings] * len(train)), np.concatenate(la), np.concatenate(ph),
                   np.concatenate(wt), np.concatenate([L.diagonal_features(h, strings) for h in train]))
    losses = model.train(600, lr=1e-3, seed=2)
    assert losses[-20:].mean() < losses[:20].mean()

    held = [ham(50000 + i) for i in range(8)]
    qb = q.Batch([q.Program(h.segmented_terms(), M, na, nb) for h in held] * 2, P, dtype=np.complex64)
    starts, evs = [], []
    hf = np.zeros(d, np.complex128)
    hf[0] = 1.0
    for i, h in enumerate(held):
        cands = L.learned_candidates(L.proposed_state(model, strings, L.diagonal_features(h, strings)))
        ptau = q.Program(ham(50000 + i, tau).segmented_terms(), M, na, nb)
        e = L.variational_energies([ptau] * (len(cands) + 1), [hf] + cands, tau)
        # the batched energies agree with the single-state helper
        assert abs(e[0] - L.variational_energy(ptau, hf, tau)) < 1e-9
        sel = int(np.argmin(e[1:]))
        starts.append(cands[sel])
        evs.append((e[0], e[1 + sel]))
        qb.upload(i, (hf * 2.0 ** (-P / 2)).astype(np.complex64))
        qb.upload(len(held) + i, (cands[sel] * 2.0 ** (-P / 2)).astype(np.complex64))
    qb.run()
    rows = []
    for i, h in enumerate(held):
        seg = h.segmented_terms()
        U = np.zeros((d, d), complex)
        for j in range(d):
            st = np.zeros(2 * d, complex)
            st[j] = 1.0
            orc.time_evolve(M, na, nb, 1, seg, st)
            U[:, j] = st[d:]
        lam, V = np.linalg.eig(U)
        E = -np.angle(lam) / dt
        k = int(np.argmin(E))
        g = V[:, k] / np.linalg.norm(V[:, k])
        j0 = int(round((-E[k] * dt / (2 * math.pi)) % 1.0 * (1 << P))) % (1 << P)
        learned = starts[i]
        e_hf, e_l = evs[i]
        s_hf = L.window_mass(qb.phase_probs(i), j0)
        s_l = L.window_mass(qb.phase_probs(len(held) + i), j0)
        chosen = s_l if e_l < e_hf else s_hf
        rows.append((abs(np.vdot(g, hf)) ** 2, abs(np.vdot(g, learned)) ** 2, s_hf, s_l, e_l < e_hf, chosen))
    r = np.array(rows, dtype=float)
    ov_hf, ov_l = np.median(r[:, 0]), np.median(r[:, 1])
    record_property("median_overlap_hf", float(ov_hf))
    record_property("median_overlap_learned", float(ov_l))
    record_property("median_success_hf", float(np.median(r[:, 2])))
    record_property("median_success_learned", float(np.median(r[:, 3])))
    record_property("learned_chosen", int(r[:, 4].sum()))
    print(f"learned vs Hartree-Fock on 8 held-out n=12 Hamiltonians: median exact overlap {ov_l:.3g} vs {ov_hf:.3g}, "
          f"median success {np.median(r[:, 3]):.3g} vs {np.median(r[:, 2]):.3g}, learned chosen {int(r[:, 4].sum())}/8")
    # the chosen start is never less likely to land in the ground window, hence never
    # slower (a candidate can be the Hartree-Fock determinant itself up to a global
    # phase, whose complex64 histogram differs from Hartree-Fock's by rounding only)
    assert np.all(r[:, 5] >= r[:, 2] * (1 - 1e-4))
    # the gain
    assert ov_l >= 100 * ov_hf
    assert (r[:, 3] > r[:, 2]).sum() >= 6
    t_hf = L.qpe_time_to_precision(float(np.median(r[:, 2])), 1e-6, dt)[0]
    t_l = L.qpe_time_to_precision(float(np.median(r[:, 5])), 1e-6, dt)[0]
    assert t_l is not None and (t_hf is None or t_l < t_hf)
