"""Learned initial state: an MLP over occupation bit strings that proposes the
QPE initial state in place of Hartree-Fock (include/qpe_gb300_mlp.h).

The model runs on the tensor cores (tcgen05 MMA with TMA-loaded BF16 operands,
FP32 accumulation in tensor memory). This module holds the host side: the
model handle, the BF16 helpers, the training-set construction from post-selected
QPE projections, and the state the model proposes for a register.
"""
from __future__ import annotations

import ctypes as C
import math

import numpy as np

from . import _native as N

NB_HIDDEN, NB_IN, NB_OUT = 256, 64, 16
# offsets of the parameter blocks (qpe_mlp_get_params layout)
_SIZES = [("W1", (256, 64)), ("b1", (256,)), ("W2", (256, 256)), ("b2", (256,)), ("W3", (256, 256)), ("b3", (256,)),
          ("W4", (16, 256)), ("b4", (16,))]


def param_layout() -> dict:
    out, off = {}, 0
    for name, shape in _SIZES:
        n = int(np.prod(shape))
        out[name] = (off, shape)
        off += n
    return out


def to_bf16_bits(x: np.ndarray) -> np.ndarray:
    """float32 -> bfloat16 bit patterns, round to nearest even."""
    u = np.ascontiguousarray(x, np.float32).view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16).astype(np.uint16)
    return r


def from_bf16_bits(b: np.ndarray) -> np.ndarray:
    return (np.asarray(b, np.uint16).astype(np.uint32) << 16).view(np.float32)


def round_bf16(x: np.ndarray) -> np.ndarray:
    return from_bf16_bits(to_bf16_bits(x))


def gemm_bf16(A: np.ndarray, B: np.ndarray, tile_n: int = 256, device: int = 0) -> np.ndarray:
    """D = A . B^T on the tensor cores (A [M, K], B [N, K], rounded to BF16)."""
    M, K = A.shape
    Nn, K2 = B.shape
    assert K == K2
    a = to_bf16_bits(A)
    b = to_bf16_bits(B)
    d = np.zeros((M, Nn), np.float32)
    N.check(N.lib().qpe_gemm_bf16(N.context(device), M, Nn, K, a.ctypes.data_as(C.POINTER(C.c_uint16)),
                                  b.ctypes.data_as(C.POINTER(C.c_uint16)), d.ctypes.data_as(C.POINTER(C.c_float)),
                                  tile_n))
    return d


def _fp(a):
    return a.ctypes.data_as(C.POINTER(C.c_float))


class AmplitudeMLP:
    """Occupation string (and n_feat extra features) -> (log|a|, phase); n_bits +
    n_feat inputs, 3 x 256 GELU, BF16."""

    def __init__(self, n_bits: int, batch: int = 8192, seed: int = 0, device: int = 0, n_feat: int = 0):
        self._lib = N.lib()
        h = C.c_void_p()
        N.check(self._lib.qpe_mlp_create2(N.context(device), n_bits, n_feat, batch, seed, C.byref(h)))
        self._h = h
        self.n_bits, self.n_feat, self.batch = n_bits, n_feat, batch
        n = C.c_uint64()
        N.check(self._lib.qpe_mlp_num_params(h, C.byref(n)))
        self.num_params = n.value

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            self._lib.qpe_mlp_destroy(h)
            self._h = None

    def get_params(self) -> np.ndarray:
        p = np.zeros(self.num_params, np.float32)
        N.check(self._lib.qpe_mlp_get_params(self._h, _fp(p)))
        return p

    def set_params(self, p: np.ndarray) -> None:
        p = np.ascontiguousarray(p, np.float32)
        assert p.size == self.num_params
        N.check(self._lib.qpe_mlp_set_params(self._h, _fp(p)))

    def _feats(self, feats, count):
        if self.n_feat == 0:
            return None
        f = np.ascontiguousarray(feats, np.float32).reshape(count, self.n_feat)
        return f

    def set_data(self, bits, log_abs, phase, weight, feats=None) -> None:
        bits = np.ascontiguousarray(bits, np.uint64)
        la, ph, w = (np.ascontiguousarray(x, np.float32) for x in (log_abs, phase, weight))
        f = self._feats(feats, bits.size)
        N.check(self._lib.qpe_mlp_set_data2(self._h, bits.ctypes.data_as(C.POINTER(C.c_uint64)),
                                            _fp(f) if f is not None else None, _fp(la), _fp(ph), _fp(w), bits.size))

    def train(self, steps: int, lr: float = 1e-3, seed: int = 0) -> np.ndarray:
        losses = np.zeros(steps, np.float32)
        N.check(self._lib.qpe_mlp_train(self._h, steps, lr, seed, _fp(losses)))
        return losses

    def forward(self, bits, feats=None) -> np.ndarray:
        bits = np.ascontiguousarray(bits, np.uint64)
        out = np.zeros((bits.size, 2), np.float32)
        f = self._feats(feats, bits.size)
        N.check(self._lib.qpe_mlp_forward2(self._h, bits.ctypes.data_as(C.POINTER(C.c_uint64)),
                                           _fp(f) if f is not None else None, bits.size, _fp(out)))
        return out

    def gradients(self, bits, log_abs, phase, weight, feats=None):
        bits = np.ascontiguousarray(bits, np.uint64)
        la, ph, w = (np.ascontiguousarray(x, np.float32) for x in (log_abs, phase, weight))
        g = np.zeros(self.num_params, np.float32)
        loss = np.zeros(1, np.float32)
        f = self._feats(feats, bits.size)
        N.check(self._lib.qpe_mlp_gradients2(self._h, bits.ctypes.data_as(C.POINTER(C.c_uint64)),
                                             _fp(f) if f is not None else None, _fp(la), _fp(ph), _fp(w), bits.size,
                                             _fp(g), _fp(loss)))
        return g, float(loss[0])

    def tensor_flops_per_step(self) -> float:
        f = C.c_double()
        N.check(self._lib.qpe_mlp_tensor_flops_per_step(self._h, C.byref(f)))
        return f.value


# ---- the learned-state pipeline ---------------------------------------------------

def colex_rank(bv: int) -> int:
    """OffsetComputer::rank (cpp/offset_computer.hpp:16-27): sum_i C(pos_i, i + 1)."""
    r, order, pos = 0, 1, 0
    while bv:
        if bv & 1:
            r += math.comb(pos, order)
            order += 1
        bv >>= 1
        pos += 1
    return r


def colex_strings(nbits: int, weight: int) -> np.ndarray:
    """The weight-`weight` strings of nbits bits in rank order."""
    from itertools import combinations
    strs = [sum(1 << i for i in c) for c in combinations(range(nbits), weight)]
    strs.sort(key=colex_rank)
    return np.array(strs, np.uint64)


def register_strings(M: int, na: int, nb: int) -> np.ndarray:
    """Occupation string of every amplitude of a block, in register order (alpha
    rank major, beta rank minor); alpha orbitals are bits 0..M-1, beta M..2M-1
    (the HalfUp convention of cpp/types.hpp:50-55)."""
    a = colex_strings(M, na)
    b = colex_strings(M, nb)
    return (a[:, None] | (b[None, :] << np.uint64(M))).ravel()


def state_targets(psi: np.ndarray, floor: float = 1e-6):
    """Training targets of one state: log|a| (floored), phase with the largest
    amplitude made real and positive, and weights |a|^2 * dim + 0.05 (mean ~1)."""
    psi = np.asarray(psi, np.complex128)
    psi = psi / np.linalg.norm(psi)
    j = int(np.argmax(np.abs(psi)))
    psi = psi * np.exp(-1j * np.angle(psi[j]))
    a = np.abs(psi)
    return (np.log(np.maximum(a, floor)).astype(np.float32), np.angle(psi).astype(np.float32),
            (a * a * len(psi) + 0.05).astype(np.float32))


# Extra inputs of the learned model per occupation string: its diagonal energy
# <x|H|x> under the string's Hamiltonian, as z = (E - E_min) / std over the
# sector (clipped at 8) and exp(-z).
N_DIAG_FEATURES = 2


def diagonal_energies(hamiltonian, strings: np.ndarray) -> np.ndarray:
    """<x|H|x> of every string x: the pp terms h_p n_p and the pqqp terms
    h_pq n_p n_q (the terms that act diagonally; bit p of x is spin orbital p)."""
    raw = hamiltonian.PrintIndexedSegmentedHamiltonianTerms()
    nso = 2 * hamiltonian.num_orbitals()
    h1 = np.zeros(nso)
    for (p, _), v in raw[0]:
        h1[p] += v
    J = np.zeros((nso, nso))
    for (p, q, _, _), v in raw[2]:
        J[p, q] += v
    occ = ((np.asarray(strings, np.uint64)[:, None] >> np.arange(nso, dtype=np.uint64)[None, :])
           & np.uint64(1)).astype(np.float64)
    return occ @ h1 + np.einsum("ij,ij->i", occ @ J, occ)


def diagonal_features(hamiltonian, strings: np.ndarray) -> np.ndarray:
    """The model's extra inputs for `strings` under `hamiltonian` ([len, 2] float32)."""
    e = diagonal_energies(hamiltonian, strings)
    z = (e - e.min()) / max(float(e.std()), 1e-12)
    return np.stack([np.minimum(z, 8.0), np.exp(-z)], axis=1).astype(np.float32)


def lowest_diagonal_state(hamiltonian, strings: np.ndarray) -> np.ndarray:
    """The determinant of lowest diagonal energy <x|H|x> (a classical start that
    needs no training), as a normalised state over `strings`."""
    e = diagonal_energies(hamiltonian, strings)
    psi = np.zeros(len(strings), np.complex128)
    psi[int(np.argmin(e))] = 1.0
    return psi


def variational_energy(program_tau, psi: np.ndarray, tau: float, device: int = 0) -> float:
    """<psi|H|psi> from one short evolution on the GPU: program_tau is the
    Hamiltonian's program at a small timestep tau (one first-order step), and
    <psi|U(tau)|psi> = exp(-i <H> tau) (1 + O(tau^2)), so <H> = -arg(...) / tau up
    to O(tau^2). Used to choose between two starts without knowing the answer."""
    from .time_evolution import DeviceState
    psi = np.asarray(psi, np.complex128)
    psi = psi / np.linalg.norm(psi)
    st = DeviceState(program_tau.num_orbitals, program_tau.n_alpha, program_tau.n_beta, 1, device=device)
    st.upload(psi)
    st.evolve(program_tau)
    u = st.download(first=len(psi), count=len(psi))
    return float(-np.angle(np.vdot(psi, u)) / tau)


def lowest_diagonal_state(hamiltonian, strings: np.ndarray) -> np.ndarray:
    """The determinant of lowest diagonal energy <x|H|x> (a classical start that
    needs no training), as a normalised state over `strings`."""
    e = diagonal_energies(hamiltonian, strings)
    psi = np.zeros(len(strings), np.complex128)
    psi[int(np.argmin(e))] = 1.0
    return psi


def variational_energy(program_tau, psi: np.ndarray, tau: float, device: int = 0) -> float:
    """<psi|H|psi> from one short evolution on the GPU: program_tau is the
    Hamiltonian's program at a small timestep tau (one first-order step), and
    <psi|U(tau)|psi> = exp(-i <H> tau) (1 + O(tau^2)), so <H> = -arg(...) / tau up
    to O(tau^2). Used to choose between starts without knowing the answer."""
    from .time_evolution import DeviceState
    psi = np.asarray(psi, np.complex128)
    psi = psi / np.linalg.norm(psi)
    st = DeviceState(program_tau.num_orbitals, program_tau.n_alpha, program_tau.n_beta, 1, device=device)
    st.upload(psi)
    st.evolve(program_tau)
    u = st.download(first=len(psi), count=len(psi))
    return float(-np.angle(np.vdot(psi, u)) / tau)


def variational_energies(programs_tau, states, tau: float, device: int = 0) -> np.ndarray:
    """variational_energy for many (program, state) pairs in one batched launch:
    a batch of one controlled power (P = 1) per pair, complex128. The batch's QIFT
    turns blocks (b0, b1) into ((b0 + b1) / sqrt 2, (b0 - b1) / sqrt 2), so
    b1 = U(tau) psi is recovered from the two blocks it returns."""
    from .batching import Batch
    states = [np.asarray(x, np.complex128) / np.linalg.norm(x) for x in states]
    bt = Batch(list(programs_tau), 1, dtype=np.complex128, device=device)
    for i, x in enumerate(states):
        bt.upload(i, x)
    bt.run()
    out = np.zeros(len(states))
    for i, x in enumerate(states):
        r = bt.download(i)
        d = len(x)
        u = (r[:d] - r[d:]) / np.sqrt(2.0)
        out[i] = -np.angle(np.vdot(x, u)) / tau
    return out


def truncated(psi: np.ndarray, m: int) -> np.ndarray:
    """psi restricted to its m largest amplitudes, renormalised."""
    psi = np.asarray(psi, np.complex128)
    keep = np.argsort(-np.abs(psi))[:m]
    out = np.zeros_like(psi)
    out[keep] = psi[keep]
    return out / np.linalg.norm(out)


# The model's candidate starts: its whole proposed state and the proposal cut
# to its m largest amplitudes; variational energy picks one of them.
CANDIDATE_TRUNCATIONS = (1, 2, 4, 8, 16, 64, 256)


def learned_candidates(psi: np.ndarray) -> list:
    return [psi] + [truncated(psi, m) for m in CANDIDATE_TRUNCATIONS if m < len(psi)]


def proposed_state(model: AmplitudeMLP, strings: np.ndarray, feats=None) -> np.ndarray:
    """The model's state over `strings` (with the features of their Hamiltonian
    when the model takes features), normalised to 1."""
    out = model.forward(strings, feats).astype(np.float64)
    amp = np.exp(out[:, 0] - out[:, 0].max()) * np.exp(1j * out[:, 1])
    return amp / np.linalg.norm(amp)


def ground_bin(probs: np.ndarray, t_power: float, rel: float = 0.02) -> int:
    """The lowest-energy local maximum of the histogram holding at least `rel`
    of the largest bin (the Fejer side lobes of one peak decay monotonically, so
    they are not local maxima)."""
    from .readout import phase_to_energy
    n = len(probs)
    thr = rel * float(probs.max())
    cand = [j for j in range(n) if probs[j] >= thr and probs[j] >= probs[(j - 1) % n] and probs[j] >= probs[(j + 1) % n]]
    return int(min(cand, key=lambda j: phase_to_energy(j / n, t_power)))


def shared_ground_bin(hists, t_power: float, rel: float = 1e-3) -> int:
    """The ground bin of one Hamiltonian from several QPE histograms (one per
    start): the lowest-energy bin that is a local maximum holding at least `rel`
    of the probability in at least one of them. The same bin then scores every
    start, so no start's own peak shape decides the target."""
    from .readout import phase_to_energy
    cand = set()
    for p in hists:
        p = np.asarray(p, np.float64)
        n = len(p)
        thr = rel * float(p.sum())
        cand |= {j for j in range(n) if p[j] >= thr and p[j] >= p[(j - 1) % n] and p[j] >= p[(j + 1) % n]}
    n = len(hists[0])
    return int(min(cand, key=lambda j: phase_to_energy(j / n, t_power)))


def qpe_time_to_precision(success: float, seconds_per_power: float, t_power: float, tol: float = 1e-3,
                          confidence: float = 0.9):
    """Time for textbook QPE to resolve the ground energy to `tol` from a start
    whose runs land in the ground window with probability `success`: a register
    of bits = ceil(log2(2 pi / (t_power * 2 tol))) ancilla qubits (bins at most
    2 tol wide), 2^bits - 1 controlled powers per run at `seconds_per_power`, and
    runs = ceil(log(1 - confidence) / log(1 - success)) so that the ground window
    is observed at least once with that confidence. Returns (seconds, runs,
    bits); seconds is None when success is 0."""
    bits = int(math.ceil(math.log2(2.0 * math.pi / (t_power * 2.0 * tol))))
    if success <= 0.0:
        return None, None, bits
    runs = 1 if success >= 1.0 else int(math.ceil(math.log(1.0 - confidence) / math.log1p(-success)))
    return runs * ((1 << bits) - 1) * seconds_per_power, runs, bits


def window_mass(probs: np.ndarray, j0: int, half: int = 1) -> float:
    n = len(probs)
    return float(sum(probs[(j0 + d) % n] for d in range(-half, half + 1)))


def subbin_energy(freq: np.ndarray, j0: int, n: int, t_power: float) -> float:
    """Energy from the histogram (or shot frequencies) around bin j0: peak bin
    refined by the amplitude ratio of its larger neighbour."""
    from .readout import phase_to_energy
    a0 = math.sqrt(max(freq[j0 % n], 0.0))
    left, right = math.sqrt(max(freq[(j0 - 1) % n], 0.0)), math.sqrt(max(freq[(j0 + 1) % n], 0.0))
    if right >= left:
        d = right / (a0 + right) if a0 + right > 0 else 0.0
    else:
        d = -left / (a0 + left) if a0 + left > 0 else 0.0
    return phase_to_energy(((j0 + d) / n) % 1.0, t_power)


def shots_to_precision(probs: np.ndarray, j0: int, t_power: float, e_target: float, tol: float = 1e-3,
                       trials: int = 16, seed: int = 0, max_shots: int = 1 << 22):
    """Smallest number of QPE shots (on a doubling grid) after which the sub-bin
    estimate from the shots landing in the ground window j0 +- 1 is within `tol`
    of e_target in at least 90% of `trials` simulated experiments. None when the
    noiseless estimate itself misses `tol` or max_shots is not enough."""
    n = len(probs)
    p = np.clip(np.asarray(probs, np.float64), 0, None)
    p = p / p.sum()
    if abs(subbin_energy(p, j0, n, t_power) - e_target) > tol:
        return None
    rng = np.random.default_rng(seed)
    shots = 16
    while shots <= max_shots:
        ok = 0
        for _ in range(trials):
            f = rng.multinomial(shots, p).astype(np.float64)
            if f[[(j0 - 1) % n, j0 % n, (j0 + 1) % n]].sum() == 0:
                continue
            # the estimate uses the peak of the observed window
            w = [(j0 + d) % n for d in (-1, 0, 1)]
            jm = w[int(np.argmax(f[w]))]
            if abs(subbin_energy(f, jm, n, t_power) - e_target) <= tol:
                ok += 1
        if ok >= 0.9 * trials:
            return shots
        shots *= 2
    return None
