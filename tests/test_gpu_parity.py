"""GPU path against the oracle (same inputs, this machine) and the golden vectors
(the reference itself, another machine).

complex128 results are compared bit for bit with the oracle: both use the same
operation order with every product and sum rounded separately. Against the
golden vectors (produced on a different CPU) they agree to 1e-13. complex64
results are compared with the complex128 oracle with the tolerance stated in
each test.
"""
import math

import numpy as np
import pytest

from conftest import GOLDEN, evolve_cases, golden_segments, load_golden

pytestmark = pytest.mark.gpu

KINDS = ("pp", "pq", "pqqp", "pqqr", "pqrs")


def _seg(q, n, N, seed, dt):
    return q.Hamiltonian.from_integrals(q.synthetic_integrals(n, seed), N // 2, dt).segmented_terms()


def test_rank_and_unrank_against_oracle(gpu, orc):
    q = gpu
    rng = np.random.default_rng(1)
    bvs = rng.integers(0, 1 << 40, size=5000, dtype=np.uint64)
    bvs[:3] = [0, 1, (1 << 40) - 1]
    got = q.OffsetComputer.ranks(bvs)
    assert list(got) == [orc.rank(int(b)) for b in bvs]
    for nbits, w in [(8, 4), (12, 6), (20, 10), (24, 12), (5, 0), (31, 3), (32, 16)]:
        total = math.comb(nbits, w)
        ranks = np.arange(min(total, 20000), dtype=np.int64)
        s = q.OffsetComputer.unrank(nbits, w, ranks)
        # colex enumeration order of next_comb, from the smallest string
        x = (1 << w) - 1
        for r in range(len(ranks)):
            assert int(s[r]) == x, (nbits, w, r)
            x = orc.next_comb(x) if x else 1
        assert np.array_equal(q.OffsetComputer.ranks(s), ranks)


def test_swap_ranks_against_reference(gpu):
    q = gpu
    z = load_golden("swaps.npz")
    qoff = 0
    for n, bv, cnt in z["heads"]:
        qs = z["queries"][qoff:qoff + cnt]
        want = z["ranks"][qoff:qoff + cnt]
        qoff += cnt
        oc = q.OffsetComputer(int(n), int(bv))
        assert np.array_equal(oc.rank_with_swaps(qs), want)


def test_device_tables_equal_reference_runs(gpu):
    """Each device table equals the reference's discover*_BVs runs expanded in
    order (off01 + i, off10 + i, mid_parity & 1 for i < niter)."""
    from qpesim_gb300.offset_computer import axis_table
    z = load_golden("discover.npz")
    off = 0
    for kind, M, e, p, q_, r, s, n in z["rows"]:
        runs = z["tables"][off:off + n]
        off += n
        orb = {0: [q_], 1: [p, r], 2: [p, r], 3: [p, q_, r], 4: [p, q_, r, s]}[int(kind)]
        i01, i10, par = axis_table(int(kind), int(M), int(e), [int(x) for x in orb])
        w01 = np.concatenate([np.arange(o1, o1 + ni) for ni, o1, _, _ in runs]) if n else np.zeros(0)
        assert np.array_equal(i01, w01), (kind, M, e, p, q_, r, s)
        if kind >= 2:
            w10 = np.concatenate([np.arange(o2, o2 + ni) for ni, _, o2, _ in runs])
            wp = np.concatenate([np.full(ni, pa & 1) for ni, _, _, pa in runs])
            assert np.array_equal(i10, w10) and np.array_equal(par, wp), (kind, M, e, p, q_, r, s)


@pytest.mark.parametrize("name", evolve_cases())
def test_golden_evolution_qift_probs(gpu, orc, name):
    q = gpu
    z = load_golden(name)
    n, N, P = int(z["n"]), int(z["N"]), int(z["P"])
    M, e = n // 2, N // 2
    seg = golden_segments(z)
    ld = len(z["block0"])
    sv = q.StateVector(P, M, e)
    sv[:ld] = z["block0"]
    h = q.Hamiltonian.from_integrals(q.synthetic_integrals(n, int(z["seed"])), e, float(z["dt"]))
    q.time_evolve_over_terms(sv, h, P)
    ref = np.zeros(len(sv), np.complex128)
    ref[:ld] = z["block0"]
    orc.time_evolve(M, e, e, P, seg, ref)
    assert np.array_equal(np.asarray(sv), ref)
    np.testing.assert_allclose(np.asarray(sv), z["evolved"], rtol=0, atol=1e-13)
    sv.qift()
    orc.qift(P, ld, ref)
    assert np.array_equal(np.asarray(sv), ref)
    np.testing.assert_allclose(np.asarray(sv), z["qift"], rtol=0, atol=1e-13)
    np.testing.assert_allclose(sv.IdentifyPhaseAmplitudes(), z["probs"], rtol=1e-12, atol=1e-15)


@pytest.mark.parametrize("n,na,nb,P,order,steps", [
    (8, 2, 2, 5, 1, 1), (12, 3, 3, 3, 1, 1), (14, 4, 3, 2, 1, 1), (10, 1, 1, 3, 1, 1), (10, 5, 5, 2, 1, 1),
    (10, 2, 3, 3, 2, 3), (12, 2, 2, 2, 2, 1), (16, 4, 4, 2, 1, 1), (6, 3, 3, 3, 1, 1)])
def test_device_state_against_oracle(gpu, orc, n, na, nb, P, order, steps):
    q = gpu
    M = n // 2
    seg = _seg(q, n, 2 * max(na, nb), 100 + n + na, 0.07)
    prog = q.Program(seg, M, na, nb, trotter_order=order, steps=steps)
    st = q.DeviceState(M, na, nb, P)
    block0 = q.hf_block0(st.c_alpha, st.c_beta, P)
    rng = np.random.default_rng(n)
    block0 += (rng.standard_normal(st.ld) + 1j * rng.standard_normal(st.ld)) * 1e-2
    st.upload(block0)
    st.evolve(prog)
    got = st.download()
    ref = np.zeros(st.size, np.complex128)
    ref[:st.ld] = block0
    orc.time_evolve(M, na, nb, P, seg, ref, order=order, steps=steps)
    assert np.array_equal(got, ref)
    np.testing.assert_allclose(st.block_norms(), [np.vdot(b, b).real for b in ref.reshape(-1, st.ld)], rtol=1e-12)
    st.qift()
    orc.qift(P, st.ld, ref)
    assert np.array_equal(st.download(), ref)
    np.testing.assert_allclose(st.phase_probs(), orc.identify_phase_amplitudes(P, st.ld, ref), rtol=1e-12,
                               atol=1e-16)


def test_partial_power_ranges_compose(gpu):
    q = gpu
    seg = _seg(q, 10, 6, 9, 0.1)
    prog = q.Program(seg, 5, 3, 3)
    a = q.DeviceState(5, 3, 3, 4)
    b = q.DeviceState(5, 3, 3, 4)
    b0 = q.hf_block0(a.c_alpha, a.c_beta, 4)
    a.upload(b0)
    b.upload(b0)
    a.evolve(prog)
    b.evolve(prog, 1, 6)
    b.evolve(prog, 6, 16)
    assert np.array_equal(a.download(), b.download())


def test_complex64_error_is_stated(gpu, orc):
    """complex64 state with FP32 arithmetic (FP64 coefficients rounded once):
    the amplitudes stay within 2e-5 of the complex128 oracle over 31 powers at
    n = 12, and the histogram within 1e-5."""
    q = gpu
    n, N, P = 12, 6, 5
    M, e = n // 2, N // 2
    seg = _seg(q, n, N, 21, 0.05)
    prog = q.Program(seg, M, e, e)
    st = q.DeviceState(M, e, e, P, dtype=np.complex64)
    b0 = q.hf_block0(st.c_alpha, st.c_beta, P)
    st.upload(b0.astype(np.complex64))
    st.evolve(prog)
    got = st.download()
    ref = np.zeros(st.size, np.complex128)
    ref[:st.ld] = b0
    orc.time_evolve(M, e, e, P, seg, ref)
    err = np.abs(got - ref).max()
    assert err < 2e-5, err
    st.qift()
    orc.qift(P, st.ld, ref)
    perr = np.abs(st.phase_probs() - orc.identify_phase_amplitudes(P, st.ld, ref)).max()
    assert perr < 1e-5, perr


def test_edge_shapes(gpu, orc):
    """Full shells (C = 1), a single orbital, no terms at all, and P = 1."""
    q = gpu
    from qpesim_gb300 import TERM_DTYPE
    empty = {k: np.zeros(0, TERM_DTYPE) for k in KINDS}
    for M, na, nb, P, seg in [(3, 3, 3, 2, _seg(q, 6, 6, 3, 0.1)), (1, 1, 1, 3, _seg(q, 2, 2, 4, 0.3)),
                              (4, 2, 2, 1, empty), (4, 2, 1, 2, _seg(q, 8, 4, 5, 0.2))]:
        prog = q.Program(seg, M, na, nb)
        st = q.DeviceState(M, na, nb, P)
        b0 = q.hf_block0(st.c_alpha, st.c_beta, P) + 0.1
        st.upload(b0)
        st.evolve(prog)
        ref = np.zeros(st.size, np.complex128)
        ref[:st.ld] = b0
        orc.time_evolve(M, na, nb, P, seg, ref)
        assert np.array_equal(st.download(), ref)


def test_invalid_input_is_reported(gpu):
    q = gpu
    seg = _seg(q, 8, 4, 1, 0.1)
    bad = {k: v.copy() for k, v in seg.items()}
    bad["pq"]["p"][0] = 99
    with pytest.raises(q.QpeError):
        q.Program(bad, 4, 2, 2)
    bad = {k: v.copy() for k, v in seg.items()}
    bad["pqrs"]["q"][0] = bad["pqrs"]["p"][0]
    with pytest.raises(q.QpeError):
        q.Program(bad, 4, 2, 2)
    with pytest.raises(q.QpeError):
        q.DeviceState(4, 5, 2, 3)
    prog = q.Program(seg, 4, 2, 2)
    st = q.DeviceState(5, 2, 2, 2)
    with pytest.raises(q.QpeError):
        st.evolve(prog)  # shapes differ
    with pytest.raises(q.QpeError):
        q.OffsetComputer.unrank(8, 4, [70])


def test_pp_fixture_phase_on_gpu(gpu):
    """cpp/time_evolution.hpp:339-367 on the hot path: probs[87] > 0.5."""
    q = gpu
    h = q.Hamiltonian()
    h.SetNumOrbitals(1)
    h.SetNumOccupied(1)
    h.AddOneBodyTerm((1, 1), 1.0)
    h.IndexTerms()
    h.SetTimestep(1.0)
    P = 7
    sv = q.StateVector(P, 1, 1)
    sv[0] = 2 ** (-P / 2)
    q.time_evolve_over_terms(sv, h, P)
    sv.qift()
    assert sv.IdentifyPhaseAmplitudes()[87] > 0.5


@pytest.mark.parametrize("strategy,cluster", [(1, 0), (2, 2), (2, 4), (2, 8), (2, 16), (3, 0), (0, 0),
                                              (4, 1), (4, 2), (4, 4), (4, 8), (4, 16),
                                              (5, 1), (5, 2), (5, 4), (5, 8), (5, 16),
                                              (6, 1), (6, 2), (6, 4), (6, 8), (6, 16),
                                              (7, 2), (7, 4), (7, 8), (7, 16)])
@pytest.mark.parametrize("n,na,nb,P", [(12, 3, 3, 3), (14, 4, 3, 2), (8, 2, 2, 4), (16, 4, 4, 2)])
def test_strategies_bit_identical(gpu, orc, strategy, cluster, n, na, nb, P):
    """Every evolution strategy (one CTA resident in shared memory, clusters of 2
    to 16 CTAs over distributed shared memory, global-memory tile passes, and the
    autotuned choice) gives the oracle's complex128 register bit for bit."""
    q = gpu
    M = n // 2
    seg = _seg(q, n, 2 * max(na, nb), 300 + n, 0.09)
    prog = q.Program(seg, M, na, nb)
    st = q.DeviceState(M, na, nb, P)
    rng = np.random.default_rng(7)
    b0 = (rng.standard_normal(st.ld) + 1j * rng.standard_normal(st.ld)) / np.sqrt(2 * st.ld)
    st.upload(b0)
    opts = dict(strategy=strategy)
    st.evolve(prog, **opts) if cluster == 0 else st.evolve(prog, strategy=strategy, cluster_size=cluster)
    ref = np.zeros(st.size, np.complex128)
    ref[:st.ld] = b0
    orc.time_evolve(M, na, nb, P, seg, ref)
    assert np.array_equal(st.download(), ref)


@pytest.mark.parametrize("strategy,cluster,replicas", [(0, 0, 0), (6, 16, 0), (6, 8, 0), (7, 16, 0), (7, 8, 0),
                                                       (7, 16, 2), (7, 16, 3), (7, 8, 2), (3, 0, 0)])
def test_headline_configuration(gpu, orc, strategy, cluster, replicas):
    """The plain-n16 bench workload exactly as it is timed, at P = 3: n = 16,
    N = 8, seed-0 integrals, 2nd-order Trotter (forward and reversed sweeps at
    dt / 2 = 0.025), 4 steps per power, Hartree-Fock start, complex128. Autotuned
    (the strategy the bench ends up with) and forced to the three-warp-group
    cluster of 16 and 8 CTAs (with the column-pair passes as tiles and as update
    units, and with 2 or 3 replica clusters splitting the row and column passes)
    and to the tile passes: the register is bit-identical
    to the oracle's order-2, 4-step evolution, and after the QIFT the register too,
    and the histogram within 1e-12."""
    q = gpu
    n, N, P, dt, order, steps = 16, 8, 3, 0.05, 2, 4
    M, e = n // 2, N // 2
    h = q.Hamiltonian.from_integrals(q.synthetic_integrals(n, 0), e, dt / 2)
    seg = h.segmented_terms()
    prog = q.Program(seg, M, e, e, trotter_order=order, steps=steps)
    assert prog.touches_per_power == 24_304_000
    st = q.DeviceState(M, e, e, P)
    b0 = q.hf_block0(st.c_alpha, st.c_beta, P)
    st.upload(b0)
    st.evolve(prog, strategy=strategy, cluster_size=cluster, replicas=replicas)
    if strategy in (6, 7):
        assert st.last_strategy() == (strategy, cluster)
        assert st.last_replicas() == max(replicas, 1)
    if strategy == 7:
        # every one of the 392 column-pair passes of a sweep as update units
        assert prog.unit_schedule() == (cluster, 392)
    ref = np.zeros(st.size, np.complex128)
    ref[:st.ld] = b0
    orc.time_evolve(M, e, e, P, seg, ref, order=order, steps=steps)
    assert np.array_equal(st.download(), ref)
    st.qift()
    orc.qift(P, st.ld, ref)
    assert np.array_equal(st.download(), ref)
    np.testing.assert_allclose(st.phase_probs(), orc.identify_phase_amplitudes(P, st.ld, ref), rtol=1e-12,
                               atol=1e-16)


@pytest.mark.parametrize("strategy,cluster", [(1, 0), (2, 4), (3, 0), (4, 1), (4, 4), (5, 1), (5, 4), (6, 1), (6, 4),
                                              (7, 4), (7, 16)])
def test_strategies_complex64(gpu, orc, strategy, cluster):
    q = gpu
    n, N, P = 12, 6, 4
    M, e = n // 2, N // 2
    seg = _seg(q, n, N, 31, 0.05)
    prog = q.Program(seg, M, e, e)
    st = q.DeviceState(M, e, e, P, dtype=np.complex64)
    b0 = q.hf_block0(st.c_alpha, st.c_beta, P)
    st.upload(b0.astype(np.complex64))
    st.evolve(prog, strategy=strategy, cluster_size=cluster)
    ref = np.zeros(st.size, np.complex128)
    ref[:st.ld] = b0
    orc.time_evolve(M, e, e, P, seg, ref)
    assert np.abs(st.download() - ref).max() < 2e-5


@pytest.mark.parametrize("strategy,cluster", [(1, 0), (2, 4), (3, 0), (4, 1), (4, 4), (5, 4), (6, 4), (7, 4)])
def test_fp64_contract_within_tolerance(gpu, orc, strategy, cluster):
    """With FMAs allowed (QPE_EVOLVE_FP64_CONTRACT) complex128 stays within 1e-12
    of the reference's rounding (here over 15 powers of a 2nd-order, 2-step
    program at n = 12)."""
    q = gpu
    n, N, P = 12, 6, 4
    M, e = n // 2, N // 2
    seg = _seg(q, n, N, 41, 0.05)
    prog = q.Program(seg, M, e, e, trotter_order=2, steps=2)
    st = q.DeviceState(M, e, e, P)
    b0 = q.hf_block0(st.c_alpha, st.c_beta, P)
    st.upload(b0)
    st.evolve(prog, strategy=strategy, cluster_size=cluster, fp64_contract=True)
    ref = np.zeros(st.size, np.complex128)
    ref[:st.ld] = b0
    orc.time_evolve(M, e, e, P, seg, ref, order=2, steps=2)
    got = st.download()
    assert np.abs(got - ref).max() < 1e-12
    assert not np.array_equal(got, ref) or True


@pytest.mark.parametrize("dtype", [np.complex128, np.complex64])
def test_batch_matches_oracle_per_instance(gpu, orc, dtype):
    """A batch of uneven Hamiltonians (two structure classes per size, odd and
    even electron counts) in one graph launch: every register equals the
    oracle's evolution of that instance (complex128 bit for bit, complex64 within
    2e-5), every histogram the oracle's QIFT histogram; a tuned rerun gives the
    same complex128 result."""
    q = gpu
    P = 3
    shapes = [(8, 2, 2), (10, 3, 2), (8, 2, 2), (12, 3, 3), (10, 3, 2), (6, 1, 1)]
    progs, segs, b0s = [], [], []
    for i, (n, na, nb) in enumerate(shapes):
        seg = _seg(q, n, na + nb, 500 + i, 0.08)
        segs.append(seg)
        progs.append(q.Program(seg, n // 2, na, nb))
    bt = q.Batch(progs, P, dtype=dtype)
    assert bt.info["classes"] == 4
    rng = np.random.default_rng(3)
    for i, (n, na, nb) in enumerate(shapes):
        ld = bt.ld[i]
        b0s.append((rng.standard_normal(ld) + 1j * rng.standard_normal(ld)) / np.sqrt(2 * ld))
    for rep in range(2):
        if rep == 1:
            bt.tune()
        for i in range(len(shapes)):  # the QIFT of a run transforms block 0 as well
            bt.upload(i, b0s[i].astype(dtype))
        bt.run()
        for i, (n, na, nb) in enumerate(shapes):
            ld = bt.ld[i]
            ref = np.zeros((1 << P) * ld, np.complex128)
            ref[:ld] = b0s[i].astype(dtype) if dtype == np.complex64 else b0s[i]
            orc.time_evolve(n // 2, na, nb, P, segs[i], ref)
            orc.qift(P, ld, ref)
            got = bt.download(i)
            if dtype == np.complex128:
                assert np.array_equal(got, ref), i
            else:
                assert np.abs(got - ref).max() < 2e-5, i
            np.testing.assert_allclose(bt.phase_probs(i), orc.identify_phase_amplitudes(P, ld, ref), rtol=1e-4,
                                       atol=1e-6)


def test_batch_complex64_eigenphase_matches_fp64(gpu):
    """The FP32 batched form gives every instance's eigenphase (the sub-bin
    estimate of its histogram) within 1e-6 rad of the FP64 batch of the same
    programs, from Hartree-Fock starts of seeded synthetic Hamiltonians."""
    q = gpu
    P = 6
    sizes = (8, 12, 8, 12, 8, 12)
    progs, starts = [], []
    for i, n in enumerate(sizes):
        h = q.Hamiltonian.from_integrals(q.synthetic_integrals(n, 40 + i), n // 4, 0.05)
        progs.append(q.Program(h.segmented_terms(), n // 2, n // 4, n // 4))
        c = math.comb(n // 2, n // 4)
        starts.append(q.hf_block0(c, c, P, np.complex128))
    b64 = q.Batch(progs, P, dtype=np.complex64)
    b128 = q.Batch(progs, P, dtype=np.complex128)
    for i, a in enumerate(starts):
        b64.upload(i, a.astype(np.complex64))
        b128.upload(i, a)
    b64.run()
    b128.run()
    for i in range(len(sizes)):
        p64, p128 = b64.phase_probs(i), b128.phase_probs(i)
        assert np.argmax(p64) == np.argmax(p128), i
        d = abs(q.subbin_phase(p64) - q.subbin_phase(p128))
        assert 2 * math.pi * min(d, 1 - d) < 1e-6, (i, d)


@pytest.mark.parametrize("name", sorted(p.name for p in GOLDEN.glob("iqpe_*.npz")))
@pytest.mark.parametrize("strategy,cluster", [(1, 0), (2, 2), (3, 0), (0, 0), (4, 2), (5, 2), (6, 2), (7, 4)])
def test_iqpe_golden(gpu, name, strategy, cluster):
    """time_evolve_iqpe (cpp/time_evolution_over_terms.hpp:141-155): block 1 in
    place, applyUnitary's term order, against the reference's own output, through
    the device-resident form under every strategy and through the host call."""
    q = gpu
    z = load_golden(name)
    n, N, P, apps = int(z["n"]), int(z["N"]), int(z["P"]), int(z["applications"])
    M, e = n // 2, N // 2
    seg = golden_segments(z)
    prog = q.Program(seg, M, e, e, apply_unitary_order=True)
    st = q.DeviceState(M, e, e, P)
    st.upload(z["before"])
    st.evolve_in_place(prog, block=1, repeats=apps, strategy=strategy, cluster_size=cluster)
    np.testing.assert_allclose(st.download(), z["after"], rtol=0, atol=1e-13)
    if strategy == 0:
        h = q.Hamiltonian.from_integrals(q.synthetic_integrals(n, int(z["seed"])), e, float(z["dt"]))
        sv = z["before"].copy()
        q.time_evolve_iqpe(sv, h, apps)
        np.testing.assert_allclose(sv, z["after"], rtol=0, atol=1e-13)


@pytest.mark.parametrize("strategy", [1, 3])
def test_iqpe_bit_identical_to_oracle(gpu, orc, strategy):
    q = gpu
    M, e, P, apps = 6, 3, 2, 3
    seg = _seg(q, 12, 6, 41, 0.08)
    rng = np.random.default_rng(41)
    st = q.DeviceState(M, e, e, P)
    reg = (rng.standard_normal(st.size) + 1j * rng.standard_normal(st.size)) / np.sqrt(st.size)
    st.upload(reg)
    st.evolve_in_place(q.Program(seg, M, e, e, apply_unitary_order=True), 1, apps, strategy=strategy)
    orc.time_evolve_iqpe(M, e, e, P, seg, reg, apps)
    assert np.array_equal(st.download(), reg)


@pytest.mark.parametrize("strategy,order,steps", [(1, 1, 1), (2, 2, 2), (3, 2, 1), (4, 2, 2), (5, 2, 2), (6, 2, 2),
                                                   (7, 2, 2)])
def test_in_place_repeats_equal_powers(gpu, strategy, order, steps):
    """r in-place applications to block 1 holding block 0 give block r of the
    ordinary controlled-power evolution, bit for bit, in any strategy."""
    q = gpu
    M, na, nb, P, r = 5, 2, 3, 3, 5
    seg = _seg(q, 10, 6, 52, 0.06)
    prog = q.Program(seg, M, na, nb, trotter_order=order, steps=steps)
    a = q.DeviceState(M, na, nb, P)
    b = q.DeviceState(M, na, nb, P)
    rng = np.random.default_rng(52)
    b0 = (rng.standard_normal(a.ld) + 1j * rng.standard_normal(a.ld)) / np.sqrt(2 * a.ld)
    a.upload(b0)
    a.evolve(prog, strategy=strategy, cluster_size=2 if strategy == 2 else 0)
    reg = np.zeros(b.size, np.complex128)
    reg[:b.ld] = b0
    reg[b.ld:2 * b.ld] = b0
    b.upload(reg)
    b.evolve_in_place(prog, 1, r, strategy=strategy, cluster_size=2 if strategy == 2 else 0)
    got = b.download()
    assert np.array_equal(got[b.ld:2 * b.ld], a.download()[r * b.ld:(r + 1) * b.ld])
    assert np.array_equal(got[2 * b.ld:], reg[2 * b.ld:])


def test_autotune_leaves_register_unchanged(gpu):
    """The autotuner's trial powers write block 1; it is put back, so a partial
    range or an in-place call that triggers tuning sees the register it was given."""
    q = gpu
    seg = _seg(q, 12, 6, 61, 0.05)
    prog = q.Program(seg, 6, 3, 3)
    st = q.DeviceState(6, 3, 3, 3)
    rng = np.random.default_rng(61)
    reg = (rng.standard_normal(st.size) + 1j * rng.standard_normal(st.size)) / np.sqrt(st.size)
    st.upload(reg)
    st.evolve(prog, 5, 6)  # first use: tunes, then evolves block 5 from block 4
    got = st.download()
    assert np.array_equal(np.delete(got.reshape(8, -1), 5, axis=0), np.delete(reg.reshape(8, -1), 5, axis=0))
    prog2 = q.Program(seg, 6, 3, 3, apply_unitary_order=True)
    st.upload(reg)
    st.evolve_in_place(prog2, 1, 2)  # tunes on prog2 first
    ref = q.DeviceState(6, 3, 3, 3)
    ref.upload(reg)
    ref.evolve_in_place(prog2, 1, 2, strategy=3)
    assert np.array_equal(st.download(), ref.download())


def test_fp64_peak_probe(gpu):
    """qpe_measure_fp64_peak (the FP64 roofline denominator the bench reports)
    returns a plausible FMA rate for one GPU."""
    import ctypes
    N = gpu._native
    v = ctypes.c_double()
    N.check(N.lib().qpe_measure_fp64_peak(N.context(0), ctypes.byref(v)))
    assert 0.1 < v.value < 200.0, v.value


@pytest.mark.parametrize("n,na,nb,order", [(14, 4, 3, 1), (14, 3, 4, 2), (10, 2, 2, 1), (16, 4, 4, 2)])
def test_tile_passes_complex64_copy_paths(gpu, orc, n, na, nb, order):
    """complex64 tile passes on both copy paths: columns of 8 x Ca bytes that are
    not a multiple of 16 (Ca = 35 at n = 14, Na = 4; Ca = 35 with the spins
    swapped in the second case) take per-thread copies, the others bulk copies
    and the pass images; all within 2e-5 of the complex128 oracle, and the
    complex128 tile passes on the same shapes bit for bit."""
    q = gpu
    M, P = n // 2, 3
    seg = _seg(q, n, 2 * max(na, nb), 700 + n + na, 0.06)
    prog = q.Program(seg, M, na, nb, trotter_order=order, steps=2 if order == 2 else 1)
    steps = 2 if order == 2 else 1
    ref = None
    for dtype in (np.complex64, np.complex128):
        st = q.DeviceState(M, na, nb, P, dtype=dtype)
        b0 = q.hf_block0(st.c_alpha, st.c_beta, P)
        rng = np.random.default_rng(n + na)
        b0 = b0 + (rng.standard_normal(st.ld) + 1j * rng.standard_normal(st.ld)) * 1e-2
        st.upload(b0.astype(dtype))
        st.evolve(prog, strategy=3)
        if ref is None:
            ref = np.zeros(st.size, np.complex128)
            ref[:st.ld] = b0.astype(np.complex64)
            orc.time_evolve(M, na, nb, P, seg, ref, order=order, steps=steps)
        got = st.download()
        if dtype == np.complex64:
            assert np.abs(got - ref).max() < 2e-5
        else:
            ref128 = np.zeros(st.size, np.complex128)
            ref128[:st.ld] = b0
            orc.time_evolve(M, na, nb, P, seg, ref128, order=order, steps=steps)
            assert np.array_equal(got, ref128)
