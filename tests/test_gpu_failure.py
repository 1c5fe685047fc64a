"""Failure detection on the GPU without a GPU fault.

Every tcgen05 / TMA wait of the library polls its mbarrier a bounded number of
times; a wait that runs out makes the kernel record an error and return, and the
call reports QPE_ERR_TIMEOUT (the reference only asserts,
cpp/offset_computer.hpp:39,47). qpe_selftest_bounded_wait runs that wait alone on
an mbarrier with nothing in flight: nobody arrives, so the wait runs out after a
few polls. The test checks the status, the message, and that the context keeps
working: the same wait with an arrival succeeds, and an evolution afterwards is
still bit-identical to the oracle.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_bounded_wait_runs_out_and_context_survives(gpu, orc):
    q = gpu
    N = q._native
    ctx = N.context(0)
    for tries in (1, 64, 4096):
        rc = N.lib().qpe_selftest_bounded_wait(ctx, tries, 0)
        assert rc == N.QPE_ERR_TIMEOUT, rc
        msg = N.lib().qpe_last_error().decode()
        assert "ran out" in msg and str(tries) in msg, msg
    assert N.lib().qpe_selftest_bounded_wait(ctx, 64, 1) == N.QPE_OK
    with pytest.raises(q.QpeError) as ei:
        N.check(N.lib().qpe_selftest_bounded_wait(ctx, 8, 0))
    assert ei.value.code == N.QPE_ERR_TIMEOUT
    # the next library calls on the same context and stream succeed
    h = q.Hamiltonian.from_integrals(q.synthetic_integrals(8, 5), 2, 0.1)
    seg = h.segmented_terms()
    prog = q.Program(seg, 4, 2, 2)
    st = q.DeviceState(4, 2, 2, 3)
    b0 = q.hf_block0(st.c_alpha, st.c_beta, 3)
    st.upload(b0)
    st.evolve(prog)
    ref = np.zeros(st.size, np.complex128)
    ref[:st.ld] = b0
    orc.time_evolve(4, 2, 2, 3, seg, ref)
    assert np.array_equal(st.download(), ref)


def test_bounded_wait_rejects_zero_limit(gpu):
    N = gpu._native
    assert N.lib().qpe_selftest_bounded_wait(N.context(0), 0, 0) == N.QPE_ERR_INVALID
