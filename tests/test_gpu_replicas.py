"""Replica clusters of the lean resident kernel (strategy 7 with replicas > 1):
2 to 8 thread-block clusters each hold the whole block, split every row and
column pass between them and exchange their results through global memory
(bounded waits, cooperative launch); column-pair passes run on every replica.
The register must be the oracle's bit for bit, as with one cluster."""
import numpy as np
import pytest

from test_gpu_parity import _seg

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("n,na,nb,P,cluster,replicas,order,steps", [
    (16, 4, 4, 2, 16, 2, 1, 1), (16, 4, 4, 2, 16, 4, 2, 2), (16, 4, 4, 2, 8, 3, 2, 1),
    (12, 3, 3, 3, 4, 2, 1, 1), (12, 3, 3, 3, 16, 3, 2, 2), (14, 4, 3, 2, 8, 2, 2, 1), (8, 2, 2, 3, 2, 2, 1, 1)])
def test_replicas_bit_identical(gpu, orc, n, na, nb, P, cluster, replicas, order, steps):
    q = gpu
    M = n // 2
    seg = _seg(q, n, 2 * max(na, nb), 500 + n, 0.07)
    prog = q.Program(seg, M, na, nb, trotter_order=order, steps=steps)
    st = q.DeviceState(M, na, nb, P)
    rng = np.random.default_rng(n + replicas)
    b0 = (rng.standard_normal(st.ld) + 1j * rng.standard_normal(st.ld)) / np.sqrt(2 * st.ld)
    st.upload(b0)
    st.evolve(prog, strategy=7, cluster_size=cluster, replicas=replicas)
    assert st.last_strategy() == (7, cluster) and st.last_replicas() == replicas
    ref = np.zeros(st.size, np.complex128)
    ref[:st.ld] = b0
    orc.time_evolve(M, na, nb, P, seg, ref, order=order, steps=steps)
    assert np.array_equal(st.download(), ref)


def test_replicas_in_place_and_complex64(gpu, orc):
    """In place (the iterative-QPE evolution) and in complex64, with 2 replicas."""
    q = gpu
    M, e, P, apps = 8, 4, 2, 3
    seg = _seg(q, 16, 8, 77, 0.05)
    st = q.DeviceState(M, e, e, P)
    rng = np.random.default_rng(77)
    reg = (rng.standard_normal(st.size) + 1j * rng.standard_normal(st.size)) / np.sqrt(st.size)
    st.upload(reg)
    st.evolve_in_place(q.Program(seg, M, e, e, apply_unitary_order=True), 1, apps, strategy=7, cluster_size=16,
                       replicas=2)
    orc.time_evolve_iqpe(M, e, e, P, seg, reg, apps)
    assert np.array_equal(st.download(), reg)
    prog = q.Program(seg, M, e, e)
    s64 = q.DeviceState(M, e, e, 3, dtype=np.complex64)
    b0 = q.hf_block0(s64.c_alpha, s64.c_beta, 3)
    s64.upload(b0.astype(np.complex64))
    s64.evolve(prog, strategy=7, cluster_size=16, replicas=2)
    one = q.DeviceState(M, e, e, 3, dtype=np.complex64)
    one.upload(b0.astype(np.complex64))
    one.evolve(prog, strategy=7, cluster_size=16)
    assert np.array_equal(s64.download(), one.download())


def test_replicas_rejected_outside_strategy_7(gpu):
    q = gpu
    seg = _seg(q, 8, 4, 3, 0.05)
    prog = q.Program(seg, 4, 2, 2)
    st = q.DeviceState(4, 2, 2, 2)
    with pytest.raises(q.QpeError):
        st.evolve(prog, strategy=6, cluster_size=2, replicas=2)
    with pytest.raises(q.QpeError):
        st.evolve(prog, strategy=7, cluster_size=2, replicas=9)
