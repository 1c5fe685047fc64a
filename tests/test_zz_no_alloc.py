"""qpe_qift_device_noalloc, the QIFT entry point that allocates nothing.

It is meant for callers that cannot let a library allocate device memory (a
host that owns all device memory through its own pool, or a latency-bound loop
that cannot afford cudaMalloc). These tests give it device buffers the test owns
(torch is only the allocator here) and check, on two calls in a row that share
the library's fixed scratch arrays, that it matches the allocating entry points:
qpe_qift and IdentifyPhaseAmplitudes on host buffers for complex128 (1e-12), and
a device register's qpe_state_qift / qpe_state_phase_probs for complex64 (the
same kernels and twiddles; 1e-6). The file is collected last.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _noalloc(q):
    lib = q._native.lib()
    fn = lib.qpe_qift_device_noalloc
    fn.restype = C.c_int
    fn.argtypes = [C.c_void_p, C.c_uint32, C.c_uint64, C.c_int, C.c_void_p, C.c_void_p]
    return fn


def _register(rng, P, ld):
    x = rng.standard_normal((1 << P) * ld) + 1j * rng.standard_normal((1 << P) * ld)
    return x / np.linalg.norm(x)


def test_noalloc_qift_matches_allocating_entry_point(gpu):
    q = gpu
    torch = pytest.importorskip("torch")
    fn = _noalloc(q)
    N = q._native
    rng = np.random.default_rng(11)
    # two calls in a row with different shapes, both through the shared scratch
    for P, ld in ((10, 300), (6, 37)):
        x = _register(rng, P, ld)
        want = x.copy()
        sv_probs = np.zeros(1 << P)
        N.check(N.lib().qpe_qift(N.context(0), P, ld, want.view(np.float64).ctypes.data_as(C.POINTER(C.c_double))))
        N.check(N.lib().qpe_identify_phase_amplitudes(
            N.context(0), P, ld, want.view(np.float64).ctypes.data_as(C.POINTER(C.c_double)),
            sv_probs.ctypes.data_as(C.POINTER(C.c_double))))
        d_state = torch.from_numpy(x.view(np.float64).copy()).cuda()
        d_probs = torch.zeros(1 << P, dtype=torch.float64, device="cuda")
        stream = torch.cuda.current_stream().cuda_stream
        N.check(fn(stream, P, ld, 0, d_state.data_ptr(), d_probs.data_ptr()))
        torch.cuda.synchronize()
        got = d_state.cpu().numpy().view(np.complex128)
        np.testing.assert_allclose(got, want, rtol=0, atol=1e-12)
        np.testing.assert_allclose(d_probs.cpu().numpy(), sv_probs, rtol=1e-12, atol=1e-15)


def test_noalloc_qift_complex64(gpu):
    q = gpu
    torch = pytest.importorskip("torch")
    fn = _noalloc(q)
    rng = np.random.default_rng(12)
    for P, M, e in ((7, 5, 2), (9, 6, 3)):
        st = q.DeviceState(M, e, e, P, dtype=np.complex64)
        x = _register(rng, P, st.ld).astype(np.complex64)
        st.upload(x)
        st.qift()
        want, want_probs = st.download(), st.phase_probs()
        d_state = torch.from_numpy(x.view(np.float32).copy()).cuda()
        d_probs = torch.zeros(1 << P, dtype=torch.float64, device="cuda")
        q._native.check(fn(torch.cuda.current_stream().cuda_stream, P, st.ld, 1, d_state.data_ptr(),
                           d_probs.data_ptr()))
        torch.cuda.synchronize()
        got = d_state.cpu().numpy().view(np.complex64)
        np.testing.assert_allclose(got, want, rtol=0, atol=1e-6)
        np.testing.assert_allclose(d_probs.cpu().numpy(), want_probs, rtol=1e-6, atol=1e-9)


def test_noalloc_rejects_oversize(gpu):
    q = gpu
    torch = pytest.importorskip("torch")
    fn = _noalloc(q)
    buf = torch.zeros(16, dtype=torch.float64, device="cuda")
    rc = fn(None, 11, 1, 0, buf.data_ptr(), buf.data_ptr())
    assert rc == 2 and b"precision" in q._native.lib().qpe_last_error()
