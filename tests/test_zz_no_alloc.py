"""qpe_qift_device_noalloc, the QIFT entry point that allocates nothing.

It is meant for callers that cannot allocate device memory when they need the
QIFT (a stream under CUDA-graph capture, a host that owns all device memory
through its own pool). This test gives it device buffers the test owns (torch is
only the allocator here) and checks, on two calls in a row that share the
library's fixed scratch array, that it matches the allocating entry point
qpe_qift (host buffers) to 1e-12, and its histogram IdentifyPhaseAmplitudes. It
lives in a file of its own, collected last.
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


def test_noalloc_qift_matches_allocating_entry_point(gpu):
    q = gpu
    torch = pytest.importorskip("torch")
    fn = _noalloc(q)
    rng = np.random.default_rng(11)
    # two calls in a row with different shapes, both through the shared scratch
    for P, ld in ((10, 300), (6, 37)):
        x = (rng.standard_normal((1 << P) * ld) + 1j * rng.standard_normal((1 << P) * ld)) / np.sqrt(ld << P)
        want = x.copy()
        sv_probs = np.zeros(1 << P)
        q._native.check(q._native.lib().qpe_qift(q._native.context(0), P, ld,
                                                 want.view(np.float64).ctypes.data_as(C.POINTER(C.c_double))))
        q._native.check(q._native.lib().qpe_identify_phase_amplitudes(
            q._native.context(0), P, ld, want.view(np.float64).ctypes.data_as(C.POINTER(C.c_double)),
            sv_probs.ctypes.data_as(C.POINTER(C.c_double))))
        d_state = torch.from_numpy(x.view(np.float64).copy()).cuda()
        d_probs = torch.zeros(1 << P, dtype=torch.float64, device="cuda")
        stream = torch.cuda.current_stream().cuda_stream
        rc = fn(stream, P, ld, 0, d_state.data_ptr(), d_probs.data_ptr())
        q._native.check(rc)
        torch.cuda.synchronize()
        got = d_state.cpu().numpy().view(np.complex128)
        np.testing.assert_allclose(got, want, rtol=0, atol=1e-12)
        np.testing.assert_allclose(d_probs.cpu().numpy(), sv_probs, rtol=1e-12, atol=1e-15)


def test_noalloc_rejects_oversize(gpu):
    q = gpu
    torch = pytest.importorskip("torch")
    fn = _noalloc(q)
    buf = torch.zeros(16, dtype=torch.float64, device="cuda")
    rc = fn(None, 11, 1, 0, buf.data_ptr(), buf.data_ptr())
    assert rc == 2 and b"precision" in q._native.lib().qpe_last_error()
