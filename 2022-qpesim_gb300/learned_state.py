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
    """Occupation string -> (log|a|, phase); n_bits inputs, 3 x 256 GELU, BF16."""

    def __init__(self, n_bits: int, batch: int = 8192, seed: int = 0, device: int = 0):
        self._lib = N.lib()
        h = C.c_void_p()
        N.check(self._lib.qpe_mlp_create(N.context(device), n_bits, batch, seed, C.byref(h)))
        self._h = h
        self.n_bits, self.batch = n_bits, batch
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

    def set_data(self, bits, log_abs, phase, weight) -> None:
        bits = np.ascontiguousarray(bits, np.uint64)
        la, ph, w = (np.ascontiguousarray(x, np.float32) for x in (log_abs, phase, weight))
        N.check(self._lib.qpe_mlp_set_data(self._h, bits.ctypes.data_as(C.POINTER(C.c_uint64)), _fp(la), _fp(ph),
                                           _fp(w), bits.size))

    def train(self, steps: int, lr: float = 1e-3, seed: int = 0) -> np.ndarray:
        losses = np.zeros(steps, np.float32)
        N.check(self._lib.qpe_mlp_train(self._h, steps, lr, seed, _fp(losses)))
        return losses

    def forward(self, bits) -> np.ndarray:
        bits = np.ascontiguousarray(bits, np.uint64)
        out = np.zeros((bits.size, 2), np.float32)
        N.check(self._lib.qpe_mlp_forward(self._h, bits.ctypes.data_as(C.POINTER(C.c_uint64)), bits.size, _fp(out)))
        return out

    def gradients(self, bits, log_abs, phase, weight):
        bits = np.ascontiguousarray(bits, np.uint64)
        la, ph, w = (np.ascontiguousarray(x, np.float32) for x in (log_abs, phase, weight))
        g = np.zeros(self.num_params, np.float32)
        loss = np.zeros(1, np.float32)
        N.check(self._lib.qpe_mlp_gradients(self._h, bits.ctypes.data_as(C.POINTER(C.c_uint64)), _fp(la), _fp(ph),
                                            _fp(w), bits.size, _fp(g), _fp(loss)))
        return g, float(loss[0])

    def tensor_flops_per_step(self) -> float:
        f = C.c_double()
        N.check(self._lib.qpe_mlp_tensor_flops_per_step(self._h, C.byref(f)))
        return f.value
