"""tcgen05 BF16 GEMM (TMA operands, TMEM accumulator) against a float64 product
of the same bf16-rounded operands: a single 128 x 64 x 64 tile (one MMA chain),
multi-tile shapes, a K loop longer than the stage ring, every tile width and
every fused epilogue."""
import ctypes as C

import numpy as np
import pytest

from uppasd_gb300 import _lib
from uppasd_gb300.bf16 import from_bf16_bits, to_bf16_bits

pytestmark = pytest.mark.gpu


def run(A, B, epi, bn, bias=None, Y=None):
    M, K = A.shape
    N = B.shape[0]
    a, b = to_bf16_bits(A), to_bf16_bits(B)
    y = None if Y is None else to_bf16_bits(Y)
    f32 = epi in (0, 1)
    Cf = np.zeros((M, N), dtype=np.float32) if f32 else None
    Cb = None if f32 else np.zeros((M, N), dtype=np.uint16)
    bb = None if bias is None else np.ascontiguousarray(bias, dtype=np.float32)
    ptr = lambda x: None if x is None else x.ctypes.data_as(C.c_void_p)
    _lib.call("uppasd_gpu_tc_gemm", M, N, K, ptr(a), ptr(b), ptr(bb), ptr(y), epi, bn, ptr(Cf), ptr(Cb))
    return Cf if f32 else from_bf16_bits(Cb)


def ref(A, B):
    a = from_bf16_bits(to_bf16_bits(A)).astype(np.float64)
    b = from_bf16_bits(to_bf16_bits(B)).astype(np.float64)
    return a @ b.T, np.abs(a) @ np.abs(b).T


@pytest.mark.parametrize("M,N,K,bn", [(128, 64, 64, 64), (256, 256, 192, 256), (384, 128, 512, 128),
                                      (128, 256, 256, 64), (512, 64, 1024, 64)])
def test_product(M, N, K, bn):
    rng = np.random.default_rng(M + N + K)
    A = rng.normal(size=(M, K)).astype(np.float32)
    B = rng.normal(size=(N, K)).astype(np.float32)
    C = run(A, B, 0, bn)
    R, S = ref(A, B)
    assert np.max(np.abs(C - R) / S) < 1e-5


def test_epilogues():
    rng = np.random.default_rng(3)
    M, N, K = 256, 128, 128
    A = rng.normal(size=(M, K)).astype(np.float32) * 0.2
    B = rng.normal(size=(N, K)).astype(np.float32) * 0.2
    bias = rng.normal(size=N).astype(np.float32) * 0.1
    R, S = ref(A, B)
    C1 = run(A, B, 1, 128, bias=bias)
    assert np.max(np.abs(C1 - (R + bias)) / (S + 1e-3)) < 1e-5
    C2 = run(A, B, 2, 64, bias=bias)
    assert np.max(np.abs(C2 - np.tanh(R + bias))) < 1e-2  # bf16 output and tanh.approx
    Y = np.tanh(rng.normal(size=(M, N))).astype(np.float32)
    Yb = from_bf16_bits(to_bf16_bits(Y)).astype(np.float64)
    C3 = run(A, B, 3, 128, Y=Y)
    want = R * (1 - Yb * Yb)
    assert np.max(np.abs(C3 - want) / (np.abs(want) + 1e-2)) < 1e-2


def test_rejects_bad_shapes():
    A = np.zeros((100, 64), dtype=np.float32)
    B = np.zeros((64, 64), dtype=np.float32)
    with pytest.raises(_lib.UppasdGpuError):
        run(A, B, 0, 64)
