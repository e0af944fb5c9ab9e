"""Bounded device waits: a wait that runs past its limit returns an error status that
the host reads, and the context stays usable.

* the replica-group barrier of the batched Monte Carlo kernel: with its poll limit set
  to 1, every CTA of a group of two or more gives up at the group's first barrier, on
  arrival, and the run returns UPPASD_GPU_ESTATE; with the default limit the next run
  works;
* the tensor-core pipeline's mbarrier wait: a self-test CTA waits on an mbarrier that
  nothing arrives at (no copy or MMA in flight) and reports code 4; a GEMM
  afterwards is correct.
"""
import ctypes as C

import numpy as np
import pytest

from uppasd_gb300 import _lib
from uppasd_gb300.batch import ReplicaBatch

pytestmark = pytest.mark.gpu


def test_replica_barrier_limit_returns_error_and_recovers():
    b = ReplicaBatch([16, 16], [900.0, 1100.0], seed=3, max_sweeps_per_launch=8)
    b.set_schedule(128, [4, 4])          # four CTAs per replica: every colour ends in a group barrier
    b.run(4, sweeps_per_launch=4)
    b.set_spin_limit(1)
    with pytest.raises(_lib.UppasdGpuError) as ei:
        b.run(16, sweeps_per_launch=8)
    assert ei.value.rc == -4 and "barrier" in str(ei.value), str(ei.value)
    b.set_spin_limit(0)
    b.run(16, sweeps_per_launch=8)       # default limit: no error
    for s in b.get_spins():
        assert np.all(np.isfinite(s)) and np.abs(np.linalg.norm(s, axis=1) - 1).max() < 1e-5
    b.close()


def test_tensor_core_wait_limit_returns_error_and_recovers():
    with pytest.raises(_lib.UppasdGpuError) as ei:
        _lib.call("uppasd_gpu_tc_wait_selftest")
    assert ei.value.rc == -4 and "code 4" in str(ei.value), str(ei.value)
    from uppasd_gb300.bf16 import from_bf16_bits, to_bf16_bits

    rng = np.random.default_rng(2)
    A = rng.normal(size=(128, 64)).astype(np.float32)
    B = rng.normal(size=(64, 64)).astype(np.float32)
    a, bb = to_bf16_bits(A), to_bf16_bits(B)
    Cf = np.zeros((128, 64), dtype=np.float32)
    _lib.call("uppasd_gpu_tc_gemm", 128, 64, 64, a.ctypes.data_as(C.c_void_p), bb.ctypes.data_as(C.c_void_p), None,
              None, 0, 64, Cf.ctypes.data_as(C.c_void_p), None)
    ref = from_bf16_bits(a).astype(np.float64) @ from_bf16_bits(bb).astype(np.float64).T
    assert np.max(np.abs(Cf - ref)) <= 1e-3
