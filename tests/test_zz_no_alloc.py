"""Allocation-free magnetisation sums (uppasd_gpu_moment_sums_noalloc).

Some callers cannot allocate device memory (a host code with its own device
pool, code running during another stream's graph capture, an embedding runtime
that reserves the device at start-up).  This entry point takes caller-owned
device input and output and uses only a fixed scratch array inside the library.
Its result must match the regular observables entry point, on two calls in a
row (the second call reuses the scratch the first one left behind).

This file is collected last on purpose, so a run that stops at the first
failure has already run every other test.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_noalloc_sums_match_observables_twice():
    import torch

    from uppasd_gb300 import _lib, lattice
    from uppasd_gb300.simulation import GpuSimulation

    lat = lattice.bcc(6, [1.3, 0.7], 2.2).with_ensembles(5)
    rng = np.random.default_rng(31)
    e0 = rng.normal(size=(5, lat.natom, 3))
    e0 /= np.linalg.norm(e0, axis=-1, keepdims=True)
    sim = GpuSimulation(lat, sdealgh=5, delta_t=1e-16, damping=0.1, temperature=300.0, emom=e0)
    sim.evolve(20)
    ref = sim.observables()
    _, emomM = sim.get_moments(full=True)
    sim.close()

    d_in = torch.from_numpy(np.ascontiguousarray(emomM)).to("cuda")
    stream = torch.cuda.Stream()
    for call in range(2):
        d_out = torch.full((5, 4), float("nan"), dtype=torch.float64, device="cuda")
        torch.cuda.synchronize()
        _lib.call("uppasd_gpu_moment_sums_noalloc", C.c_void_p(d_in.data_ptr()), lat.natom, 5,
                  C.c_void_p(d_out.data_ptr()), C.c_void_p(stream.cuda_stream))
        stream.synchronize()
        out = d_out.cpu().numpy()
        assert np.allclose(out[:, :3], ref["mvec"], rtol=1e-12, atol=1e-10), (call, out[:, :3], ref["mvec"])
        assert np.allclose(out[:, 3], ref["mabs"], rtol=1e-12, atol=1e-14), (call, out[:, 3], ref["mabs"])
        # and against a direct sum of the moments it was given
        tot = emomM.sum(axis=1)
        assert np.allclose(out[:, :3], tot, rtol=1e-12, atol=1e-10), (call, out[:, :3], tot)
        assert np.allclose(out[:, 3], np.linalg.norm(tot, axis=-1) / lat.natom, rtol=1e-12, atol=1e-14)


def test_noalloc_rejects_too_many_ensembles():
    import torch

    from uppasd_gb300 import _lib

    d_in = torch.zeros((65, 4, 3), dtype=torch.float64, device="cuda")
    d_out = torch.zeros((65, 4), dtype=torch.float64, device="cuda")
    with pytest.raises(_lib.UppasdGpuError) as ei:
        _lib.call("uppasd_gpu_moment_sums_noalloc", C.c_void_p(d_in.data_ptr()), 4, 65,
                  C.c_void_p(d_out.data_ptr()), None)
    assert ei.value.rc == -1
    assert "65" in str(ei.value)
