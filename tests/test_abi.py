"""The C ABI library: it loads, exports every symbol include/uppasd_gpu.h
declares, and rejects malformed input with a status code before touching the
GPU (so these run on CPU-only hosts)."""
import ctypes as C
import os
import re
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def lib():
    from uppasd_gb300 import build as b
    b.build()
    from uppasd_gb300 import _lib
    return _lib.load()


def declared_functions():
    hdr = open(os.path.join(ROOT, "include", "uppasd_gpu.h")).read()
    return sorted(set(re.findall(r"\b(uppasd_gpu_[a-z_0-9]+)\s*\(", hdr)))


def test_every_declared_symbol_is_exported(lib):
    out = subprocess.run(["nm", "-D", "--defined-only", os.path.join(ROOT, "uppasd_gb300", "libuppasd_gb300.so")],
                         capture_output=True, text=True, check=True).stdout
    exported = set(l.split()[-1] for l in out.splitlines() if l.strip())
    missing = [f for f in declared_functions() if f not in exported]
    assert not missing, missing
    from uppasd_gb300 import _lib
    assert set(declared_functions()) == set(_lib.exported_symbols())


def _good_inputs():
    from uppasd_gb300 import lattice, _lib
    lat = lattice.bcc(2, [1.3, 0.7])
    N = lat.natom
    keep = []

    def k(a, dt):
        a = np.ascontiguousarray(a, dtype=dt)
        keep.append(a)
        return a.ctypes.data_as(_lib.I32P if dt == np.int32 else _lib.F64P)

    c = _lib.Consts(natom=N, mensemble=1, max_no_neigh=lat.max_no_neigh, nham=lat.nham, sdealgh=5,
                    delta_t=1e-16, bn=1.0, temprescale=1.0)
    emom = np.zeros((1, N, 3))
    emom[..., 2] = 1
    a = _lib.Arrays(nlist=k(lat.nlist, np.int32), nlistsize=k(lat.nlistsize, np.int32), ncoup=k(lat.ncoup, np.float64),
                    aham=k(lat.aham, np.int32), external_field=k(lat.extfield, np.float64),
                    mmom=k(lat.mmom, np.float64), lambda1_array=k(np.full(N, 0.1), np.float64),
                    temp_array=k(np.zeros(N), np.float64), emom=k(emom, np.float64))
    return lat, c, a, keep


@pytest.mark.parametrize("field,value", [("natom", 0), ("sdealgh", 3), ("delta_t", -1.0), ("nham", 0),
                                         ("gpu_rng", 7), ("precision", 5)])
def test_init_rejects_bad_constants(lib, field, value):
    lat, c, a, keep = _good_inputs()
    setattr(c, field, value)
    h = C.c_void_p()
    rc = lib.uppasd_gpu_init(C.byref(c), C.byref(a), C.byref(h))
    assert rc == -1
    assert h.value is None
    assert lib.uppasd_gpu_last_error()


def test_init_rejects_out_of_range_neighbour(lib):
    from uppasd_gb300 import _lib
    lat, c, a, keep = _good_inputs()
    bad = lat.nlist.copy()
    bad[0, 0] = lat.natom + 5
    bad = np.ascontiguousarray(bad, dtype=np.int32)
    a.nlist = bad.ctypes.data_as(_lib.I32P)
    h = C.c_void_p()
    assert lib.uppasd_gpu_init(C.byref(c), C.byref(a), C.byref(h)) == -1
    assert b"nlist" in lib.uppasd_gpu_last_error()


def test_init_rejects_missing_arrays(lib):
    lat, c, a, keep = _good_inputs()
    a.ncoup = None
    h = C.c_void_p()
    assert lib.uppasd_gpu_init(C.byref(c), C.byref(a), C.byref(h)) == -1
    lat, c, a, keep = _good_inputs()
    c.do_dm = 1
    c.max_no_dmneigh = 4
    assert lib.uppasd_gpu_init(C.byref(c), C.byref(a), C.byref(h)) == -1


def test_null_arguments(lib):
    assert lib.uppasd_gpu_init(None, None, None) == -1
    assert lib.uppasd_gpu_finalize(None) == -1
    assert lib.uppasd_gpu_sd_run(None, 1) == -1
    assert lib.uppasd_gpu_mc_run(None, b"H", 1.0, 1) == -1
    info = np.zeros(8, dtype=np.int64)
    assert lib.uppasd_gpu_path_info(None, info.ctypes.data_as(C.POINTER(C.c_int64))) == -1


def test_mcbatch_rejects_bad_tables(lib):
    from uppasd_gb300 import _lib
    js = np.array([1.3, 0.7])
    h = C.c_void_p()

    def create(L, T, nrep=None, spl=64, mom=2.2):
        L = np.ascontiguousarray(L, dtype=np.int32)
        T = np.ascontiguousarray(T, dtype=np.float64)
        n = len(L) if nrep is None else nrep
        return lib.uppasd_gpu_mcbatch_create(n, L.ctypes.data_as(_lib.I32P), T.ctypes.data_as(_lib.F64P), None,
                                             js.ctypes.data_as(_lib.F64P), mom, None, 1, 0, spl, C.byref(h))

    assert create([5], [500.0]) == -1          # odd L
    assert create([2], [500.0]) == -1          # too small
    assert create([8], [-1.0]) == -1           # negative temperature
    assert create([8], [500.0], nrep=0) == -1  # empty table
    assert create([8], [500.0], spl=0) == -1   # no sweeps per launch
    assert create([8], [500.0], mom=0.0) == -1
    assert h.value is None
    assert lib.uppasd_gpu_last_error()
    for fn, args in [("uppasd_gpu_mcbatch_run", (None, 1, 1, 0)), ("uppasd_gpu_mcbatch_destroy", (None,)),
                     ("uppasd_gpu_mcbatch_stats", (None, None, None, None)), ("uppasd_gpu_mcbatch_check", (None,)),
                     ("uppasd_gpu_mcbatch_get_spins", (None, None)), ("uppasd_gpu_mcbatch_set_sweep", (None, 0))]:
        assert getattr(lib, fn)(*args) == -1, fn


def test_host_block_and_dipole_reject_bad_calls(lib):
    """sd_run_io and set_dipole refuse a null simulation and bad arguments with -1
    before any device work."""
    from uppasd_gb300 import _lib
    buf = np.zeros(3, dtype=np.float64)
    p = buf.ctypes.data_as(_lib.F64P)
    assert lib.uppasd_gpu_sd_run_io(None, p, 10, p, None) == -1
    assert lib.uppasd_gpu_set_dipole(None, 1, 2.87e-10, None, 1, 1, 1, 1, p, p) == -1
    assert lib.uppasd_gpu_last_error()
