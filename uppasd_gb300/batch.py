"""Batched replica Monte Carlo: many bcc J1/J2 replicas (temperatures x sizes)
in one persistent launch, through the C ABI ``uppasd_gpu_mcbatch_*``.

This is the replica table that the reference's temperature loops run one
system at a time (mc_mphase, MonteCarlo/mc_driver.f90:234-420, and the replica
list of MonteCarlo/pt_driver.f90:58-367).  Observables per sweep: E (mRy/atom,
Hamiltonian/energy.f90:60-405) and M (muB/atom, Measurement/measurements.f90:211-235);
derived cumulants use the reference's formulas (``analysis.cumulants``).
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import _lib
from .analysis import cumulants, tau_int

DEFAULT_CACHE = os.path.join(os.path.dirname(os.path.abspath(__file__)), ".tune_cache")


def _i32(a):
    return np.ascontiguousarray(a, dtype=np.int32)


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


class ReplicaBatch:
    def __init__(self, L, temperature, heatbath=True, j_shells_mry=(1.3, 0.7), mom: float = 2.2, bfield=None,
                 seed: int = 1, series_len: int = 0, max_sweeps_per_launch: int = 256, first_id: int = 0):
        """first_id: the id of this batch's first replica in a larger table that is split
        over processes (``replicas.partition``); its chains are then those of the whole
        table's replicas first_id, first_id + 1, ..."""
        self.lib = _lib.load()
        self.L = _i32(L)
        self.T = _f64(temperature)
        if self.L.shape != self.T.shape or self.L.ndim != 1:
            raise ValueError("L and temperature must be 1-D of equal length")
        self.nrep = int(self.L.size)
        hb = np.broadcast_to(np.asarray(heatbath, dtype=np.int32), (self.nrep,))
        self.heatbath = _i32(hb)
        self.natoms = 2 * self.L.astype(np.int64) ** 3
        self.mom = float(mom)
        self.series_len = int(series_len)
        self.max_spl = int(max_sweeps_per_launch)
        js = _f64(j_shells_mry)
        bf = None if bfield is None else _f64(bfield)
        h = C.c_void_p()
        _lib.call("uppasd_gpu_mcbatch_create", self.nrep, self._p(self.L, _lib.I32P), self._p(self.T),
                  self._p(self.heatbath, _lib.I32P), self._p(js), self.mom,
                  None if bf is None else self._p(bf), seed, self.series_len, self.max_spl, C.byref(h))
        self.h = h
        self._keep = (js, bf)
        self.first_id = int(first_id)
        if self.first_id:
            _lib.call("uppasd_gpu_mcbatch_set_replica_ids", self.h, self.first_id)

    @staticmethod
    def _p(a, t=_lib.F64P):
        return a.ctypes.data_as(t)

    # ---- schedule ----
    def schedule(self):
        """(register build, threads per CTA, CTAs per replica)."""
        bld, t = C.c_int32(), C.c_int32()
        c = np.zeros(self.nrep, dtype=np.int32)
        _lib.call("uppasd_gpu_mcbatch_get_schedule", self.h, C.byref(bld), C.byref(t), self._p(c, _lib.I32P))
        return int(bld.value), int(t.value), c

    def set_schedule(self, threads: int, ctas_per_rep, reg_build: int = 0):
        c = _i32(ctas_per_rep)
        _lib.call("uppasd_gpu_mcbatch_set_schedule", self.h, int(reg_build), int(threads), self._p(c, _lib.I32P))

    def autotune(self, sweeps_per_trial: int = 20, cache: str | None = DEFAULT_CACHE) -> float:
        ms = C.c_float()
        _lib.call("uppasd_gpu_mcbatch_autotune", self.h, int(sweeps_per_trial),
                  None if cache is None else cache.encode(), C.byref(ms))
        return float(ms.value)

    def set_stream(self, stream_ptr: int | None):
        _lib.call("uppasd_gpu_mcbatch_set_stream", self.h, C.c_void_p(stream_ptr or 0))

    # ---- sweeps ----
    def run(self, nsweeps: int, sweeps_per_launch: int = 100, measure: bool = False):
        spl = min(int(sweeps_per_launch), self.max_spl)
        _lib.call("uppasd_gpu_mcbatch_run", self.h, int(nsweeps), spl, 1 if measure else 0)

    def enqueue(self, nsweeps: int, sweeps_per_launch: int = 100, measure: bool = False):
        spl = min(int(sweeps_per_launch), self.max_spl)
        _lib.call("uppasd_gpu_mcbatch_enqueue", self.h, int(nsweeps), spl, 1 if measure else 0)

    def check(self):
        _lib.call("uppasd_gpu_mcbatch_check", self.h)

    def set_sweep(self, sweep: int):
        _lib.call("uppasd_gpu_mcbatch_set_sweep", self.h, int(sweep))

    def set_spin_limit(self, limit: int = 0):
        """Poll limit of the replica-group barrier's wait (0: the default); 1 makes every
        CTA of a multi-CTA group give up at the group's first barrier (the error path)."""
        _lib.call("uppasd_gpu_mcbatch_set_spin_limit", self.h, int(limit))

    # ---- replica exchange ----
    def set_exchange(self, enable: bool = True):
        """Swap temperatures between ladder neighbours (same L) after every launch."""
        _lib.call("uppasd_gpu_mcbatch_set_exchange", self.h, 1 if enable else 0)

    def exchange_state(self):
        """(slot_of_replica, pairs (n, 2) of slots, attempts, accepts)."""
        n = C.c_int32()
        _lib.call("uppasd_gpu_mcbatch_exchange_state", self.h, None, C.byref(n), None, None, None)
        slot = np.zeros(self.nrep, dtype=np.int32)
        pairs = np.zeros((max(n.value, 1), 2), dtype=np.int32)
        att = np.zeros(max(n.value, 1), dtype=np.int64)
        acc = np.zeros(max(n.value, 1), dtype=np.int64)
        _lib.call("uppasd_gpu_mcbatch_exchange_state", self.h, self._p(slot, _lib.I32P), C.byref(n),
                  self._p(pairs, _lib.I32P), att.ctypes.data_as(C.POINTER(C.c_int64)),
                  acc.ctypes.data_as(C.POINTER(C.c_int64)))
        k = n.value
        return slot, pairs[:k], att[:k], acc[:k]

    # ---- results ----
    def raw_stats(self):
        acc = np.zeros((self.nrep, 10))
        ns = np.zeros(self.nrep, dtype=np.int64)
        last = np.zeros((self.nrep, 4))
        _lib.call("uppasd_gpu_mcbatch_stats", self.h, self._p(acc), ns.ctypes.data_as(C.POINTER(C.c_int64)),
                  self._p(last))
        return acc, ns, last

    def stats(self):
        acc, ns, last = self.raw_stats()
        out = cumulants(acc[:, 0], acc[:, 1], acc[:, 2], acc[:, 3], acc[:, 4], acc[:, 5], self.natoms, self.T)
        out["n"] = ns
        out["last"] = last
        out["Mvec"] = acc[:, 6:9] / np.maximum(acc[:, :1], 1)
        return out

    def series(self):
        """(nrep, n, 2) measured (E, |M|) per sweep, oldest first (the last series_len sweeps)."""
        if self.series_len <= 0:
            raise ValueError("created without a series buffer")
        buf = np.zeros((self.nrep, self.series_len, 2))
        _lib.call("uppasd_gpu_mcbatch_series", self.h, self._p(buf))
        _, ns, _ = self.raw_stats()
        n = int(ns.min())
        if n <= self.series_len:
            return buf[:, :n]
        k = n % self.series_len
        return np.concatenate([buf[:, k:], buf[:, :k]], axis=1)

    def tau_int(self, c: float = 6.0):
        """Per replica: the larger of tau_int(E) and tau_int(|M|), in sweeps."""
        s = self.series()
        return np.array([max(tau_int(s[r, :, 0], c)[0], tau_int(s[r, :, 1], c)[0]) for r in range(self.nrep)])

    def reset_stats(self):
        _lib.call("uppasd_gpu_mcbatch_reset_stats", self.h)

    # ---- spins (reference layout per replica: (natom, 3) rows = Fortran (3, natom)) ----
    def get_spins(self):
        flat = np.zeros(int(3 * self.natoms.sum()))
        _lib.call("uppasd_gpu_mcbatch_get_spins", self.h, self._p(flat))
        out, o = [], 0
        for n in self.natoms:
            out.append(flat[o:o + 3 * n].reshape(n, 3))
            o += 3 * n
        return out

    def put_spins(self, spins):
        flat = _f64(np.concatenate([np.asarray(s, dtype=np.float64).reshape(-1) for s in spins]))
        if flat.size != 3 * self.natoms.sum():
            raise ValueError("spin arrays do not match the replica table")
        _lib.call("uppasd_gpu_mcbatch_put_spins", self.h, self._p(flat))

    def close(self):
        if self.h:
            _lib.call("uppasd_gpu_mcbatch_destroy", self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
