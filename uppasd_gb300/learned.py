"""Learned 4x4-patch proposal with exact Metropolis-Hastings acceptance
(C ABI ``uppasd_gpu_proposal_*``), acting on a ``GpuSimulation``'s spins
beside its heat bath (``GpuSimulation.relax("H", ...)``).

Workflow: thermalise with the heat bath, ``collect()`` windows of heat-bath
configurations, ``train()`` on them, then alternate heat-bath and learned
sweeps (``sweep()``); every learned move is accepted with
min(1, exp(-beta dE) q(old) / q(new)), so the chain samples the Boltzmann
distribution whatever the network has learned.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib

N_FEAT, N_HID, N_OUT = 192, 256, 64
W_SHAPES = [(N_HID, N_FEAT), (N_HID, N_HID), (N_HID, N_HID), (N_OUT, N_HID)]
B_SHAPES = [(N_HID,), (N_HID,), (N_HID,), (N_OUT,)]


def unpack(vec):
    """Parameter vector -> ([W1..W4], [b1..b4])."""
    ws, bs, o = [], [], 0
    for s in W_SHAPES:
        n = s[0] * s[1]
        ws.append(vec[o:o + n].reshape(s))
        o += n
    for s in B_SHAPES:
        bs.append(vec[o:o + s[0]])
        o += s[0]
    return ws, bs


def pack(ws, bs):
    return np.concatenate([np.asarray(w, dtype=np.float32).ravel() for w in ws] +
                          [np.asarray(b, dtype=np.float32).ravel() for b in bs])


class LearnedProposal:
    def __init__(self, sim, L: int, eta_scale: float = 16.0, data_capacity: int = 0, seed: int = 1):
        self.sim = sim
        self.L = int(L)
        self.eta_scale = float(eta_scale)
        h = C.c_void_p()
        _lib.call("uppasd_gpu_proposal_create", sim._h, self.L, self.eta_scale, int(data_capacity), int(seed),
                  C.byref(h))
        self.h = h
        n = C.c_int64()
        _lib.call("uppasd_gpu_proposal_nparams", self.h, C.byref(n))
        self.nparams = int(n.value)

    def get_params(self):
        v = np.zeros(self.nparams, dtype=np.float32)
        _lib.call("uppasd_gpu_proposal_get_params", self.h, v.ctypes.data_as(C.c_void_p))
        return v

    def set_params(self, v):
        v = np.ascontiguousarray(v, dtype=np.float32)
        _lib.call("uppasd_gpu_proposal_set_params", self.h, v.ctypes.data_as(C.c_void_p))

    def masks(self):
        n = sum(a * b for a, b in W_SHAPES)
        m = np.zeros(n, dtype=np.float32)
        _lib.call("uppasd_gpu_proposal_get_masks", self.h, m.ctypes.data_as(C.c_void_p))
        out, o = [], 0
        for s in W_SHAPES:
            out.append(m[o:o + s[0] * s[1]].reshape(s))
            o += s[0] * s[1]
        return out

    def forward(self, x):
        x = np.ascontiguousarray(x, dtype=np.float32)
        out = np.zeros((x.shape[0], N_OUT), dtype=np.float32)
        _lib.call("uppasd_gpu_proposal_forward", self.h, x.ctypes.data_as(C.c_void_p), x.shape[0],
                  out.ctypes.data_as(C.c_void_p))
        return out

    def loss_grad(self, x):
        x = np.ascontiguousarray(x, dtype=np.float32)
        loss = C.c_double()
        g = np.zeros(self.nparams, dtype=np.float32)
        _lib.call("uppasd_gpu_proposal_loss_grad", self.h, x.ctypes.data_as(C.c_void_p), x.shape[0],
                  C.byref(loss), g.ctypes.data_as(C.c_void_p))
        return float(loss.value), g

    def collect(self):
        _lib.call("uppasd_gpu_proposal_collect", self.h)

    def train(self, nsteps: int, rows: int = 16384, lr: float = 1e-3):
        losses = np.zeros(max(int(nsteps), 1))
        _lib.call("uppasd_gpu_proposal_train", self.h, int(nsteps), int(rows), float(lr),
                  losses.ctypes.data_as(C.c_void_p))
        return losses[:nsteps]

    def sweep(self, temperature: float, nsweeps: int = 1):
        """Learned sweeps; returns (accepted, proposed, summed accepted energy change in J)."""
        a, p, de = C.c_int64(), C.c_int64(), C.c_double()
        _lib.call("uppasd_gpu_proposal_sweep", self.h, float(temperature), int(nsweeps), C.byref(a), C.byref(p),
                  C.byref(de))
        return int(a.value), int(p.value), float(de.value)

    def mix(self, temperature: float, ncycles: int, hb_per_cycle: int = 1):
        """ncycles of (hb_per_cycle structured heat-bath sweeps + one learned sweep), one sync."""
        a, p, de = C.c_int64(), C.c_int64(), C.c_double()
        _lib.call("uppasd_gpu_proposal_mix", self.h, float(temperature), int(ncycles), int(hb_per_cycle),
                  C.byref(a), C.byref(p), C.byref(de))
        return int(a.value), int(p.value), float(de.value)

    def mix_temps(self, temps, ncycles: int, hb_per_cycle: int = 1):
        """mix() with one temperature per ensemble of the simulation."""
        t = np.ascontiguousarray(temps, dtype=np.float64)
        a, p, de = C.c_int64(), C.c_int64(), C.c_double()
        _lib.call("uppasd_gpu_proposal_mix_temps", self.h, t.ctypes.data_as(_lib.F64P), int(ncycles),
                  int(hb_per_cycle), C.byref(a), C.byref(p), C.byref(de))
        return int(a.value), int(p.value), float(de.value)

    def close(self):
        if getattr(self, "h", None) is not None and self.h.value:
            _lib.call("uppasd_gpu_proposal_destroy", self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
