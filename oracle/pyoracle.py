"""ctypes driver for the CPU oracle (liboracle.so).

TEST INFRASTRUCTURE ONLY: used by tests/, by ``__graft_entry__.smoke()`` as
the checker and by ``bench.py``'s CPU-baseline leg.  The product library never
imports this module.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "liboracle.so")
# the timed build (-O3, default contraction): the CPU baseline, never the checker
LIB_FAST = os.path.join(HERE, "liboracle_fast.so")

_lib = None
_lib_fast = None

I32P = C.POINTER(C.c_int32)
F64P = C.POINTER(C.c_double)


class OrcMT(C.Structure):
    _fields_ = [("mti", C.c_int32), ("mt", C.c_uint64 * 624)]


class OrcZig(C.Structure):
    _fields_ = [("z", OrcMT), ("kn", C.c_int32 * 128), ("fn", C.c_double * 128), ("wn", C.c_double * 128)]


class OrcHam(C.Structure):
    _fields_ = [
        ("natom", C.c_int), ("mensemble", C.c_int), ("max_no_neigh", C.c_int), ("nham", C.c_int),
        ("nlist", I32P), ("nlistsize", I32P), ("ncoup", F64P), ("aham", I32P),
        ("do_dm", C.c_int), ("max_no_dmneigh", C.c_int), ("dmlist", I32P), ("dmlistsize", I32P),
        ("dm_vect", F64P), ("do_aniso", C.c_int), ("taniso", I32P), ("eaniso", F64P),
        ("kaniso", F64P), ("sb", F64P), ("extfield", F64P),
        ("do_jtensor", C.c_int), ("j_tens", F64P),
        ("do_dip", C.c_int), ("dip_na", C.c_int), ("dip_n1", C.c_int), ("dip_n2", C.c_int), ("dip_n3", C.c_int),
        ("dip_cell", F64P), ("dip_bas", F64P), ("dip_alat", C.c_double), ("dip_work", F64P),
    ]


class OrcLLG(C.Structure):
    _fields_ = [
        ("sdealgh", C.c_int), ("delta_t", C.c_double), ("bn", C.c_double), ("temprescale", C.c_double),
        ("lambda1", F64P), ("temp", F64P), ("landeg", F64P), ("noise_mode", C.c_int),
        ("zig", C.POINTER(OrcZig)), ("noise", F64P), ("seed", C.c_uint64), ("step", C.c_int64),
        ("relaxtime", C.c_double), ("perp", C.c_int),
    ]


class OrcState(C.Structure):
    _fields_ = [("emom", F64P), ("emom2", F64P), ("emomM", F64P), ("mmom", F64P),
                ("b2eff", F64P), ("beff", F64P), ("ranv", F64P), ("mpast", F64P)]


class OrcCumulant(C.Structure):
    _fields_ = [("cumuw", C.c_double), ("cumutotw", C.c_double), ("avrgmcum", C.c_double),
                ("avrgm2cum", C.c_double), ("avrgm4cum", C.c_double), ("avrgecum", C.c_double),
                ("avrge2cum", C.c_double), ("navrgcum", C.c_int)]


NOISE_NONE, NOISE_ZIGGURAT, NOISE_ARRAY, NOISE_PHILOX = 0, 1, 2, 3


def build() -> str:
    subprocess.run(["make", "-s", "-C", HERE, "liboracle.so", "liboracle_fast.so"], check=True)
    return LIB


def load(fast: bool = False):
    """The parity build (default) or, with fast=True, the -O3 build used to time the
    CPU baseline."""
    global _lib, _lib_fast
    if fast:
        if _lib_fast is None:
            if not os.path.exists(LIB_FAST):
                build()
            _lib_fast = _declare(C.CDLL(LIB_FAST))
        return _lib_fast
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB):
        build()
    _lib = _declare(C.CDLL(LIB))
    return _lib


def _declare(lib):
    lib.orc_mt_init.argtypes = [C.POINTER(OrcMT), C.c_int32]
    lib.orc_mt_rand64.argtypes = [C.POINTER(OrcMT)]
    lib.orc_mt_rand64.restype = C.c_uint64
    lib.orc_mt_real2.argtypes = [C.POINTER(OrcMT)]
    lib.orc_mt_real2.restype = C.c_double
    lib.orc_mt_real1.argtypes = [C.POINTER(OrcMT)]
    lib.orc_mt_real1.restype = C.c_double
    lib.orc_zig_setup.argtypes = [C.POINTER(OrcZig), C.c_int32]
    lib.orc_zig_nor.argtypes = [C.POINTER(OrcZig)]
    lib.orc_zig_nor.restype = C.c_double
    lib.orc_zig_fill.argtypes = [C.POINTER(OrcZig), F64P, C.c_int64]
    lib.orc_philox4x32_10.argtypes = [C.POINTER(C.c_uint32), C.POINTER(C.c_uint32), C.POINTER(C.c_uint32)]
    lib.orc_philox_normal3.argtypes = [C.c_uint64, C.c_int64, C.c_int32, C.c_int64, C.c_uint32, F64P]
    lib.orc_philox_uniform4.argtypes = [C.c_uint64, C.c_int64, C.c_int32, C.c_int64, C.c_uint32, F64P]
    lib.orc_effective_field.argtypes = [C.POINTER(OrcHam), F64P, F64P]
    lib.orc_effective_field.restype = C.c_double
    lib.orc_sd_step.argtypes = [C.POINTER(OrcHam), C.POINTER(OrcLLG), C.POINTER(OrcState)]
    lib.orc_sd_step.restype = C.c_int
    lib.orc_llg_draw_normals.argtypes = [C.POINTER(OrcLLG), C.c_int, C.c_int, F64P]
    lib.orc_initmag_random.argtypes = [C.POINTER(OrcMT), C.c_int, C.c_int, F64P, F64P, F64P]
    lib.orc_choose_random_atom_x.argtypes = [C.POINTER(OrcMT), C.c_int, I32P]
    lib.orc_mc_evolve_ref.argtypes = [C.POINTER(OrcHam), C.c_char, C.c_double, C.c_double, I32P,
                                      C.POINTER(OrcMT), C.POINTER(OrcZig), F64P, F64P, F64P, F64P]
    lib.orc_mc_sweep_checkerboard.argtypes = [C.POINTER(OrcHam), C.c_char, C.c_double, I32P, I32P, C.c_int,
                                              C.c_uint64, C.c_int64, F64P, F64P, F64P]
    lib.orc_mc_sweep_checkerboard_temps.argtypes = [C.POINTER(OrcHam), C.c_char, C.c_double, F64P, I32P, I32P,
                                                    C.c_int, C.c_uint64, C.c_int64, F64P, F64P, F64P]
    lib.orc_mavg.argtypes = [C.c_int, C.c_int, F64P, F64P, F64P]
    lib.orc_energy.argtypes = [C.POINTER(OrcHam), F64P, F64P, F64P, F64P, F64P, F64P]
    lib.orc_cumulant_update.argtypes = [C.POINTER(OrcCumulant), C.c_int, C.c_int, F64P, C.c_double, F64P, F64P]
    lib.orc_set_threads.argtypes = [C.c_int]
    lib.orc_get_threads.restype = C.c_int
    lib.orc_set_units.argtypes = [C.c_double] * 4
    lib.orc_dipole_field.argtypes = [C.POINTER(OrcHam), F64P, F64P]
    return lib


SI_UNITS = (1.760859644e11, 1.38064852e-23, 9.274009994e-24, 2.179872325e-21)   # gama, k_bolt, mub, mry
ATOMIC_UNITS = (1.0, 1.0, 1.0, 1.0)   # aunits 'Y' (Input/inputhandler.f90:1685-1704)


class units:
    """Context manager: the oracle computes with (gama, k_bolt, mub, mry) inside the
    block and with SI units again after it."""

    def __init__(self, values):
        self.values = tuple(float(v) for v in values)

    def __enter__(self):
        load().orc_set_units(*self.values)
        return self

    def __exit__(self, *exc):
        load().orc_set_units(*SI_UNITS)
        return False


def _p(a, t=F64P):
    return a.ctypes.data_as(t) if a is not None else None


class Oracle:
    """Holds one Hamiltonian and one spin state in the reference's layout."""

    def __init__(self, lat, threads: int = 0, fast: bool = False, dipole_alat: float = 0.0):
        """dipole_alat > 0 adds the brute-force dipole-dipole field (do_dip = 1) with that
        lattice constant (m), on the lattice's cell and basis."""
        self.lib = load(fast)
        self.lib.orc_set_threads(threads)
        self.lat = lat
        N, M = lat.natom, lat.mensemble
        self._keep = []

        def keep(a, dtype):
            a = np.ascontiguousarray(a, dtype=dtype)
            self._keep.append(a)
            return a

        h = OrcHam()
        h.natom, h.mensemble = N, M
        h.max_no_neigh, h.nham = lat.max_no_neigh, lat.nham
        h.nlist = _p(keep(lat.nlist, np.int32), I32P)
        h.nlistsize = _p(keep(lat.nlistsize, np.int32), I32P)
        h.ncoup = _p(keep(lat.ncoup, np.float64))
        h.aham = _p(keep(lat.aham, np.int32), I32P)
        h.do_dm = lat.do_dm
        if lat.do_dm:
            h.max_no_dmneigh = lat.dmlist.shape[1]
            h.dmlist = _p(keep(lat.dmlist, np.int32), I32P)
            h.dmlistsize = _p(keep(lat.dmlistsize, np.int32), I32P)
            h.dm_vect = _p(keep(lat.dm_vect, np.float64))
        h.do_aniso = lat.do_aniso
        if lat.do_aniso:
            h.taniso = _p(keep(lat.taniso, np.int32), I32P)
            h.eaniso = _p(keep(lat.eaniso, np.float64))
            h.kaniso = _p(keep(lat.kaniso, np.float64))
            h.sb = _p(keep(lat.sb if lat.sb is not None else np.zeros(N), np.float64))
        if getattr(lat, "j_tens", None) is not None:
            h.do_jtensor = 1
            h.j_tens = _p(keep(lat.j_tens, np.float64))
        self.extfield = keep(np.broadcast_to(lat.extfield, (M, N, 3)), np.float64)
        h.extfield = _p(self.extfield)
        if dipole_alat > 0.0:
            cell, bas = lat.dipole_geometry()
            h.do_dip = 1
            h.dip_na = lat.nbasis
            h.dip_n1, h.dip_n2, h.dip_n3 = lat.cells
            h.dip_cell = _p(keep(cell, np.float64))
            h.dip_bas = _p(keep(bas, np.float64))
            h.dip_alat = float(dipole_alat)
            h.dip_work = _p(keep(np.zeros((M, N, 3)), np.float64))
        self.ham = h
        self.mmom = keep(np.broadcast_to(lat.mmom, (M, N)), np.float64)
        shape3 = (M, N, 3)
        self.emom = np.zeros(shape3)
        self.emom2 = np.zeros(shape3)
        self.emomM = np.zeros(shape3)
        self.beff = np.zeros(shape3)
        self.b2eff = np.zeros(shape3)
        self.ranv = np.zeros(shape3)
        self.mpast = np.zeros(shape3)
        st = OrcState()
        st.emom, st.emom2, st.emomM = _p(self.emom), _p(self.emom2), _p(self.emomM)
        st.mmom, st.b2eff, st.beff, st.ranv = _p(self.mmom), _p(self.b2eff), _p(self.beff), _p(self.ranv)
        st.mpast = _p(self.mpast)
        self.state = st
        self.zig = None
        self.mt = None

    # ---- state ----
    def set_moments(self, emom):
        emom = np.asarray(emom, dtype=np.float64).reshape(self.emom.shape)
        self.emom[...] = emom
        self.emom2[...] = emom
        self.emomM[...] = emom * self.mmom[..., None]
        self.mpast[...] = 0.0   # LLGI starts without a previous step (llgi.f90:295)

    def init_random(self, seed: int):
        """initmag 1 from a fresh mtprng stream seeded with `seed` (rng_init)."""
        self.mt = OrcMT()
        self.lib.orc_mt_init(C.byref(self.mt), seed)
        self.lib.orc_initmag_random(C.byref(self.mt), self.lat.natom, self.lat.mensemble, _p(self.mmom),
                                    _p(self.emom), _p(self.emomM))
        self.emom2[...] = self.emom
        self.mpast[...] = 0.0

    def setup_ziggurat(self, seed: int):
        self.zig = OrcZig()
        self.lib.orc_zig_setup(C.byref(self.zig), seed)

    # ---- field / energy ----
    def field(self):
        e = self.lib.orc_effective_field(C.byref(self.ham), _p(self.emomM), _p(self.beff))
        return self.beff.copy(), e

    def energy(self):
        M = self.lat.mensemble
        out = [np.zeros(M) for _ in range(5)]
        self.lib.orc_energy(C.byref(self.ham), _p(self.emomM), *[_p(o) for o in out])
        return {"total": out[0], "xc": out[1], "dm": out[2], "ani": out[3], "ext": out[4]}

    def dipole_field(self):
        """The brute-force dipolar field of the current full moments, (M, N, 3)."""
        out = np.zeros(self.emom.shape)
        self.lib.orc_dipole_field(C.byref(self.ham), _p(self.emomM), _p(out))
        return out

    def mavg(self):
        M = self.lat.mensemble
        mv = np.zeros((M, 3))
        ma = np.zeros(M)
        self.lib.orc_mavg(self.lat.natom, M, _p(self.emomM), _p(mv), _p(ma))
        return mv, ma

    # ---- LLG ----
    def make_llg(self, sdealgh, delta_t, lambda1, temp, landeg=1.0, noise_mode=NOISE_PHILOX, seed=0, bn=1.0,
                 relaxtime=0.0, perp=False):
        N = self.lat.natom
        self._lam = np.ascontiguousarray(np.broadcast_to(np.asarray(lambda1, dtype=np.float64), (N,)))
        self._temp = np.ascontiguousarray(np.broadcast_to(np.asarray(temp, dtype=np.float64), (N,)))
        self._g = np.ascontiguousarray(np.broadcast_to(np.asarray(landeg, dtype=np.float64), (N,)))
        p = OrcLLG()
        p.sdealgh, p.delta_t, p.bn, p.temprescale = sdealgh, delta_t, bn, 1.0
        p.lambda1, p.temp, p.landeg = _p(self._lam), _p(self._temp), _p(self._g)
        p.noise_mode = noise_mode
        p.seed = seed
        p.step = 0
        p.relaxtime = relaxtime
        p.perp = 1 if perp else 0
        if noise_mode == NOISE_ZIGGURAT:
            if self.zig is None:
                raise ValueError("setup_ziggurat() first")
            p.zig = C.pointer(self.zig)
        self.llg = p
        return p

    def sd_step(self, noise=None):
        if noise is not None:
            self._noise = np.ascontiguousarray(noise, dtype=np.float64)
            self.llg.noise = _p(self._noise)
        rc = self.lib.orc_sd_step(C.byref(self.ham), C.byref(self.llg), C.byref(self.state))
        if rc != 0:
            raise RuntimeError(f"orc_sd_step failed ({rc})")
        self.llg.step += 1

    def draw_normals(self):
        out = np.zeros(self.emom.shape)
        self.lib.orc_llg_draw_normals(C.byref(self.llg), self.lat.natom, self.lat.mensemble, _p(out))
        return out

    # ---- MC ----
    def mc_sweep_ref(self, mode: str, temperature: float, iflip_a):
        if self.mt is None or self.zig is None:
            raise ValueError("seed the uniform and ziggurat streams first")
        return self.lib.orc_mc_evolve_ref(C.byref(self.ham), mode.encode(), temperature, 1.0,
                                          _p(np.ascontiguousarray(iflip_a, dtype=np.int32), I32P),
                                          C.byref(self.mt), C.byref(self.zig), _p(self.emom), _p(self.emomM),
                                          _p(self.mmom), _p(self.beff))

    def choose_random_atom_x(self):
        out = np.zeros(self.lat.natom, dtype=np.int32)
        self.lib.orc_choose_random_atom_x(C.byref(self.mt), self.lat.natom, _p(out, I32P))
        return out

    def mc_sweep_checkerboard(self, mode: str, temperature: float, colour_sites, colour_start, seed: int, sweep: int,
                              temps=None):
        """One checkerboard sweep; temps: one temperature per ensemble (overrides temperature)."""
        cs = np.ascontiguousarray(colour_sites, dtype=np.int32)
        st = np.ascontiguousarray(colour_start, dtype=np.int32)
        tk = None if temps is None else np.ascontiguousarray(temps, dtype=np.float64)
        return self.lib.orc_mc_sweep_checkerboard_temps(C.byref(self.ham), mode.encode(), temperature, _p(tk),
                                                        _p(cs, I32P), _p(st, I32P), len(st) - 1, seed, sweep,
                                                        _p(self.emom), _p(self.emomM), _p(self.mmom))

    def pt_iphase(self, temps, nsweeps: int, pt_step: int, colour_sites, colour_start, seed: int, sweep0: int = 0):
        """pt_iphase (pt_driver.f90:58-367) with the ensembles as replicas on the checkerboard
        heat bath: swap attempts every pt_step sweeps during the first 90 %, positions
        (r, r + 1) for r = 0, 2, ... then 1, 3, ..., one Philox uniform per position
        (position, 0, step, stream 8), acceptance min(1, exp((e2 - e1)(b2 - b1))) on the
        per-atom energies in J.  Returns (temps, trials, accepted, lowest-energy replica)."""
        kb = 1.38064852e-23
        T = np.array(temps, dtype=np.float64)
        M = self.lat.mensemble
        trial = hit = 0
        for step in range(1, nsweeps + 1):
            self.mc_sweep_checkerboard("H", 0.0, colour_sites, colour_start, seed, sweep0 + step - 1, temps=T)
            if step % pt_step or step / nsweeps >= 0.90:
                continue
            ene = self.energy()["total"] * 2.179872325e-21
            u = [uniform4(seed, r, 0, step, 8)[0] for r in range(M)]
            for ishift in (0, 1):
                for r in range(ishift, M - 1, 2):
                    trial += 1
                    b1, b2 = 1.0 / kb / (T[r] + 1e-15), 1.0 / kb / (T[r + 1] + 1e-15)
                    prob = min(1.0, np.exp((ene[r + 1] - ene[r]) * (b2 - b1)))
                    if u[r] <= prob:
                        T[r], T[r + 1] = T[r + 1], T[r]
                        hit += 1
        ene = self.energy()["total"]
        return T, trial, hit, int(np.argmin(ene))


def uniform4(seed: int, site: int, ens: int, step: int, stream: int):
    """The four (0, 1) uniforms of one Philox draw (site, ensemble, step, stream)."""
    lib = load()
    u = np.zeros(4)
    lib.orc_philox_uniform4(seed, site, ens, step, stream, _p(u))
    return u


def philox(ctr, key):
    lib = load()
    c = (C.c_uint32 * 4)(*ctr)
    k = (C.c_uint32 * 2)(*key)
    o = (C.c_uint32 * 4)()
    lib.orc_philox4x32_10(c, k, o)
    return list(o)


def mt_stream(seed: int, n: int, kind: str = "real2"):
    lib = load()
    s = OrcMT()
    lib.orc_mt_init(C.byref(s), seed)
    f = {"real2": lib.orc_mt_real2, "real1": lib.orc_mt_real1, "u32": lib.orc_mt_rand64}[kind]
    return np.array([f(C.byref(s)) for _ in range(n)])


def ziggurat_stream(seed: int, n: int):
    lib = load()
    z = OrcZig()
    lib.orc_zig_setup(C.byref(z), seed)
    out = np.zeros(n)
    lib.orc_zig_fill(C.byref(z), _p(out), n)
    return out
