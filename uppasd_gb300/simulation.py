"""Host-side mirror of the reference's interface to the spin-update hot path.

``GpuSimulation`` plays the role of the reference's ``CudaMdSimulation``
(gpu_files/cudaMdSimulation.cu) behind the Fortran driver, and exposes the
calls the reference's Python layer makes (uppasd/simulator.py:
``get_moments``, ``put_moments``, ``get_fields``, ``relax``, ``evolve``) on top
of the C ABI in include/uppasd_gpu.h.  Arrays cross the boundary in the
reference's layout: (mensemble, natom, 3) C-ordered, i.e. Fortran
(3, natom, mensemble).
"""
from __future__ import annotations

import ctypes as C
from typing import Optional

import numpy as np

from . import _lib
from .lattice import Lattice

SOLVERS = {"midpoint": 1, "heun": 4, "depondt": 5, "sib": 6, "sisph": 7, "llgi": 11}


def _ptr(a, t=_lib.F64P):
    return a.ctypes.data_as(t) if a is not None else None


class GpuSimulation:
    """One Hamiltonian and `mensemble` spin replicas resident on the GPU.

    precision: 0 FP64 throughout (any neighbour list, every solver); 1 / 2 the structured
    bcc kernels (FP32 gather, FP64 / double-single master; periodic bcc, up to four
    shells and two species, Depondt); 3 / 4 FP32 gather over any neighbour list with an
    FP64 / double-single master (every solver)."""

    def __init__(self, lat: Lattice, sdealgh: int = 5, delta_t: float = 1e-16, damping=0.1,
                 temperature=0.0, landeg=1.0, seed: int = 1, emom: Optional[np.ndarray] = None,
                 precision: int = 0, gpu_rng: int = 0, bn: float = 1.0, relaxtime: float = 0.0,
                 perp: bool = False):
        if isinstance(sdealgh, str):
            sdealgh = SOLVERS[sdealgh]
        self.lat = lat
        N, M = lat.natom, lat.mensemble
        self._keep = []

        def keep(a, dtype):
            a = np.ascontiguousarray(a, dtype=dtype)
            self._keep.append(a)
            return a

        c = _lib.Consts()
        c.natom, c.mensemble = N, M
        c.max_no_neigh, c.nham = lat.max_no_neigh, lat.nham
        c.do_dm = lat.do_dm
        c.max_no_dmneigh = lat.dmlist.shape[1] if lat.do_dm else 0
        c.do_aniso = lat.do_aniso
        c.sdealgh = int(sdealgh)
        c.delta_t, c.bn, c.temprescale = float(delta_t), float(bn), 1.0
        c.gpu_rng_seed = int(seed)
        c.gpu_rng = int(gpu_rng)
        c.precision = int(precision)
        if lat.cells[0] > 0:
            c.n1, c.n2, c.n3 = lat.cells
            c.na = lat.nbasis
        a = _lib.Arrays()
        a.nlist = _ptr(keep(lat.nlist, np.int32), _lib.I32P)
        a.nlistsize = _ptr(keep(lat.nlistsize, np.int32), _lib.I32P)
        a.ncoup = _ptr(keep(lat.ncoup, np.float64))
        a.aham = _ptr(keep(lat.aham, np.int32), _lib.I32P)
        if lat.do_dm:
            a.dmlist = _ptr(keep(lat.dmlist, np.int32), _lib.I32P)
            a.dmlistsize = _ptr(keep(lat.dmlistsize, np.int32), _lib.I32P)
            a.dm_vect = _ptr(keep(lat.dm_vect, np.float64))
        if lat.do_aniso:
            a.taniso = _ptr(keep(lat.taniso, np.int32), _lib.I32P)
            a.eaniso = _ptr(keep(lat.eaniso, np.float64))
            a.kaniso = _ptr(keep(lat.kaniso, np.float64))
            a.sb = _ptr(keep(lat.sb if lat.sb is not None else np.zeros(N), np.float64))
        a.external_field = _ptr(keep(np.broadcast_to(lat.extfield, (M, N, 3)), np.float64))
        self.mmom = keep(np.broadcast_to(lat.mmom, (M, N)), np.float64)
        a.mmom = _ptr(self.mmom)
        a.lambda1_array = _ptr(keep(np.broadcast_to(np.asarray(damping, float), (N,)), np.float64))
        a.temp_array = _ptr(keep(np.broadcast_to(np.asarray(temperature, float), (N,)), np.float64))
        a.landeg = _ptr(keep(np.broadcast_to(np.asarray(landeg, float), (N,)), np.float64))
        if emom is None:
            emom = np.zeros((M, N, 3))
            emom[..., 2] = 1.0
        a.emom = _ptr(keep(np.broadcast_to(emom, (M, N, 3)), np.float64))
        if lat.species is not None:
            a.species = _ptr(keep(lat.species, np.int32), _lib.I32P)
        h = C.c_void_p()
        _lib.call("uppasd_gpu_init", C.byref(c), C.byref(a), C.byref(h))
        self._h = h
        self._keep = []  # init copied everything it needs
        if lat.j_tens is not None:
            self.set_jtensor(lat.j_tens)
        if relaxtime:
            _lib.call("uppasd_gpu_set_relaxtime", self._h, float(relaxtime))
        if perp:
            _lib.call("uppasd_gpu_set_perp", self._h, 1)

    def set_jtensor(self, j_tens: Optional[np.ndarray]):
        """Exchange tensor in the Fortran image (nham, mnn, 3, 3) = j_tens(3,3,mnn,nham);
        None returns to the scalar couplings."""
        if j_tens is None:
            _lib.call("uppasd_gpu_set_jtensor", self._h, None)
            return
        jt = np.ascontiguousarray(j_tens, dtype=np.float64)
        if jt.shape != (self.lat.nham, self.lat.max_no_neigh, 3, 3):
            raise ValueError(f"j_tens must be (nham, mnn, 3, 3), got {jt.shape}")
        _lib.call("uppasd_gpu_set_jtensor", self._h, _ptr(jt))

    def set_dipole(self, do_dip: int, alat: float = 2.87e-10, coord: Optional[np.ndarray] = None):
        """Dipole-dipole field (input keyword do_dip): 0 off, 1 brute force, 3 FFT.

        alat is the lattice constant in metres.  Brute force sums over `coord` (natom, 3),
        Cartesian in units of alat, when given, else over the lattice's cell grid
        (Lattice.dipole_geometry); the FFT form always uses the cell grid.  FP64 path only.
        """
        if do_dip == 0:
            _lib.call("uppasd_gpu_set_dipole", self._h, 0, 0.0, None, 0, 0, 0, 0, None, None)
            return
        cell, bas = self.lat.dipole_geometry()
        n1, n2, n3 = (int(v) for v in self.lat.cells)
        cell = np.ascontiguousarray(cell, dtype=np.float64)
        bas = np.ascontiguousarray(bas, dtype=np.float64)
        cp = None
        if coord is not None:
            coord = np.ascontiguousarray(coord, dtype=np.float64)
            if coord.shape != (self.lat.natom, 3):
                raise ValueError(f"coord must be (natom, 3), got {coord.shape}")
            cp = _ptr(coord)
        _lib.call("uppasd_gpu_set_dipole", self._h, int(do_dip), float(alat), cp, int(self.lat.nbasis), n1, n2, n3,
                  _ptr(cell), _ptr(bas))

    # -- lifecycle --
    def close(self):
        if getattr(self, "_h", None) is not None and self._h.value:
            _lib.call("uppasd_gpu_finalize", self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    # -- state (uppasd/simulator.py get_moments / put_moments / get_fields) --
    def put_moments(self, emom):
        e = np.ascontiguousarray(np.broadcast_to(emom, (self.lat.mensemble, self.lat.natom, 3)), dtype=np.float64)
        _lib.call("uppasd_gpu_put_moments", self._h, _ptr(e))

    def get_moments(self, full: bool = False, out: Optional[np.ndarray] = None):
        """Unit moments (mensemble, natom, 3); with full=True also the full moments.
        `out`: a C-contiguous float64 array of that shape to copy into (e.g. pinned
        host memory, which the device-to-host copy reads at full speed)."""
        shape = (self.lat.mensemble, self.lat.natom, 3)
        if out is not None:
            if out.shape != shape or out.dtype != np.float64 or not out.flags.c_contiguous:
                raise ValueError(f"out must be a C-contiguous float64 array of shape {shape}")
            e = out
        else:
            e = np.empty(shape)
        em = np.empty(shape) if full else None
        _lib.call("uppasd_gpu_get_moments", self._h, _ptr(e), _ptr(em))
        return (e, em) if full else e

    def get_coords(self):
        """Atom positions (natom, 3), as the reference simulator's get_coords."""
        return self.lat.coords

    def get_fields(self):
        b = np.empty((self.lat.mensemble, self.lat.natom, 3))
        _lib.call("uppasd_gpu_get_field", self._h, _ptr(b))
        return b

    def set_temperature(self, temperature):
        t = np.ascontiguousarray(np.broadcast_to(np.asarray(temperature, float), (self.lat.natom,)))
        _lib.call("uppasd_gpu_set_temperature", self._h, _ptr(t))

    def set_units(self, gama: float, k_bolt: float, mub: float, mry: float):
        """The physical constants every path computes with (SI until set)."""
        _lib.call("uppasd_gpu_set_units", self._h, float(gama), float(k_bolt), float(mub), float(mry))

    def set_atomic_units(self):
        """aunits = 'Y': gama, k_bolt, mub and mry all 1 (Input/inputhandler.f90:1685-1704)."""
        self.set_units(1.0, 1.0, 1.0, 1.0)

    def set_step(self, step: int):
        _lib.call("uppasd_gpu_set_step", self._h, int(step))

    def set_noise(self, normals: Optional[np.ndarray]):
        """Inject N(0,1) numbers, shape (nsteps, mensemble, natom, 3) (reference draw order)."""
        if normals is None:
            _lib.call("uppasd_gpu_set_noise", self._h, None, 0)
            return
        n = np.ascontiguousarray(normals, dtype=np.float64)
        _lib.call("uppasd_gpu_set_noise", self._h, _ptr(n), n.shape[0])

    # -- dynamics (sd_mphase) and Monte Carlo (mc_mphase) --
    def evolve(self, nsteps: int):
        _lib.call("uppasd_gpu_sd_run", self._h, int(nsteps))

    def run_io(self, emom_in: Optional[np.ndarray], nsteps: int, out: Optional[np.ndarray] = None,
               out_full: Optional[np.ndarray] = None):
        """put_moments(emom_in) + evolve(nsteps) + get_moments into `out` (and the full
        moments into `out_full`) as one call; the arrays are C-contiguous float64
        (mensemble, natom, 3).  With page-locked arrays on the structured path the
        ensembles' copies overlap the other ensembles' steps (same result)."""
        shape = (self.lat.mensemble, self.lat.natom, 3)
        arrs = []
        for a in (emom_in, out, out_full):
            if a is not None and (a.shape != shape or a.dtype != np.float64 or not a.flags.c_contiguous):
                raise ValueError(f"arrays must be C-contiguous float64 of shape {shape}")
            arrs.append(_ptr(a) if a is not None else None)
        _lib.call("uppasd_gpu_sd_run_io", self._h, arrs[0], int(nsteps), arrs[1], arrs[2])

    def sd_run_measured(self, nsteps: int, every: int, fn):
        """nsteps steps with fn(step, emom, emomM) after every `every` of them; the arrays are
        (mensemble, natom, 3) views of library memory, valid during the call (copy to keep).
        Each snapshot's transfer to the host overlaps the next block of steps.  A truthy
        return value of fn stops the run after the block in flight."""
        shape = (self.lat.mensemble, self.lat.natom, 3)
        count = 3 * self.lat.natom * self.lat.mensemble
        stopped = []

        def cb(step, pe, pm, user):
            try:
                e = np.ctypeslib.as_array(pe, shape=(count,)).reshape(shape)
                m = np.ctypeslib.as_array(pm, shape=(count,)).reshape(shape)
                if fn(int(step), e, m):
                    stopped.append(int(step))
                    return 1
                return 0
            except Exception as exc:  # an exception ends the run; it is raised after it
                stopped.append(exc)
                return 1

        c_cb = _lib.MEASURE_CB(cb)
        rc = _lib.load().uppasd_gpu_sd_run_measured(self._h, int(nsteps), int(every), c_cb, None)
        if stopped and isinstance(stopped[-1], Exception):
            raise stopped[-1]
        if rc < 0:
            msg = _lib.load().uppasd_gpu_last_error()
            raise _lib.UppasdGpuError("uppasd_gpu_sd_run_measured", rc, msg.decode() if msg else "")
        return rc

    def relax(self, mode: str = "M", temperature: float = 0.0, nsweeps: int = 1, structured: bool = False):
        """Monte Carlo sweeps: mode 'M' (Metropolis, T >= 0) or 'H' (heat bath, T > 0); the
        defaults are those of the reference simulator's relax (uppasd/simulator.py), a
        zero-temperature Metropolis sweep.  structured=True runs the square-lattice heat
        bath (FP32 draws, uniform couplings recognised at the first call)."""
        if structured:
            if mode != "H":
                raise ValueError("the structured path is a heat bath")
            L = int(round(np.sqrt(self.lat.natom)))
            _lib.call("uppasd_gpu_mc_run_square", self._h, L, float(temperature), int(nsweeps))
            return
        _lib.call("uppasd_gpu_mc_run", self._h, mode.encode()[:1], float(temperature), int(nsweeps))

    def relax_temps(self, mode: str, temps, nsweeps: int):
        """Monte Carlo sweeps with one temperature per ensemble."""
        t = np.ascontiguousarray(temps, dtype=np.float64)
        if t.shape != (self.lat.mensemble,):
            raise ValueError("one temperature per ensemble")
        _lib.call("uppasd_gpu_mc_run_temps", self._h, mode.encode()[:1], _ptr(t), int(nsweeps))

    def relax_temps_square(self, temps, nsweeps: int):
        """Structured square-lattice heat bath (uppasd_gpu_mc_run_square) with one
        temperature per ensemble."""
        t = np.ascontiguousarray(temps, dtype=np.float64)
        if t.shape != (self.lat.mensemble,):
            raise ValueError("one temperature per ensemble")
        _lib.call("uppasd_gpu_mc_run_square_temps", self._h, int(self.lat.cells[0]), _ptr(t), int(nsweeps))

    def parallel_tempering(self, temps, nsweeps: int, pt_step: int = 1):
        """pt_iphase with the ensembles as replicas: returns (temperatures per replica at the
        end, swap trials, accepted swaps, replica of lowest energy)."""
        t = np.array(temps, dtype=np.float64)
        if t.shape != (self.lat.mensemble,):
            raise ValueError("one temperature per ensemble")
        nt, nh, sel = C.c_int64(), C.c_int64(), C.c_int32()
        _lib.call("uppasd_gpu_pt_run", self._h, _ptr(t), int(nsweeps), int(pt_step), C.byref(nt), C.byref(nh),
                  C.byref(sel))
        return t, nt.value, nh.value, sel.value

    def set_stream(self, cuda_stream_handle: int):
        """Issue all work on the caller's CUDA stream (0 = the library's own)."""
        _lib.call("uppasd_gpu_set_stream", self._h, C.c_void_p(cuda_stream_handle or None))

    def time_kernels(self, nrep: int = 5):
        """Mean device ms per launch: predictor, corrector, whole step (advances nrep steps)."""
        ms = np.zeros(3)
        _lib.call("uppasd_gpu_time_kernels", self._h, int(nrep), _ptr(ms))
        return {"predict_ms": ms[0], "correct_ms": ms[1], "step_ms": ms[2]}

    def path_info(self):
        """Which path and data forms init chose: precision, structured stencil path, and on
        the FP32-gather path the site classes (0: per-site lists), distinct coupling rows,
        chemical types the exchange is looked up by (0: none), uniform external field;
        device bytes allocated."""
        info = np.zeros(8, dtype=np.int64)
        _lib.call("uppasd_gpu_path_info", self._h, info.ctypes.data_as(C.POINTER(C.c_int64)))
        keys = ("precision", "structured", "site_classes", "coupling_rows", "chemical_types", "uniform_field",
                "device_bytes")
        return {k: int(v) for k, v in zip(keys, info)}

    def observables(self):
        M = self.lat.mensemble
        mv = np.empty((M, 3))
        ma = np.empty(M)
        en = np.empty(M)
        _lib.call("uppasd_gpu_observables", self._h, _ptr(mv), _ptr(ma), _ptr(en))
        return {"mvec": mv, "mabs": ma, "energy": en}

    def energy_terms(self):
        """Per-ensemble energy terms in mRy/atom: dict of (mensemble,) arrays
        total, xc (the pair energy with an exchange tensor), ani, dm, ext."""
        t = np.empty((self.lat.mensemble, 5))
        _lib.call("uppasd_gpu_energy_terms", self._h, _ptr(t))
        return dict(zip(("total", "xc", "ani", "dm", "ext"), t.T.copy()))

    def calculate_energy(self) -> float:
        """The reference simulator's calculate_energy (uppasd/simulator.py): the total
        energy in mRy per atom, averaged over the ensembles as calc_energy prints it;
        also kept in ``self.energy``."""
        self.energy = float(np.mean(self.energy_terms()["total"]))
        return self.energy


def device_info():
    sm = C.c_int32()
    ma = C.c_int32()
    mi = C.c_int32()
    mem = C.c_int64()
    _lib.call("uppasd_gpu_device_info", C.byref(sm), C.byref(ma), C.byref(mi), C.byref(mem))
    return {"sm_count": sm.value, "cc": (ma.value, mi.value), "hbm_bytes": mem.value}
