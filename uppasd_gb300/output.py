"""Reference-compatible output files, so runs through this library can be checked
by the reference's own regression harness (its tests read these files by column).

* ``AveragesFile``  -- ``averages.<simid>.out`` of prn_avrg
  (Measurement/prn_averages.f90:566-651): per measurement, the ensemble means of
  the average moment vector and of its norm, and the ensemble standard deviation
  of the norm; header ``(a8,6a16)``, rows ``(i8,6es16.8)`` (``(es12.4,6es16.8)``
  with real time).
* ``CumulantsFile`` -- ``cumulants.<simid>.out`` of calc_and_print_cumulant
  (prn_averages.f90:919-1095): running averages whose weights grow by one per
  sample, Binder cumulant, susceptibility and specific heat in the reference's
  units, written every ``cumu_buff`` samples; rows ``(i8,10es16.8)``.
* ``TotEnergyFile`` -- ``totenergy.<simid>.out`` (and ``stdenergy.<simid>.out`` for
  several ensembles) of calc_energy (Hamiltonian/energy.f90:407-500): the ensemble mean
  of each energy term in mRy/atom, header ``(a8,16a20)`` and rows ``(i8,14es16.8)``;
  with an exchange tensor the pair-energy layout, header ``(a8,11a16)``, rows
  ``(i8,11es16.8)``.  The deviation file holds calculate_mean_and_deviation's value
  (:577-602): the ensemble variance over M - 1, times mub/mry.
* ``ProjAvgsFile`` -- ``projavgs.<simid>.out`` of prn_proj_avrg
  (prn_averages.f90:662-804): averages projected per atom type ('Y') or per basis
  atom ('A'), see ``projected_averages``.
* ``write_restart`` -- the legacy ``restart.<simid>.out`` of prnrestart
  (System/restart.f90:720-751): ``(i8)`` step, then ``(i8,i8,2x,4es16.8)`` per atom.
* ``write_restart_std`` -- the restart file of prn_mag_conf_iter with type 'R'
  (System/restart.f90:186-246), what the reference writes and reads by default
  (do_mom_legacy = 'N'): a seven-line header, then ``(i8,i8,i8,2x,4es16.8)`` per atom.
* ``read_restart`` -- read_mag_conf_std (System/restart.f90:320-381) for either layout:
  moments normalised as there, the step from the file.
* ``sd_run_with_averages`` -- the measurement cadence of sd_mphase: a row every
  ``avrg_step`` steps starting at iteration 0.
"""
from __future__ import annotations

import math
import os
from typing import Optional

import numpy as np

KBOLT = 1.38064852e-23
MUB = 9.274009994e-24
MRY = 2.179872325e-21
DBL_TOLERANCE = float(np.float32(1e-14))


def fortran_es(x: float, width: int = 16, digits: int = 8) -> str:
    """Fortran ``ESw.d``: one digit before the point; exponents beyond two digits drop the E."""
    s = f"{float(x):.{digits}E}"
    mant, exp = s.split("E")
    e = int(exp)
    tail = f"E{e:+03d}" if abs(e) < 100 else f"{e:+04d}"
    return (mant + tail).rjust(width)


def fortran_a(s: str, width: int) -> str:
    """Fortran ``Aw`` output: right-justified in the field, truncated on the right."""
    return s[:width].rjust(width)


class AveragesFile:
    HEADER = ("#Iter", "<M>_x", "<M>_y", "<M>_z", "<M>", "M_{stdv}")

    def __init__(self, path: str, real_time: bool = False):
        self.path = path
        self.real_time = real_time
        self._first = not os.path.exists(path)

    def write(self, index, mvec_per_atom):
        """mvec_per_atom: (Mensemble, 3) = sum of emomM over atoms / Natom per ensemble."""
        mv = np.asarray(mvec_per_atom, dtype=np.float64).reshape(-1, 3)
        m = np.sqrt(np.sum(mv * mv, axis=1))
        mvm = mv.mean(axis=0)
        mm = m.mean()
        ms = np.mean(m * m) - mm * mm  # the reference divides by Mensemble, not Mensemble - 1
        ms = 0.0 if ms < DBL_TOLERANCE else math.sqrt(ms)
        with open(self.path, "a") as f:
            if self._first:
                head = ("Time[s]",) + self.HEADER[1:] if self.real_time else self.HEADER
                f.write(fortran_a(head[0], 12 if self.real_time else 8) +
                        "".join(fortran_a(h, 16) for h in head[1:]) + "\n")
                self._first = False
            lead = fortran_es(index, 12, 4) if self.real_time else f"{int(index):8d}"
            f.write(lead + "".join(fortran_es(v) for v in (*mvm, mm, ms)) + "\n")


class CumulantsFile:
    HEADER = ("#Iter", "<M>", "<M^2>", "<M^4>", "U_{Binder}", "\\chi", "C_v(tot)", "<E>", "<E_{exc}>",
              "<E_{lsf}>")

    def __init__(self, path: str, natom: int, temperature: float, cumu_buff: int = 1):
        self.path, self.natom, self.temp, self.cumu_buff = path, int(natom), float(temperature), int(cumu_buff)
        self.cumuw = self.cumutotw = 0.0
        self.m = self.m2 = self.m4 = self.e = self.e2 = self.exc = 0.0
        self.navrgcum = 0
        self.mensemble = None
        self._first = not os.path.exists(path)

    def add(self, mabs, energy=None, energy_xc=None):
        """One measurement: |M| per ensemble (muB/atom), total (and exchange) energy per
        ensemble in mRy/atom or None.  Returns the row (<M>, <M^2>, <M^4>, U, chi, Cv, <E>,
        <E_exc>, <E_lsf>) after the update."""
        mabs = np.atleast_1d(np.asarray(mabs, dtype=np.float64))
        self.mensemble = mabs.size
        cumulant = chi = cv = 0.0
        for k in range(mabs.size):
            me = mabs[k]
            self.cumuw += 1.0
            w0, w = self.cumutotw, self.cumuw
            self.m = (self.m * w0 + me * w) / (w0 + w)
            self.m2 = (self.m2 * w0 + me * me * w) / (w0 + w)
            self.m4 = (self.m4 * w0 + me ** 4 * w) / (w0 + w)
            cumulant = 1.0 - self.m4 / 3.0 / (self.m2 * self.m2)
            if self.temp > 0.0:
                chi = (self.m2 - self.m * self.m) * MUB * MUB * self.natom / (KBOLT * KBOLT) / self.temp
            else:
                chi = (self.m2 - self.m * self.m) * self.natom * MUB * MUB / KBOLT
            if energy is not None and self.temp > 0.0:
                en = float(np.atleast_1d(energy)[k])
                self.e = (self.e * w0 + en * w) / (w0 + w)
                self.e2 = (self.e2 * w0 + en * en * w) / (w0 + w)
                if energy_xc is not None:
                    ex = float(np.atleast_1d(energy_xc)[k])
                    self.exc = (self.exc * w0 + ex * w) / (w0 + w)
                cv = (self.e2 - self.e * self.e) * MRY * MRY * self.natom / (KBOLT * KBOLT) / (self.temp ** 2)
            self.navrgcum += 1
            self.cumutotw += self.cumuw
        row = (self.m, self.m2, self.m4, cumulant, chi, cv, self.e, self.exc, 0.0)
        n = self.navrgcum // self.mensemble
        if (n - 1) % self.cumu_buff == 0:
            with open(self.path, "a") as f:
                if self._first:
                    f.write(fortran_a(self.HEADER[0], 8) + "".join(fortran_a(h, 16) for h in self.HEADER[1:]) + "\n")
                    self._first = False
                f.write(f"{n:8d}" + "".join(fortran_es(v) for v in row) + "\n")
        return row


class TotEnergyFile:
    HEADER = ("#Iter", "Tot", "Exc", "Ani", "DM", "PD", "BiqDM", "BQ", "Dip", "Zeeman", "LSF", "Chir", "Ring", "SA")
    HEADER_TENSOR = ("#Iter", "Tot", "Heis-Tens", "Ani", "PD", "BiqDM", "BQ", "Dip", "Zeeman", "LSF", "Chir",
                     "Ring")

    def __init__(self, path: str, tensor: bool = False, std_path: Optional[str] = None):
        self.path, self.std_path, self.tensor = path, std_path, bool(tensor)
        self._first = {p: not os.path.exists(p) for p in (path, std_path) if p}

    def _columns(self, t):
        """Term values in the file's column order; terms absent from this library are 0."""
        z = np.zeros_like(t["total"])
        if self.tensor:
            return [t["total"], t["xc"], t["ani"], z, z, z, z, t["ext"], z, z, z]
        return [t["total"], t["xc"], t["ani"], t["dm"], z, z, z, z, t["ext"], z, z, z, z]

    def _write(self, path, index, vals):
        with open(path, "a") as f:
            if self._first[path]:
                head = self.HEADER_TENSOR if self.tensor else self.HEADER
                w = 16 if self.tensor else 20
                f.write(fortran_a(head[0], 8) + "".join(fortran_a(h, w) for h in head[1:]) + "\n")
                self._first[path] = False
            f.write(f"{int(index):8d}" + "".join(fortran_es(v) for v in vals) + "\n")

    def write(self, index, terms):
        """terms: dict of per-ensemble arrays in mRy/atom (GpuSimulation.energy_terms())."""
        cols = [np.atleast_1d(np.asarray(c, dtype=np.float64)) for c in self._columns(terms)]
        m = cols[0].size
        fcinv = MUB / MRY
        means = [c.mean() if m > 1 else c[0] for c in cols]
        self._write(self.path, index, means)
        if self.std_path and m > 1:
            # calculate_mean_and_deviation works on the unscaled values and scales once
            devs = [np.sum((c / fcinv - mu / fcinv) ** 2) / (m - 1.0) * fcinv for c, mu in zip(cols, means)]
            self._write(self.std_path, index, devs)
        return means


def projected_averages(emomM, types, ncells: int, mode: str = "Y"):
    """The rows of prn_proj_avrg (Measurement/prn_averages.f90:462-513, :662-804): the
    moments summed per basis atom (atom i belongs to basis atom mod(i-1, NA)+1), divided
    by the number of cells and summed per atom type (mode 'Y') or kept per basis atom
    ('A'); then per projection the ensemble means of the vector and of its norm and the
    ensemble deviation of the norm.  emomM (Mensemble, Natom, 3); types: the type of
    each basis atom (1-based).  Returns (nproj, 5) rows <M>, M_stdv, <M>_x, <M>_y, <M>_z."""
    e = np.asarray(emomM, dtype=np.float64)
    types = np.asarray(types, dtype=np.int64)
    na = types.size
    per_b = np.stack([e[:, b::na].sum(axis=1) for b in range(na)], axis=1) / ncells   # (M, NA, 3)
    if mode.upper() == "Y":
        proj = np.stack([per_b[:, types == t].sum(axis=1) for t in range(1, int(types.max()) + 1)], axis=1)
    elif mode.upper() == "A":
        proj = per_b
    else:
        raise ValueError("mode is 'Y' (per type) or 'A' (per basis atom)")
    norm = np.sqrt(np.sum(proj * proj, axis=2))                                       # (M, nproj)
    mm = norm.mean(axis=0)
    ms = np.mean(norm * norm, axis=0) - mm * mm
    ms = np.where(ms < 0.0, 0.0, np.sqrt(np.maximum(ms, 0.0)))
    return np.column_stack([mm, ms, proj.mean(axis=0)])


class ProjAvgsFile:
    """``projavgs.<simid>.out`` of prn_proj_avrg: header ``(a8,a,5a16)``, per projection a
    row ``(i8,i8,5es16.8)`` (``(es16.4,i8,5es16.8)`` with real time)."""
    HEADER = ("#Iter", "Proj", "<M>", "M_{stdv}", "<M>_x", "<M>_y", "<M>_z")

    def __init__(self, path: str, types, ncells: int, mode: str = "Y", real_time: bool = False):
        self.path, self.types, self.ncells, self.mode, self.real_time = path, types, int(ncells), mode, real_time
        self._first = not os.path.exists(path)

    def write(self, index, emomM):
        rows = projected_averages(emomM, self.types, self.ncells, self.mode)
        with open(self.path, "a") as f:
            if self._first:
                head = ("Time[s]",) + self.HEADER[1:] if self.real_time else self.HEADER
                f.write(fortran_a(head[0], 16 if self.real_time else 8) + head[1] +
                        "".join(fortran_a(h, 16) for h in head[2:]) + "\n")
                self._first = False
            lead = fortran_es(index, 16, 4) if self.real_time else f"{int(index):8d}"
            for k, r in enumerate(rows):
                f.write(lead + f"{k + 1:8d}" + "".join(fortran_es(v) for v in r) + "\n")
        return rows


def write_restart(path: str, mstep: int, emom, mmom):
    """emom (Mensemble, Natom, 3) unit vectors, mmom (Mensemble, Natom)."""
    emom = np.asarray(emom, dtype=np.float64)
    mmom = np.broadcast_to(np.asarray(mmom, dtype=np.float64), emom.shape[:2])
    with open(path, "w") as f:
        f.write(f"{int(mstep):8d}\n")
        for k in range(emom.shape[0]):
            for i in range(emom.shape[1]):
                f.write(f"{k + 1:8d}{i + 1:8d}  " + fortran_es(mmom[k, i]) +
                        "".join(fortran_es(v) for v in emom[k, i]) + "\n")


def write_restart_std(path: str, mstep: int, emom, mmom, mode: str = "S"):
    """emom (Mensemble, Natom, 3) unit vectors, mmom (Mensemble, Natom)."""
    emom = np.asarray(emom, dtype=np.float64)
    mmom = np.broadcast_to(np.asarray(mmom, dtype=np.float64), emom.shape[:2])
    m, n = emom.shape[:2]
    with open(path, "w") as f:
        f.write("#" * 80 + "\n")
        f.write("# File type: R\n")
        f.write(f"# Simulation type: {mode}\n")
        f.write(f"# Number of atoms:  {n:8d}\n")
        f.write(f"# Number of ensembles:  {m:8d}\n")
        f.write("#" * 80 + "\n")
        f.write("".join(fortran_a(h, w) for h, w in (("# iter", 8), ("ens", 8), ("iatom", 8), ("|Mom|", 16),
                                                      ("M_x", 16), ("M_y", 16), ("M_z", 16))) + "\n")
        for k in range(m):
            for i in range(n):
                f.write(f"{int(mstep):8d}{k + 1:8d}{i + 1:8d}  " + fortran_es(mmom[k, i]) +
                        "".join(fortran_es(v) for v in emom[k, i]) + "\n")


def read_restart(path: str, natom: int, mensemble: int):
    """(step, emom (Mensemble, Natom, 3) normalised, mmom (Mensemble, Natom)) from either the
    standard (seven header lines) or the legacy restart layout."""
    with open(path) as f:
        lines = f.read().splitlines()
    if lines and lines[0].startswith("#"):
        rows = [ln.split() for ln in lines[7:] if ln.strip()]
        step = int(rows[0][0])
        vals = np.array([[float(v) for v in r[3:7]] for r in rows[:natom * mensemble]])
    else:
        step = int(lines[0].split()[0])
        rows = [ln.split() for ln in lines[1:] if ln.strip()]
        vals = np.array([[float(v) for v in r[2:6]] for r in rows[:natom * mensemble]])
    if vals.shape[0] != natom * mensemble:
        raise ValueError(f"{path}: {vals.shape[0]} moments, expected {natom * mensemble}")
    vals = vals.reshape(mensemble, natom, 4)
    e = vals[..., 1:4]
    e = e / np.sqrt(np.sum(e * e, axis=-1))[..., None]
    return step, np.ascontiguousarray(e), np.ascontiguousarray(vals[..., 0])


def read_columns(path: str):
    """The reference harness's reading: whitespace-split rows, '#' lines skipped."""
    rows = []
    with open(path) as f:
        for line in f:
            if line.strip() and not line.lstrip().startswith("#"):
                rows.append([float(v) for v in line.split()])
    return np.array(rows)


def sd_run_with_averages(sim, nsteps: int, avrg_step: int, path: str):
    """sd_mphase's measurement cadence: a row at iteration 0 and every avrg_step steps
    (mstep - 1 divisible by avrg_step), then the steps up to the next measurement."""
    f = AveragesFile(path)
    natom = sim.lat.natom
    it = 0
    while it <= nsteps:
        full = sim.get_moments(full=True)
        emomM = full[1] if isinstance(full, tuple) else full
        f.write(it, emomM.sum(axis=1) / natom)
        if it == nsteps:
            break
        n = min(avrg_step, nsteps - it)
        sim.evolve(n)
        it += n
    return f
