"""The reference's input directory: ``inpsd.dat`` and the tables it names, read into a
lattice, an initial state and the run parameters.

Keywords follow read_parameters (Input/inputhandler.f90:52-1678): a line's first token is
the keyword, compared in lower case; lines starting with ``%``, ``#``, ``*``, ``=`` or
``!`` are comments; a keyword's values are read list-directed from the rest of its line
and, when that line holds too few, the lines after it (``cell`` spans three); file names
are the next token; unknown keywords are skipped with their line.  Fortran ``d``
exponents are accepted.  The tables: posfile rows ``isite itype x y z`` (with do_ralloy 1
``isite itype ichem conc x y z``), momfile rows ``isite ichem mom ex ey ez``, the
exchange, dm and anisotropy files as ``lattice.from_tables`` takes them.  Only what the
spin-update path uses is interpreted; everything else is kept in ``raw``.
"""
from __future__ import annotations

import os
import struct
from typing import Optional

import numpy as np

from . import lattice as _lattice
from . import output as _output

_COMMENT = ("%", "#", "*", "=", "!")
# keyword: (number of values, kind) read list-directed
_VALUES = {
    "ncell": (3, int), "bc": (3, str), "cell": (9, float), "sym": (1, int), "maptype": (1, int),
    "posfiletype": (1, str), "do_ralloy": (1, int), "tseed": (1, int), "aunits": (1, str),
    "do_reduced": (1, str), "mensemble": (1, int), "initmag": (1, int), "sdealgh": (1, int),
    "temp": (1, float), "timestep": (1, float), "damping": (1, float), "nstep": (1, int),
    "mode": (1, str), "hfield": (3, float), "mcnstep": (1, int), "do_jtensor": (1, int),
    "alat": (1, float), "do_dip": (1, int), "simid": (1, str), "gpu_rng_seed": (1, int),
    "ip_mode": (1, str), "ip_nphase": (1, int), "ip_mcanneal": (1, int), "avrg_step": (1, int),
    "cumu_step": (1, int), "cumu_buff": (1, int), "plotenergy": (1, int),
    "theta0": (1, float), "phi0": (1, float), "mavg0": (1, float),
}
_FILES = ("posfile", "momfile", "exchange", "dm", "anisotropy", "restartfile")


def _num(tok: str) -> float:
    return float(tok.replace("d", "e").replace("D", "e"))


def _convert(tok: str, kind):
    if kind is int:
        return int(_num(tok))
    if kind is float:
        return _num(tok)
    return tok.strip("'\"")


def read_inpsd(path: str) -> dict:
    """The keywords of an inpsd.dat file: known ones converted (see the module doc), the
    tokens of every keyword in ``raw``; ``ip_nphase`` brings its phase rows (nstep, temp,
    timestep, damping) as ``ip_phases``."""
    lines = [ln.split() for ln in open(path)]
    out, raw = {}, {}
    i = 0
    while i < len(lines):
        t = lines[i]
        i += 1
        if not t or t[0].startswith(_COMMENT):
            continue
        key, rest = t[0].lower(), t[1:]
        raw.setdefault(key, rest)
        if key in _FILES:
            if rest:
                out[key] = rest[0].strip("'\"")
            continue
        if key not in _VALUES:
            continue
        n, kind = _VALUES[key]
        vals = list(rest)
        while len(vals) < n and i < len(lines):  # list-directed: continue on the next lines
            vals += lines[i]
            i += 1
        vals = [_convert(v, kind) for v in vals[:n]]
        out[key] = vals[0] if n == 1 else vals
        if key == "ip_nphase":
            phases = []
            for _ in range(out[key]):
                row = lines[i]
                i += 1
                phases.append([int(_num(row[0]))] + [_num(v) for v in row[1:4]])
            out["ip_phases"] = phases
    out["raw"] = raw
    return out


def _rows(path: str):
    out = []
    for ln in open(path):
        t = ln.split()
        if t and not t[0].startswith(_COMMENT):
            out.append([_num(v) for v in t])
    return out


def load_system(directory: str, inpsd: str = "inpsd.dat", mensemble: Optional[int] = None):
    """(lattice, emom (mensemble, natom, 3), params) of a reference input directory.

    The lattice is ``lattice.from_tables`` of the tables inpsd.dat names (random alloys
    with do_ralloy 1, their chemical types drawn from tseed as the reference draws them),
    with Mensemble copies and hfield as the external field of every spin.  emom follows
    Initmag (default 4): 1 the reference's random start on its stream after rng_init(tseed)
    (after the alloy's chemical draws), 2 random in the cone of theta0, phi0 (or mavg0) on
    the same stream, 3 the momfile directions, 4 the restart file (directions and moment
    lengths); other values are refused.  params holds the run keywords: mode,
    SDEalgh, Temp, timestep (the reference's REAL(4) default 1e-16 when absent), damping,
    Nstep, mcNstep, Initmag, tseed, ip phases, simid and the rest of ``read_inpsd``."""
    k = read_inpsd(os.path.join(directory, inpsd))

    def table(key):
        return _rows(os.path.join(directory, k[key])) if key in k else None

    for need in ("ncell", "cell", "posfile", "momfile", "exchange"):
        if need not in k:
            raise ValueError(f"{inpsd}: keyword {need} missing")
    cell = np.asarray(k["cell"], dtype=np.float64).reshape(3, 3)
    bc = [str(b).upper() for b in k.get("bc", ["P", "P", "P"])]
    ralloy = int(k.get("do_ralloy", 0)) == 1
    pos, mom = table("posfile"), table("momfile")
    chemistry = None
    if ralloy:
        geo, chemistry = {}, {}
        for r in pos:  # isite itype ichem conc x y z
            isite = int(r[0])
            geo.setdefault(isite, (int(r[1]), r[4], r[5], r[6]))
            chemistry.setdefault(isite, {})[int(r[2])] = r[3]
        moms = {(int(r[0]), int(r[1])): r[2:6] for r in mom}
        chemistry = {s: [(c, conc, *moms[(s, c)]) for c, conc in sorted(chemistry[s].items())]
                     for s in sorted(chemistry)}
        sites = [(geo[s][0], geo[s][1], geo[s][2], geo[s][3], 1.0, 1.0, 0.0, 0.0) for s in sorted(geo)]
    else:
        p = {int(r[0]): r for r in pos}          # isite itype x y z
        m = {int(r[0]): r for r in mom}          # isite ichem mom ex ey ez
        sites = [(p[s][1], p[s][2], p[s][3], p[s][4], *m[s][2:6]) for s in sorted(p)]
    tseed = int(k.get("tseed", 1))
    initmag = int(k.get("initmag", 4))
    if initmag not in (1, 2, 3, 4):
        raise ValueError(f"Initmag {initmag} is not read (1 to 4 are)")
    # the main stream after rng_init(tseed): the alloy's chemical draws, then Initmag 1
    stream = _lattice.MtprngStream(tseed)
    ncells = int(np.prod(k["ncell"]))
    achtype = None
    if ralloy:
        conc = [[r[1] for r in chemistry[s]] for s in sorted(chemistry)]
        achtype = _lattice.random_chemistry(ncells, conc, uniform=stream.real2(len(conc) * ncells))
    lat, emom = _lattice.from_tables(
        cell, tuple(k["ncell"]), bc, sites, table("exchange"), sym=int(k.get("sym", 0)),
        dmfile=table("dm"), kfile=table("anisotropy"),
        reduce=str(k.get("do_reduced", "N")).upper() == "Y", maptype=int(k.get("maptype", 1)),
        aunits=str(k.get("aunits", "N")).upper() == "Y", posfiletype=str(k.get("posfiletype", "C")).upper(),
        tensor=int(k.get("do_jtensor", 0)) == 1, chemistry=chemistry, achtype=achtype)
    M = int(mensemble if mensemble is not None else k.get("mensemble", 1))
    lat = lat.with_ensembles(M)
    if "hfield" in k:
        lat.extfield = np.ascontiguousarray(np.broadcast_to(np.asarray(k["hfield"], dtype=np.float64),
                                                            (M, lat.natom, 3)))
    if initmag in (1, 2):
        nfull = len(sites) * ncells
        u = (_lattice.initmag_random(nfull, stream) if initmag == 1 else
             _lattice.initmag_cone(nfull, stream, float(k.get("theta0", 0.0)), float(k.get("phi0", 0.0)),
                                   float(k.get("mavg0", -1.0))))
        emom = u[achtype > 0] if ralloy else u
        emom = np.ascontiguousarray(np.broadcast_to(emom[None], (M, lat.natom, 3)))
    elif initmag == 4:
        if "restartfile" not in k:
            raise ValueError("Initmag 4 (the default) needs a restartfile")
        _, emom, mm = _output.read_restart(os.path.join(directory, k["restartfile"]), lat.natom, M)
        lat.mmom = mm
    else:
        emom = np.ascontiguousarray(np.broadcast_to(emom[:1], (M, lat.natom, 3)))
    params = {key: v for key, v in k.items() if key not in ("raw",)}
    params.setdefault("timestep", struct.unpack("f", struct.pack("f", 1.0e-16))[0])
    params.setdefault("mode", "S")
    params.setdefault("sdealgh", 1)
    params.setdefault("tseed", tseed)
    params.setdefault("initmag", initmag)
    params["raw"] = k["raw"]
    return lat, emom, params
