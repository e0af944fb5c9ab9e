"""The reference's input directory read by ``inputs.load_system``: inpsd.dat keywords
with the reference's parsing rules (case, comment markers, values continued on the next
lines, Fortran d exponents, unknown keywords skipped) and the tables it names give the
same lattice as ``lattice.from_tables`` handed the same tables, for a bcc ferromagnet with
anisotropy and an external field and for a random alloy (do_ralloy 1, tseed).  The input
files are written here; their numbers are this test's own."""
import numpy as np
import pytest

from uppasd_gb300 import inputs, lattice


def _write(d, name, text):
    (d / name).write_text(text)


def test_bcc_directory(tmp_path):
    _write(tmp_path, "inpsd.dat", """simid  bccTest
% a comment line
ncell  4 4 4        System size
BC     P P P        Boundary conditions
Cell   1.00000 0.00000 0.00000
       0.00000 1.00000 0.00000
       0.00000 0.00000 1.00000
SYM    1
posfile   ./pos.dat
momfile   ./mom.dat
exchange  ./jij.dat
anisotropy ./k.dat
do_prnstruct 1
Mensemble 3
Initmag 3
mode S
SDEalgh 5
Temp 250.0
timestep 2.0d-16
damping 0.05
Nstep 1200
hfield 0.0 0.0 1.5
ip_mode S
ip_nphase 2
100 10.0 1d-16 0.5
200 5.0 2d-16 0.1
""")
    _write(tmp_path, "pos.dat", "1 1 0.0 0.0 0.0\n2 1 0.5 0.5 0.5\n")
    _write(tmp_path, "mom.dat", "1 1 2.2 0.0 0.0 1.0\n2 1 2.2 0.0 0.0 1.0\n")
    _write(tmp_path, "jij.dat", "# isite jsite r J\n1 1 0.5 0.5 0.5 1.30\n1 1 1.0 0.0 0.0 0.70\n")
    _write(tmp_path, "k.dat", "1 1 0.02 0.0 0.0 0.0 1.0 0.0\n2 1 0.02 0.0 0.0 0.0 1.0 0.0\n")
    lat, emom, par = inputs.load_system(str(tmp_path))
    want, e0 = lattice.from_tables(np.eye(3), (4, 4, 4), "PPP",
                                   [(1, 0.0, 0.0, 0.0, 2.2, 0.0, 0.0, 1.0), (1, 0.5, 0.5, 0.5, 2.2, 0.0, 0.0, 1.0)],
                                   [(1, 1, 0.5, 0.5, 0.5, 1.3), (1, 1, 1.0, 0.0, 0.0, 0.7)], sym=1,
                                   kfile=[(1, 1, 0.02, 0.0, 0.0, 0.0, 1.0, 0.0), (2, 1, 0.02, 0.0, 0.0, 0.0, 1.0, 0.0)])
    assert lat.mensemble == 3 and lat.natom == want.natom == 128
    for name in ("nlist", "nlistsize", "ncoup", "taniso", "kaniso", "eaniso"):
        assert np.array_equal(getattr(lat, name), getattr(want, name)), name
    assert np.array_equal(lat.mmom, np.broadcast_to(want.mmom[:1], (3, 128)))
    assert np.array_equal(lat.extfield, np.broadcast_to([0.0, 0.0, 1.5], (3, 128, 3)))
    assert np.array_equal(emom, np.broadcast_to(e0[:1], (3, 128, 3)))
    assert par["sdealgh"] == 5 and par["mode"] == "S" and par["nstep"] == 1200
    assert par["temp"] == 250.0 and par["timestep"] == 2.0e-16 and par["damping"] == 0.05
    assert par["simid"] == "bccTest" and par["initmag"] == 3
    assert par["ip_phases"] == [[100, 10.0, 1e-16, 0.5], [200, 5.0, 2e-16, 0.1]]
    assert "do_prnstruct" in par["raw"]


def test_defaults(tmp_path):
    _write(tmp_path, "inpsd.dat", "ncell 2 2 2\ncell 1 0 0 0 1 0 0 0 1\nposfile p\nmomfile m\nexchange j\n"
                                  "initmag 3\n")
    _write(tmp_path, "p", "1 1 0 0 0\n")
    _write(tmp_path, "m", "1 1 1.0 1 0 0\n")
    _write(tmp_path, "j", "1 1 1 0 0 1.0\n")
    lat, _, par = inputs.load_system(str(tmp_path))
    assert lat.natom == 8 and lat.mensemble == 1
    # the reference's default time step is a REAL(4) literal
    assert par["timestep"] == float(np.float32(1e-16)) and par["sdealgh"] == 1 and par["mode"] == "S"
    with pytest.raises(ValueError):
        _write(tmp_path, "inpsd.dat", "ncell 2 2 2\nposfile p\n")
        inputs.load_system(str(tmp_path))


def test_random_alloy_directory(tmp_path):
    _write(tmp_path, "inpsd.dat", """ncell 6 6 6
BC P P P
cell 1.0 0.0 0.0
     0.0 1.0 0.0
     0.0 0.0 1.0
Sym 1
maptype 2
do_ralloy 1
tseed 11
Initmag 1
posfile ./posfile
momfile ./momfile
exchange ./jfile
""")
    _write(tmp_path, "posfile", "1 1 1 0.70 0.0 0.0 0.0\n1 1 2 0.30 0.0 0.0 0.0\n"
                                "2 1 1 0.40 0.5 0.5 0.5\n2 1 2 0.60 0.5 0.5 0.5\n")
    _write(tmp_path, "momfile", "1 1 2.00 1 0 0\n1 2 1.50 0 1 0\n2 1 2.00 1 0 0\n2 2 1.50 0 1 0\n")
    jrows = [(1, 1, 1, 1, 0.5, 0.5, 0.5, 1.1), (1, 1, 1, 2, 0.5, 0.5, 0.5, 0.6), (1, 1, 2, 1, 0.5, 0.5, 0.5, 0.6),
             (1, 1, 2, 2, 0.5, 0.5, 0.5, -0.4), (1, 1, 1, 1, 1.0, 0.0, 0.0, 0.3)]
    _write(tmp_path, "jfile", "".join(" ".join(str(v) for v in r) + "\n" for r in jrows))
    lat, emom, par = inputs.load_system(str(tmp_path))
    chem = {1: [(1, 0.7, 2.0, 1, 0, 0), (2, 0.3, 1.5, 0, 1, 0)], 2: [(1, 0.4, 2.0, 1, 0, 0), (2, 0.6, 1.5, 0, 1, 0)]}
    want, e0 = lattice.from_tables(np.eye(3), (6, 6, 6), "PPP", [(1, 0, 0, 0, 1, 1, 0, 0), (1, .5, .5, .5, 1, 1, 0, 0)],
                                   jrows, sym=1, maptype=2, chemistry=chem, tseed=11)
    for name in ("nlist", "nlistsize", "ncoup", "species", "mmom"):
        assert np.array_equal(getattr(lat, name), getattr(want, name)), name
    assert np.array_equal(lat.meta["achtype"], lattice.random_chemistry(216, [(0.7, 0.3), (0.4, 0.6)], seed=11))
    # on 125 cells 0.7 / 0.3 round to 88 + 38 atoms: more than the cells, refused
    with pytest.raises(ValueError):
        lattice.random_chemistry(125, [(0.7, 0.3)], seed=11)
    assert par["tseed"] == 11 and par["do_ralloy"] == 1 and par["initmag"] == 1
    # Initmag 1 on the same stream, after the 2 x 216 chemical draws
    s = lattice.MtprngStream(11)
    s.real2(2 * 216)
    assert np.array_equal(emom[0], lattice.initmag_random(432, s))


def test_restart_start(tmp_path):
    """Initmag 4 (the default): directions and moment lengths from the restart file."""
    _write(tmp_path, "inpsd.dat", "ncell 2 2 1\ncell 1 0 0 0 1 0 0 0 1\nposfile p\nmomfile m\nexchange j\n"
                                  "restartfile ./restart.in\nMensemble 2\n")
    _write(tmp_path, "p", "1 1 0 0 0\n")
    _write(tmp_path, "m", "1 1 1.0 1 0 0\n")
    _write(tmp_path, "j", "1 1 1 0 0 1.0\n")
    rng = np.random.default_rng(2)
    e = rng.normal(size=(2, 4, 3))
    e /= np.linalg.norm(e, axis=-1, keepdims=True)
    mm = 1.0 + rng.random((2, 4))
    from uppasd_gb300 import output
    output.write_restart_std(str(tmp_path / "restart.in"), 0, e, mm)
    lat, emom, par = inputs.load_system(str(tmp_path))
    assert par["initmag"] == 4 and lat.mensemble == 2
    assert np.allclose(emom, e, atol=1e-8) and np.allclose(lat.mmom, mm, atol=1e-8)
    _write(tmp_path, "inpsd.dat", "ncell 2 2 1\ncell 1 0 0 0 1 0 0 0 1\nposfile p\nmomfile m\nexchange j\n"
                                  "initmag 6\n")
    with pytest.raises(ValueError):
        inputs.load_system(str(tmp_path))


def test_cone_start(tmp_path):
    """Initmag 2: two draws per atom in the cone theta0 (radians) about z; mavg0 >= 0
    replaces the cone by theta0 = 2 acos(mavg0), phi0 = 2 pi."""
    _write(tmp_path, "p", "1 1 0 0 0\n")
    _write(tmp_path, "m", "1 1 1.0 1 0 0\n")
    _write(tmp_path, "j", "1 1 1 0 0 1.0\n")
    base = "ncell 4 4 4\ncell 1 0 0 0 1 0 0 0 1\nposfile p\nmomfile m\nexchange j\ninitmag 2\ntseed 9\n"
    _write(tmp_path, "inpsd.dat", base + "theta0 0.3\nphi0 6.283185307179586\n")
    _, emom, _ = inputs.load_system(str(tmp_path))
    r = lattice.mtprng_real2(9, 128).reshape(64, 2)
    want = np.stack([np.sin(0.3 * r[:, 0]) * np.cos(2 * np.pi * r[:, 1]),
                     np.sin(0.3 * r[:, 0]) * np.sin(2 * np.pi * r[:, 1]), np.cos(0.3 * r[:, 0])], axis=1)
    assert np.array_equal(emom[0], want)
    assert np.all(emom[0, :, 2] >= np.cos(0.3) - 1e-15)
    _write(tmp_path, "inpsd.dat", base + "mavg0 0.9\n")
    _, emom, _ = inputs.load_system(str(tmp_path))
    assert np.all(emom[0, :, 2] >= np.cos(2 * np.arccos(0.9)) - 1e-15)


def _fmt(v):
    return repr(float(v)) if isinstance(v, float) else str(v)


def _write_case(d, inp, extra=""):
    """A pinned regression case's tables written back out as an input directory (the
    tables stored in the golden fixture, in the reference's file layouts)."""
    sites = inp["sites"]
    _write(d, "posfile", "".join(f"{i + 1} {int(s[0])} {s[1]} {s[2]} {s[3]}\n" for i, s in enumerate(sites)))
    _write(d, "momfile", "".join(f"{i + 1} 1 {s[4]} {s[5]} {s[6]} {s[7]}\n" for i, s in enumerate(sites)))
    _write(d, "jfile", "".join(" ".join(_fmt(v) for v in r) + "\n" for r in inp["jfile"]))
    text = (f"ncell {' '.join(str(n) for n in inp['ncell'])}\nBC {' '.join(inp['bc'])}\n"
            "cell " + "\n     ".join(" ".join(repr(float(v)) for v in row) for row in inp["cell"]) + "\n"
            f"Sym {inp['sym']}\nmaptype {inp['maptype']}\nposfiletype {inp['posfiletype']}\n"
            "posfile ./posfile\nmomfile ./momfile\nexchange ./jfile\n"
            f"Initmag {inp['initmag']}\nSDEalgh {inp['sdealgh']}\nTemp {inp['temp']}\n"
            f"timestep {inp['timestep']!r}\ndamping {inp['damping']}\nmode S\nNstep {inp['nstep']}\n")
    for key, name, word in (("kfile", "kfile", "anisotropy"), ("dmfile", "dmfile", "dm")):
        if key in inp:
            _write(d, name, "".join(" ".join(_fmt(v) for v in r) + "\n" for r in inp[key]))
            text += f"{word} ./{name}\n"
    if inp.get("aunits"):
        text += "aunits Y\n"
    if "restart" in inp:   # rows |m|, m_x, m_y, m_z per atom, written in the standard layout
        from uppasd_gb300 import output
        r = np.asarray(inp["restart"], dtype=np.float64)
        output.write_restart_std(str(d / "restart.in"), 0, r[None, :, 1:4], r[None, :, 0])
        text += "restartfile ./restart.in\n"
    if "ip_phases" in inp:
        text += f"ip_mode S\nip_nphase {len(inp['ip_phases'])}\n" + "".join(
            f"{int(n)} {t!r} {dt!r} {dmp!r}\n" for n, t, dt, dmp in inp["ip_phases"])
    _write(d, "inpsd.dat", text + extra)


@pytest.mark.parametrize("case,steps,pin", [("heisstripe", 1190, "heisstripe_iter1190"),
                                            ("scsurf", 800, "scsurf_iter800"),
                                            ("heischain", 1000, "heischain_iter1000")])
def test_pinned_case_through_the_reader(tmp_path, case, steps, pin):
    """Pinned regression cases end to end through the reader: the tables of tests/HeisStripe
    (vacuum edges, anisotropy), tests/SCsurf (atomic units, maptype 2, DM and anisotropy)
    and tests/HeisChain (a restart-file start, Initmag 4, and an initial phase) written as
    input directories, read by load_system (Initmag 1 drawn from the default tseed), run on
    the oracle with each directory's phases, solver, time steps and damping: <m> equals the
    reference's printed value."""
    import json
    import os
    from oracle import pyoracle as po
    here = os.path.dirname(os.path.abspath(__file__))
    pins = json.load(open(os.path.join(here, "golden", "reference_pins.json")))
    _write_case(tmp_path, pins["inputs"][case])
    lat, e0, par = inputs.load_system(str(tmp_path))
    with po.units(po.ATOMIC_UNITS if str(par.get("aunits", "N")).upper() == "Y" else po.SI_UNITS):
        o = po.Oracle(lat, threads=1)
        o.set_moments(e0)
        o.setup_ziggurat(par["tseed"])
        if str(par.get("ip_mode", "N")).upper() == "S":
            for nstep, temp, dt, damping in par.get("ip_phases", []):
                o.make_llg(par["sdealgh"], dt, damping, temp, 1.0, noise_mode=po.NOISE_ZIGGURAT)
                for _ in range(int(nstep)):
                    o.sd_step()
        o.make_llg(par["sdealgh"], par["timestep"], par["damping"], par["temp"], 1.0, noise_mode=po.NOISE_ZIGGURAT)
        for _ in range(steps):
            o.sd_step()
        mv, ma = o.mavg()
    got = np.array(list(mv[0] / lat.natom) + [ma[0]])
    pin = pins[pin]
    exp = np.asarray(pin["expected"])
    printed = 0.5 * 10.0 ** (np.floor(np.log10(np.abs(exp) + 1e-300)) - 8)
    assert np.all(np.abs(got - exp) <= 1e-8 + printed), (got, exp)
