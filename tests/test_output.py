"""Reference-format output files (uppasd_gb300/output.py): Fortran ES/A editing,
the cumulant bookkeeping against the oracle's restatement of
calc_and_print_cumulant (itself pinned to the reference's cumulant rows), and
round trips through the reference harness's column reading."""
import ctypes as C

import numpy as np

from oracle import pyoracle as po
from uppasd_gb300 import output


def test_fortran_edit_descriptors():
    assert output.fortran_es(1.5) == "  1.50000000E+00"
    assert output.fortran_es(-1.23e-4) == " -1.23000000E-04"
    assert output.fortran_es(0.0) == "  0.00000000E+00"
    assert output.fortran_es(1e-120) == "  1.00000000-120"
    assert output.fortran_es(2.5e3, 12, 4) == "  2.5000E+03"
    assert output.fortran_a("#Iter", 8) == "   #Iter"


def test_cumulants_match_oracle(tmp_path):
    rng = np.random.default_rng(4)
    natom, M, T = 128, 2, 640.0
    cu = po.OrcCumulant()
    lib = po.load()
    f = output.CumulantsFile(str(tmp_path / "cumulants.test.out"), natom, T)
    out = (C.c_double * 6)()
    for _ in range(30):
        e = rng.normal(size=(M, natom, 3)) + np.array([0.0, 0.0, 1.0])
        e /= np.linalg.norm(e, axis=-1, keepdims=True)
        emomM = np.ascontiguousarray(2.2 * e)
        en = rng.normal(size=M) - 7.0
        lib.orc_cumulant_update(C.byref(cu), natom, M, emomM.ctypes.data_as(po.F64P), T,
                                np.ascontiguousarray(en).ctypes.data_as(po.F64P), out)
        mabs = np.linalg.norm(emomM.sum(axis=1), axis=1) / natom
        row = f.add(mabs, en)
        assert np.allclose(row[:6], list(out), rtol=1e-12, atol=0)
    cols = output.read_columns(str(tmp_path / "cumulants.test.out"))
    assert cols.shape == (30, 10) and cols[-1, 0] == 30
    assert np.allclose(cols[-1, 1:7], list(out), rtol=1e-8)


def test_averages_and_restart_round_trip(tmp_path):
    rng = np.random.default_rng(2)
    p = str(tmp_path / "averages.test.out")
    f = output.AveragesFile(p)
    mv = rng.normal(size=(3, 3))
    f.write(0, mv)
    f.write(100, mv * 0.5)
    cols = output.read_columns(p)
    m = np.linalg.norm(mv, axis=1)
    assert cols.shape == (2, 6) and cols[1, 0] == 100
    assert np.allclose(cols[0, 1:4], mv.mean(axis=0), rtol=1e-8)
    assert np.isclose(cols[0, 4], m.mean(), rtol=1e-8)
    assert np.isclose(cols[0, 5], np.sqrt(np.mean(m * m) - m.mean() ** 2), rtol=1e-7)
    e = rng.normal(size=(2, 5, 3))
    e /= np.linalg.norm(e, axis=-1, keepdims=True)
    r = str(tmp_path / "restart.test.out")
    output.write_restart(r, 1234, e, np.full((2, 5), 2.2))
    lines = open(r).read().splitlines()
    assert lines[0].strip() == "1234" and len(lines) == 11
    vals = np.array([[float(v) for v in ln.split()] for ln in lines[1:]])
    assert np.allclose(vals[:, 3:], e.reshape(-1, 3), atol=1e-8) and np.all(vals[:, 2] == 2.2)


def test_totenergy_layout_and_deviation(tmp_path):
    rng = np.random.default_rng(5)
    terms = {k: rng.normal(size=4) for k in ("xc", "ani", "dm", "ext")}
    terms["total"] = terms["xc"] + terms["ani"] + terms["dm"] + terms["ext"]
    f = output.TotEnergyFile(str(tmp_path / "totenergy.t.out"), std_path=str(tmp_path / "stdenergy.t.out"))
    f.write(0, terms)
    f.write(10, terms)
    lines = open(tmp_path / "totenergy.t.out").read().splitlines()
    assert len(lines[0]) == 8 + 13 * 20 and lines[0].split()[:3] == ["#Iter", "Tot", "Exc"]
    assert all(len(l) == 8 + 13 * 16 for l in lines[1:])
    cols = output.read_columns(str(tmp_path / "totenergy.t.out"))
    assert cols[:, 0].tolist() == [0, 10]
    want = [terms[k].mean() for k in ("total", "xc", "ani", "dm")] + [0.0] * 4 + [terms["ext"].mean()]
    assert np.allclose(cols[0, 1:10], want, rtol=1e-8, atol=1e-12)
    fc = output.MUB / output.MRY
    std = output.read_columns(str(tmp_path / "stdenergy.t.out"))
    assert np.isclose(std[0, 1], np.var(terms["total"] / fc, ddof=1) * fc, rtol=1e-8)
    t = output.TotEnergyFile(str(tmp_path / "totenergy.j.out"), tensor=True)
    t.write(0, terms)
    lines = open(tmp_path / "totenergy.j.out").read().splitlines()
    assert lines[0].split()[2] == "Heis-Tens" and len(lines[0]) == 8 + 11 * 16
    assert len(lines[1]) == 8 + 11 * 16


def test_restart_layouts_round_trip(tmp_path, pins):
    """The reference's default restart layout (prn_mag_conf_iter) and the legacy one read back
    by read_restart as read_mag_conf_std does; the HeisChain start file's moments (taken from
    the reference's tests/HeisChain/startmom) survive a write and a read to the printed digits."""
    rows = np.asarray(pins["inputs"]["heischain"]["restart"])
    e = rows[:, 1:4][None]
    m = rows[:, 0][None]
    for writer, name in ((output.write_restart_std, "restart.std.out"), (output.write_restart, "restart.leg.out")):
        p = str(tmp_path / name)
        writer(p, 0, e, m)
        step, e2, m2 = output.read_restart(p, rows.shape[0], 1)
        assert step == 0 and np.array_equal(m2, m)
        assert np.max(np.abs(e2 - e / np.linalg.norm(e, axis=-1, keepdims=True))) < 1e-8
    lines = open(tmp_path / "restart.std.out").read().splitlines()
    assert lines[0] == "#" * 80 and lines[1] == "# File type: R" and len(lines) == 7 + rows.shape[0]
    assert lines[7].split()[:3] == ["0", "1", "1"] and len(lines[7]) == 24 + 2 + 4 * 16


def test_lattice_coordinates(pins):
    """Positions in the reference's numbering: the HeisStripe tables (x fastest), the bcc
    pair basis and the kagome basis."""
    from uppasd_gb300 import lattice
    inp = pins["inputs"]["heisstripe"]
    lat, _ = lattice.from_tables(inp["cell"], inp["ncell"], inp["bc"], inp["sites"], inp["jfile"], sym=inp["sym"])
    c = lat.coords
    i = np.arange(lat.natom)
    assert np.array_equal(c, np.stack([i % 10, np.zeros_like(i), i // 10], axis=1).astype(float))
    b = lattice.bcc(3, [1.0], 1.0).coords
    assert np.allclose(b[1], [0.5, 0.5, 0.5]) and np.allclose(b[2], [1.0, 0.0, 0.0])
    k = lattice.kagome(2).coords
    assert np.allclose(k[1], [0.5, 0.0, 0.0]) and np.allclose(k[3], [1.0, 0.0, 0.0])
    assert np.allclose(np.linalg.norm(k[2]), 0.5)
