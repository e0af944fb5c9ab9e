"""The CPU oracle against the reference's own golden vectors.

Each case replays a regression case of UppASD's test suite
(tests/regulartests.yaml) through the oracle and compares with the value the
reference printed, using the suite's own comparison (``similar``: |d| <= 1e-8 plus the
9-significant-digit print rounding,
``sloppy``: |d| <= 2e-2 and relative < 2e-2; tests/bergtest.py:42-75).
"""
import ctypes as C
import os

import numpy as np
import pytest

from oracle import pyoracle as po
from uppasd_gb300 import lattice


def _check(got, pin):
    exp = np.asarray(pin["expected"], dtype=np.float64)
    got = np.asarray(got, dtype=np.float64)
    if pin["comparison"] == "similar":
        # The golden values are printed with 9 significant digits (es16.8), so
        # the comparison allows that rounding on top of the suite's 1e-8.
        printed = 0.5 * 10.0 ** (np.floor(np.log10(np.abs(exp) + 1e-300)) - 8)
        assert np.all(np.abs(got - exp) <= 1e-8 + printed), (got, exp)
    else:
        assert np.all((np.abs(got - exp) <= 2e-2) & (np.abs((got - exp) / exp) < 2e-2)), (got, exp)


@pytest.mark.parametrize("solver,name", [(1, "solvers_midpoint"), (4, "solvers_heun"), (5, "solvers_depondt")])
def test_solvers_chain_T0(pins, solver, name):
    """tests/Solvers: 100-spin chain, random start from mtprng seed 1, T=0, 8000 steps."""
    inp = pins["inputs"]["solvers"]
    n = inp["ncell"][2]
    lat = lattice.chain(n, inp["j_mry"], inp["mom"])
    o = po.Oracle(lat, threads=1)
    o.init_random(inp["tseed_default"])
    o.setup_ziggurat(inp["tseed_default"])
    o.make_llg(solver, inp["timestep"], inp["damping"], inp["temp"], 1.0, noise_mode=po.NOISE_ZIGGURAT)
    for _ in range(inp["nstep_checked"]):
        o.sd_step()
    mv, ma = o.mavg()
    _check(list(mv[0] / n) + [ma[0]], pins[name])


def _bccfe(pins):
    inp = pins["inputs"]["bccfe"]
    lat = lattice.bcc(inp["ncell"][0], inp["j_mry"], inp["mom"])
    o = po.Oracle(lat, threads=1)
    e = np.zeros((1, lat.natom, 3))
    e[..., :] = inp["emom0"]
    o.set_moments(e)
    o.mt = po.OrcMT()
    o.lib.orc_mt_init(C.byref(o.mt), inp["tseed"])
    o.setup_ziggurat(inp["tseed"])
    return inp, lat, o


def _cumulant_row(o, lat, inp, step_fn, row_wanted):
    """Replays the measurement loop order: measure (cumulant every cumu_step),
    energy every avrg_step, then one step (sd_driver.f90:554-579, mc_driver.f90:321-366)."""
    cum = po.OrcCumulant()
    energy = np.zeros(1)
    out = np.zeros(6)
    row = 0
    s = 0
    while True:
        s += 1
        if s % inp["cumu_step"] == 0:
            o.lib.orc_cumulant_update(C.byref(cum), lat.natom, 1, po._p(o.emomM), inp["temp"], po._p(energy), po._p(out))
            row += 1
            if row == row_wanted:
                return out
        if (s - 1) % inp["avrg_step"] == 0:
            energy[:] = o.energy()["total"]
        step_fn(s)


def test_bccfe_sd_T500(pins):
    """tests/bccFe mode S: midpoint at 500 K with the ziggurat stream (tseed 5)."""
    inp, lat, o = _bccfe(pins)
    o.make_llg(1, inp["ip_timestep"], inp["ip_damping"], inp["ip_temp"], 1.0, noise_mode=po.NOISE_ZIGGURAT)
    for _ in range(inp["ip_nstep"]):
        o.sd_step()
    mv, ma = o.mavg()
    _check(list(mv[0] / lat.natom) + [ma[0]], pins["bccfe_sd_iter0"])
    o.llg.delta_t = float(np.float32(inp["timestep_default_real4"]))
    for _ in range(2700):
        o.sd_step()
    mv, ma = o.mavg()
    _check(list(mv[0] / lat.natom) + [ma[0]], pins["bccfe_sd_iter2700"])


def test_bccfe_sd_cumulants(pins):
    inp, lat, o = _bccfe(pins)
    o.make_llg(1, inp["ip_timestep"], inp["ip_damping"], inp["ip_temp"], 1.0, noise_mode=po.NOISE_ZIGGURAT)
    for _ in range(inp["ip_nstep"]):
        o.sd_step()
    o.llg.delta_t = float(np.float32(inp["timestep_default_real4"]))
    out = _cumulant_row(o, lat, inp, lambda s: o.sd_step(), 41)
    _check(out, pins["bccfe_sd_cumulants"])


def _mc_initial_phase(o, mode, nsweep, temp):
    """mc_iphase (mc_driver.f90:45-140): permutation redrawn every nsweep/10 sweeps."""
    iflip = o.choose_random_atom_x()
    for s in range(1, nsweep + 1):
        o.mc_sweep_ref(mode, temp, iflip)
        if s % (nsweep // 10) == 0:
            iflip = o.choose_random_atom_x()


@pytest.mark.parametrize("mode,prefix", [("M", "bccfe_mc"), ("H", "bccfe_hb")])
def test_bccfe_mc(pins, mode, prefix):
    inp, lat, o = _bccfe(pins)
    _mc_initial_phase(o, mode, inp["ip_nstep"], inp["ip_temp"])
    mv, ma = o.mavg()
    got0 = list(mv[0] / lat.natom) + [ma[0]]
    pin0 = pins[prefix + "_iter0"]
    _check(got0[-len(pin0["expected"]):], pin0)
    iflip = o.choose_random_atom_x()
    nstep = 3000
    for s in range(1, 2701):
        o.mc_sweep_ref(mode, inp["temp"], iflip)
        if s % (nstep // 10) == 0:
            iflip = o.choose_random_atom_x()
    mv, ma = o.mavg()
    got = list(mv[0] / lat.natom) + [ma[0]]
    pin = pins[prefix + "_iter2700"]
    _check(got[-len(pin["expected"]):], pin)


def test_bccfe_mc_cumulants(pins):
    inp, lat, o = _bccfe(pins)
    _mc_initial_phase(o, "M", inp["ip_nstep"], inp["ip_temp"])
    state = {"iflip": o.choose_random_atom_x()}
    nstep = 3000

    def step(s):
        o.mc_sweep_ref("M", inp["temp"], state["iflip"])
        if s % (nstep // 10) == 0:
            state["iflip"] = o.choose_random_atom_x()

    out = _cumulant_row(o, lat, inp, step, 41)
    _check(out, pins["bccfe_mc_cumulants"])


def from_tables(inp):
    """The lattice of a reference test directory, from the tables make_golden.py stored."""
    return lattice.from_tables(inp["cell"], inp["ncell"], inp["bc"], inp["sites"], inp["jfile"], sym=inp["sym"],
                               dmfile=inp.get("dmfile"), kfile=inp.get("kfile"), reduce=inp["do_reduced"],
                               maptype=inp.get("maptype", 1), aunits=inp.get("aunits", False),
                               posfiletype=inp.get("posfiletype", "C"), tensor=bool(inp.get("do_jtensor", 0)))


def restart_moments(inp):
    """Initmag 4: the restart file's moments, normalised (System/restart.f90:320-381)."""
    r = np.asarray(inp["restart"], dtype=np.float64)
    return (r[:, 1:4] / np.sqrt(np.sum(r[:, 1:4] ** 2, axis=1))[:, None])[None]


def _energy_columns(e, pin):
    cols = {"E_tot": e["total"], "E_xc": e["xc"], "E_ani": e["ani"], "E_DM": e["dm"]}
    return [float(cols[c][0]) for c in pin["extract"]]


def test_heisstripe(pins):
    """tests/HeisStripe: 10 x 1 x 100 simple-cubic stripe, vacuum in x and y (edge atoms keep 3
    of the 4 neighbours the cubic images of (0, 0, 1) give), uniaxial anisotropy along y,
    midpoint at T = 0 from the mtprng initmag-1 draw: <m> after 1190 steps and the
    totenergy columns E_tot, E_xc, E_ani after 1460."""
    inp = pins["inputs"]["heisstripe"]
    lat, _ = from_tables(inp)
    assert sorted(set(lat.nlistsize.tolist())) == [3, 4]
    o = po.Oracle(lat, threads=1)
    o.init_random(inp["tseed_default"])
    o.setup_ziggurat(inp["tseed_default"])
    o.make_llg(inp["sdealgh"], inp["timestep"], inp["damping"], inp["temp"], 1.0, noise_mode=po.NOISE_ZIGGURAT)
    for _ in range(1190):
        o.sd_step()
    mv, ma = o.mavg()
    _check(list(mv[0] / lat.natom) + [ma[0]], pins["heisstripe_iter1190"])
    for _ in range(1460 - 1190):
        o.sd_step()
    _check(_energy_columns(o.energy(), pins["heisstripe_energy1460"]), pins["heisstripe_energy1460"])


def test_kagome(pins):
    """tests/kagome: 12 x 12 kagome cells, exchange and DMI from the jfile / dmfile, reduced
    Hamiltonian (three coupling rows), Initmag 3, midpoint at T = 0: the trajectory of
    atom 2 after 2400 steps and <m> after 13000."""
    inp = pins["inputs"]["kagome"]
    lat, e0 = from_tables(inp)
    assert lat.nham == 3 and lat.do_dm
    o = po.Oracle(lat, threads=1)
    o.set_moments(e0)
    o.setup_ziggurat(inp["tseed_default"])
    o.make_llg(inp["sdealgh"], inp["timestep"], inp["damping"], inp["temp"], 1.0, noise_mode=po.NOISE_ZIGGURAT)
    for _ in range(2400):
        o.sd_step()
    pin = pins["kagome_traj2400"]
    _check([2.0] + list(o.emom[0, 1]) + [o.mmom[0, 1]], pin)
    for _ in range(13000 - 2400):
        o.sd_step()
    mv, ma = o.mavg()
    _check(list(mv[0] / lat.natom) + [ma[0]], pins["kagome_iter13000"])


def test_heischain(pins):
    """tests/HeisChain: 100-spin chain from its restart file (Initmag 4), an initial phase of
    20000 midpoint steps at 0.1 K with damping 4 on the ziggurat stream, then undamped T = 0
    precession: <m> after 1000 measurement steps and E_tot after 1400."""
    inp = pins["inputs"]["heischain"]
    lat, _ = from_tables(inp)
    o = po.Oracle(lat, threads=1)
    o.set_moments(restart_moments(inp))
    o.setup_ziggurat(inp["tseed_default"])
    for nstep, temp, dt, damping in inp["ip_phases"]:
        o.make_llg(inp["sdealgh"], dt, damping, temp, 1.0, noise_mode=po.NOISE_ZIGGURAT)
        for _ in range(int(nstep)):
            o.sd_step()
    o.make_llg(inp["sdealgh"], inp["timestep"], inp["damping"], inp["temp"], 1.0, noise_mode=po.NOISE_ZIGGURAT)
    for _ in range(1000):
        o.sd_step()
    mv, ma = o.mavg()
    _check(list(mv[0] / lat.natom) + [ma[0]], pins["heischain_iter1000"])
    for _ in range(400):
        o.sd_step()
    _check(_energy_columns(o.energy(), pins["heischain_energy1400"]), pins["heischain_energy1400"])


def test_heischainaf(pins, tmp_path):
    """tests/HeisChainAF: ferrimagnetic chain, two basis atoms of moments 1 and 2, two shells
    per type from the cubic images of the jfile vectors, midpoint at T = 0 from the mtprng
    initmag-1 draw: <m> after 1000 steps, E_tot after 1500 and the per-type projected
    averages after 5000, read back from a projavgs file by the suite's columns."""
    inp = pins["inputs"]["heischainaf"]
    lat, _ = from_tables(inp)
    o = po.Oracle(lat, threads=1)
    o.init_random(inp["tseed_default"])
    o.setup_ziggurat(inp["tseed_default"])
    o.make_llg(inp["sdealgh"], inp["timestep"], inp["damping"], inp["temp"], 1.0, noise_mode=po.NOISE_ZIGGURAT)
    for _ in range(1000):
        o.sd_step()
    mv, ma = o.mavg()
    _check(list(mv[0] / lat.natom) + [ma[0]], pins["heischainaf_iter1000"])
    for _ in range(500):
        o.sd_step()
    _check(_energy_columns(o.energy(), pins["heischainaf_energy1500"]), pins["heischainaf_energy1500"])
    for _ in range(3500):
        o.sd_step()
    check_projavgs(o.emomM, lat, inp, pins, str(tmp_path / "projavgs.AF_WireT.out"))


def check_projavgs(emomM, lat, inp, pins, path):
    from uppasd_gb300 import output
    types = [int(s[0]) for s in inp["sites"]]
    output.ProjAvgsFile(path, types, int(np.prod(inp["ncell"]))).write(5000, emomM)
    cols = ["#_Iter.", "#_Atom", "M_avg", "M_avg_d", "M_avg_x", "M_avg_y", "M_avg_z"]
    rows = output.read_columns(path)
    for t in (1, 2):
        row = dict(zip(cols, rows[(rows[:, 0] == 5000) & (rows[:, 1] == t)][0]))
        pin = pins["heischainaf_proj5000_type%d" % t]
        _check([row[c] for c in pin["extract"]], pin)


def test_feco(pins):
    """tests/FeCo: B2 FeCo, 6^3 cells, two species of moments 2.72 and 1.72, 258 neighbours per
    atom from a maptype-2 exchange table (cell offsets), reduced Hamiltonian, Initmag 3 with
    canted sublattices, midpoint at T = 0 with damping 0.001: the cumulant row 221 (sampled
    every 20 steps) and <M> after 4700 steps, both compared as the suite does (``sloppy``).
    The cumulants agree with the reference's to all printed digits; <M> differs by 2e-4."""
    inp = pins["inputs"]["feco"]
    lat, e0 = from_tables(inp)
    assert lat.nham == 2 and lat.max_no_neigh == 258
    o = po.Oracle(lat, threads=1)
    o.set_moments(e0)
    o.setup_ziggurat(inp["tseed_default"])
    o.make_llg(inp["sdealgh"], inp["timestep"], inp["damping"], inp["temp"], 1.0, noise_mode=po.NOISE_ZIGGURAT)
    steps = {"n": 0}

    def step(s):
        o.sd_step()
        steps["n"] += 1

    out = _cumulant_row(o, lat, inp, step, 221)
    _check(out[:4], pins["feco_cumulants221"])
    assert np.allclose(out[:4], pins["feco_cumulants221"]["expected"], rtol=5e-9, atol=0)
    for _ in range(4700 - steps["n"]):
        o.sd_step()
    mv, ma = o.mavg()
    _check([ma[0]], pins["feco_iter4700"])


def test_scsurf_atomic_units(pins):
    """tests/SCsurf: 16 x 16 square monolayer in atomic units (aunits 'Y': gama = k_bolt =
    mub = mry = 1), antiferromagnetic exchange, DMI and anisotropy from maptype-2 tables,
    time step 0.01, midpoint at T = 0 from the mtprng initmag-1 draw: <m> after 800 steps."""
    inp = pins["inputs"]["scsurf"]
    assert inp["aunits"]
    lat, _ = from_tables(inp)
    with po.units(po.ATOMIC_UNITS):
        o = po.Oracle(lat, threads=1)
        o.init_random(inp["tseed_default"])
        o.setup_ziggurat(inp["tseed_default"])
        o.make_llg(inp["sdealgh"], inp["timestep"], inp["damping"], inp["temp"], 1.0, noise_mode=po.NOISE_ZIGGURAT)
        for _ in range(800):
            o.sd_step()
        mv, ma = o.mavg()
    _check(list(mv[0] / lat.natom) + [ma[0]], pins["scsurf_iter800"])


# The reference's GPU cases (tests/cudatests.yaml) run its CUDA path (gpu_mode 1), whose only
# integrator is Depondt (gpu_files/cudaDepondtIntegrator.cu) whatever SDEalgh says; with
# SDEalgh 5 the oracle reproduces their cumulant rows to all printed digits.  Their <M> rows
# for bccFe_cuda and FeCo_cuda do not follow from those same runs (the suite compares them
# ``sloppy``) and are kept at that bound.
GPU_CASES = [("kagome_cuda", 1300, 171), ("bccfe_cuda", 1700, 41), ("feco_cuda", 4700, 221)]


def replay_reference_gpu_case(pins, name, mavg_at, cumulant_row, run):
    """Drives `run(nsteps)` (advance) and returns (<M> row at mavg_at, cumulant row) with the
    sampling order of sd_mphase: a cumulant sample every cumu_step steps, taken before the step."""
    from uppasd_gb300 import output
    inp = pins["inputs"][name]
    cf = output.CumulantsFile(os.devnull, 1, inp["temp"], 10 ** 9)
    done, mrow, crow = 0, None, None
    for row in range(1, max(cumulant_row, mavg_at // inp["cumu_step"] + 1) + 1):
        target = row * inp["cumu_step"] - 1
        if mrow is None and mavg_at <= target:
            run["step"](mavg_at - done)
            done = mavg_at
            mrow = run["mavg"]()
        run["step"](target - done)
        done = target
        if row <= cumulant_row:
            out = cf.add(np.linalg.norm(run["mavg"]()[:3]))
            if row == cumulant_row:
                crow = out[:4]
    return mrow, crow


def check_reference_gpu_case(pins, name, mrow, crow):
    exact = pins[name + "_cumulants%d" % {"kagome_cuda": 171, "bccfe_cuda": 41, "feco_cuda": 221}[name]]
    _check(crow, exact)
    assert np.allclose(crow, exact["expected"], rtol=5e-9, atol=0), (crow, exact["expected"])
    mpin = pins[name + "_iter%d" % {"kagome_cuda": 1300, "bccfe_cuda": 1700, "feco_cuda": 4700}[name]]
    _check(mrow[-len(mpin["expected"]):], mpin)


@pytest.mark.parametrize("name,mavg_at,cumulant_row", GPU_CASES)
def test_reference_gpu_cases(pins, name, mavg_at, cumulant_row):
    """kagome_cuda (SKKR exchange tensors from a 9-column jfile, direct coordinates, 13068
    atoms), bccFe_cuda (four cubic shells, two sublattice directions) and FeCo_cuda, all at
    T = 0 with Depondt."""
    inp = pins["inputs"][name]
    lat, e0 = from_tables(inp)
    o = po.Oracle(lat)
    if inp["initmag"] == 1:
        o.init_random(inp["tseed_default"])
    else:
        o.set_moments(e0)
    o.setup_ziggurat(inp["tseed_default"])
    o.make_llg(5, inp["timestep"], inp["damping"], inp["temp"], 1.0, noise_mode=po.NOISE_ZIGGURAT)

    def step(n):
        for _ in range(n):
            o.sd_step()

    def mavg():
        mv, ma = o.mavg()
        return list(mv[0] / lat.natom) + [ma[0]]

    mrow, crow = replay_reference_gpu_case(pins, name, mavg_at, cumulant_row, {"step": step, "mavg": mavg})
    check_reference_gpu_case(pins, name, mrow, crow)


def test_from_tables_matches_the_bcc_builder(pins):
    """The table-driven builder on the bccFe_cuda tables (one type, two sites, four cubic
    shells) gives the same neighbours and couplings as the bcc builder, site by site, and
    the cubic images of the first two shells come in the order get_fullnnlist keeps them."""
    inp = pins["inputs"]["bccfe_cuda"]
    lat, _ = from_tables(inp)
    js = [r[5] for r in inp["jfile"]]
    ref = lattice.bcc(inp["ncell"][0], js, inp["sites"][0][4])
    assert lat.natom == ref.natom and np.array_equal(lat.nlistsize, ref.nlistsize)
    for i in range(lat.natom):
        a = sorted(zip(lat.nlist[i, :lat.nlistsize[i]], lat.ncoup[i, :lat.nlistsize[i]]))
        b = sorted(zip(ref.nlist[i, :ref.nlistsize[i]], ref.ncoup[i, :ref.nlistsize[i]]))
        assert [x[0] for x in a] == [x[0] for x in b]
        assert np.allclose([x[1] for x in a], [x[1] for x in b], rtol=1e-14, atol=0)
    img = [tuple(v) for v in lattice.cubic_images((0.5, 0.5, 0.5))]
    assert len(img) == 8 and img[0] == (0.5, 0.5, 0.5) and img[-1] == (-0.5, -0.5, -0.5)
    assert [tuple(v) for v in lattice.cubic_images((1.0, 0.0, 0.0))][:2] == [(1.0, 0.0, 0.0), (-1.0, 0.0, 0.0)]
