"""The CPU oracle against the reference's own golden vectors.

Each case replays a regression case of UppASD's test suite
(tests/regulartests.yaml) through the oracle and compares with the value the
reference printed, using the suite's own comparison (``similar``: |d| <= 1e-8 plus the
9-significant-digit print rounding,
``sloppy``: |d| <= 2e-2 and relative < 2e-2; tests/bergtest.py:42-75).
"""
import ctypes as C

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
