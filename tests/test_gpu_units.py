"""Physical constants set through uppasd_gpu_set_units reach every path of a simulation.

The LLG paths see gama only through dt * gama (noise amplitudes 2 lambda k_bolt /
(dt gama mub), rotation angles |B| dt gama), Monte Carlo sees k_bolt only through k_bolt * T,
and energies in mRy scale with mub / mry.  Doubling gama while halving dt (and relaxtime),
or doubling k_bolt while halving T, changes no floating-point value, so the runs must be
bit-identical to the SI ones; doubling mry halves the energies exactly.  The reference's
aunits case itself (all constants 1) is pinned by tests/SCsurf in test_gpu_golden.py.
"""
import numpy as np
import pytest

from uppasd_gb300 import _lib, lattice
from uppasd_gb300.simulation import GpuSimulation

pytestmark = pytest.mark.gpu
SI = (1.760859644e11, 1.38064852e-23, 9.274009994e-24, 2.179872325e-21)


def _rand_unit(rng, shape):
    e = rng.normal(size=shape)
    return e / np.linalg.norm(e, axis=-1, keepdims=True)


def _lattice(kind):
    if kind == "alloy":
        return lattice.bcc_alloy(6, seed=3).with_ensembles(2)
    return lattice.square_dmi(16, 1.0, 0.3, -0.05, 0.5, 1.0).with_ensembles(2)


@pytest.mark.parametrize("prec,solver,kind", [(0, 1, "square"), (0, 4, "square"), (0, 5, "square"), (0, 6, "square"),
                                              (0, 7, "square"), (0, 11, "square"), (3, 1, "square"), (3, 5, "square"),
                                              (3, 7, "square"), (3, 11, "square"),
                                              (1, 5, "alloy"), (2, 5, "alloy")])
def test_llg_time_scale(prec, solver, kind):
    lat = _lattice(kind)
    e0 = _rand_unit(np.random.default_rng(7), (2, lat.natom, 3))
    tau = 1e-15 if solver == 11 else 0.0
    out = []
    for scale in (1.0, 2.0):
        sim = GpuSimulation(lat, sdealgh=solver, delta_t=1e-16 / scale, damping=0.1, temperature=200.0, seed=5,
                            emom=e0, precision=prec, relaxtime=tau / scale)
        if scale != 1.0:
            sim.set_units(SI[0] * scale, SI[1], SI[2], SI[3])
        sim.evolve(40)
        out.append(sim.get_moments())
        sim.close()
    assert np.array_equal(out[0], out[1])


@pytest.mark.parametrize("prec,mode,structured", [(0, "H", False), (0, "M", False), (3, "H", False), (3, "M", False),
                                                  (0, "H", True)])
def test_mc_temperature_scale(prec, mode, structured):
    lat = _lattice("square")
    if structured:   # the structured square heat bath takes no anisotropy
        lat.taniso = lat.eaniso = lat.kaniso = lat.sb = None
    e0 = _rand_unit(np.random.default_rng(8), (2, lat.natom, 3))
    out, en = [], []
    for scale in (1.0, 2.0):
        sim = GpuSimulation(lat, emom=e0, seed=9, precision=prec, sdealgh=5)
        if scale != 1.0:
            sim.set_units(SI[0], SI[1] * scale, SI[2], SI[3] * scale)
        # 40 K and 20 K both absorb the + 1e-15 of the Metropolis acceptance
        sim.relax(mode, 40.0 / scale, 3, structured=structured)
        out.append(sim.get_moments())
        en.append(sim.energy_terms()["total"] * scale)
        sim.close()
    assert np.array_equal(out[0], out[1])
    assert np.array_equal(en[0], en[1])


def test_parallel_tempering_scale():
    lat = _lattice("square").with_ensembles(4)
    e0 = _rand_unit(np.random.default_rng(10), (4, lat.natom, 3))
    # temperatures whose halves still absorb the reference's + 1e-15 in the swap rule
    temps = np.array([50.0, 100.0, 200.0, 400.0])
    res = []
    for scale in (1.0, 2.0):
        sim = GpuSimulation(lat, emom=e0, seed=11, sdealgh=5)
        if scale != 1.0:
            sim.set_units(SI[0], SI[1] * scale, SI[2], SI[3] * scale)
        t, trials, swaps, best = sim.parallel_tempering(temps / scale, 20, 2)
        res.append((sim.get_moments(), t * scale, trials, swaps, best))
        sim.close()
    assert np.array_equal(res[0][0], res[1][0])
    assert np.array_equal(res[0][1], res[1][1]) and res[0][2:] == res[1][2:]


def test_set_units_rejects_bad_values():
    sim = GpuSimulation(_lattice("square"), sdealgh=5)
    for bad in ((0.0, 1.0, 1.0, 1.0), (1.0, -1.0, 1.0, 1.0), (1.0, 1.0, float("nan"), 1.0)):
        with pytest.raises(_lib.UppasdGpuError) as ex:
            sim.set_units(*bad)
        assert ex.value.rc == -1
    sim.close()


def test_structured_set_temperature():
    """The structured path takes the thermal amplitude by value: set_temperature refreshes
    it (the run equals one created at that temperature) and refuses a non-uniform one."""
    lat = _lattice("alloy")
    e0 = _rand_unit(np.random.default_rng(12), (2, lat.natom, 3))
    out = []
    for t0 in (0.0, 300.0):
        sim = GpuSimulation(lat, sdealgh=5, temperature=t0, seed=13, emom=e0, precision=1)
        sim.evolve(3)
        sim.put_moments(e0)
        sim.set_step(0)
        sim.set_temperature(300.0)
        sim.evolve(30)
        out.append(sim.get_moments())
        if t0 == 0.0:
            t = np.full(lat.natom, 300.0)
            t[0] = 310.0
            with pytest.raises(_lib.UppasdGpuError) as ex:
                sim.set_temperature(t)
            assert ex.value.rc == -7
        sim.close()
    assert np.array_equal(out[0], out[1])
