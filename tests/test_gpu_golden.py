"""The GPU's FP64 path against the reference's own golden values (tests/regulartests.yaml):
HeisStripe (vacuum edges, ragged neighbour lists, uniaxial anisotropy, totenergy columns),
kagome (DMI, reduced Hamiltonian), HeisChain (restart start, initial phase on the
reference's ziggurat stream, undamped precession), HeisChainAF (two moments, per-type
projected averages), FeCo (maptype-2 table, 258 neighbours, reduced, cumulants), SCsurf
(atomic units through uppasd_gpu_set_units) and the suite's GPU cases kagome_cuda (exchange
tensors), bccFe_cuda and FeCo_cuda.  Lattices are built from the reference's
input tables by ``lattice.from_tables``; start states the reference draws from its own
generators (mtprng initmag 1, ziggurat noise) come from the oracle's restatement of them.
Same comparison as the suite (``similar``: 1e-8 plus the 9-digit print rounding)."""
import numpy as np
import pytest

from oracle import pyoracle as po
from test_oracle_golden import (GPU_CASES, _check, _energy_columns, check_projavgs, check_reference_gpu_case,
                                from_tables, replay_reference_gpu_case, restart_moments)
from uppasd_gb300.simulation import GpuSimulation

pytestmark = pytest.mark.gpu


def _mavg(sim, lat):
    e = sim.get_moments()
    m = np.sum(e[0] * lat.mmom[0][:, None], axis=0) / lat.natom
    return list(m) + [np.linalg.norm(m)]


def test_heisstripe_on_gpu(pins):
    inp = pins["inputs"]["heisstripe"]
    lat, _ = from_tables(inp)
    o = po.Oracle(lat)
    o.init_random(inp["tseed_default"])
    sim = GpuSimulation(lat, sdealgh=inp["sdealgh"], delta_t=inp["timestep"], damping=inp["damping"],
                        temperature=inp["temp"], emom=o.emom.copy())
    sim.evolve(1190)
    _check(_mavg(sim, lat), pins["heisstripe_iter1190"])
    sim.evolve(1460 - 1190)
    _check(_energy_columns(sim.energy_terms(), pins["heisstripe_energy1460"]), pins["heisstripe_energy1460"])
    sim.close()


def test_kagome_on_gpu(pins):
    inp = pins["inputs"]["kagome"]
    lat, e0 = from_tables(inp)
    sim = GpuSimulation(lat, sdealgh=inp["sdealgh"], delta_t=inp["timestep"], damping=inp["damping"],
                        temperature=inp["temp"], emom=e0)
    sim.evolve(2400)
    _check([2.0] + list(sim.get_moments()[0, 1]) + [lat.mmom[0, 1]], pins["kagome_traj2400"])
    sim.evolve(13000 - 2400)
    _check(_mavg(sim, lat), pins["kagome_iter13000"])
    sim.close()


def test_heischain_on_gpu(pins):
    inp = pins["inputs"]["heischain"]
    lat, _ = from_tables(inp)
    e = restart_moments(inp)
    (nstep, temp, dt, damping), = inp["ip_phases"]
    nstep = int(nstep)
    normals = po.ziggurat_stream(inp["tseed_default"], nstep * 3 * lat.natom).reshape(nstep, 1, lat.natom, 3)
    sim = GpuSimulation(lat, sdealgh=inp["sdealgh"], delta_t=dt, damping=damping, temperature=temp, emom=e)
    sim.set_noise(normals)
    sim.evolve(nstep)
    e = sim.get_moments()
    sim.close()
    # measurement phase: new damping and temperature; midpoint carries no state but the moments
    sim = GpuSimulation(lat, sdealgh=inp["sdealgh"], delta_t=inp["timestep"], damping=inp["damping"],
                        temperature=inp["temp"], emom=e)
    sim.evolve(1000)
    _check(_mavg(sim, lat), pins["heischain_iter1000"])
    sim.evolve(400)
    _check(_energy_columns(sim.energy_terms(), pins["heischain_energy1400"]), pins["heischain_energy1400"])
    sim.close()


def test_heischainaf_on_gpu(pins, tmp_path):
    inp = pins["inputs"]["heischainaf"]
    lat, _ = from_tables(inp)
    o = po.Oracle(lat)
    o.init_random(inp["tseed_default"])
    sim = GpuSimulation(lat, sdealgh=inp["sdealgh"], delta_t=inp["timestep"], damping=inp["damping"],
                        temperature=inp["temp"], emom=o.emom.copy())
    sim.evolve(1000)
    _check(_mavg(sim, lat), pins["heischainaf_iter1000"])
    sim.evolve(500)
    _check(_energy_columns(sim.energy_terms(), pins["heischainaf_energy1500"]), pins["heischainaf_energy1500"])
    sim.evolve(3500)
    e = sim.get_moments()
    check_projavgs(e * lat.mmom[..., None], lat, inp, pins, str(tmp_path / "projavgs.AF_WireT.out"))
    sim.close()


def test_feco_on_gpu(pins, tmp_path):
    from uppasd_gb300 import output
    inp = pins["inputs"]["feco"]
    lat, e0 = from_tables(inp)
    sim = GpuSimulation(lat, sdealgh=inp["sdealgh"], delta_t=inp["timestep"], damping=inp["damping"],
                        temperature=inp["temp"], emom=e0)
    cf = output.CumulantsFile(str(tmp_path / "cumulants.test"), lat.natom, inp["temp"], inp["cumu_buff"])
    done = 0
    for row in range(221):
        # sample `row + 1` is taken before step (row + 1) * cumu_step runs
        target = (row + 1) * inp["cumu_step"] - 1
        sim.evolve(target - done)
        done = target
        out = cf.add(np.linalg.norm(_mavg(sim, lat)[:3]))
    _check(out[:4], pins["feco_cumulants221"])
    assert np.allclose(out[:4], pins["feco_cumulants221"]["expected"], rtol=5e-9, atol=0)
    sim.evolve(4700 - done)
    _check([_mavg(sim, lat)[3]], pins["feco_iter4700"])
    sim.close()


def test_scsurf_atomic_units_on_gpu(pins):
    inp = pins["inputs"]["scsurf"]
    lat, _ = from_tables(inp)
    with po.units(po.ATOMIC_UNITS):
        o = po.Oracle(lat)
        o.init_random(inp["tseed_default"])
    sim = GpuSimulation(lat, sdealgh=inp["sdealgh"], delta_t=inp["timestep"], damping=inp["damping"],
                        temperature=inp["temp"], emom=o.emom.copy())
    sim.set_atomic_units()
    sim.evolve(800)
    _check(_mavg(sim, lat), pins["scsurf_iter800"])
    sim.close()


@pytest.mark.parametrize("name,mavg_at,cumulant_row", GPU_CASES)
def test_reference_gpu_cases_on_gpu(pins, name, mavg_at, cumulant_row):
    """The reference's own GPU cases (its CUDA path integrates with Depondt)."""
    inp = pins["inputs"][name]
    lat, e0 = from_tables(inp)
    if inp["initmag"] == 1:
        o = po.Oracle(lat)
        o.init_random(inp["tseed_default"])
        e0 = o.emom.copy()
    sim = GpuSimulation(lat, sdealgh=5, delta_t=inp["timestep"], damping=inp["damping"], temperature=inp["temp"],
                        emom=e0)
    mrow, crow = replay_reference_gpu_case(pins, name, mavg_at, cumulant_row,
                                           {"step": lambda n: sim.evolve(n) if n else None,
                                            "mavg": lambda: _mavg(sim, lat)})
    check_reference_gpu_case(pins, name, mrow, crow)
    sim.close()
