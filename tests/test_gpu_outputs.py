"""The drop-in's measurement files pass the reference's own regression check:
tests/Solvers (midpoint, Heun, Depondt) run on the GPU with the averages file
written in the reference's format (sd_mphase cadence), read back by columns the
way the reference harness does, row of iteration 8000 against the expected
values of tests/regulartests.yaml (the suite's 'similar' tolerance)."""
import numpy as np
import pytest

from oracle import pyoracle as po
from uppasd_gb300 import lattice, output
from uppasd_gb300.simulation import GpuSimulation

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("solver,name", [(1, "solvers_midpoint"), (4, "solvers_heun"), (5, "solvers_depondt")])
def test_solvers_averages_file_passes_reference_check(pins, solver, name, tmp_path):
    inp = pins["inputs"]["solvers"]
    n = inp["ncell"][2]
    lat = lattice.chain(n, inp["j_mry"], inp["mom"])
    o = po.Oracle(lat)
    o.init_random(inp["tseed_default"])
    sim = GpuSimulation(lat, sdealgh=solver, delta_t=inp["timestep"], damping=inp["damping"],
                        temperature=0.0, emom=o.emom.copy())
    path = str(tmp_path / f"averages.{solver}")
    output.sd_run_with_averages(sim, inp["nstep_checked"], 100, path)
    sim.close()
    cols = output.read_columns(path)
    row = cols[cols[:, 0] == inp["nstep_checked"]][0]
    exp = np.array(pins[name]["expected"])
    got = row[1:5]
    assert np.all(np.abs(got - exp) <= 1e-8 + 0.5 * 10.0 ** (np.floor(np.log10(np.abs(exp))) - 8)), (got, exp)


@pytest.mark.parametrize("kind", ["square_dmi", "kagome_tensor"])
def test_energy_terms_match_oracle_and_write_totenergy(tmp_path, kind):
    from uppasd_gb300 import lattice as lt
    lat = (lt.square_dmi(16, 1.0, 0.3, -0.05, 0.5, 1.0) if kind == "square_dmi"
           else lt.kagome(8, -1.0, 0.1, 0.05, 1.0, 0.2)).with_ensembles(3)
    rng = np.random.default_rng(51)
    e0 = rng.normal(size=(3, lat.natom, 3))
    e0 /= np.linalg.norm(e0, axis=-1, keepdims=True)
    sim = GpuSimulation(lat, emom=e0)
    t = sim.energy_terms()
    o = po.Oracle(lat)
    o.set_moments(e0)
    ref = o.energy()
    for k in ("total", "xc", "dm", "ani", "ext"):
        assert np.allclose(t[k], ref[k], rtol=1e-12, atol=1e-13), k
    f = output.TotEnergyFile(str(tmp_path / "totenergy.x.out"), tensor=lat.j_tens is not None)
    f.write(0, t)
    row = output.read_columns(str(tmp_path / "totenergy.x.out"))[0]
    assert np.isclose(row[1], ref["total"].mean(), rtol=1e-8)
    assert np.isclose(sim.calculate_energy(), ref["total"].mean(), rtol=1e-12) and sim.energy == sim.calculate_energy()
    sim.close()
