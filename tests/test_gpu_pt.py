"""Per-ensemble temperatures and parallel tempering (pt_iphase with the ensembles as
replicas) on the GPU against the oracle's restatement: the FP64 path takes the same
swaps and ends in the same states (1e-12); precision 3 runs the same schedule with
its FP32 heat bath."""
import numpy as np
import pytest

from oracle import pyoracle as po
from uppasd_gb300 import lattice
from uppasd_gb300.simulation import GpuSimulation

pytestmark = pytest.mark.gpu


def _state(lat, seed):
    e = np.random.default_rng(seed).normal(size=(lat.mensemble, lat.natom, 3))
    return e / np.linalg.norm(e, axis=-1, keepdims=True)


@pytest.mark.parametrize("mode", ["H", "M"])
def test_mc_run_temps_chain(mode):
    lat = lattice.square_dmi(16, 1.0, 0.3, -0.05, 0.5, 1.0).with_ensembles(3)
    e0 = _state(lat, 71)
    temps = [8.0, 20.0, 45.0]
    sim = GpuSimulation(lat, emom=e0, seed=19)
    sim.relax_temps(mode, temps, 3)
    g = sim.get_moments()
    sim.close()
    o = po.Oracle(lat)
    o.set_moments(e0)
    _, order, start = lattice.greedy_colouring(lat)
    for sw in range(3):
        o.mc_sweep_checkerboard(mode, 0.0, order, start, 19, sw, temps=temps)
    assert np.max(np.abs(g - o.emom)) <= 1e-12


def test_parallel_tempering_matches_oracle():
    lat = lattice.square_dmi(16, 1.0, 0.3, -0.05, 0.5, 1.0).with_ensembles(6)
    e0 = _state(lat, 72)
    temps = [3.0, 6.0, 10.0, 15.0, 22.0, 30.0]
    sim = GpuSimulation(lat, emom=e0, seed=23)
    T, trial, hit, sel = sim.parallel_tempering(temps, 60, 2)
    g = sim.get_moments()
    sim.close()
    o = po.Oracle(lat)
    o.set_moments(e0)
    _, order, start = lattice.greedy_colouring(lat)
    To, to, ho, so = o.pt_iphase(temps, 60, 2, order, start, 23)
    assert np.array_equal(T, To) and (trial, hit, sel) == (to, ho, so)
    assert hit > 0 and sorted(T) == temps
    assert np.max(np.abs(g - o.emom)) <= 1e-12


def test_parallel_tempering_precision3_runs_the_schedule():
    lat = lattice.kagome(8).with_ensembles(4)
    e0 = _state(lat, 73)
    sim = GpuSimulation(lat, emom=e0, seed=29, precision=3, sdealgh=5)
    T, trial, hit, sel = sim.parallel_tempering([5.0, 10.0, 20.0, 40.0], 40, 2)
    g = sim.get_moments()
    sim.close()
    assert trial == 17 * 3 and 0 <= hit <= trial and sorted(T) == [5.0, 10.0, 20.0, 40.0] and 0 <= sel < 4
    assert np.max(np.abs(np.linalg.norm(g, axis=-1) - 1.0)) < 1e-12
