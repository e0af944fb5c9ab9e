"""Reduced Hamiltonian (aHam(i) = anumb(i), nHam = NA) on the GPU: the coupling rows are
read through aham in every kernel, so a reduced table gives bit-identical results to the
full one on each path (FP64 LLG and Monte Carlo, structured bcc LLG, structured square
heat bath), and the FP64 path matches the oracle run on the reduced table."""
import numpy as np
import pytest

from oracle import pyoracle as po
from uppasd_gb300 import lattice
from uppasd_gb300.simulation import GpuSimulation

pytestmark = pytest.mark.gpu


def _rand_unit(rng, shape):
    e = rng.normal(size=shape)
    return e / np.linalg.norm(e, axis=-1, keepdims=True)


LATTICES = {
    "bcc": lambda: lattice.bcc(4, [1.3, 0.7], 2.2),
    "square_dmi": lambda: lattice.square_dmi(16, 1.0, 0.3, -0.05, 0.5, 1.0),
    "kagome_tensor": lambda: lattice.kagome(8, -1.0, 0.1, 0.05, 1.0, 0.2),
}


def _run(lat, e0, **kw):
    sim = GpuSimulation(lat, sdealgh=5, delta_t=1e-16, damping=0.1, temperature=200.0, seed=3, emom=e0, **kw)
    sim.evolve(100)
    sim.relax("M", 40.0, 2)
    out = sim.get_moments(), sim.observables()["energy"]
    sim.close()
    return out


@pytest.mark.parametrize("kind", sorted(LATTICES))
def test_reduced_fp64_path(kind):
    full = LATTICES[kind]().with_ensembles(2)
    red = lattice.reduced(full)
    e0 = _rand_unit(np.random.default_rng(41), (2, full.natom, 3))
    mf, ef = _run(full, e0)
    mr, er = _run(red, e0)
    assert np.array_equal(mf, mr) and np.array_equal(ef, er)
    o = po.Oracle(red)
    o.set_moments(e0)
    o.make_llg(5, 1e-16, 0.1, 200.0, 1.0, noise_mode=po.NOISE_PHILOX, seed=3)
    for _ in range(100):
        o.sd_step()
    _, order, start = lattice.greedy_colouring(red)
    for sw in range(2):
        o.mc_sweep_checkerboard("M", 40.0, order, start, 3, sw)
    assert np.max(np.abs(mr - o.emom)) <= 1e-9


def test_reduced_structured_bcc_llg():
    full = lattice.bcc(6, [1.3, 0.7], 2.2)
    e0 = _rand_unit(np.random.default_rng(42), (1, full.natom, 3))
    runs = []
    for lat in (full, lattice.reduced(full)):
        sim = GpuSimulation(lat, sdealgh=5, delta_t=1e-16, damping=0.1, temperature=300.0, seed=8, emom=e0,
                            precision=1)
        sim.evolve(64)
        runs.append(sim.get_moments())
        sim.close()
    assert np.array_equal(runs[0], runs[1])


def test_reduced_structured_square_heat_bath():
    full = lattice.square_dmi(32, 1.0, 0.3, 0.0, 0.5, 1.0).with_ensembles(2)
    e0 = _rand_unit(np.random.default_rng(43), (2, full.natom, 3))
    runs = []
    for lat in (full, lattice.reduced(full)):
        sim = GpuSimulation(lat, emom=e0, seed=12)
        sim.relax("H", 5.0, 20, structured=True)
        runs.append(sim.get_moments())
        sim.close()
    assert np.array_equal(runs[0], runs[1])
