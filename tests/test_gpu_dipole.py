"""GPU dipole-dipole field (do_dip 1 and 3) through the C ABI against the oracle.

The field alone to 1e-12 (brute force) and 1e-10 (FFT) of its largest component, on
cubic, skewed and non-cubic cell grids; FP64 LLG trajectories with the field on within
1e-9 per spin component of the oracle's after 200 steps; the energy with the dipolar
term; checkerboard Monte Carlo chains with the field against the oracle's.
"""
import numpy as np
import pytest

from oracle import pyoracle as po
from uppasd_gb300 import _lib, lattice
from uppasd_gb300.simulation import GpuSimulation

from test_oracle_dipole import ALAT, coords_of, grid_lattice, pair_sum, rand_moments

pytestmark = pytest.mark.gpu
TOL_FIELD = {1: 1e-12, 3: 1e-10}
TOL_TRAJ = 1e-9

GRIDS = [
    ((4, 4, 4), [[0, 0, 0], [0.5, 0.5, 0.5]], np.eye(3)),
    ((3, 4, 5), [[0, 0, 0], [0.5, 0.3, 0.2]], [[1.0, 0.0, 0.0], [0.5, 0.8660254037844386, 0.0], [0.1, 0.2, 1.3]]),
    ((6, 2, 1), [[0, 0, 0], [0.5, 0, 0], [0, 0.5, 0]], [[1.0, 0.0, 0.0], [0.5, 0.8660254037844386, 0.0], [0, 0, 1.0]]),
]


@pytest.mark.parametrize("mode", [1, 3])
@pytest.mark.parametrize("grid", range(len(GRIDS)))
def test_field_matches_oracle(mode, grid):
    cells, basis, cell = GRIDS[grid]
    lat = grid_lattice(*cells, basis, cell, mensemble=2)
    e = rand_moments(np.random.default_rng(10 + grid), lat)
    sim = GpuSimulation(lat, emom=e)
    sim.set_dipole(mode, ALAT)
    b = sim.get_fields()  # no exchange: the dipolar field alone
    o = po.Oracle(lat, dipole_alat=ALAT)
    o.set_moments(e)
    ref = o.dipole_field()
    scale = np.max(np.abs(ref))
    assert scale > 0
    assert np.max(np.abs(b - ref)) <= TOL_FIELD[mode] * scale
    sim.set_dipole(0)
    assert np.max(np.abs(sim.get_fields())) == 0.0
    sim.close()


def test_brute_force_caller_coordinates():
    """do_dip = 1 over the caller's coordinates (setup_qdip takes coord)."""
    lat = grid_lattice(4, 3, 2, [[0, 0, 0]], np.eye(3), mensemble=1)
    rng = np.random.default_rng(4)
    coord = coords_of(lat) + 0.2 * rng.uniform(-1, 1, size=(lat.natom, 3))
    e = rand_moments(rng, lat)
    sim = GpuSimulation(lat, emom=e)
    sim.set_dipole(1, ALAT, coord=coord)
    b = sim.get_fields()
    _, em = sim.get_moments(full=True)
    ref = pair_sum(coord, em, ALAT)
    assert np.max(np.abs(b - ref)) <= 1e-12 * np.max(np.abs(ref))
    sim.close()


@pytest.mark.parametrize("mode", [1, 3])
@pytest.mark.parametrize("solver, temp", [(5, 0.0), (5, 300.0), (1, 300.0)])
def test_llg_with_dipoles_200_steps(mode, solver, temp):
    lat = lattice.bcc(4, [1.3, 0.7], 2.2).with_ensembles(2)
    e0 = rand_moments(np.random.default_rng(5), lat)
    sim = GpuSimulation(lat, sdealgh=solver, delta_t=1e-16, damping=0.1, temperature=temp, seed=9, emom=e0)
    sim.set_dipole(mode, ALAT)
    o = po.Oracle(lat, dipole_alat=ALAT)
    o.set_moments(e0)
    o.make_llg(solver, 1e-16, 0.1, temp, 1.0, noise_mode=po.NOISE_PHILOX, seed=9)
    nsteps = 200
    sim.evolve(nsteps)
    for _ in range(nsteps):
        o.sd_step()
    g = sim.get_moments()
    assert np.max(np.abs(g - o.emom)) <= TOL_TRAJ
    # the dipolar field moves the trajectory far beyond the tolerance
    o0 = po.Oracle(lat)
    o0.set_moments(e0)
    o0.make_llg(solver, 1e-16, 0.1, temp, 1.0, noise_mode=po.NOISE_PHILOX, seed=9)
    for _ in range(nsteps):
        o0.sd_step()
    assert np.max(np.abs(o0.emom - o.emom)) > 1e3 * TOL_TRAJ
    sim.close()


@pytest.mark.parametrize("mode", [1, 3])
def test_energy_and_field_with_exchange(mode):
    lat = lattice.bcc(4, [1.3, 0.7], 2.2).with_ensembles(2)
    e = rand_moments(np.random.default_rng(6), lat)
    sim = GpuSimulation(lat, emom=e)
    sim.set_dipole(mode, ALAT)
    o = po.Oracle(lat, dipole_alat=ALAT)
    o.set_moments(e)
    ref_b, _ = o.field()
    assert np.max(np.abs(sim.get_fields() - ref_b)) <= 1e-12 * np.max(np.abs(ref_b))
    ref_e = o.energy()["total"]
    got = sim.energy_terms()["total"]
    assert np.allclose(got, ref_e, rtol=1e-11, atol=0)
    sim.close()


@pytest.mark.parametrize("mode", ["M", "H"])
@pytest.mark.parametrize("do_dip", [1, 3])
def test_monte_carlo_chain_with_dipoles(mode, do_dip):
    """Checkerboard Metropolis (field of the sweep's start in the external field) and heat
    bath (field refreshed before each colour) against the oracle's chain, per spin."""
    # weak exchange at low temperature: dipolar energies comparable to k_B T
    lat = lattice.bcc(4, [0.02, 0.01], 2.2).with_ensembles(2)
    e0 = rand_moments(np.random.default_rng(8), lat)
    T = 5.0
    sim = GpuSimulation(lat, emom=e0, seed=123)
    sim.set_dipole(do_dip, ALAT)
    sim.relax(mode, T, 3)
    o = po.Oracle(lat, dipole_alat=ALAT)
    o.set_moments(e0)
    _, order, start = lattice.greedy_colouring(lat)
    for sw in range(3):
        o.mc_sweep_checkerboard(mode, T, order, start, 123, sw)
    tol = 1e-12 if do_dip == 1 else 1e-9
    assert np.max(np.abs(sim.get_moments() - o.emom)) <= tol
    # the dipolar field changes the chain
    o0 = po.Oracle(lat)
    o0.set_moments(e0)
    for sw in range(3):
        o0.mc_sweep_checkerboard(mode, T, order, start, 123, sw)
    assert np.max(np.abs(o0.emom - o.emom)) > 1e-6
    sim.close()


def test_square_heat_bath_and_learned_refuse_while_on():
    lat = lattice.square_dmi(16, 1.0, 0.3, 0.0, 0.5, 1.0)
    sim = GpuSimulation(lat)
    sim.set_dipole(1, ALAT)
    with pytest.raises(_lib.UppasdGpuError) as ei:
        sim.relax("H", 20.0, 1, structured=True)
    assert ei.value.rc == -7
    sim.set_dipole(0)
    sim.relax("H", 20.0, 1, structured=True)
    sim.close()


def test_rejects_structured_path_and_bad_grid():
    lat = lattice.bcc(6, [1.3, 0.7], 2.2)
    sim = GpuSimulation(lat, precision=2)
    with pytest.raises(_lib.UppasdGpuError) as ei:
        sim.set_dipole(3, ALAT)
    assert ei.value.rc == -7
    sim.close()
    sim = GpuSimulation(lat)
    with pytest.raises(_lib.UppasdGpuError) as ei:
        _lib.call("uppasd_gpu_set_dipole", sim._h, 3, ALAT, None, 2, 6, 6, 5, None, None)
    assert ei.value.rc == -1
    sim.close()
