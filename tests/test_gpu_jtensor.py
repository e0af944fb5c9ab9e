"""GPU exchange-tensor path (do_jtensor = 1) through the C ABI against the oracle.

* kagome lattice with a full per-bond tensor (isotropic + symmetric anisotropic +
  antisymmetric parts): field and energies to 1e-12, LLG trajectories to 1e-9 after
  1000 steps (FP64 bar), checkerboard Monte Carlo chains to 1e-12;
* an isotropic tensor reproduces the scalar exchange run bit for bit on the GPU;
* scope: the structured paths refuse a tensor Hamiltonian with -7.
"""
import numpy as np
import pytest

from oracle import pyoracle as po
from uppasd_gb300 import _lib, lattice
from uppasd_gb300.simulation import GpuSimulation

pytestmark = pytest.mark.gpu
TOL = 1e-9


def _rand_unit(rng, shape):
    e = rng.normal(size=shape)
    return e / np.linalg.norm(e, axis=-1, keepdims=True)


def _kagome(M=2):
    return lattice.kagome(8, -1.0, 0.1, 0.05, 1.0, 0.2).with_ensembles(M)


def test_kagome_field_and_energy_match_oracle():
    lat = _kagome(3)
    e0 = _rand_unit(np.random.default_rng(21), (3, lat.natom, 3))
    sim = GpuSimulation(lat, emom=e0)
    o = po.Oracle(lat)
    o.set_moments(e0)
    b, _ = o.field()
    assert np.max(np.abs(sim.get_fields() - b)) <= 1e-12 * max(1.0, np.abs(b).max())
    obs = sim.observables()
    assert np.allclose(obs["energy"], o.energy()["total"], rtol=1e-12, atol=1e-14)
    sim.close()


@pytest.mark.parametrize("solver,temp", [(1, 0.0), (4, 0.0), (5, 0.0), (5, 300.0), (1, 300.0), (7, 0.0)])
def test_kagome_llg_1000_steps(solver, temp):
    lat = _kagome(2)
    e0 = _rand_unit(np.random.default_rng(22), (2, lat.natom, 3))
    sim = GpuSimulation(lat, sdealgh=solver, delta_t=1e-16, damping=0.05, temperature=temp, seed=17, emom=e0)
    o = po.Oracle(lat)
    o.set_moments(e0)
    o.make_llg(solver, 1e-16, 0.05, temp, 1.0, noise_mode=po.NOISE_PHILOX, seed=17)
    sim.evolve(1000)
    for _ in range(1000):
        o.sd_step()
    assert np.max(np.abs(sim.get_moments() - o.emom)) <= TOL
    sim.close()


@pytest.mark.parametrize("mode", ["M", "H"])
def test_kagome_checkerboard_chain_parity(mode):
    lat = _kagome(2)
    e0 = _rand_unit(np.random.default_rng(23), (2, lat.natom, 3))
    sim = GpuSimulation(lat, emom=e0, seed=99)
    sim.relax(mode, 30.0, 4)
    o = po.Oracle(lat)
    o.set_moments(e0)
    _, order, start = lattice.greedy_colouring(lat)
    for sw in range(4):
        o.mc_sweep_checkerboard(mode, 30.0, order, start, 99, sw)
    assert np.max(np.abs(sim.get_moments() - o.emom)) <= 1e-12
    sim.close()


def test_isotropic_tensor_reproduces_scalar_run_bit_for_bit():
    lat = lattice.bcc(4, [1.3, 0.7], 2.2).with_ensembles(2)
    e0 = _rand_unit(np.random.default_rng(24), (2, lat.natom, 3))
    runs = []
    for L in (lat, lattice.with_isotropic_tensor(lat)):
        sim = GpuSimulation(L, sdealgh=5, delta_t=1e-16, damping=0.1, temperature=300.0, seed=5, emom=e0)
        sim.evolve(200)
        sim.relax("H", 400.0, 3)
        runs.append((sim.get_moments(), sim.observables()["energy"]))
        sim.close()
    assert np.array_equal(runs[0][0], runs[1][0])
    assert np.array_equal(runs[0][1], runs[1][1])


def test_tensor_switch_and_scope():
    lat = lattice.square_dmi(16, 1.0, 0.3, 0.0, 0.5, 1.0).with_ensembles(2)
    e0 = _rand_unit(np.random.default_rng(25), (2, lat.natom, 3))
    sim = GpuSimulation(lat, emom=e0)
    f_scalar = sim.get_fields()
    sim.relax("H", 10.0, 2, structured=True)            # recognised as uniform square
    sim.put_moments(e0)
    sim.set_jtensor(lattice.with_isotropic_tensor(lat).j_tens)
    assert np.array_equal(sim.get_fields(), f_scalar)
    with pytest.raises(_lib.UppasdGpuError) as ex:
        sim.relax("H", 10.0, 2, structured=True)
    assert ex.value.rc == -7
    sim.set_jtensor(None)
    assert np.array_equal(sim.get_fields(), f_scalar)
    sim.relax("H", 10.0, 2, structured=True)
    sim.close()
    fast = GpuSimulation(lattice.bcc_alloy(6, seed=9), sdealgh=5, precision=1)
    with pytest.raises(_lib.UppasdGpuError) as ex:
        fast.set_jtensor(lattice.with_isotropic_tensor(fast.lat).j_tens)
    assert ex.value.rc == -7
    fast.close()


@pytest.mark.parametrize("prec,tol", [(0, 1e-9), (3, 2e-4)])
def test_block_form_runs_like_separate_terms(prec, tol):
    """Exchange and DMI folded into 3x3 blocks (the reference's sparse path's form) run on
    the tensor gather and follow the separate-term run: 1e-9 after 1000 FP64 steps, FP32
    scale at precision 3 after 100."""
    lat = lattice.square_dmi(32, 1.0, 0.3, -0.05, 0.5, 1.0).with_ensembles(2)
    e0 = _rand_unit(np.random.default_rng(83), (2, lat.natom, 3))
    n = 1000 if prec == 0 else 100
    out = []
    for L in (lat, lattice.fold_dm_into_tensor(lat)):
        sim = GpuSimulation(L, sdealgh=1, delta_t=1e-16, damping=0.1, temperature=50.0, seed=4, emom=e0,
                            precision=prec)
        sim.evolve(n)
        out.append(sim.get_moments())
        sim.close()
    assert np.max(np.abs(out[0] - out[1])) <= tol
