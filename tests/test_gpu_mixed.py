"""Precision 3: FP32 gather over the caller's neighbour lists with the FP64 state as
master (renormalised in FP64 every step), on Hamiltonians outside the structured bcc
path: exchange (scalar or tensor), DMI, anisotropy and Zeeman, midpoint and Depondt.
Precision 4: the same with a double-single master (hi = the FP32 mirror, lo a residual,
renormalised in error-free FP32 arithmetic); the tests run on both.

The field, thermal field and rotation run in FP32, so trajectories are compared with
the FP64 oracle at FP32-scale tolerances that grow with the step count (a random
start at T = 0 amplifies a 1e-7 perturbation to ~1e-5 in 100 steps); spin norms are
held to 1e-12.
"""
import numpy as np
import pytest

from oracle import pyoracle as po
from uppasd_gb300 import _lib, lattice
from uppasd_gb300.simulation import GpuSimulation

pytestmark = pytest.mark.gpu
CHECKPOINTS = {10: 2e-6, 100: 2e-5}
THERMAL_TOL = 2e-4


def _rand_unit(rng, shape):
    e = rng.normal(size=shape)
    return e / np.linalg.norm(e, axis=-1, keepdims=True)


def _pair(lat, solver, temp, e0, seed=31, damping=0.05, prec=3):
    sim = GpuSimulation(lat, sdealgh=solver, delta_t=1e-16, damping=damping, temperature=temp, seed=seed,
                        emom=e0, precision=prec)
    o = po.Oracle(lat)
    o.set_moments(e0)
    o.make_llg(solver, 1e-16, damping, temp, 1.0, noise_mode=po.NOISE_PHILOX, seed=seed)
    return sim, o


@pytest.mark.parametrize("prec", [3, 4])
@pytest.mark.parametrize("kind,solver", [("square_dmi_aniso", 1), ("square_dmi_aniso", 5), ("kagome_tensor", 5),
                                         ("kagome_tensor", 1)])
def test_T0_against_oracle(kind, solver, prec):
    lat = (lattice.square_dmi(32, 1.0, 0.3, -0.05, 0.5, 1.0) if kind == "square_dmi_aniso"
           else lattice.kagome(12, -1.0, 0.1, 0.05, 1.0, 0.2)).with_ensembles(2)
    e0 = _rand_unit(np.random.default_rng(41), (2, lat.natom, 3))
    sim, o = _pair(lat, solver, 0.0, e0, prec=prec)
    done = 0
    for n, tol in CHECKPOINTS.items():
        sim.evolve(n - done)
        for _ in range(n - done):
            o.sd_step()
        done = n
        g = sim.get_moments()
        assert np.max(np.abs(g - o.emom)) <= tol, (n, np.max(np.abs(g - o.emom)))
        assert np.max(np.abs(np.linalg.norm(g, axis=-1) - 1.0)) <= 1e-12
    sim.close()


@pytest.mark.parametrize("prec", [3, 4])
@pytest.mark.parametrize("solver", [1, 5])
def test_thermal_philox_against_oracle(solver, prec):
    lat = lattice.square_dmi(32, 1.0, 0.3, -0.05, 0.5, 1.0).with_ensembles(2)
    e0 = _rand_unit(np.random.default_rng(42), (2, lat.natom, 3))
    sim, o = _pair(lat, solver, 50.0, e0, prec=prec)
    sim.evolve(200)
    for _ in range(200):
        o.sd_step()
    assert np.max(np.abs(sim.get_moments() - o.emom)) <= THERMAL_TOL
    sim.close()


@pytest.mark.parametrize("prec", [3, 4])
def test_injected_noise_against_oracle(prec):
    lat = lattice.kagome(12).with_ensembles(1)
    e0 = _rand_unit(np.random.default_rng(43), (1, lat.natom, 3))
    nsteps = 100
    normals = po.ziggurat_stream(3, nsteps * 3 * lat.natom).reshape(nsteps, 1, lat.natom, 3)
    sim = GpuSimulation(lat, sdealgh=5, delta_t=1e-16, damping=0.05, temperature=100.0, emom=e0, precision=prec)
    sim.set_noise(normals)
    sim.evolve(nsteps)
    o = po.Oracle(lat)
    o.set_moments(e0)
    o.make_llg(5, 1e-16, 0.05, 100.0, 1.0, noise_mode=po.NOISE_ARRAY)
    for s in range(nsteps):
        o.sd_step(noise=normals[s])
    assert np.max(np.abs(sim.get_moments() - o.emom)) <= THERMAL_TOL
    sim.close()


def test_agrees_with_structured_path_on_the_alloy():
    lat = lattice.bcc_alloy(6, seed=9).with_ensembles(2)
    e0 = _rand_unit(np.random.default_rng(44), (2, lat.natom, 3))
    out = []
    for prec in (1, 3, 4):
        sim = GpuSimulation(lat, sdealgh=5, delta_t=1e-16, damping=0.1, temperature=300.0, seed=21, emom=e0,
                            precision=prec)
        sim.evolve(100)
        out.append(sim.get_moments())
        sim.close()
    assert np.max(np.abs(out[0] - out[1])) <= 1e-4
    assert np.max(np.abs(out[0] - out[2])) <= 1e-4


def test_state_changes_between_runs_are_seen():
    """put_moments, FP64 and structured Monte Carlo between LLG runs: precision 3 follows
    the same sequence as the FP64 path to FP32 accuracy."""
    lat = lattice.square_dmi(16, 1.0, 0.3, 0.0, 0.5, 1.0).with_ensembles(2)
    rng = np.random.default_rng(45)
    e0, e1 = _rand_unit(rng, (2, lat.natom, 3)), _rand_unit(rng, (2, lat.natom, 3))
    res = []
    for prec in (0, 3, 4):
        sim = GpuSimulation(lat, sdealgh=1, delta_t=1e-16, damping=0.1, temperature=0.0, seed=9, emom=e0,
                            precision=prec)
        sim.evolve(20)
        sim.relax("H", 30.0, 1)
        sim.evolve(20)
        sim.relax("H", 30.0, 2, structured=True)
        sim.evolve(20)
        sim.put_moments(e1)
        sim.evolve(20)
        res.append(sim.get_moments())
        sim.close()
    assert np.max(np.abs(res[0] - res[1])) <= 1e-4
    assert np.max(np.abs(res[0] - res[2])) <= 1e-4


@pytest.mark.parametrize("solver,prec", [(4, 3), (6, 3), (7, 3), (11, 3), (4, 4), (6, 4), (7, 4), (11, 4)])
def test_other_solvers_T0_against_oracle(solver, prec):
    lat = lattice.square_dmi(32, 1.0, 0.3, -0.05, 0.5, 1.0).with_ensembles(2)
    e0 = _rand_unit(np.random.default_rng(47), (2, lat.natom, 3))
    tau = 1e-15 if solver == 11 else 0.0
    sim = GpuSimulation(lat, sdealgh=solver, delta_t=1e-16, damping=0.05, temperature=0.0, seed=31, emom=e0,
                        precision=prec, relaxtime=tau)
    o = po.Oracle(lat)
    o.set_moments(e0)
    o.make_llg(solver, 1e-16, 0.05, 0.0, 1.0, noise_mode=po.NOISE_PHILOX, seed=31, relaxtime=tau)
    done = 0
    for n, tol in CHECKPOINTS.items():
        sim.evolve(n - done)
        for _ in range(n - done):
            o.sd_step()
        done = n
        g = sim.get_moments()
        assert np.max(np.abs(g - o.emom)) <= tol, (n, np.max(np.abs(g - o.emom)))
        assert np.max(np.abs(np.linalg.norm(g, axis=-1) - 1.0)) <= 1e-12
    sim.close()


@pytest.mark.parametrize("solver,prec", [(1, 3), (4, 3), (5, 3), (6, 3), (7, 3), (11, 3), (1, 4), (4, 4), (5, 4),
                                         (6, 4), (7, 4), (11, 4)])
def test_perp_against_oracle(solver, prec):
    lat = lattice.square_dmi(32, 1.0, 0.3, -0.05, 0.5, 1.0).with_ensembles(2)
    e0 = _rand_unit(np.random.default_rng(48), (2, lat.natom, 3))
    tau = 1e-15 if solver == 11 else 0.0
    sim = GpuSimulation(lat, sdealgh=solver, delta_t=1e-16, damping=0.05, temperature=50.0, seed=33, emom=e0,
                        precision=prec, relaxtime=tau, perp=True)
    o = po.Oracle(lat)
    o.set_moments(e0)
    o.make_llg(solver, 1e-16, 0.05, 50.0, 1.0, noise_mode=po.NOISE_PHILOX, seed=33, relaxtime=tau, perp=True)
    sim.evolve(100)
    for _ in range(100):
        o.sd_step()
    assert np.max(np.abs(sim.get_moments() - o.emom)) <= THERMAL_TOL
    sim.close()


def test_scope():
    lat = lattice.bcc_alloy(6, seed=9)
    sim = GpuSimulation(lat, sdealgh=5, precision=1)
    with pytest.raises(_lib.UppasdGpuError) as ex:
        _lib.call("uppasd_gpu_set_perp", sim._h, 1)
    assert ex.value.rc == -7
    sim.close()


def _alloy_runs(lat, e0, prec, solver):
    """20 Philox steps at 300 K, then 2 heat-bath and 2 Metropolis sweeps: the path
    info and the state after each stage."""
    sim = GpuSimulation(lat, sdealgh=solver, delta_t=1e-16, damping=0.1, temperature=300.0, seed=21, emom=e0,
                        precision=prec)
    info = sim.path_info()
    sim.evolve(20)
    out = [sim.get_moments()]
    sim.relax("H", 300.0, 2)
    out.append(sim.get_moments())
    sim.relax("M", 300.0, 2)
    out.append(sim.get_moments())
    sim.close()
    return info, out


@pytest.mark.parametrize("prec,solver", [(3, 5), (4, 5), (4, 1)])
def test_chemical_classes_reproduce_the_per_site_lists(prec, solver, monkeypatch):
    """Random bcc alloy (14^3 cells, four shells, couplings from a (type_i, type_j, shell)
    table): every site's coupling row differs, so the plain site classes give way to the
    per-site lists; with the chemical types the sites fall into classes keyed on their
    own type and the neighbours' couplings are looked up by type.  Both forms give the
    same LLG trajectory and Monte Carlo chains bit for bit, and the LLG steps follow the
    FP64 oracle within the thermal tolerance."""
    lat = lattice.bcc_alloy(14, seed=9).with_ensembles(2)
    e0 = _rand_unit(np.random.default_rng(47), (2, lat.natom, 3))
    info, got = _alloy_runs(lat, e0, prec, solver)
    assert info["chemical_types"] == 2
    assert 0 < info["site_classes"] <= lat.natom // 8
    monkeypatch.setenv("UPPASD_CHEMICAL_CLASSES", "0")
    info0, ref = _alloy_runs(lat, e0, prec, solver)
    assert info0["chemical_types"] == 0 and info0["site_classes"] == 0
    for a, b in zip(got, ref):
        assert np.array_equal(a, b)
    o = po.Oracle(lat)
    o.set_moments(e0)
    o.make_llg(solver, 1e-16, 0.1, 300.0, 1.0, noise_mode=po.NOISE_PHILOX, seed=21)
    for _ in range(20):
        o.sd_step()
    assert np.max(np.abs(got[0] - o.emom)) <= THERMAL_TOL


def test_chemical_classes_need_type_resolved_couplings():
    """One coupling that is not a function of the neighbour's type: the per-site lists
    stay; with couplings that are, the classes are taken (and the simulation reports it)."""
    lat = lattice.bcc_alloy(14, seed=9)
    sim = GpuSimulation(lat, sdealgh=5, precision=3)
    assert sim.path_info()["chemical_types"] == 2
    sim.close()
    lat.ncoup = lat.ncoup.copy()
    lat.ncoup[5, 3] *= 1.01
    sim = GpuSimulation(lat, sdealgh=5, precision=3)
    info = sim.path_info()
    sim.close()
    assert info["chemical_types"] == 0 and info["site_classes"] == 0


@pytest.mark.parametrize("prec", [3, 4])
@pytest.mark.parametrize("kind", ["kagome_tensor", "square_dmi_aniso"])
def test_heat_bath_chain_against_oracle(kind, prec):
    """mc_run 'H' at precision 3: the FP64 path's checkerboard chain (same colouring,
    same Philox draws) with the field and the draw in FP32, per spin within 2e-4
    after 3 sweeps."""
    lat = (lattice.kagome(12, -1.0, 0.1, 0.05, 1.0, 0.2) if kind == "kagome_tensor"
           else lattice.square_dmi(32, 1.0, 0.3, -0.05, 0.5, 1.0)).with_ensembles(2)
    e0 = _rand_unit(np.random.default_rng(46), (2, lat.natom, 3))
    T = 30.0
    sim = GpuSimulation(lat, emom=e0, seed=61, precision=prec, sdealgh=5)
    sim.relax("H", T, 3)
    g = sim.get_moments()
    sim.close()
    o = po.Oracle(lat)
    o.set_moments(e0)
    _, order, start = lattice.greedy_colouring(lat)
    for sw in range(3):
        o.mc_sweep_checkerboard("H", T, order, start, 61, sw)
    assert np.max(np.abs(g - o.emom)) < 2e-4


@pytest.mark.parametrize("prec", [3, 4])
@pytest.mark.parametrize("kind", ["kagome_tensor", "square_dmi_aniso"])
def test_metropolis_sweep_follows_the_fp64_chain(kind, prec):
    """mc_run 'M' at precision 3 makes the FP64 path's trials (same Philox words, same
    colouring) and decisions with the energy change in FP32: after one sweep from the same
    state nearly every spin agrees with the FP64 chain to FP32 rounding (a decision can
    differ where the energy change sits at the acceptance threshold), norms stay 1."""
    lat = (lattice.kagome(12, -1.0, 0.1, 0.05, 1.0, 0.2) if kind == "kagome_tensor"
           else lattice.square_dmi(32, 1.0, 0.3, -0.05, 0.5, 1.0)).with_ensembles(2)
    e0 = _rand_unit(np.random.default_rng(49), (2, lat.natom, 3))
    out = []
    for p in (prec, 0):
        sim = GpuSimulation(lat, emom=e0, seed=63, precision=p, sdealgh=5)
        sim.relax("M", 30.0, 1)
        out.append(sim.get_moments())
        sim.close()
    d = np.max(np.abs(out[0] - out[1]), axis=-1)
    assert np.mean(d < 1e-5) > 0.98, np.mean(d < 1e-5)
    assert np.mean(np.max(np.abs(out[0] - e0), axis=-1) > 1e-3) > 0.05   # the sweep moved spins
    assert np.max(np.abs(np.linalg.norm(out[0], axis=-1) - 1.0)) <= 1e-12


def test_metropolis_statistics_match_the_fp64_path():
    """E and |M| of FP32-energy Metropolis chains agree with the FP64 path's within 3 sigma
    (8 ensembles, 40 samples each after thermalisation, errors from the spread of the
    ensemble means)."""
    lat = lattice.square_dmi(24, 1.0, 0.3, -0.05, 0.5, 1.0).with_ensembles(8)
    e0 = _rand_unit(np.random.default_rng(50), (8, lat.natom, 3))
    stats = []
    for prec, seed in ((0, 71), (3, 72)):
        sim = GpuSimulation(lat, emom=e0, seed=seed, precision=prec, sdealgh=5)
        sim.relax("M", 40.0, 300)
        es, ms = [], []
        for _ in range(40):
            sim.relax("M", 40.0, 10)
            obs = sim.observables()
            es.append(obs["energy"])
            ms.append(obs["mabs"])
        sim.close()
        es, ms = np.mean(es, axis=0), np.mean(ms, axis=0)   # one mean per ensemble
        stats.append((es.mean(), es.std(ddof=1) / np.sqrt(8), ms.mean(), ms.std(ddof=1) / np.sqrt(8)))
    (e0m, e0s, m0m, m0s), (e3m, e3s, m3m, m3s) = stats
    assert abs(e0m - e3m) <= 3 * np.hypot(e0s, e3s), stats
    assert abs(m0m - m3m) <= 3 * np.hypot(m0s, m3s), stats


@pytest.mark.parametrize("prec", [3, 4])
@pytest.mark.parametrize("solver", [1, 5])
def test_T0_per_site_field_and_anisotropy(solver, prec):
    """Precision 3 with nothing uniform: a random external field per site and per
    ensemble (the per-site branch of the FP32 field, not the single uniform entry),
    per-site uniaxial and cubic anisotropy with random axes and constants (one FP32
    anisotropy row per site), and every site's exchange row scaled differently (one
    coupling row per site): against the FP64 oracle at T = 0."""
    rng = np.random.default_rng(44)
    lat = lattice.square_dmi(16, 1.0, 0.3, -0.05, 0.5, 1.0).with_ensembles(2)
    N = lat.natom
    lat.extfield = rng.normal(scale=2.0, size=(2, N, 3))
    lat.taniso = rng.choice([1, 2, 7], size=N).astype(np.int32)
    lat.eaniso = _rand_unit(rng, (N, 3))
    lat.kaniso = lat.kaniso.copy()
    lat.kaniso[:, 0] *= rng.uniform(0.5, 2.0, size=N)
    lat.kaniso[:, 1] = lat.kaniso[:, 0] * rng.uniform(-0.5, 0.5, size=N)
    lat.sb = rng.uniform(0.0, 1.0, size=N)
    lat.ncoup = lat.ncoup * rng.uniform(0.8, 1.2, size=(N, 1))
    e0 = _rand_unit(np.random.default_rng(45), (2, N, 3))
    sim, o = _pair(lat, solver, 0.0, e0, prec=prec)
    done = 0
    for n, tol in CHECKPOINTS.items():
        sim.evolve(n - done)
        for _ in range(n - done):
            o.sd_step()
        done = n
        g = sim.get_moments()
        err = float(np.max(np.abs(g - o.emom)))
        print(f"per-site field/anisotropy solver {solver} steps {n}: {err:.3e}")
        assert err <= tol, (n, err)
        assert np.max(np.abs(np.linalg.norm(g, axis=-1) - 1.0)) <= 1e-12
    sim.close()



@pytest.mark.parametrize("solver", [1, 4, 5, 11])
def test_precision4_reads_leave_the_trajectory_unchanged(solver):
    """The double-single master is converted to e / eM whenever the caller reads them
    (get_moments, observables, energy terms, the field); the master itself is not touched,
    so a run with reads between its blocks is bit-identical to one without."""
    lat = lattice.kagome(12, -1.0, 0.1, 0.05, 1.0, 0.2).with_ensembles(2)
    e0 = _rand_unit(np.random.default_rng(52), (2, lat.natom, 3))
    out = []
    for reads in (False, True):
        sim = GpuSimulation(lat, sdealgh=solver, delta_t=1e-16, damping=0.05, temperature=50.0, seed=5, emom=e0,
                            precision=4, relaxtime=1e-15 if solver == 11 else 0.0)
        for _ in range(4):
            sim.evolve(25)
            if reads:
                sim.get_moments(full=True)
                sim.observables()
                sim.energy_terms()
                sim.get_fields()
        out.append(sim.get_moments(full=True))
        sim.close()
    assert np.array_equal(out[0][0], out[1][0]) and np.array_equal(out[0][1], out[1][1])
    assert np.max(np.abs(np.linalg.norm(out[0][0], axis=-1) - 1.0)) <= 1e-12
