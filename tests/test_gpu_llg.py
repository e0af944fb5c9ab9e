"""GPU LLG parity: the CUDA path through the C ABI against the CPU oracle.

Tolerance: FP64 trajectories within 1e-9 per spin component
after 1000 steps, at T = 0 and with fixed injected noise.  Runs on a GB300.
"""
import ctypes as C

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


def _pair(lat, solver, dt, damping, temp, seed, e0, noise_mode):
    sim = GpuSimulation(lat, sdealgh=solver, delta_t=dt, damping=damping, temperature=temp, seed=seed, emom=e0)
    o = po.Oracle(lat)
    o.set_moments(e0)
    o.make_llg(solver, dt, damping, temp, 1.0, noise_mode=noise_mode, seed=seed)
    return sim, o


@pytest.mark.parametrize("solver", [1, 4, 5, 6, 7])
def test_bcc_T0_1000_steps(solver):
    lat = lattice.bcc(4, [1.3, 0.7], 2.2).with_ensembles(2)
    e0 = _rand_unit(np.random.default_rng(1), (2, lat.natom, 3))
    nsteps = 1000 if solver not in (6, 7) else 200
    sim, o = _pair(lat, solver, 1e-16, 0.1, 0.0, 5, e0, po.NOISE_PHILOX)
    sim.evolve(nsteps)
    for _ in range(nsteps):
        o.sd_step()
    g = sim.get_moments()
    assert np.max(np.abs(g - o.emom)) <= TOL
    sim.close()


@pytest.mark.parametrize("solver", [1, 5, 7])
def test_bcc_philox_T300_1000_steps(solver):
    lat = lattice.bcc(4, [1.3, 0.7], 2.2).with_ensembles(2)
    e0 = _rand_unit(np.random.default_rng(2), (2, lat.natom, 3))
    sim, o = _pair(lat, solver, 1e-16, 0.1, 300.0, 77, e0, po.NOISE_PHILOX)
    sim.evolve(1000)
    for _ in range(1000):
        o.sd_step()
    g = sim.get_moments()
    assert np.max(np.abs(g - o.emom)) <= TOL
    sim.close()


@pytest.mark.parametrize("solver", [1, 4, 5, 7])
def test_injected_reference_noise_1000_steps(solver):
    """The reference's own ziggurat normal stream injected into the GPU."""
    lat = lattice.bcc(3, [1.3, 0.7], 2.2)
    e0 = _rand_unit(np.random.default_rng(3), (1, lat.natom, 3))
    nsteps = 1000
    normals = po.ziggurat_stream(5, nsteps * 3 * lat.natom).reshape(nsteps, 1, lat.natom, 3)
    sim = GpuSimulation(lat, sdealgh=solver, delta_t=1e-16, damping=0.1, temperature=300.0, emom=e0)
    sim.set_noise(normals)
    sim.evolve(nsteps)
    o = po.Oracle(lat)
    o.set_moments(e0)
    o.make_llg(solver, 1e-16, 0.1, 300.0, 1.0, noise_mode=po.NOISE_ARRAY)
    for s in range(nsteps):
        o.sd_step(noise=normals[s])
    assert np.max(np.abs(sim.get_moments() - o.emom)) <= TOL
    sim.close()


@pytest.mark.parametrize("temp", [0.0, 50.0])
def test_square_dmi_aniso_zeeman_midpoint(temp):
    """Config-1 Hamiltonian (J, interfacial DMI, uniaxial K, Zeeman) on a 32^2 patch."""
    lat = lattice.square_dmi(32, 1.0, 0.3, -0.05, 0.5, 1.0)
    e0 = _rand_unit(np.random.default_rng(4), (1, lat.natom, 3))
    sim, o = _pair(lat, 1, 1e-16, 0.05, temp, 9, e0, po.NOISE_PHILOX)
    sim.evolve(1000)
    for _ in range(1000):
        o.sd_step()
    assert np.max(np.abs(sim.get_moments() - o.emom)) <= TOL
    sim.close()


def test_alloy_four_shells_depondt():
    lat = lattice.bcc_alloy(4, seed=3)
    e0 = _rand_unit(np.random.default_rng(5), (1, lat.natom, 3))
    sim, o = _pair(lat, 5, 1e-16, 0.1, 300.0, 3, e0, po.NOISE_PHILOX)
    sim.evolve(500)
    for _ in range(500):
        o.sd_step()
    assert np.max(np.abs(sim.get_moments() - o.emom)) <= TOL
    sim.close()


def test_field_and_observables_match_oracle():
    lat = lattice.square_dmi(16, 1.0, 0.3, -0.05, 0.5, 1.0).with_ensembles(3)
    e0 = _rand_unit(np.random.default_rng(6), (3, lat.natom, 3))
    sim = GpuSimulation(lat, emom=e0)
    o = po.Oracle(lat)
    o.set_moments(e0)
    b, _ = o.field()
    gb = sim.get_fields()
    assert np.max(np.abs(gb - b)) <= 1e-12 * max(1.0, np.abs(b).max())
    obs = sim.observables()
    mv, ma = o.mavg()
    en = o.energy()["total"]
    assert np.allclose(obs["mvec"], mv, rtol=0, atol=1e-10)
    assert np.allclose(obs["mabs"], ma, rtol=1e-13, atol=1e-14)
    assert np.allclose(obs["energy"], en, rtol=1e-12, atol=1e-14)
    sim.close()


@pytest.mark.parametrize("solver,name", [(1, "solvers_midpoint"), (4, "solvers_heun"), (5, "solvers_depondt")])
def test_gpu_reproduces_reference_solvers_golden(pins, solver, name):
    """tests/Solvers on the GPU: the start state is the reference's mtprng initmag-1 draw."""
    inp = pins["inputs"]["solvers"]
    n = inp["ncell"][2]
    lat = lattice.chain(n, inp["j_mry"], inp["mom"])
    o = po.Oracle(lat)
    o.init_random(inp["tseed_default"])
    sim = GpuSimulation(lat, sdealgh=solver, delta_t=inp["timestep"], damping=inp["damping"],
                        temperature=0.0, emom=o.emom.copy())
    sim.evolve(inp["nstep_checked"])
    e = sim.get_moments()
    m = e[0].sum(axis=0) / n
    got = np.array(list(m) + [np.linalg.norm(m)])
    exp = np.array(pins[name]["expected"])
    assert np.all(np.abs(got - exp) <= 1e-8 + 0.5 * 10.0 ** (np.floor(np.log10(np.abs(exp))) - 8))
    sim.close()


def test_gpu_reproduces_reference_bccfe_T500_golden(pins):
    """tests/bccFe mode S on the GPU with the reference's ziggurat stream injected."""
    inp = pins["inputs"]["bccfe"]
    lat = lattice.bcc(inp["ncell"][0], inp["j_mry"], inp["mom"])
    e0 = np.zeros((1, lat.natom, 3))
    e0[..., :] = inp["emom0"]
    n_ip = inp["ip_nstep"]
    normals = po.ziggurat_stream(inp["tseed"], n_ip * 3 * lat.natom).reshape(n_ip, 1, lat.natom, 3)
    sim = GpuSimulation(lat, sdealgh=1, delta_t=inp["ip_timestep"], damping=inp["ip_damping"],
                        temperature=inp["ip_temp"], emom=e0)
    sim.set_noise(normals)
    sim.evolve(n_ip)
    e = sim.get_moments()
    m = e[0].sum(axis=0) / lat.natom * inp["mom"]
    got = np.array(list(m) + [np.linalg.norm(m)])
    exp = np.array(pins["bccfe_sd_iter0"]["expected"])
    assert np.all(np.abs(got - exp) <= 1e-8 + 0.5 * 10.0 ** (np.floor(np.log10(np.abs(exp))) - 8)), (got, exp)
    sim.close()


def test_noise_statistics_philox():
    """The in-kernel Philox thermal field pulls |M| below saturation at 300 K."""
    lat = lattice.bcc(6, [1.3, 0.7], 2.2).with_ensembles(4)
    e0 = np.zeros((4, lat.natom, 3))
    e0[..., 2] = 1.0
    sim = GpuSimulation(lat, sdealgh=5, delta_t=1e-16, damping=0.1, temperature=300.0, seed=1, emom=e0)
    sim.evolve(2000)
    ma = sim.observables()["mabs"]
    assert np.all(ma < 2.2) and np.all(ma > 1.5)
    sim.close()


@pytest.mark.parametrize("kind,temp,tau", [("bcc", 0.0, 0.0), ("bcc", 0.0, 2e-15), ("bcc", 300.0, 2e-15),
                                           ("kagome_tensor", 100.0, 1e-15)])
def test_llgi_1000_steps(kind, temp, tau):
    """SDEalgh 11 (inertial LLG) through the C ABI against the oracle."""
    lat = (lattice.bcc(4, [1.3, 0.7], 2.2) if kind == "bcc" else lattice.kagome(8)).with_ensembles(2)
    e0 = _rand_unit(np.random.default_rng(8), (2, lat.natom, 3))
    sim = GpuSimulation(lat, sdealgh=11, delta_t=1e-16, damping=0.05, temperature=temp, seed=13, emom=e0,
                        relaxtime=tau)
    o = po.Oracle(lat)
    o.set_moments(e0)
    o.make_llg(11, 1e-16, 0.05, temp, 1.0, noise_mode=po.NOISE_PHILOX, seed=13, relaxtime=tau)
    sim.evolve(1000)
    for _ in range(1000):
        o.sd_step()
    assert np.max(np.abs(sim.get_moments() - o.emom)) <= TOL
    # a new state starts without a previous step, as a fresh run does
    sim.put_moments(e0)
    sim.set_step(0)
    sim.evolve(10)
    o.set_moments(e0)
    o.llg.step = 0
    for _ in range(10):
        o.sd_step()
    assert np.max(np.abs(sim.get_moments() - o.emom)) <= TOL
    sim.close()


@pytest.mark.parametrize("solver", [1, 4, 5, 6, 7, 11])
def test_perp_projection(solver):
    """Input perp = 'Y': the field loses its component along emom before each half-step."""
    lat = lattice.square_dmi(16, 1.0, 0.3, -0.05, 0.5, 1.0).with_ensembles(2)
    e0 = _rand_unit(np.random.default_rng(9), (2, lat.natom, 3))
    nsteps = 300 if solver != 6 else 100
    sim = GpuSimulation(lat, sdealgh=solver, delta_t=1e-16, damping=0.1, temperature=50.0, seed=21, emom=e0,
                        relaxtime=1e-15 if solver == 11 else 0.0, perp=True)
    o = po.Oracle(lat)
    o.set_moments(e0)
    o.make_llg(solver, 1e-16, 0.1, 50.0, 1.0, noise_mode=po.NOISE_PHILOX, seed=21,
               relaxtime=1e-15 if solver == 11 else 0.0, perp=True)
    sim.evolve(nsteps)
    for _ in range(nsteps):
        o.sd_step()
    assert np.max(np.abs(sim.get_moments() - o.emom)) <= TOL
    # the projection changes the trajectory of a finite step
    ref = po.Oracle(lat)
    ref.set_moments(e0)
    ref.make_llg(solver, 1e-16, 0.1, 50.0, 1.0, noise_mode=po.NOISE_PHILOX, seed=21,
                 relaxtime=1e-15 if solver == 11 else 0.0)
    for _ in range(nsteps):
        ref.sd_step()
    assert np.max(np.abs(ref.emom - o.emom)) > 1e-12
    sim.close()


@pytest.mark.parametrize("prec", [0, 1])
def test_page_locked_buffers_read_and_written_in_place(prec):
    """put_moments / get_moments with page-locked caller buffers (read and written by the
    conversion kernels directly) give exactly what the staged path for pageable buffers gives."""
    torch = pytest.importorskip("torch")
    lat = lattice.bcc(6, [1.3, 0.7], 2.2).with_ensembles(3)
    e0 = _rand_unit(np.random.default_rng(21), (3, lat.natom, 3))
    pinned_in = torch.empty(e0.shape, dtype=torch.float64, pin_memory=True).numpy()
    pinned_in[...] = e0
    pinned_out = torch.empty(e0.shape, dtype=torch.float64, pin_memory=True).numpy()
    pinned_m = torch.empty(e0.shape, dtype=torch.float64, pin_memory=True).numpy()
    res = []
    for src, pinned in ((e0.copy(), False), (pinned_in, True)):
        sim = GpuSimulation(lat, sdealgh=5, temperature=300.0, seed=3, emom=e0, precision=prec)
        sim.put_moments(src)
        sim.evolve(20)
        if pinned:
            out = sim.get_moments(out=pinned_out)
            e, em = sim.get_moments(full=True)
            _lib.call("uppasd_gpu_get_moments", sim._h, pinned_out.ctypes.data_as(_lib.F64P),
                      pinned_m.ctypes.data_as(_lib.F64P))
            res.append((np.array(out), pinned_out.copy(), pinned_m.copy(), e, em))
        else:
            e, em = sim.get_moments(full=True)
            res.append((e, e, em, e, em))
        sim.close()
    for a, b in zip(res[0], res[1]):
        assert np.array_equal(a, b)


@pytest.mark.parametrize("prec", [0, 1])
def test_measured_run_equals_blocks_of_steps(prec):
    """sd_run_measured hands over the same states, at the same steps, as blocks of sd_run
    followed by get_moments; a callback that asks to stop ends the run after the block in
    flight."""
    lat = lattice.bcc_alloy(6, seed=4).with_ensembles(2)
    e0 = _rand_unit(np.random.default_rng(22), (2, lat.natom, 3))
    make = lambda: GpuSimulation(lat, sdealgh=5, temperature=300.0, seed=8, emom=e0, precision=prec)
    a, snaps = make(), []
    a.sd_run_measured(53, 10, lambda st, e, m: snaps.append((st, e.copy(), m.copy())))
    b = make()
    assert [s[0] for s in snaps] == [10, 20, 30, 40, 50]
    for st, e, m in snaps:
        b.evolve(10)
        eb, mb = b.get_moments(full=True)
        assert np.array_equal(e, eb) and np.array_equal(m, mb), st
    b.evolve(3)
    assert np.array_equal(a.get_moments(), b.get_moments())
    c, seen = make(), []
    rc = c.sd_run_measured(100, 10, lambda st, e, m: seen.append(st) or st == 20)
    assert rc == 1 and seen == [10, 20]
    d = make()
    d.evolve(30)
    assert np.array_equal(c.get_moments(), d.get_moments())
    for s in (a, b, c, d):
        s.close()
