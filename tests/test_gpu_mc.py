"""GPU Monte Carlo: checkerboard sweeps against the oracle.

* exact chain parity: the CUDA sweep and the oracle's restatement of the same
  checkerboard chain (same Philox draws, same colouring) agree per spin to 1e-12;
* statistical parity: GPU heat bath / Metropolis against the reference's own
  chain (random-permutation order, mtprng + ziggurat draws) on E and |M|,
  within 3 sigma of the combined binning error.
"""
import ctypes as C

import numpy as np
import pytest

from oracle import pyoracle as po
from uppasd_gb300 import _lib, lattice
from uppasd_gb300.simulation import GpuSimulation

pytestmark = pytest.mark.gpu


def _rand_unit(rng, shape):
    e = rng.normal(size=shape)
    return e / np.linalg.norm(e, axis=-1, keepdims=True)


@pytest.mark.parametrize("mode", ["M", "H"])
@pytest.mark.parametrize("kind", ["bcc", "square"])
def test_checkerboard_chain_parity(mode, kind):
    if kind == "bcc":
        lat = lattice.bcc(4, [1.3, 0.7], 2.2).with_ensembles(2)
    else:
        lat = lattice.square_dmi(16, 1.0, 0.3, -0.05, 0.5, 1.0).with_ensembles(2)
    e0 = _rand_unit(np.random.default_rng(7), (2, lat.natom, 3))
    T = 400.0 if kind == "bcc" else 20.0
    sim = GpuSimulation(lat, emom=e0, seed=123)
    sim.relax(mode, T, 3)
    o = po.Oracle(lat)
    o.set_moments(e0)
    _, order, start = lattice.greedy_colouring(lat)
    for sw in range(3):
        o.mc_sweep_checkerboard(mode, T, order, start, 123, sw)
    g = sim.get_moments()
    assert np.max(np.abs(g - o.emom)) <= 1e-12
    sim.close()


def _binned(x, nbin=20):
    x = np.asarray(x)
    b = x[: len(x) // nbin * nbin].reshape(nbin, -1).mean(axis=1)
    return b.mean(), b.std(ddof=1) / np.sqrt(nbin)


@pytest.mark.parametrize("mode", ["H", "M"])
def test_statistics_match_reference_chain(mode):
    lat = lattice.bcc(6, [1.3, 0.7], 2.2)
    T = 900.0
    ntherm, nmeas = 500, 3000
    # reference chain on the CPU (oracle), its own RNG streams
    o = po.Oracle(lat)
    # random start: from an exactly collinear state flip_h's field frame degenerates
    # (zcp = zsp = 0 when the field lies on z) and the heat bath never leaves the z axis
    e0 = np.random.default_rng(17).normal(size=(1, lat.natom, 3))
    e0 /= np.linalg.norm(e0, axis=-1, keepdims=True)
    o.set_moments(e0)
    o.mt = po.OrcMT()
    o.lib.orc_mt_init(C.byref(o.mt), 17)
    o.setup_ziggurat(17)
    iflip = o.choose_random_atom_x()
    ref_e, ref_m = [], []
    for s in range(ntherm + nmeas):
        o.mc_sweep_ref(mode, T, iflip)
        if (s + 1) % 100 == 0:
            iflip = o.choose_random_atom_x()
        if s >= ntherm:
            ref_e.append(o.energy()["total"][0])
            ref_m.append(o.mavg()[1][0])
    # GPU checkerboard chain, 8 replicas
    latg = lat.with_ensembles(8)
    sim = GpuSimulation(latg, emom=np.broadcast_to(e0, (8, lat.natom, 3)), seed=99)
    sim.relax(mode, T, ntherm)
    ge, gm = [], []
    for s in range(nmeas // 4):
        sim.relax(mode, T, 4)
        obs = sim.observables()
        ge.append(obs["energy"].mean())
        gm.append(obs["mabs"].mean())
    sim.close()
    for ref, gpu in ((ref_e, ge), (ref_m, gm)):
        mr, sr = _binned(ref)
        mg, sg = _binned(gpu)
        assert abs(mr - mg) <= 3.0 * np.hypot(sr, sg), (mr, sr, mg, sg)


def test_square_structured_heat_bath_matches_oracle_chain():
    """The structured square-lattice heat bath is the checkerboard chain (x + y even,
    then odd) of the FP64 path with FP32 draws: per spin within 2e-4 after 3 sweeps."""
    lat = lattice.square_dmi(16, 1.0, 0.3, 0.0, 5.0, 1.0).with_ensembles(2)
    e0 = _rand_unit(np.random.default_rng(8), (2, lat.natom, 3))
    T = 40.0
    sim = GpuSimulation(lat, emom=e0, seed=77)
    sim.relax("H", T, 3, structured=True)
    g = sim.get_moments()
    sim.close()
    o = po.Oracle(lat)
    o.set_moments(e0)
    idx = np.arange(lat.natom)
    par = (idx % 16 + idx // 16) % 2
    order = np.concatenate([idx[par == 0], idx[par == 1]]).astype(np.int32)
    start = np.array([0, (par == 0).sum(), lat.natom], dtype=np.int32)
    for sw in range(3):
        o.mc_sweep_checkerboard("H", T, order, start, 77, sw)
    assert np.max(np.abs(g - o.emom)) < 2e-4


def test_square_structured_statistics_match_fp64_path():
    lat = lattice.square_dmi(16, 1.0, 0.3, 0.0, 5.0, 1.0).with_ensembles(32)
    T = 40.0
    out = []
    for structured in (False, True):
        sim = GpuSimulation(lat, emom=_rand_unit(np.random.default_rng(9 + structured), (32, lat.natom, 3)),
                            seed=5 + structured)
        sim.relax("H", T, 300, structured=structured)
        es = []
        for _ in range(300):
            sim.relax("H", T, 2, structured=structured)
            es.append(sim.observables()["energy"].copy())
        sim.close()
        per_chain = np.array(es).mean(axis=0)
        out.append((per_chain.mean(), per_chain.std(ddof=1) / np.sqrt(per_chain.size)))
    (a, sa), (b, sb) = out
    assert abs(a - b) <= 3 * np.hypot(sa, sb), out


def test_square_structured_refuses_other_lattices():
    from uppasd_gb300 import _lib
    lat = lattice.bcc(4, [1.3, 0.7], 2.2)
    sim = GpuSimulation(lat)
    with pytest.raises(_lib.UppasdGpuError) as ei:
        _lib.call("uppasd_gpu_mc_run_square", sim._h, 8, 100.0, 1)
    assert ei.value.rc == -7
    sim.close()


def test_square_mirror_follows_every_state_change():
    """The structured square path reads an FP32 mirror of the spins: FP64 sweeps, LLG
    steps and put_moments in between must all be seen by the next structured sweep."""
    lat = lattice.square_dmi(16, 1.0, 0.3, 0.0, 5.0, 1.0).with_ensembles(2)
    rng = np.random.default_rng(18)
    e0, e1 = _rand_unit(rng, (2, lat.natom, 3)), _rand_unit(rng, (2, lat.natom, 3))
    T = 40.0
    sim = GpuSimulation(lat, emom=e0, seed=77, sdealgh=5, delta_t=1e-16, damping=0.1, temperature=0.0)
    sim.relax("H", T, 2, structured=True)
    sim.relax("H", T, 1)
    sim.evolve(5)
    sim.relax("H", T, 2, structured=True)
    g1 = sim.get_moments()
    sim.put_moments(e1)
    sim.relax("H", T, 1, structured=True)
    g2 = sim.get_moments()
    sim.close()
    o = po.Oracle(lat)
    o.set_moments(e0)
    o.make_llg(5, 1e-16, 0.1, 0.0, 1.0, noise_mode=po.NOISE_PHILOX, seed=77)
    _, order, start = lattice.greedy_colouring(lat)
    for sw in range(3):
        o.mc_sweep_checkerboard("H", T, order, start, 77, sw)
    for _ in range(5):
        o.sd_step()
    for sw in (3, 4):
        o.mc_sweep_checkerboard("H", T, order, start, 77, sw)
    assert np.max(np.abs(g1 - o.emom)) < 2e-4
    o.set_moments(e1)
    o.mc_sweep_checkerboard("H", T, order, start, 77, 5)
    assert np.max(np.abs(g2 - o.emom)) < 2e-4


@pytest.mark.parametrize("prec", [0, 3])
def test_zero_temperature_metropolis_never_raises_the_energy(prec):
    """relax() with the reference simulator's defaults (Metropolis at T = 0): every taken
    move lowers or keeps the energy, so each sweep's total energy does not rise; the heat
    bath refuses T = 0."""
    lat = lattice.square_dmi(24, 1.0, 0.3, -0.05, 0.5, 1.0).with_ensembles(2)
    rng = np.random.default_rng(91)
    e0 = rng.normal(size=(2, lat.natom, 3))
    e0 /= np.linalg.norm(e0, axis=-1, keepdims=True)
    sim = GpuSimulation(lat, emom=e0, seed=5, precision=prec, sdealgh=5)
    e_prev = sim.observables()["energy"]
    for _ in range(5):
        sim.relax()
        e_now = sim.observables()["energy"]
        assert np.all(e_now <= e_prev + 1e-9 * np.abs(e_prev)), (e_prev, e_now)
        e_prev = e_now
    with pytest.raises(_lib.UppasdGpuError):
        sim.relax("H", 0.0)
    sim.close()


@pytest.mark.parametrize("mode", ["H", "M"])
def test_binder_and_susceptibility_near_tc(mode):
    """Near the L = 6 lattice's ordering temperature (U_L falls from 0.66 to 0.49 between
    1200 and 1400 K) the Binder cumulant and the susceptibility are at their most
    sensitive: the FP64 checkerboard chain (32 replicas) against the reference's
    random-permutation chain (four independent chains, mtprng + ziggurat), within 3 sigma
    of the combined jackknife errors."""
    from uppasd_gb300 import analysis

    lat = lattice.bcc(6, [1.3, 0.7], 2.2)
    T = 1300.0
    ntherm, nmeas = 1000, 12000
    kchi = analysis.MUB ** 2 * lat.natom / analysis.KBOLT ** 2 / T

    def binder(m2, m4):
        return 1.0 - m4 / 3.0 / (m2 * m2)

    def chi(m, m2):
        return (m2 - m * m) * kchi

    # reference chains: blocks of each chain are the jackknife units
    ref_m = []
    for seed in (17, 18, 19, 20):
        o = po.Oracle(lat, threads=1)
        e0 = _rand_unit(np.random.default_rng(seed), (1, lat.natom, 3))
        o.set_moments(e0)
        o.mt = po.OrcMT()
        o.lib.orc_mt_init(C.byref(o.mt), seed)
        o.setup_ziggurat(seed)
        iflip = o.choose_random_atom_x()
        ms = []
        for s in range(ntherm + nmeas):
            o.mc_sweep_ref(mode, T, iflip)
            if (s + 1) % 100 == 0:
                iflip = o.choose_random_atom_x()
            if s >= ntherm:
                ms.append(o.mavg()[1][0])
        ref_m.append(np.array(ms))
    ref_m = np.concatenate(ref_m)  # 4 chains back to back: 80 blocks of 600 sweeps
    ref = {"U": analysis.jackknife(binder, [ref_m ** 2, ref_m ** 4], nbin=80),
           "chi": analysis.jackknife(chi, [ref_m, ref_m ** 2], nbin=80)}
    # GPU: independent replicas are the jackknife units
    nrep = 32
    latg = lat.with_ensembles(nrep)
    sim = GpuSimulation(latg, emom=_rand_unit(np.random.default_rng(5), (nrep, lat.natom, 3)), seed=71)
    sim.relax(mode, T, ntherm)
    gm = []
    for _ in range(nmeas // 2):
        sim.relax(mode, T, 2)
        gm.append(sim.observables()["mabs"].copy())
    sim.close()
    gm = np.array(gm).T.reshape(-1)  # replica-major: one block per replica
    gpu = {"U": analysis.jackknife(binder, [gm ** 2, gm ** 4], nbin=nrep),
           "chi": analysis.jackknife(chi, [gm, gm ** 2], nbin=nrep)}
    for k in ("U", "chi"):
        (gv, ge), (rv, re_) = gpu[k], ref[k]
        print(f"{mode} T={T} {k}: GPU {gv:.5g} +- {ge:.2g}, reference chain {rv:.5g} +- {re_:.2g}")
        assert abs(gv - rv) <= 3.0 * np.hypot(ge, re_), (k, gv, ge, rv, re_)
