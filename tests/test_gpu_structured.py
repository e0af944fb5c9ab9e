"""Structured mixed-precision LLG path (precision 1: FP64 master, 2: double-single
master) against the FP64 CPU oracle.

The field gather, thermal field and rotation run in FP32, so trajectories are
compared with an FP32-scale tolerance; the spin norm, which the higher-precision
master renormalises every step, is held to 1e-12.
"""
import numpy as np
import pytest

from oracle import pyoracle as po
from uppasd_gb300 import lattice
from uppasd_gb300._lib import UppasdGpuError
from uppasd_gb300.simulation import GpuSimulation

pytestmark = pytest.mark.gpu

# Max per-component deviation from the FP64 oracle.  The FP32 gather and
# rotation inject ~1e-7 relative error per step; from a random start at T = 0 the
# dynamics amplify it (a 1e-7 perturbation of the FP64 oracle's own start grows
# to ~3e-5 in 1000 steps), so the bound widens with the step count.
CHECKPOINTS = {10: 2e-6, 100: 2e-5, 1000: 5e-3}
THERMAL_TOL = 2e-4   # T = 300 K, 200 steps (FP32 vs FP64 Box-Muller noise on top)


def _rand_unit(rng, shape):
    e = rng.normal(size=shape)
    return e / np.linalg.norm(e, axis=-1, keepdims=True)


def _sim(lat, prec, temp, e0, seed=21):
    return GpuSimulation(lat, sdealgh=5, delta_t=1e-16, damping=0.1, temperature=temp, seed=seed, emom=e0,
                         precision=prec)


def _oracle(lat, temp, e0, seed=21):
    o = po.Oracle(lat)
    o.set_moments(e0)
    o.make_llg(5, 1e-16, 0.1, temp, 1.0, noise_mode=po.NOISE_PHILOX, seed=seed)
    return o


def _run(lat, prec, temp, nsteps, e0, seed=21):
    sim = _sim(lat, prec, temp, e0, seed)
    sim.evolve(nsteps)
    e = sim.get_moments()
    sim.close()
    return e


@pytest.mark.parametrize("prec", [1, 2])
@pytest.mark.parametrize("kind", ["bcc2", "alloy4", "alloy4_L5"])
def test_structured_vs_oracle(prec, kind):
    """L = 6 runs the z-marching kernels (compile-time pitches, factorised
    couplings); L = 5 runs the general gather kernels with runtime pitches."""
    if kind == "bcc2":
        lat = lattice.bcc(6, [1.3, 0.7], 2.2).with_ensembles(2)
    elif kind == "alloy4":
        lat = lattice.bcc_alloy(6, seed=4).with_ensembles(2)
    else:
        lat = lattice.bcc_alloy(5, seed=4).with_ensembles(2)
    e0 = _rand_unit(np.random.default_rng(8), (2, lat.natom, 3))
    sim, o = _sim(lat, prec, 0.0, e0), _oracle(lat, 0.0, e0)
    done = 0
    for n, tol in sorted(CHECKPOINTS.items()):
        sim.evolve(n - done)
        for _ in range(n - done):
            o.sd_step()
        done = n
        g = sim.get_moments()
        err = np.max(np.abs(g - o.emom))
        print(f"prec={prec} {kind} T=0 steps={n}: max|GPU-oracle| = {err:.3e}")
        assert err <= tol
        assert np.max(np.abs(np.linalg.norm(g, axis=-1) - 1.0)) <= 1e-12
    sim.close()
    g = _run(lat, prec, 300.0, 200, e0)
    o = _oracle(lat, 300.0, e0)
    for _ in range(200):
        o.sd_step()
    err = np.max(np.abs(g - o.emom))
    print(f"prec={prec} {kind} T=300 steps=200: max|GPU-oracle| = {err:.3e}")
    assert err <= THERMAL_TOL
    assert np.max(np.abs(np.linalg.norm(g, axis=-1) - 1.0)) <= 1e-12


def test_master_variants_agree():
    lat = lattice.bcc_alloy(6, seed=9).with_ensembles(1)
    e0 = _rand_unit(np.random.default_rng(10), (1, lat.natom, 3))
    a = _run(lat, 1, 300.0, 500, e0)
    b = _run(lat, 2, 300.0, 500, e0)
    assert np.max(np.abs(a - b)) <= 1e-4


def test_structured_refuses_unsupported_hamiltonian():
    lat = lattice.square_dmi(16)
    with pytest.raises(UppasdGpuError) as ei:
        GpuSimulation(lat, sdealgh=5, precision=1)
    assert ei.value.rc == -7


def test_structured_observables_and_mc_roundtrip():
    """Observables and MC sweeps read the structured master state."""
    lat = lattice.bcc(6, [1.3, 0.7], 2.2).with_ensembles(2)
    e0 = _rand_unit(np.random.default_rng(11), (2, lat.natom, 3))
    sim = GpuSimulation(lat, sdealgh=5, delta_t=1e-16, damping=0.1, temperature=0.0, emom=e0, precision=2)
    sim.evolve(10)
    e = sim.get_moments()
    o = po.Oracle(lat)
    o.set_moments(e)
    obs = sim.observables()
    assert np.allclose(obs["energy"], o.energy()["total"], rtol=1e-10, atol=1e-12)
    sim.relax("H", 500.0, 2)
    sim.evolve(10)
    e2 = sim.get_moments()
    assert np.max(np.abs(np.linalg.norm(e2, axis=-1) - 1.0)) <= 1e-12
    sim.close()


def _pinned(shape):
    torch = pytest.importorskip("torch")
    return torch.empty(shape, dtype=torch.float64, pin_memory=True).numpy()


@pytest.mark.parametrize("prec", [0, 1, 2, 3, 4])
@pytest.mark.parametrize("M", [3, 8])
@pytest.mark.parametrize("pinned", [True, False])
def test_run_io_equals_put_run_get(prec, M, pinned):
    """sd_run_io (pipelined over ensemble groups with page-locked arrays on the structured
    path, the three calls in turn otherwise) gives exactly what put_moments + sd_run +
    get_moments give, and keeps the step counter."""
    lat = lattice.bcc_alloy(6, seed=3).with_ensembles(M)
    rng = np.random.default_rng(40 + M)
    e0 = _rand_unit(rng, (M, lat.natom, 3))
    e1 = _rand_unit(rng, (M, lat.natom, 3))
    shape = (M, lat.natom, 3)
    a = _sim(lat, prec, 300.0, e0, seed=8)
    b = _sim(lat, prec, 300.0, e0, seed=8)
    a.evolve(3)
    b.evolve(3)
    a.put_moments(e1)
    a.evolve(7)
    ea, ema = a.get_moments(full=True)
    mk = _pinned if pinned else np.empty
    inp, out, outm = mk(shape), mk(shape), mk(shape)
    inp[...] = e1
    b.run_io(inp, 7, out, outm)
    assert np.array_equal(out, ea) and np.array_equal(outm, ema)
    # a second block from the resident state: the counters continue
    a.evolve(5)
    b.run_io(None, 5, out)
    assert np.array_equal(out, a.get_moments())
    # no steps: the conversions in and out alone
    a.put_moments(e1)
    b.run_io(inp, 0, out)
    assert np.array_equal(out, a.get_moments())
    a.close()
    b.close()
