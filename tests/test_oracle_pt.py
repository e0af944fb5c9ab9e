"""The oracle's restatement of pt_iphase (pt_driver.f90:58-367) with ensembles as replicas."""
import numpy as np

from oracle import pyoracle as po
from uppasd_gb300 import lattice


def _setup(M=4, seed=0):
    lat = lattice.square_dmi(8, 1.0, 0.3, -0.05, 0.5, 1.0).with_ensembles(M)
    e = np.random.default_rng(seed).normal(size=(M, lat.natom, 3))
    e /= np.linalg.norm(e, axis=-1, keepdims=True)
    o = po.Oracle(lat, threads=1)
    o.set_moments(e)
    _, order, start = lattice.greedy_colouring(lat)
    return lat, o, order, start


def test_equal_temperatures_swap_always_and_trials_follow_the_schedule():
    _, o, order, start = _setup()
    T, trial, hit, _ = o.pt_iphase([20.0] * 4, 40, 2, order, start, 7)
    # swap steps 2, 4, ..., 34 (the first 90 %), pairs (0,1), (2,3), then (1,2)
    assert trial == 17 * 3 and hit == trial
    assert np.all(T == 20.0)


def test_temperatures_come_back_permuted():
    _, o, order, start = _setup(M=6, seed=1)
    temps = [4.0, 8.0, 12.0, 16.0, 24.0, 32.0]
    T, trial, hit, sel = o.pt_iphase(temps, 60, 3, order, start, 11)
    assert sorted(T) == temps
    assert 0 <= hit <= trial and 0 <= sel < 6


def test_per_ensemble_temperatures_match_separate_runs():
    """One sweep with temps[k] per ensemble equals sweeps at each temperature alone."""
    lat, o, order, start = _setup(M=2, seed=2)
    e0 = o.emom.copy()
    o.mc_sweep_checkerboard("H", 0.0, order, start, 5, 0, temps=[10.0, 30.0])
    both = o.emom.copy()
    for k, T in enumerate((10.0, 30.0)):
        p = po.Oracle(lat, threads=1)
        p.set_moments(e0)
        p.mc_sweep_checkerboard("H", T, order, start, 5, 0)
        assert np.array_equal(p.emom[k], both[k])
