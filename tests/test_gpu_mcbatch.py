"""Batched replica Monte Carlo (one persistent launch over uneven replicas).

* chain parity: each replica's checkerboard chain equals the oracle's
  restatement of the same chain (same colours, same Philox draws) within the
  FP32 gather's error, for heat bath, Metropolis and a mixed table;
* the chain does not depend on the schedule (CTAs per replica, block size):
  the spins are bit-identical after the same sweeps;
* the per-sweep observables built from exact update deltas equal the oracle's
  energy and magnetisation of the final state;
* statistics: E, |M|, Binder cumulant and susceptibility of the batched chain
  agree with the reference's own chain (random-permutation order, mtprng +
  ziggurat) within 3 sigma;
* the autotuner installs a valid schedule and reuses its cache.
"""
import ctypes as C

import numpy as np
import pytest

from oracle import pyoracle as po
from uppasd_gb300 import analysis, lattice
from uppasd_gb300.batch import ReplicaBatch

pytestmark = pytest.mark.gpu

J = [1.3, 0.7]


def colour_order(L):
    idx = np.arange(2 * L ** 3)
    b = idx % 2
    cell = idx // 2
    x, y, z = cell % L, (cell // L) % L, cell // (L * L)
    p = (x + y + z) & 1
    order, start = [], [0]
    for c in range(4):
        sel = idx[(b == c >> 1) & (p == (c & 1))]
        order.append(sel)
        start.append(start[-1] + sel.size)
    return np.concatenate(order), np.array(start)


@pytest.mark.parametrize("modes", ["H", "M", "mixed"])
def test_batch_chain_matches_oracle(modes):
    L = [4, 6, 4]
    T = [500.0, 900.0, 1300.0]
    hb = {"H": [1, 1, 1], "M": [0, 0, 0], "mixed": [1, 0, 1]}[modes]
    b = ReplicaBatch(L, T, heatbath=hb, seed=321, max_sweeps_per_launch=8)
    s0 = b.get_spins()
    b.run(3, sweeps_per_launch=2)  # one graph replay and one direct launch
    s1 = b.get_spins()
    b.close()
    for r in range(3):
        lat = lattice.bcc(L[r], J, 2.2).with_ensembles(r + 1)
        o = po.Oracle(lat)
        o.set_moments(np.broadcast_to(s0[r], (r + 1, lat.natom, 3)))
        order, start = colour_order(L[r])
        for sw in range(3):
            o.mc_sweep_checkerboard("H" if hb[r] else "M", T[r], order, start, 321, sw)
        d = np.abs(o.emom[r] - s1[r]).max()
        assert d < 2e-4, (r, d)
        assert np.abs(np.linalg.norm(s1[r], axis=1) - 1).max() < 1e-6


def test_chain_independent_of_schedule():
    L = [4, 8, 6, 4]
    T = [600.0, 800.0, 1000.0, 1200.0]
    a = ReplicaBatch(L, T, heatbath=[1, 0, 1, 0], seed=77, max_sweeps_per_launch=8)
    b = ReplicaBatch(L, T, heatbath=[1, 0, 1, 0], seed=77, max_sweeps_per_launch=8)
    a.set_schedule(64, [1, 5, 3, 2], reg_build=2)
    b.set_schedule(256, [2, 1, 1, 1], reg_build=0)
    a.run(5, sweeps_per_launch=5)
    b.run(5, sweeps_per_launch=2)
    for sa, sb in zip(a.get_spins(), b.get_spins()):
        assert np.array_equal(sa, sb)
    a.close()
    b.close()


def test_observables_equal_oracle_of_final_state():
    L = [4, 6]
    T = [700.0, 1100.0]
    b = ReplicaBatch(L, T, seed=5, series_len=64, bfield=[0.0, 0.0, 2.0])
    b.run(10, sweeps_per_launch=4, measure=True)
    st = b.stats()
    spins = b.get_spins()
    s = b.series()
    assert s.shape == (2, 10, 2)
    for r in range(2):
        lat = lattice.bcc(L[r], J, 2.2)
        lat.extfield[..., 2] = 2.0
        o = po.Oracle(lat)
        o.set_moments(spins[r][None])
        E = o.energy()["total"][0]
        mv, ma = o.mavg()
        assert abs(st["last"][r, 0] - E) <= 1e-5 * abs(E) + 1e-8, (st["last"][r, 0], E)
        assert np.allclose(st["last"][r, 1:], mv[0] / lat.natom, atol=1e-6)  # oracle mvec is the sum
        assert abs(s[r, -1, 0] - st["last"][r, 0]) < 1e-12
        assert abs(s[r, -1, 1] - ma[0]) < 1e-6
        assert abs(st["E"][r] - s[r, :, 0].mean()) < 1e-9 * abs(st["E"][r])
        assert abs(st["M"][r] - s[r, :, 1].mean()) < 1e-9
    assert (st["n"] == 10).all()
    b.close()


def _reference_chain(L, T, mode, ntherm, nmeas, seed):
    lat = lattice.bcc(L, J, 2.2)
    o = po.Oracle(lat)
    # random start: from an exactly collinear state flip_h's field frame degenerates
    # (zcp = zsp = 0 when the field lies on z) and the heat bath never leaves the z axis
    e0 = np.random.default_rng(seed).normal(size=(1, lat.natom, 3))
    e0 /= np.linalg.norm(e0, axis=-1, keepdims=True)
    o.set_moments(e0)
    o.mt = po.OrcMT()
    o.lib.orc_mt_init(C.byref(o.mt), seed)
    o.setup_ziggurat(seed)
    iflip = o.choose_random_atom_x()
    es, ms = [], []
    for s in range(ntherm + nmeas):
        o.mc_sweep_ref(mode, T, iflip)
        if (s + 1) % 100 == 0:
            iflip = o.choose_random_atom_x()
        if s >= ntherm:
            es.append(o.energy()["total"][0])
            ms.append(o.mavg()[1][0])
    return np.array(es), np.array(ms)


def _binder(m2, m4):
    return 1.0 - m4 / 3.0 / (m2 * m2)


@pytest.mark.parametrize("mode", ["H", "M"])
def test_statistics_match_reference_chain(mode):
    L, T = 6, 900.0
    ntherm, nmeas = 500, 3000
    natom = 2 * L ** 3
    re, rm = _reference_chain(L, T, mode, ntherm, nmeas, 17)
    nrep = 16
    b = ReplicaBatch([L] * nrep, [T] * nrep, heatbath=1 if mode == "H" else 0, seed=99, series_len=nmeas)
    b.run(ntherm, sweeps_per_launch=100)
    b.run(nmeas, sweeps_per_launch=100, measure=True)
    s = b.series()
    st = b.stats()
    b.close()
    # GPU: independent replicas -> mean and spread over replicas
    def over_replicas(v):
        return v.mean(), v.std(ddof=1) / np.sqrt(v.size)
    g = {
        "E": over_replicas(s[:, :, 0].mean(axis=1)),
        "M": over_replicas(s[:, :, 1].mean(axis=1)),
        "U": over_replicas(_binder((s[:, :, 1] ** 2).mean(1), (s[:, :, 1] ** 4).mean(1))),
        "chi": over_replicas(st["chi"]),
    }
    kchi = analysis.MUB ** 2 * natom / analysis.KBOLT ** 2 / T
    ref = {
        "E": analysis.binned_mean(re),
        "M": analysis.binned_mean(rm),
        "U": analysis.jackknife(lambda a, c: _binder(a, c), [rm ** 2, rm ** 4]),
        "chi": analysis.jackknife(lambda a, c: (c - a * a) * kchi, [rm, rm ** 2]),
    }
    for k in g:
        (gm, ge), (rmn, rerr) = g[k], ref[k]
        assert abs(gm - rmn) <= 3.0 * np.hypot(ge, rerr), (k, gm, ge, rmn, rerr)


def test_autotune_installs_and_caches(tmp_path):
    L = [4, 6, 8, 10, 4, 12]
    T = list(np.linspace(600.0, 1400.0, 6))
    cache = str(tmp_path / "tune")
    a = ReplicaBatch(L, T, seed=9, max_sweeps_per_launch=16)
    ms = a.autotune(sweeps_per_trial=4, cache=cache)
    bld, t, c = a.schedule()
    assert ms > 0 and bld in (0, 1, 2) and t in (64, 128, 256) and c.min() >= 1
    assert open(cache).read().count("mcbatch-v2") == 1
    a.run(8, sweeps_per_launch=8)
    assert all(np.abs(np.linalg.norm(s, axis=1) - 1).max() < 1e-6 for s in a.get_spins())
    b = ReplicaBatch(L, T, seed=9, max_sweeps_per_launch=16)
    b.autotune(sweeps_per_trial=4, cache=cache)
    bld2, t2, c2 = b.schedule()
    assert bld2 == bld and t2 == t and np.array_equal(c2, c)
    a.close()
    b.close()


def test_full_replica_table_invariants():
    """The 64-replica temperature x size table: norms stay 1 and the incremental
    energy of every replica equals the recount of its final state."""
    Ls = [16, 24, 32, 48]
    Ts = np.linspace(600.0, 1400.0, 16)
    L = [l for l in Ls for _ in Ts]
    T = [t for _ in Ls for t in Ts]
    b = ReplicaBatch(L, T, seed=2024, series_len=16)
    b.run(30, sweeps_per_launch=10, measure=True)
    st = b.stats()
    spins = b.get_spins()
    for r in (0, 17, 40, 63):
        assert np.abs(np.linalg.norm(spins[r], axis=1) - 1).max() < 1e-6
        lat = lattice.bcc(L[r], J, 2.2)
        o = po.Oracle(lat)
        o.set_moments(spins[r][None])
        E = o.energy()["total"][0]
        assert abs(st["last"][r, 0] - E) <= 2e-5 * abs(E), (r, st["last"][r, 0], E)
    b.close()


def test_replica_exchange_keeps_the_distribution():
    """Temperature swaps between ladder neighbours: the slots stay a permutation
    within each size, swaps are accepted, and per-temperature E and |M| agree with
    the same table run without exchange within 3 sigma (independent replicas per
    temperature on each side)."""
    Ts = list(np.linspace(900.0, 1500.0, 8))
    copies = 24
    L = [6] * (8 * copies)
    T = Ts * copies
    res = {}
    for ex in (False, True):
        b = ReplicaBatch(L, T, seed=41 + ex, series_len=2000, max_sweeps_per_launch=16)
        if ex:
            # exchange within each copy of the ladder only: build one batch per copy
            b.close()
            stats = []
            for c in range(copies):
                bb = ReplicaBatch([6] * 8, Ts, seed=100 + c, series_len=2000, max_sweeps_per_launch=16)
                bb.set_exchange(True)
                bb.run(400, 4)
                bb.run(2000, 4, measure=True)
                slot, pairs, att, acc = bb.exchange_state()
                assert sorted(slot.tolist()) == list(range(8))
                assert att.sum() > 0 and acc.sum() > 0
                stats.append(bb.series())
                bb.close()
            s = np.concatenate(stats, axis=0)  # (copies*8, n, 2), slot order per copy
        else:
            b.run(400, 4)
            b.run(2000, 4, measure=True)
            s = b.series()
            b.close()
        per_t = s.reshape(copies, 8, -1, 2).mean(axis=2)  # (copies, T, 2)
        res[ex] = (per_t.mean(axis=0), per_t.std(axis=0, ddof=1) / np.sqrt(copies))
    (m0, s0), (m1, s1) = res[False], res[True]
    assert np.all(np.abs(m0 - m1) <= 3.0 * np.hypot(s0, s1) + 1e-12), (m0, m1, s0, s1)


def test_split_table_reproduces_the_whole_table():
    """A table split into shares (one per GPU on a multi-GPU machine) with replica ids
    continuing across shares: every replica's chain, and so its spins and
    accumulators, equals the one it has in the whole table."""
    L = [4, 6, 4, 6, 4, 4]
    T = [500.0, 800.0, 1000.0, 1200.0, 1300.0, 1500.0]
    whole = ReplicaBatch(L, T, seed=61, series_len=8, max_sweeps_per_launch=4)
    whole.run(6, sweeps_per_launch=4, measure=True)
    sw, (aw, nw, lw) = whole.get_spins(), whole.raw_stats()
    whole.close()
    parts = [ReplicaBatch(L[:3], T[:3], seed=61, series_len=8, max_sweeps_per_launch=4, first_id=0),
             ReplicaBatch(L[3:], T[3:], seed=61, series_len=8, max_sweeps_per_launch=4, first_id=3)]
    sp, ap = [], []
    for b in parts:
        b.run(6, sweeps_per_launch=4, measure=True)
        sp += b.get_spins()
        ap.append(b.raw_stats()[0])
        b.close()
    for r in range(len(L)):
        assert np.array_equal(sw[r], sp[r]), r
    assert np.allclose(np.concatenate(ap), aw, rtol=1e-12, atol=0)
