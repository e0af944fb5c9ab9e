"""Host statistics: Sokal's tau_int on processes with known autocorrelation,
jackknife, and the reference's cumulant formulas against the oracle's running
form (calc_and_print_cumulant)."""
import numpy as np

from uppasd_gb300 import analysis


def ar1(phi, n, seed):
    rng = np.random.default_rng(seed)
    e = rng.normal(size=n)
    x = np.empty(n)
    x[0] = e[0] / np.sqrt(1 - phi * phi)
    for i in range(1, n):
        x[i] = phi * x[i - 1] + e[i]
    return x


def test_tau_int_uncorrelated():
    t, W = analysis.tau_int(np.random.default_rng(1).normal(size=50000))
    assert abs(t - 0.5) < 0.05


def test_tau_int_ar1():
    for phi in (0.5, 0.9):
        exact = (1 + phi) / (2 * (1 - phi))
        x = ar1(phi, 200000, 3)
        t, W = analysis.tau_int(x)
        err = analysis.tau_int_error(t, W, x.size)
        assert abs(t - exact) < 4 * err + 0.02 * exact, (phi, t, exact, err)


def test_jackknife_linear_matches_binned():
    x = np.random.default_rng(4).normal(size=4000)
    m, e = analysis.jackknife(lambda a: a, [x])
    bm, be = analysis.binned_mean(x)
    assert abs(m - bm) < 1e-12 and abs(e - be) < 1e-9


def test_cumulants_match_oracle_running_form():
    from oracle import pyoracle as po
    import ctypes as C
    rng = np.random.default_rng(8)
    natom, nsamp, T = 16, 50, 700.0
    lib = po.load()
    cu = po.OrcCumulant() if hasattr(po, "OrcCumulant") else None
    if cu is None:
        import pytest
        pytest.skip("oracle exposes no cumulant struct")
    out = (C.c_double * 6)()
    ms, es = [], []
    for k in range(nsamp):
        e = rng.normal(size=(natom, 3)) + np.array([0, 0, 2.0])
        e /= np.linalg.norm(e, axis=1, keepdims=True)
        emomM = np.ascontiguousarray(2.2 * e)
        en = np.array([rng.normal()])
        lib.orc_cumulant_update(C.byref(cu), natom, 1, emomM.ctypes.data_as(po.F64P), T,
                                en.ctypes.data_as(po.F64P), out)
        ms.append(np.linalg.norm(emomM.sum(axis=0)) / natom)
        es.append(en[0])
    ms, es = np.array(ms), np.array(es)
    c = analysis.cumulants(nsamp, es.sum(), (es ** 2).sum(), ms.sum(), (ms ** 2).sum(), (ms ** 4).sum(), natom, T)
    # running weights grow by one per sample: the oracle's averages are weighted, not plain
    w = np.arange(1, nsamp + 1, dtype=np.float64)
    wm = lambda v: (w * v).sum() / w.sum()
    assert abs(out[0] - wm(ms)) < 1e-12
    assert abs(out[1] - wm(ms ** 2)) < 1e-12
    u = 1 - wm(ms ** 4) / 3 / wm(ms ** 2) ** 2
    assert abs(out[3] - u) < 1e-12
    assert abs(c["binder"] - (1 - (ms ** 4).mean() / 3 / (ms ** 2).mean() ** 2)) < 1e-12


def test_topological_charge_of_a_skyrmion_and_uniform_states():
    from uppasd_gb300.analysis import topological_charge
    L = 32
    y, x = np.mgrid[0:L, 0:L]
    r = np.hypot(x - L / 2 + 0.5, y - L / 2 + 0.5)
    th = np.pi * np.exp(-(r / 5) ** 2)
    ph = np.arctan2(y - L / 2 + 0.5, x - L / 2 + 0.5)
    e = np.stack([np.sin(th) * np.cos(ph), np.sin(th) * np.sin(ph), np.cos(th)], -1).reshape(L * L, 3)
    assert abs(topological_charge(e, L) + 1.0) < 1e-9          # one skyrmion, core against +z
    assert abs(topological_charge(-e, L) - 1.0) < 1e-9         # the reversed texture
    two = np.stack([e, np.tile([0.0, 0.0, 1.0], (L * L, 1))])
    assert np.allclose(topological_charge(two, L), [-1.0, 0.0], atol=1e-9)
