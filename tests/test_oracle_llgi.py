"""SDEalgh 11 (LLGI, Evolution/llgi.f90) in the oracle.

* two steps against an independent numpy restatement that solves A m = B with
  numpy.linalg.solve instead of the explicit adjugate of llgiheun (1e-12);
* relaxtime = 0 converges to the Depondt solution at first order in dt;
* the spin norm stays 1 to rounding.
"""
import numpy as np

from oracle import pyoracle as po
from uppasd_gb300 import lattice

GAMA = 1.760859644e11


def _rand_unit(rng, shape):
    e = rng.normal(size=shape)
    return e / np.linalg.norm(e, axis=-1, keepdims=True)


def _solve_step(lam, dt, tau, et, e1, h):
    beta = -lam * (1.0 + tau / dt)
    zeta = -lam * (tau / dt)
    dtg = -dt * GAMA
    out = np.empty_like(e1)
    for n in range(e1.shape[0]):
        x, y, z = e1[n]
        A = np.array([[1.0, -beta * z, beta * y], [beta * z, 1.0, -beta * x], [-beta * y, beta * x, 1.0]])
        B = e1[n] + dtg * np.cross(e1[n], h[n]) + zeta * np.cross(et[n], e1[n])
        out[n] = np.linalg.solve(A, B)
    return out


def test_two_steps_match_numpy_restatement():
    lat = lattice.bcc(2, [1.3, 0.7], 2.2)
    e0 = _rand_unit(np.random.default_rng(61), (1, lat.natom, 3))
    dt, lam, tau = 1e-16, 0.1, 2e-15
    o = po.Oracle(lat, threads=1)
    o.set_moments(e0)
    o.make_llg(11, dt, lam, 0.0, relaxtime=tau)
    f = po.Oracle(lat, threads=1)
    m, mpast = e0[0].copy(), np.zeros_like(e0[0])
    mm = lat.mmom[0][:, None]
    for _ in range(2):
        o.sd_step()
        f.set_moments(m[None])
        b1 = f.field()[0][0]
        pred = _solve_step(lam, dt, tau, mpast, m, b1)
        f.emomM[0] = pred * mm
        b2 = f.field()[0][0]
        corr = _solve_step(lam, dt, tau, mpast, m, 0.5 * b2 + 0.5 * b1)
        mpast = m
        m = corr / np.linalg.norm(corr, axis=1, keepdims=True)
    assert np.max(np.abs(o.emom[0] - m)) <= 1e-12


def test_zero_relaxtime_converges_to_depondt():
    lat = lattice.bcc(2, [1.3, 0.7], 2.2)
    e0 = _rand_unit(np.random.default_rng(62), (1, lat.natom, 3))
    out = {}
    for alg, dt, n in ((5, 1e-18, 2000), (11, 2e-18, 1000), (11, 1e-18, 2000)):
        o = po.Oracle(lat, threads=1)
        o.set_moments(e0)
        o.make_llg(alg, dt, 0.1, 0.0)
        for _ in range(n):
            o.sd_step()
        out[(alg, dt)] = o.emom.copy()
        assert np.abs(np.linalg.norm(o.emom, axis=-1) - 1.0).max() < 1e-14
    d1 = np.abs(out[(11, 2e-18)] - out[(5, 1e-18)]).max()
    d2 = np.abs(out[(11, 1e-18)] - out[(5, 1e-18)]).max()
    assert d2 < 0.6 * d1 and d2 < 1e-3


def test_perp_projection_is_a_small_change_per_step():
    """perp = 'Y' removes the field along emom: each solver's step changes by far less
    than the step itself (the parallel part does not drive the LLG equation)."""
    lat = lattice.bcc(2, [1.3, 0.7], 2.2)
    e0 = _rand_unit(np.random.default_rng(63), (1, lat.natom, 3))
    for alg in (1, 4, 5, 6, 11):
        out = []
        for perp in (False, True):
            o = po.Oracle(lat, threads=1)
            o.set_moments(e0)
            o.make_llg(alg, 1e-17, 0.1, 0.0, perp=perp)
            o.sd_step()
            out.append(o.emom.copy())
        step = np.abs(out[0] - e0).max()
        diff = np.abs(out[0] - out[1]).max()
        assert 0.0 < diff < 0.2 * step, (alg, diff, step)
