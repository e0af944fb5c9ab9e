"""SDEalgh 7 (semi-implicit spherical midpoint, sispht / sisphf in Evolution/sphmidpoint.f90)
in the oracle.

* three steps against an independent numpy restatement that solves the predictor's and the
  corrector's fixed points by Newton's method on e' = e + dtg u x a1, u = (e + e')/|e + e'|,
  instead of the reference's plain iteration (agreement to 1e-11, the iteration's tolerance
  being 1e-12 per component);
* it converges to the midpoint solver (SDEalgh 1) at first order in dt;
* the norm: at the fixed point e' - e = dtg u x a1 is orthogonal to e' + e, so |e'| = |e|;
  what remains is the iteration's 1e-12 tolerance (3.8e-13 after 100 steps here).
"""
import numpy as np

from oracle import pyoracle as po
from uppasd_gb300 import lattice

GAMA = 1.760859644e11


def _rand_unit(rng, shape):
    e = rng.normal(size=shape)
    return e / np.linalg.norm(e, axis=-1, keepdims=True)


def _fixed_point(e1, a1, dtg):
    """Root of g(x) = x - e1 - dtg (u(x) x a1), u = (e1 + x)/|e1 + x|, by Newton with a
    finite-difference Jacobian (T = 0: no noise term)."""
    x = e1.copy()
    for _ in range(30):
        def g(v):
            w = e1 + v
            return v - e1 - dtg * np.cross(w / np.linalg.norm(w), a1)
        r = g(x)
        J = np.empty((3, 3))
        h = 1e-7
        for c in range(3):
            d = np.zeros(3)
            d[c] = h
            J[:, c] = (g(x + d) - g(x - d)) / (2 * h)
        x = x - np.linalg.solve(J, r)
    return x


def _step(lat, f, e, lam, dt):
    """One sispht + sisphf step of the whole lattice at T = 0 in numpy."""
    mm = lat.mmom[0][:, None]
    dtg = dt * GAMA / (1.0 + lam * lam)
    f.set_moments(e[None])
    b1 = f.field()[0][0]
    mid = np.empty_like(e)
    for n in range(e.shape[0]):
        a1 = -b1[n] - lam * np.cross(e[n], b1[n])
        x = _fixed_point(e[n], a1, dtg)
        mid[n] = (e[n] + x) / np.linalg.norm(e[n] + x)
    f.emomM[0] = mid * mm
    b2 = f.field()[0][0]
    out = np.empty_like(e)
    for n in range(e.shape[0]):
        a1 = -b2[n] - lam * np.cross(mid[n], b2[n])
        out[n] = _fixed_point(e[n], a1, dtg)
    return out


def test_three_steps_match_newton_restatement():
    lat = lattice.square_dmi(4, 1.0, 0.3, -0.05, 0.5, 1.0)
    e0 = _rand_unit(np.random.default_rng(71), (1, lat.natom, 3))
    dt, lam = 1e-16, 0.1
    o = po.Oracle(lat, threads=1)
    o.set_moments(e0)
    o.make_llg(7, dt, lam, 0.0)
    f = po.Oracle(lat, threads=1)
    e = e0[0].copy()
    for _ in range(3):
        o.sd_step()
        e = _step(lat, f, e, lam, dt)
    assert np.max(np.abs(o.emom[0] - e)) <= 1e-11


def test_converges_to_midpoint():
    lat = lattice.bcc(2, [1.3, 0.7], 2.2)
    e0 = _rand_unit(np.random.default_rng(72), (1, lat.natom, 3))
    diffs = []
    for dt in (4e-16, 2e-16, 1e-16):
        out = {}
        for alg in (1, 7):
            o = po.Oracle(lat, threads=1)
            o.set_moments(e0)
            o.make_llg(alg, dt, 0.1, 0.0)
            for _ in range(int(round(2e-14 / dt))):
                o.sd_step()
            out[alg] = o.emom.copy()
        diffs.append(np.max(np.abs(out[1] - out[7])))
    # first order at least: halving dt at least roughly halves the difference
    assert diffs[1] < 0.7 * diffs[0] and diffs[2] < 0.7 * diffs[1], diffs
    assert diffs[2] < 1e-4


def test_norm_kept_to_the_iteration_tolerance():
    lat = lattice.bcc(2, [1.3, 0.7], 2.2)
    e0 = _rand_unit(np.random.default_rng(73), (1, lat.natom, 3))
    o = po.Oracle(lat, threads=1)
    o.set_moments(e0)
    o.make_llg(7, 1e-16, 0.1, 0.0)
    for _ in range(100):
        o.sd_step()
    assert np.max(np.abs(np.linalg.norm(o.emom[0], axis=1) - 1.0)) < 1e-11
