"""Statistics of Monte Carlo series: the reference's cumulant formulas and the
integrated autocorrelation time.

* ``cumulants`` forms <M>, <M^2>, <M^4>, the Binder cumulant, the susceptibility
  and the specific heat from plain sample moments, with the expressions and
  units of calc_and_print_cumulant (Measurement/prn_averages.f90:960-990):
  U_L = 1 - <M^4> / (3 <M^2>^2), chi = (<M^2> - <M>^2) muB^2 N / kB^2 / T,
  C_v = (<E^2> - <E>^2) mRy^2 N / kB^2 / T^2.
* ``tau_int`` is Sokal's windowed estimator: rho(t) from the FFT of the
  centred series, tau(W) = 1/2 + sum_{t=1..W} rho(t), W the first window with
  W >= c tau(W) (c = 6); an uncorrelated series gives 1/2, so n / (2 tau) is
  the number of independent samples.
"""
from __future__ import annotations

import numpy as np

KBOLT = 1.38064852e-23
MUB = 9.274009994e-24
MRY = 2.179872325e-21


def cumulants(n, sE, sE2, sM, sM2, sM4, natom, temperature):
    n = np.asarray(n, dtype=np.float64)
    with np.errstate(invalid="ignore", divide="ignore"):
        m, m2, m4 = sM / n, sM2 / n, sM4 / n
        e, e2 = sE / n, sE2 / n
        binder = 1.0 - m4 / 3.0 / (m2 * m2)
        chi = (m2 - m * m) * MUB * MUB * natom / (KBOLT * KBOLT) / temperature
        cv = (e2 - e * e) * MRY * MRY * natom / (KBOLT * KBOLT) / (temperature * temperature)
    return {"M": m, "M2": m2, "M4": m4, "E": e, "E2": e2, "binder": binder, "chi": chi, "cv": cv}


def autocorrelation(x):
    x = np.asarray(x, dtype=np.float64)
    n = x.size
    y = x - x.mean()
    f = np.fft.rfft(y, n=2 * n)
    acf = np.fft.irfft(f * np.conj(f))[:n]
    if acf[0] <= 0.0:
        return np.zeros(n)
    return acf / acf[0]


def tau_int(x, c: float = 6.0):
    """Integrated autocorrelation time (in samples) and its window."""
    rho = autocorrelation(x)
    n = rho.size
    if n < 4 or not np.any(rho):
        return 0.5, 0
    csum = 0.5 + np.cumsum(rho[1:])
    w = np.arange(1, n)
    ok = np.nonzero(w >= c * csum)[0]
    W = int(w[ok[0]]) if ok.size else n - 1
    return float(max(csum[W - 1], 0.5)), W


def tau_int_error(tau, W, n):
    """Sokal's variance estimate: var(tau) ~ 2 (2W + 1) / n * tau^2."""
    return float(np.sqrt(2.0 * (2 * W + 1) / n) * tau)


def binned_mean(x, nbin: int = 20):
    """Mean and its standard error from `nbin` equal blocks."""
    x = np.asarray(x, dtype=np.float64)
    m = x.size // nbin * nbin
    b = x[:m].reshape(nbin, -1).mean(axis=1)
    return float(b.mean()), float(b.std(ddof=1) / np.sqrt(nbin))


def jackknife(fn, columns, nbin: int = 20):
    """Jackknife estimate and error of fn(*block_means) over `nbin` blocks of the columns."""
    cols = [np.asarray(c, dtype=np.float64) for c in columns]
    m = min(c.size for c in cols) // nbin * nbin
    blocks = [c[:m].reshape(nbin, -1).sum(axis=1) for c in cols]
    tot = [b.sum() for b in blocks]
    full = fn(*[t / m for t in tot])
    k = m // nbin
    loo = np.array([fn(*[(t - b[i]) / (m - k) for t, b in zip(tot, blocks)]) for i in range(nbin)])
    err = np.sqrt((nbin - 1) / nbin * np.sum((loo - loo.mean()) ** 2))
    return float(full), float(err)


def topological_charge(emom, L: int):
    """Skyrmion number of each configuration of an L x L square monolayer with periodic
    edges (site i = x + L y), from unit spins of shape (..., L*L, 3): every plaquette
    split into two triangles, each contributing its signed solid angle
    2 atan2(a.(b x c), 1 + a.b + b.c + c.a) (Berg and Luescher), summed and divided by 4 pi."""
    s = np.asarray(emom, dtype=np.float64)
    s = s.reshape(s.shape[:-2] + (L, L, 3))           # [..., y, x, 3]
    a = s
    b = np.roll(s, -1, axis=-2)                       # (x + 1, y)
    c = np.roll(b, -1, axis=-3)                       # (x + 1, y + 1)
    d = np.roll(s, -1, axis=-3)                       # (x, y + 1)

    def omega(p, q, r):
        num = np.einsum("...k,...k->...", p, np.cross(q, r))
        den = 1.0 + np.einsum("...k,...k->...", p, q) + np.einsum("...k,...k->...", q, r) + \
            np.einsum("...k,...k->...", r, p)
        return 2.0 * np.arctan2(num, den)

    tot = omega(a, b, c) + omega(a, c, d)
    return tot.sum(axis=(-2, -1)) / (4.0 * np.pi)
