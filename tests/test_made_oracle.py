"""CPU restatement of the learned proposal (oracle/made_oracle.py): its analytic
gradient against central finite differences, the autoregressive structure of
its masks, the vMF normalisation, and the patch energy change against the
oracle's full-lattice energy."""
import numpy as np
import pytest

from oracle import made_oracle as mo


def test_gradient_matches_finite_differences():
    vec = mo.random_params(1, scale_out=1.0).astype(np.float64)
    X = mo.random_windows(8, 2).astype(np.float64)
    loss, g = mo.loss_grad(vec, X, 3.0)
    rng = np.random.default_rng(0)
    m = np.concatenate([mm.ravel() for mm in mo.masks()] + [np.ones(256 * 3 + 64)])
    idx = rng.choice(np.nonzero(m)[0], 40, replace=False)
    h = 1e-6
    for i in idx:
        vp, vm = vec.copy(), vec.copy()
        vp[i] += h
        vm[i] -= h
        fd = (mo.loss_grad(vp, X, 3.0)[0] - mo.loss_grad(vm, X, 3.0)[0]) / (2 * h)
        assert abs(fd - g[i]) <= 1e-6 + 1e-5 * abs(fd), (i, fd, g[i])


def test_outputs_are_autoregressive():
    vec = mo.random_params(3, scale_out=1.0)
    X = mo.random_windows(4, 4).astype(np.float64)
    O0 = mo.forward(vec, X)[0]
    pos = mo.interior_positions()
    for grp in range(4):
        X1 = X.copy()
        for s in range(16):
            if mo.patch_group(s // 4, s % 4) == grp:
                X1[:, pos[s] * 3:pos[s] * 3 + 3] *= -1.0
        O1 = mo.forward(vec, X1)[0]
        for s in range(16):
            g_out = mo.patch_group(s // 4, s % 4)
            changed = np.max(np.abs(O1[:, 3 * s:3 * s + 3] - O0[:, 3 * s:3 * s + 3])) > 0
            assert changed == (g_out > grp), (grp, s)


@pytest.mark.parametrize("kappa", [1e-9, 0.3, 5.0, 200.0])
def test_vmf_normalised(kappa):
    # integrate exp(log vMF) over the sphere in (cos theta, phi) about eta
    t = np.linspace(-1, 1, 200001)
    eta = np.array([0.0, 0.0, kappa])
    x = np.stack([np.sqrt(1 - t * t), np.zeros_like(t), t], axis=1)
    dens = np.exp(mo.log_vmf(eta[None, :], x))
    total = 2 * np.pi * np.trapezoid(dens, t)
    assert abs(total - 1.0) < 2e-3


def test_patch_energy_change_matches_full_energy():
    from oracle import pyoracle as po
    from uppasd_gb300 import lattice
    lat = lattice.square_dmi(8, 1.0, 0.3, 0.0, 20.0, 1.0)
    rng = np.random.default_rng(5)
    e = rng.normal(size=(1, lat.natom, 3))
    e /= np.linalg.norm(e, axis=-1, keepdims=True)
    o = po.Oracle(lat)
    o.set_moments(e)
    E0 = o.energy()["total"][0] * lat.natom
    newp = rng.normal(size=(16, 3))
    newp /= np.linalg.norm(newp, axis=1, keepdims=True)
    dE = mo.patch_energy_change(lat, e * lat.mmom[0][None, :, None], 0, 4, 4, newp)
    e2 = e.copy()
    for s in range(16):
        i = (4 + s % 4) % 8 + 8 * ((4 + s // 4) % 8)
        e2[0, i] = newp[s]
    o.set_moments(e2)
    E1 = o.energy()["total"][0] * lat.natom
    # orc_energy is in mRy per atom; dE in T muB -> mRy: * muB / mRy
    assert abs((E1 - E0) - dE * mo_mub_over_mry()) < 1e-9 * max(1.0, abs(E1 - E0))


def mo_mub_over_mry():
    return 9.274009994e-24 / 2.179872325e-21
