"""The reduced Hamiltonian (do_reduced = 'Y', aHam(i) = anumb(i)) in the oracle: one
coupling row per basis atom gives bit-identical fields, energies, LLG steps and Monte
Carlo sweeps to the full (aHam(i) = i) form on translation-invariant lattices."""
import numpy as np
import pytest

from oracle import pyoracle as po
from uppasd_gb300 import lattice


def _rand_unit(rng, shape):
    e = rng.normal(size=shape)
    return e / np.linalg.norm(e, axis=-1, keepdims=True)


LATTICES = {
    "bcc": lambda: lattice.bcc(3, [1.3, 0.7], 2.2),
    "square_dmi": lambda: lattice.square_dmi(8, 1.0, 0.3, -0.05, 0.5, 1.0),
    "kagome_tensor": lambda: lattice.kagome(4, -1.0, 0.1, 0.05, 1.0, 0.2),
}


@pytest.mark.parametrize("kind", sorted(LATTICES))
def test_reduced_equals_full_bit_for_bit(kind):
    full = LATTICES[kind]().with_ensembles(2)
    red = lattice.reduced(full)
    assert red.nham == full.nbasis < full.nham
    e0 = _rand_unit(np.random.default_rng(31), (2, full.natom, 3))
    a, b = po.Oracle(full, threads=1), po.Oracle(red, threads=1)
    for o in (a, b):
        o.set_moments(e0)
    assert np.array_equal(a.field()[0], b.field()[0])
    assert np.array_equal(a.energy()["total"], b.energy()["total"])
    for o in (a, b):
        o.make_llg(5, 1e-16, 0.1, 100.0, 1.0, noise_mode=po.NOISE_PHILOX, seed=4)
        for _ in range(10):
            o.sd_step()
    assert np.array_equal(a.emom, b.emom)
    _, order, start = lattice.greedy_colouring(full)
    for sw in range(2):
        a.mc_sweep_checkerboard("H", 50.0, order, start, 8, sw)
        b.mc_sweep_checkerboard("H", 50.0, order, start, 8, sw)
    assert np.array_equal(a.emom, b.emom)


def test_reduced_refuses_a_random_alloy():
    with pytest.raises(ValueError):
        lattice.reduced(lattice.bcc_alloy(3, seed=1))
