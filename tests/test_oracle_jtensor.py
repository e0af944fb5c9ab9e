"""The oracle's exchange-tensor path (do_jtensor = 1) on the CPU.

* an isotropic tensor J_ab = ncoup delta_ab reproduces the scalar exchange bit for
  bit (field, energy, LLG steps, Monte Carlo sweeps): the tensor rows add only exact
  zeros on top of the scalar products;
* the tensor field equals an independent numpy restatement of tensor_field
  (Hamiltonian/hamiltonianactions.f90:499-542) on the kagome tensor lattice;
* the pair energy is -1/2 sum m_i . b_i (energy.f90:244-247) and, with J_ji = J_ij^T,
  the Metropolis energy change of one spin matches a full-energy difference.
"""
import numpy as np
import pytest

from oracle import pyoracle as po
from uppasd_gb300 import lattice
from uppasd_gb300.lattice import MRY, MUB


def _rand_unit(rng, shape):
    e = rng.normal(size=shape)
    return e / np.linalg.norm(e, axis=-1, keepdims=True)


def _numpy_tensor_field(lat, emomM):
    J = np.swapaxes(lat.j_tens, -1, -2)          # [ih, slot, a, b]
    ih = lat.aham - 1
    nl = lat.nlist - 1
    b = np.zeros_like(emomM)
    for s in range(lat.max_no_neigh):
        on = s < lat.nlistsize[ih]
        mj = emomM[:, nl[:, s], :]               # (M, N, 3)
        b += np.where(on[None, :, None], np.einsum("nab,mnb->mna", J[ih, s], mj), 0.0)
    return b


def test_isotropic_tensor_is_the_scalar_exchange_bit_for_bit():
    lat = lattice.bcc(3, [1.3, 0.7], 2.2).with_ensembles(2)
    lt = lattice.with_isotropic_tensor(lat)
    e0 = _rand_unit(np.random.default_rng(11), (2, lat.natom, 3))
    a, b = po.Oracle(lat, threads=1), po.Oracle(lt, threads=1)
    for o in (a, b):
        o.set_moments(e0)
    fa, ea = a.field()
    fb, eb = b.field()
    assert np.array_equal(fa, fb) and ea == eb
    assert all(np.array_equal(a.energy()[k], b.energy()[k]) for k in ("total", "xc"))
    for o in (a, b):
        o.make_llg(5, 1e-16, 0.1, 300.0, 1.0, noise_mode=po.NOISE_PHILOX, seed=3)
        for _ in range(20):
            o.sd_step()
    assert np.array_equal(a.emom, b.emom)
    _, order, start = lattice.greedy_colouring(lat)
    for mode in ("M", "H"):
        for sw in range(3):
            a.mc_sweep_checkerboard(mode, 500.0, order, start, 9, sw)
            b.mc_sweep_checkerboard(mode, 500.0, order, start, 9, sw)
        assert np.array_equal(a.emom, b.emom)


def test_kagome_tensor_field_matches_numpy_restatement():
    lat = lattice.kagome(6, -1.0, 0.1, 0.05, 1.0, 0.3).with_ensembles(2)
    e0 = _rand_unit(np.random.default_rng(12), (2, lat.natom, 3))
    o = po.Oracle(lat, threads=1)
    o.set_moments(e0)
    f, _ = o.field()
    ref = _numpy_tensor_field(lat, o.emomM) + lat.extfield
    assert np.max(np.abs(f - ref)) <= 1e-12 * np.abs(ref).max()
    # the tensor is not symmetric per bond but J_ji = J_ij^T
    J = np.swapaxes(lat.j_tens, -1, -2)
    assert np.abs(J - np.swapaxes(J, -1, -2)).max() > 0.0
    # the pair energy is -1/2 sum m.b_exchange, in mRy per atom
    en = o.energy()
    bx = _numpy_tensor_field(lat, o.emomM)
    exc = -0.5 * np.einsum("mni,mni->m", o.emomM, bx) / lat.natom * MUB / MRY
    assert np.allclose(en["xc"], exc, rtol=1e-12, atol=0)
    assert np.all(en["dm"] == 0.0)


def test_kagome_metropolis_moves_follow_the_pair_energy():
    """Single-spin Metropolis on the tensor Hamiltonian: every accepted move at T -> 0+
    lowers the pair energy, so a cold quench from a random state decreases it."""
    lat = lattice.kagome(6).with_ensembles(1)
    o = po.Oracle(lat, threads=1)
    o.set_moments(_rand_unit(np.random.default_rng(13), (1, lat.natom, 3)))
    _, order, start = lattice.greedy_colouring(lat)
    e_prev = o.energy()["total"][0]
    for sw in range(5):
        o.mc_sweep_checkerboard("M", 1e-3, order, start, 21, sw)
        e = o.energy()["total"][0]
        assert e <= e_prev + 1e-12
        e_prev = e


def test_block_form_of_exchange_and_dmi():
    """lattice.fold_dm_into_tensor, the 3x3 block form of the reference's sparse path: the
    tensor path with exchange and DMI folded gives the field of the separate terms (1e-12
    relative) and the same midpoint trajectory (1e-10 after 300 steps), on the square DMI
    lattice with anisotropy and Zeeman and on the kagome case's reduced tables."""
    import json, os
    pins = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "reference_pins.json")))
    kin = pins["inputs"]["kagome"]
    kag, _ = lattice.from_tables(kin["cell"], kin["ncell"], kin["bc"], kin["sites"], kin["jfile"],
                                 dmfile=kin["dmfile"], reduce=True)
    for lat in (lattice.square_dmi(12, 1.0, 0.3, -0.05, 0.5, 1.0), kag):
        folded = lattice.fold_dm_into_tensor(lat)
        e0 = np.random.default_rng(81).normal(size=(1, lat.natom, 3))
        e0 /= np.linalg.norm(e0, axis=-1, keepdims=True)
        res = []
        for L in (lat, folded):
            o = po.Oracle(L, threads=1)
            o.set_moments(e0)
            b = o.field()[0].copy()
            o.make_llg(1, 1e-16, 0.1, 0.0)
            for _ in range(300):
                o.sd_step()
            res.append((b, o.emom.copy()))
        scale = np.max(np.abs(res[0][0]))
        assert np.max(np.abs(res[0][0] - res[1][0])) <= 1e-12 * scale
        assert np.max(np.abs(res[0][1] - res[1][1])) <= 1e-10


def test_block_form_needs_dm_neighbours_among_the_exchange_ones():
    lat = lattice.square_dmi(4, 1.0, 0.3, 0.0, 0.0, 1.0)
    lat.dmlist = lat.dmlist.copy()
    lat.dmlist[0, 0] = 11   # not a neighbour of atom 1
    with pytest.raises(ValueError):
        lattice.fold_dm_into_tensor(lat)
    with pytest.raises(ValueError):
        lattice.fold_dm_into_tensor(lattice.bcc(2, [1.0]))
