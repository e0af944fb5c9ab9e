"""The oracle's dipole-dipole field (do_dip = 1) pinned on the CPU.

The reference's regression inputs run with do_dip = 0, so no golden vector of the
dipolar field exists.  The oracle's brute-force sum (dipolar_field with the tensor of
dipoleMatrix, Hamiltonian/dipolecommon.f90:51-84, :114-143) is pinned instead by
  * the closed form of two point dipoles (mu0/4pi) (3 (m.r) r / r^5 - m / r^3),
  * an independent numpy restatement of the same pair sum,
  * a numpy restatement of the FFT form (fftdipole_fftw.f90: moments zero-padded to
    2 N - 1 cells per axis, the tensor at the shifted separations, one 3 x 3 product
    per wave vector), which equals the pair sum on every cell grid, also non-cubic ones.
"""
import dataclasses

import numpy as np
import pytest

from oracle import pyoracle as po
from uppasd_gb300 import lattice

MUB = 9.274009994e-24  # J/T, Parameters/constants.f90
MRY = 2.179872325e-21  # J
ALAT = 2.87e-10


def grid_lattice(n1, n2, n3, basis, cell, mensemble=1, mom=2.0):
    """A lattice of n1 x n2 x n3 cells with the given basis and cell vectors (rows) and
    no exchange: only the geometry the dipolar field sums over."""
    basis = np.asarray(basis, dtype=np.float64)
    na = len(basis)
    lat = lattice.chain(na * n1 * n2 * n3, 0.0, mom)
    lat = dataclasses.replace(lat, cells=(n1, n2, n3), nbasis=na,
                              meta={"cell": np.asarray(cell, dtype=np.float64).tolist(), "basis": basis.tolist()})
    return lat.with_ensembles(mensemble)


def coords_of(lat):
    cell, bas = lat.dipole_geometry()
    n1, n2, n3 = lat.cells
    na = lat.nbasis
    i = np.arange(lat.natom)
    I0, c = i % na, i // na
    I1, I2, I3 = c % n1, (c // n1) % n2, c // (n1 * n2)
    return I1[:, None] * cell[0] + I2[:, None] * cell[1] + I3[:, None] * cell[2] + bas[I0]


def pair_sum(coord, emomM, alat):
    """B_i = sum_{j != i} fac (3 R (R.m_j) - R^2 m_j) / R^5, R = r_i - r_j (units of alat)."""
    fac = 1e-7 / alat**3 * MUB
    R = coord[:, None, :] - coord[None, :, :]
    R2 = np.einsum("ijq,ijq->ij", R, R)
    rm5 = np.where(R2 > 1e-9, np.maximum(R2, 1e-9)**-2.5, 0.0) * fac  # zero on the diagonal
    out = np.empty_like(emomM)
    for k in range(emomM.shape[0]):
        rm = np.einsum("ijq,jq->ij", R, emomM[k])
        out[k] = 3.0 * np.einsum("ij,ij,ijq->iq", rm5, rm, R) - np.einsum("ij,ij,jq->iq", rm5, R2, emomM[k])
    return out


def fft_sum(lat, emomM, alat):
    """The FFT form of the same sum on the cell grid (fftdipole_fftw.f90)."""
    fac = 1e-7 / alat**3 * MUB
    cell, bas = lat.dipole_geometry()
    n = np.array(lat.cells)
    na = lat.nbasis
    p = 2 * n - 1
    M = emomM.shape[0]
    # moments on the padded grid, axes (k, a, comp, I3, I2, I1)
    m = emomM.reshape(M, n[2], n[1], n[0], na, 3).transpose(0, 4, 5, 1, 2, 3)
    mp = np.zeros((M, na, 3, p[2], p[1], p[0]))
    mp[:, :, :, :n[2], :n[1], :n[0]] = m
    mk = np.fft.rfftn(mp, axes=(3, 4, 5))
    # separations of the padded index per axis: I for I < n, I - (2 n - 1) otherwise
    s = [np.where(np.arange(p[d]) < n[d], np.arange(p[d]), np.arange(p[d]) - p[d]) for d in range(3)]
    S3, S2, S1 = np.meshgrid(s[2], s[1], s[0], indexing="ij")
    base = S1[..., None] * cell[0] + S2[..., None] * cell[1] + S3[..., None] * cell[2]
    fk = np.zeros((M, na, 3) + mk.shape[3:], dtype=complex)
    for a in range(na):
        for b in range(na):
            R = base + bas[a] - bas[b]
            R2 = np.einsum("...q,...q->...", R, R)
            rm5 = np.where(R2 > 1e-9, np.maximum(R2, 1e-9)**-2.5, 0.0) * fac
            Q = 3.0 * rm5[..., None, None] * R[..., :, None] * R[..., None, :]
            Q -= (rm5 * R2)[..., None, None] * np.eye(3)
            Qk = np.fft.rfftn(Q, axes=(0, 1, 2))
            fk[:, a] += np.einsum("xyzvu,kuxyz->kvxyz", Qk, mk[:, b])
    f = np.fft.irfftn(fk, s=tuple(p[::-1]), axes=(3, 4, 5))[:, :, :, :n[2], :n[1], :n[0]]
    return f.transpose(0, 3, 4, 5, 1, 2).reshape(M, lat.natom, 3)


def rand_moments(rng, lat):
    e = rng.normal(size=(lat.mensemble, lat.natom, 3))
    e /= np.linalg.norm(e, axis=-1, keepdims=True)
    return e


def oracle_field(lat, e):
    o = po.Oracle(lat, dipole_alat=ALAT)
    o.set_moments(e)
    return o.dipole_field(), o.emomM.copy()


@pytest.mark.parametrize("m_dir, expect", [((0.0, 0.0, 1.0), 2.0), ((1.0, 0.0, 0.0), -1.0)])
def test_two_dipoles_closed_form(m_dir, expect):
    """On the axis of a dipole its field is (mu0/4pi) 2 m / r^3; beside it -(mu0/4pi) m / r^3."""
    lat = grid_lattice(1, 1, 2, [[0.0, 0.0, 0.0]], np.eye(3), mom=2.2)
    e = np.broadcast_to(np.array(m_dir), (1, 2, 3)).copy()
    B, _ = oracle_field(lat, e)
    m = 2.2 * MUB  # J/T
    closed = 1e-7 * m / ALAT**3 * expect
    comp = int(np.argmax(np.abs(m_dir)))
    for i in range(2):
        assert B[0, i, comp] == pytest.approx(closed, rel=1e-14)
        assert np.all(np.abs(np.delete(B[0, i], comp)) < 1e-18 * abs(closed))


def test_pair_sum_bcc():
    lat = grid_lattice(3, 3, 3, [[0, 0, 0], [0.5, 0.5, 0.5]], np.eye(3), mensemble=2)
    e = rand_moments(np.random.default_rng(1), lat)
    B, emomM = oracle_field(lat, e)
    ref = pair_sum(coords_of(lat), emomM, ALAT)
    assert np.max(np.abs(B - ref)) <= 1e-13 * np.max(np.abs(ref))


@pytest.mark.parametrize("cells, basis, cell", [
    ((3, 3, 3), [[0, 0, 0], [0.5, 0.5, 0.5]], np.eye(3)),
    ((3, 4, 5), [[0, 0, 0], [0.5, 0.3, 0.2]], [[1.0, 0.0, 0.0], [0.5, 0.8660254037844386, 0.0], [0.1, 0.2, 1.3]]),
    ((5, 2, 1), [[0, 0, 0], [0.5, 0, 0], [0, 0.5, 0]], [[1.0, 0.0, 0.0], [0.5, 0.8660254037844386, 0.0], [0, 0, 1.0]]),
])
def test_fft_form_equals_pair_sum(cells, basis, cell):
    lat = grid_lattice(*cells, basis, cell, mensemble=2)
    e = rand_moments(np.random.default_rng(2), lat)
    B, emomM = oracle_field(lat, e)
    f = fft_sum(lat, emomM, ALAT)
    assert np.max(np.abs(B - f)) <= 1e-12 * np.max(np.abs(B))


def test_dipole_in_effective_field_and_energy():
    """beff = B_dip + exchange + ...; E gains -1/2 m.B_dip per atom (energy.f90:286-291)."""
    base = lattice.bcc(3, [1.3, 0.7], 2.2).with_ensembles(2)
    e = rand_moments(np.random.default_rng(3), base)
    o0 = po.Oracle(base)
    o0.set_moments(e)
    o1 = po.Oracle(base, dipole_alat=ALAT)
    o1.set_moments(e)
    b0, _ = o0.field()
    b1, _ = o1.field()
    bd = o1.dipole_field()
    assert np.max(np.abs(b1 - (bd + b0))) <= 1e-12 * np.max(np.abs(b0))
    e0 = o0.energy()["total"]
    e1 = o1.energy()["total"]
    edip = -0.5 * np.einsum("kiq,kiq->k", o1.emomM, bd) / base.natom * MUB / MRY
    assert np.allclose(e1 - e0, edip, rtol=1e-9, atol=0)
