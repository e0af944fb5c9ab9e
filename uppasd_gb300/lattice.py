"""Synthetic lattices in the reference's Hamiltonian layout.

The arrays built here are what UppASD's setup leaves in ``ham_t``
(Hamiltonian/hamiltoniandatatype.f90:14-100) and the moment module:

* ``nlist``      (natom, mnn)      -- Fortran ``nlist(mnn, natom)``, 1-based
* ``nlistsize``  (nham,)
* ``ncoup``      (nham, mnn)       -- J * 2 mRy/muB / (m_i m_j)
  (Hamiltonian/hamiltonianinit.f90:1041-1068, lexp = 1)
* ``dmlist``, ``dmlistsize``, ``dm_vect`` (nham, mnn_dm, 3) -- same scaling
* ``taniso``, ``eaniso`` (natom, 3), ``kaniso`` (natom, 2) = mRy/muB * K / m^2
  (hamiltonianinit.f90:895-909)
* ``extfield``  (mensemble, natom, 3)
* ``mmom``      (mensemble, natom)
* ``j_tens``    (nham, mnn, 3, 3)  -- Fortran ``j_tens(3,3,mnn,nham)``: element
  ``[ih, j, b, a]`` is J_ab of neighbour slot j, same scaling as ncoup; when set it
  replaces ncoup (do_jtensor = 1, Hamiltonian/hamiltoniandata.f90:138)

Every array is C-ordered with the Fortran axes reversed, so the memory image is
exactly the Fortran column-major array and can be handed to the C ABI as is.
Atoms are numbered like the reference: i = I0 + NA*(I1 + N1*(I2 + N2*I3))
(System/geometry.f90:445-453), 0-based here.
"""
from __future__ import annotations

from dataclasses import dataclass, field
from typing import Optional

import numpy as np

MRY = 2.179872325e-21
MUB = 9.274009994e-24
FC = MRY / MUB
FC2 = 2.0 * MRY / MUB


@dataclass
class Lattice:
    natom: int
    mensemble: int
    nlist: np.ndarray
    nlistsize: np.ndarray
    ncoup: np.ndarray
    aham: np.ndarray
    mmom: np.ndarray
    extfield: np.ndarray
    dmlist: Optional[np.ndarray] = None
    dmlistsize: Optional[np.ndarray] = None
    dm_vect: Optional[np.ndarray] = None
    taniso: Optional[np.ndarray] = None
    eaniso: Optional[np.ndarray] = None
    kaniso: Optional[np.ndarray] = None
    sb: Optional[np.ndarray] = None
    j_tens: Optional[np.ndarray] = None
    # geometry hints for structured kernels (cells along x, y, z and basis size)
    cells: tuple = (0, 0, 0)
    nbasis: int = 1
    periodic: tuple = (True, True, True)
    # neighbour offsets per basis atom: (nbasis, mnn, 4) = (dx, dy, dz, basis_j)
    stencil: Optional[np.ndarray] = None
    species: Optional[np.ndarray] = None   # (natom,) chemical type, 0-based
    meta: dict = field(default_factory=dict)

    @property
    def max_no_neigh(self) -> int:
        return self.nlist.shape[1]

    @property
    def nham(self) -> int:
        return self.ncoup.shape[0]

    @property
    def do_dm(self) -> int:
        return 1 if self.dmlist is not None else 0

    @property
    def do_aniso(self) -> int:
        return 1 if self.taniso is not None else 0

    @property
    def coords(self) -> np.ndarray:
        """Atom positions (natom, 3) in the reference's numbering, from the cell vectors and
        basis positions the builder recorded (``meta['cell']``, ``meta['basis']``, Cartesian;
        the identity cell and the stencil builders' basis otherwise)."""
        cell = np.asarray(self.meta.get("cell", np.eye(3)), dtype=np.float64)
        basis = np.asarray(self.meta.get("basis", _DEFAULT_BASIS.get(self.nbasis, np.zeros((1, 3)))),
                           dtype=np.float64)
        n1, n2, _ = self.cells
        idx = np.arange(self.natom)
        b, c = idx % self.nbasis, idx // self.nbasis
        frac = np.stack([c % n1, (c // n1) % n2, c // (n1 * n2)], axis=1).astype(np.float64)
        return frac @ cell + basis[b]

    def dipole_geometry(self):
        """(cell (3, 3), basis (nbasis, 3)): rows of `cell` are the cell vectors C1, C2, C3,
        rows of `basis` the basis positions, Cartesian in units of the lattice constant
        (the geometry the dipolar field is summed over)."""
        cell = np.asarray(self.meta.get("cell", np.eye(3)), dtype=np.float64)
        basis = np.asarray(self.meta.get("basis", _DEFAULT_BASIS.get(self.nbasis, np.zeros((1, 3)))),
                           dtype=np.float64)
        return np.ascontiguousarray(cell), np.ascontiguousarray(basis)

    def with_ensembles(self, mensemble: int) -> "Lattice":
        """Same Hamiltonian, `mensemble` copies of the moment arrays."""
        lat = Lattice(**{k: getattr(self, k) for k in self.__dataclass_fields__})
        lat.mensemble = mensemble
        lat.mmom = np.ascontiguousarray(np.broadcast_to(self.mmom[:1], (mensemble, self.natom)))
        lat.extfield = np.ascontiguousarray(np.broadcast_to(self.extfield[:1], (mensemble, self.natom, 3)))
        return lat


# basis positions (Cartesian, identity cell) of the stencil builders: one atom at the
# origin, or the bcc pair
_DEFAULT_BASIS = {1: np.zeros((1, 3)), 2: np.array([[0.0, 0.0, 0.0], [0.5, 0.5, 0.5]])}


def _site_index(b, x, y, z, nb, n1, n2):
    return b + nb * (x + n1 * (y + n2 * z))


def _build_from_stencil(cells, nbasis, periodic, stencil, coup_fn, natom):
    """Neighbour lists from a translation-invariant stencil.

    stencil: list over basis atoms of lists of (dx, dy, dz, bj, shell) tuples.
    coup_fn(i_idx, j_idx, shell) -> coupling array (vectorised over sites).
    Sites whose neighbour falls outside a non-periodic boundary drop it, like
    the reference's neighbour map with vacuum boundaries.
    """
    n1, n2, n3 = cells
    mnn = max(len(s) for s in stencil)
    # built slot-major (one contiguous row per slot), transposed to (natom, mnn) at the end
    nlist_t = np.zeros((mnn, natom), dtype=np.int32)
    nsize = np.zeros(natom, dtype=np.int32)
    ncoup_t = np.zeros((mnn, natom), dtype=np.float64)
    idx = np.arange(natom, dtype=np.int64)
    b = idx % nbasis
    cell = idx // nbasis
    x = cell % n1
    y = (cell // n1) % n2
    z = cell // (n1 * n2)
    for bi in range(nbasis):
        sel = np.nonzero(b == bi)[0]
        xs, ys, zs = x[sel], y[sel], z[sel]
        for s, (dx, dy, dz, bj, shell) in enumerate(stencil[bi]):
            xx, yy, zz = xs + dx, ys + dy, zs + dz
            ok = np.ones(sel.size, dtype=bool)
            for ax, (vv, nn, per) in enumerate(((xx, n1, periodic[0]), (yy, n2, periodic[1]), (zz, n3, periodic[2]))):
                if per:
                    vv %= nn
                else:
                    ok &= (vv >= 0) & (vv < nn)
            j = _site_index(bj, xx, yy, zz, nbasis, n1, n2)
            if ok.all():
                # every site keeps this neighbour: the slot is the same for all of them
                slot = nsize[sel[0]] if sel.size else 0
                nlist_t[slot, sel] = (j + 1).astype(np.int32)
                ncoup_t[slot, sel] = coup_fn(sel, j, shell)
                nsize[sel] += 1
                continue
            rows = sel[ok]
            slot = nsize[rows]
            nlist_t[slot, rows] = (j[ok] + 1).astype(np.int32)
            ncoup_t[slot, rows] = coup_fn(rows, j[ok], shell)
            nsize[rows] += 1
    return np.ascontiguousarray(nlist_t.T), nsize, np.ascontiguousarray(ncoup_t.T)


def chain(n: int, j_mry: float, mom: float = 1.0, periodic: bool = True) -> Lattice:
    """1D chain along z, one atom per cell (tests/Solvers and tests/HeisChain setup)."""
    stencil = [[(0, 0, 1, 0, 1), (0, 0, -1, 0, 1)]]
    coup = lambda i, j, sh: np.full(i.shape, j_mry * FC2 / mom / mom)
    nlist, nsize, ncoup = _build_from_stencil((1, 1, n), 1, (False, False, periodic), stencil, coup, n)
    return Lattice(natom=n, mensemble=1, nlist=nlist, nlistsize=nsize, ncoup=ncoup,
                   aham=np.arange(1, n + 1, dtype=np.int32), mmom=np.full((1, n), mom),
                   extfield=np.zeros((1, n, 3)), cells=(1, 1, n), nbasis=1,
                   periodic=(False, False, periodic),
                   stencil=np.array([[s[:4] for s in stencil[0]]], dtype=np.int32))


# bcc shells in units of the conventional cell, expressed as (cell offset, basis)
# for basis 0 at (0,0,0) and basis 1 at (1/2,1/2,1/2).
def _bcc_shells(nshell: int):
    out = [[], []]
    vecs = []
    # shell 1: (+-1/2, +-1/2, +-1/2); shell 2: (+-1,0,0); shell 3: (+-1,+-1,0); shell 4: (+-3/2,+-1/2,+-1/2)
    half = [(sx * 0.5, sy * 0.5, sz * 0.5) for sx in (1, -1) for sy in (1, -1) for sz in (1, -1)]
    vecs.append(half)
    s2 = []
    for ax in range(3):
        for sg in (1, -1):
            v = [0, 0, 0]
            v[ax] = sg
            s2.append(tuple(float(t) for t in v))
    vecs.append(s2)
    s3 = []
    for a, bb in ((0, 1), (0, 2), (1, 2)):
        for sa in (1, -1):
            for sb_ in (1, -1):
                v = [0, 0, 0]
                v[a] = sa
                v[bb] = sb_
                s3.append(tuple(float(t) for t in v))
    vecs.append(s3)
    s4 = []
    for ax in range(3):
        for sa in (1.5, -1.5):
            for s1 in (0.5, -0.5):
                for s2_ in (0.5, -0.5):
                    v = [0.0, 0.0, 0.0]
                    v[ax] = sa
                    others = [t for t in range(3) if t != ax]
                    v[others[0]] = s1
                    v[others[1]] = s2_
                    s4.append(tuple(v))
    vecs.append(s4)
    for bi, off in ((0, 0.0), (1, 0.5)):
        for sh in range(nshell):
            for v in vecs[sh]:
                p = (off + v[0], off + v[1], off + v[2])
                # target basis: integer -> 0, half-integer -> 1
                bj = 0 if abs(p[0] - round(p[0])) < 1e-9 else 1
                o = 0.0 if bj == 0 else 0.5
                d = tuple(int(round(p[t] - o)) for t in range(3))
                out[bi].append((d[0], d[1], d[2], bj, sh + 1))
    return out


def bcc(L: int, j_shells_mry, mom: float = 2.2) -> Lattice:
    """bcc ferromagnet, L^3 conventional cells, 2-atom basis, periodic."""
    nsh = len(j_shells_mry)
    st = _bcc_shells(nsh)
    natom = 2 * L ** 3
    coup = lambda i, j, sh: np.full(i.shape, j_shells_mry[sh - 1] * FC2 / mom / mom)
    nlist, nsize, ncoup = _build_from_stencil((L, L, L), 2, (True, True, True), st, coup, natom)
    return Lattice(natom=natom, mensemble=1, nlist=nlist, nlistsize=nsize, ncoup=ncoup,
                   aham=np.arange(1, natom + 1, dtype=np.int32), mmom=np.full((1, natom), mom),
                   extfield=np.zeros((1, natom, 3)), cells=(L, L, L), nbasis=2,
                   stencil=np.array([[s[:4] for s in b] for b in st], dtype=np.int32),
                   meta={"shells": [[s[4] for s in b] for b in st]})


def bcc_alloy(L: int, seed: int, j_pair_mry=((1.3, 1.8), (1.8, 0.9)), decay: float = 0.5,
              nshell: int = 4, moms=(2.2, 1.6), conc: float = 0.5) -> Lattice:
    """Random binary alloy on bcc: species drawn from `seed`, J(shell) = J_ab * decay^(shell-1)."""
    st = _bcc_shells(nshell)
    natom = 2 * L ** 3
    rng = np.random.default_rng(seed)
    species = (rng.random(natom) >= conc).astype(np.int8)   # 0 = A, 1 = B
    mom_of = np.asarray(moms, dtype=np.float64)[species]
    jp = np.asarray(j_pair_mry, dtype=np.float64)

    def coup(i, j, sh):
        jv = jp[species[i], species[j]] * decay ** (sh - 1)
        return jv * FC2 / mom_of[i] / mom_of[j]

    nlist, nsize, ncoup = _build_from_stencil((L, L, L), 2, (True, True, True), st, coup, natom)
    return Lattice(natom=natom, mensemble=1, nlist=nlist, nlistsize=nsize, ncoup=ncoup,
                   aham=np.arange(1, natom + 1, dtype=np.int32), mmom=mom_of[None, :].copy(),
                   extfield=np.zeros((1, natom, 3)), cells=(L, L, L), nbasis=2,
                   stencil=np.array([[s[:4] for s in b] for b in st], dtype=np.int32),
                   species=species,
                   meta={"shells": [[s[4] for s in b] for b in st], "j_pair_mry": jp.tolist(),
                         "decay": decay, "moms": list(moms)})


def square_dmi(L: int, j_mry: float = 1.0, d_mry: float = 0.3, k_mry: float = -0.05,
               bz: float = 0.5, mom: float = 1.0) -> Lattice:
    """Square monolayer, 4 nn exchange, interfacial DMI D_ij = D (z x r_ij),
    uniaxial anisotropy along z (energy +K (m.e)^2, so K < 0 is an easy axis),
    Zeeman field along z.  Periodic in-plane."""
    stencil = [[(1, 0, 0, 0, 1), (-1, 0, 0, 0, 1), (0, 1, 0, 0, 1), (0, -1, 0, 0, 1)]]
    natom = L * L
    coup = lambda i, j, sh: np.full(i.shape, j_mry * FC2 / mom / mom)
    nlist, nsize, ncoup = _build_from_stencil((L, L, 1), 1, (True, True, False), stencil, coup, natom)
    # DMI: same neighbour order; D vector = D * (z x r)
    dm = np.zeros((natom, 4, 3))
    for s, (dx, dy, dz, bj, sh) in enumerate(stencil[0]):
        r = np.array([dx, dy, dz], dtype=np.float64)
        dv = np.cross(np.array([0.0, 0.0, 1.0]), r)
        dm[:, s, :] = dv * d_mry * FC2 / mom / mom
    taniso = np.ones(natom, dtype=np.int32)
    e = np.array([0.0, 0.0, 1.0])
    eaniso = np.tile(e / np.sqrt(e @ e + 1.0e-15), (natom, 1))
    kaniso = np.zeros((natom, 2))
    kaniso[:, 0] = FC * k_mry / (mom * mom)
    ext = np.zeros((1, natom, 3))
    ext[..., 2] = bz
    return Lattice(natom=natom, mensemble=1, nlist=nlist, nlistsize=nsize, ncoup=ncoup,
                   aham=np.arange(1, natom + 1, dtype=np.int32), mmom=np.full((1, natom), mom),
                   extfield=ext, dmlist=nlist.copy(), dmlistsize=nsize.copy(), dm_vect=dm,
                   taniso=taniso, eaniso=eaniso, kaniso=kaniso, sb=np.zeros(natom),
                   cells=(L, L, 1), nbasis=1, periodic=(True, True, False),
                   stencil=np.array([[s[:4] for s in stencil[0]]], dtype=np.int32))


def cubic_images(r, tol: float = 1.0e-5):
    """The distinct images of bond vector r under the 48 cubic operations, in the order
    get_symops (isym = 1) generates the operations and get_fullnnlist keeps the first of
    equal images (Hamiltonian/neighbourmap.f90:392-414, :560-640)."""
    r = np.asarray(r, dtype=np.float64)
    out = []
    for i in (1, 2, 3):
        for js in (1, -1):
            for x in (0, 1):
                for y in (0, 1):
                    for z in (0, 1):
                        s = np.zeros((3, 3))
                        s[0, (i - js) % 3] = (-1.0) ** x
                        s[1, i % 3] = (-1.0) ** y
                        s[2, (i + js) % 3] = (-1.0) ** z
                        t = s @ r
                        if all(np.sum((t - u) ** 2) >= tol for u in out):
                            out.append(t)
    return out


def _table_neighbours(cell, ncell, periodic, pos, types, shells):
    """Neighbour lists of a Bravais lattice with a basis, in the reference's order.

    shells[t] lists (image vectors, neighbour type or None) per shell of atom type t.
    For each atom, shells in order, images in order; a neighbour outside a vacuum
    boundary is dropped and one already in the list is not added again (map_multiple
    off), as setup_nm and setup_neighbour_hamiltonian do (Hamiltonian/neighbourmap.f90:
    180-300, Hamiltonian/hamiltonianinit.f90:1044-1092).  Returns 1-based nlist,
    nlistsize and, per slot, the shell index (0-based, -1 when empty)."""
    na = len(pos)
    n1, n2, n3 = ncell
    natom = na * n1 * n2 * n3
    cmat = np.asarray(cell, dtype=np.float64).T   # columns C1, C2, C3
    stencil = []
    for b in range(na):
        st = []
        for k, (images, jtype) in enumerate(shells[types[b]]):
            for v in images:
                for b2 in range(na):
                    if jtype is not None and types[b2] != jtype:
                        continue
                    f = np.linalg.solve(cmat, pos[b] + v - pos[b2])
                    if np.all(np.abs(f - np.rint(f)) < 1.0e-4):
                        d = np.rint(f).astype(np.int64)
                        st.append((int(d[0]), int(d[1]), int(d[2]), b2, k))
                        break
        stencil.append(st)
    mnn = max(1, max(len(s) for s in stencil))
    nlist = np.zeros((natom, mnn), dtype=np.int32)
    shell = np.full((natom, mnn), -1, dtype=np.int32)
    nsize = np.zeros(natom, dtype=np.int32)
    idx = np.arange(natom, dtype=np.int64)
    bb, cidx = idx % na, idx // na
    x, y, z = cidx % n1, (cidx // n1) % n2, cidx // (n1 * n2)
    dims = (n1, n2, n3)
    for b in range(na):
        sel = np.nonzero(bb == b)[0]
        earlier = []
        for dx, dy, dz, b2, k in stencil[b]:
            # an earlier entry can give the same neighbour only with the same basis atom and
            # offsets equal on open axes, congruent modulo the cells on periodic ones; without
            # one the duplicate test below finds nothing and is skipped
            clash = any(q[3] == b2 and all(((d - e) % n == 0) if per else d == e
                                           for d, e, n, per in zip((dx, dy, dz), q[:3], dims, periodic))
                        for q in earlier)
            earlier.append((dx, dy, dz, b2))
            xx, yy, zz = x[sel] + dx, y[sel] + dy, z[sel] + dz
            ok = np.ones(sel.size, dtype=bool)
            for vv, nn, per in ((xx, n1, periodic[0]), (yy, n2, periodic[1]), (zz, n3, periodic[2])):
                if per:
                    vv %= nn
                else:
                    ok &= (vv >= 0) & (vv < nn)
            j = _site_index(b2, xx, yy, zz, na, n1, n2) + 1
            rows, j = sel[ok], j[ok]
            if clash:
                fresh = ~np.any(nlist[rows] == j[:, None].astype(np.int32), axis=1)
                rows, j = rows[fresh], j[fresh]
            slot = nsize[rows]
            nlist[rows, slot] = j
            shell[rows, slot] = k
            nsize[rows] += 1
    return nlist, nsize, shell


_MT_N, _MT_M = 624, 397
_U64 = 0xFFFFFFFFFFFFFFFF


def _mt_twist(mt: np.ndarray) -> None:
    """One regeneration of the 624 words in place (mtprng_rand64, RNG/mtprng.f90:213-232),
    in the three dependency-free blocks of the sequential loops."""
    upper, lower, one = np.uint64(0x80000000), np.uint64(0x7FFFFFFF), np.uint64(1)
    mag1 = np.uint64(-1727483681 & _U64)

    def mix(a, b, c):
        y = (a & upper) | (b & lower)
        return c ^ (y >> one) ^ np.where((y & one) != 0, mag1, np.uint64(0))

    old = mt.copy()
    k = _MT_N - _MT_M  # 227
    mt[0:k] = mix(old[0:k], old[1:k + 1], old[_MT_M:_MT_N])
    mt[k:2 * k] = mix(old[k:2 * k], old[k + 1:2 * k + 1], mt[0:k])
    mt[2 * k:_MT_N - 1] = mix(old[2 * k:_MT_N - 1], old[2 * k + 1:_MT_N], mt[k:_MT_M - 1])
    mt[_MT_N - 1] = mix(old[_MT_N - 1:], mt[0:1], mt[_MT_M - 1:_MT_M])[0]


class MtprngStream:
    """The reference's main uniform stream: mtprng_rand_real2 draws after
    mtprng_init(seed) (RNG/mtprng.f90:118-138, 191-246, 309-325), as rng_uniform gives them
    after rng_init(tseed) (RNG/randomnumbers.f90:106-146).  Its Mersenne twister keeps
    INT64 words with a sign-extended mag01 and masks to 32 bits only inside the tempering,
    so a regenerated word's upper bits leak into the first tempering shift: not textbook
    MT19937 after the first 624 draws.  ``real2(n)`` returns the next n draws; draws a
    consumer looked at but did not use stay for the next (``_fill`` / ``pos``)."""

    def __init__(self, seed: int):
        self.mt = np.zeros(_MT_N, dtype=np.uint64)
        p = seed & _U64
        self.mt[0] = np.uint64(p)
        for i in range(1, _MT_N):
            p = (1812433253 * (p ^ (p >> 30)) + i) & 0xFFFFFFFF
            self.mt[i] = np.uint64(p)
        self.buf = np.empty(0)
        self.pos = 0

    def _block(self) -> np.ndarray:
        _mt_twist(self.mt)
        tb, tc = np.uint64(-1658038656 & _U64), np.uint64(-272236544 & _U64)
        m32 = np.uint64(0xFFFFFFFF)
        r = self.mt.copy()
        r ^= r >> np.uint64(11)
        r = m32 & (r ^ ((r << np.uint64(7)) & tb))
        r = m32 & (r ^ ((r << np.uint64(15)) & tc))
        r ^= r >> np.uint64(18)
        return r.astype(np.float64) * (1.0 / 4294967296.0)

    def _fill(self, n: int) -> None:
        """At least n draws buffered from pos on."""
        have = self.buf.size - self.pos
        if have >= n:
            return
        blocks = [self.buf[self.pos:]]
        for _ in range((n - have + _MT_N - 1) // _MT_N):
            blocks.append(self._block())
        self.buf = np.concatenate(blocks)
        self.pos = 0

    def real2(self, n: int) -> np.ndarray:
        self._fill(n)
        out = self.buf[self.pos:self.pos + n].copy()
        self.pos += n
        return out


def mtprng_real2(seed: int, n: int) -> np.ndarray:
    """The first n draws of the reference's stream after rng_init(seed) (``MtprngStream``)."""
    return MtprngStream(seed).real2(n)


def initmag_random(natom: int, stream: MtprngStream, chunk: int = 65536) -> np.ndarray:
    """Initmag 1 (magninit, System/magnetizationinit.f90:141-170): per atom of the full list,
    in order, three draws give x, y, z = 2 (r - 1/2); while outside the unit sphere, three
    more give x, y, z = (r - 1/2) (the reference's factor 1 on a retry, so a retry always
    lands inside); normalised.  Returns (natom, 3) unit vectors; the stream moves past the
    draws used."""
    out = np.empty((natom, 3))
    for a0 in range(0, natom, chunk):
        na = min(chunk, natom - a0)
        stream._fill(6 * na)   # at most two tries per atom
        buf = stream.buf[stream.pos:stream.pos + 6 * na].tolist()
        k = 0
        for i in range(a0, a0 + na):
            x, y, z = 2.0 * (buf[k] - 0.50), 2.0 * (buf[k + 1] - 0.50), 2.0 * (buf[k + 2] - 0.50)
            k += 3
            while x * x + y * y + z * z > 1.0:
                x, y, z = 1.0 * (buf[k] - 0.50), 1.0 * (buf[k + 1] - 0.50), 1.0 * (buf[k + 2] - 0.50)
                k += 3
            n = np.sqrt(x * x + y * y + z * z)
            out[i, 0], out[i, 1], out[i, 2] = x / n, y / n, z / n
        stream.pos += k
    return out


def initmag_cone(natom: int, stream: MtprngStream, theta0: float, phi0: float,
                 mavg0: float = -1.0) -> np.ndarray:
    """Initmag 2 (magninit, System/magnetizationinit.f90:187-228): per atom of the full list,
    in order, two draws r1, r2 give u = (sin(theta0 r1) cos(phi0 r2), sin(theta0 r1)
    sin(phi0 r2), cos(theta0 r1)), angles in radians; mavg0 >= 0 sets phi0 = 2 pi and
    theta0 = 2 acos(mavg0).  Returns (natom, 3) unit vectors."""
    if mavg0 >= 0.0:
        phi0, theta0 = 2.0 * np.pi, 2.0 * np.arccos(mavg0)
    r = stream.real2(2 * natom).reshape(natom, 2)
    th, ph = theta0 * r[:, 0], phi0 * r[:, 1]
    return np.stack([np.sin(th) * np.cos(ph), np.sin(th) * np.sin(ph), np.cos(th)], axis=1)


def _nint(x: float) -> int:
    """Fortran nint of a non-negative real: the nearest integer, halves away from zero."""
    q = int(x)
    return q + 1 if x - q >= 0.5 else q


def random_chemistry(ncells: int, conc, seed: Optional[int] = None, uniform=None) -> np.ndarray:
    """Chemical types of a random alloy as setup_chemicaldata assigns them
    (System/geometry.f90:190-329): for each basis site ia in turn, ncells uniform draws
    (``uniform``, else the reference's stream after rng_init(seed): ``mtprng_real2``); the
    cells taken in order of decreasing draw (maxloc, the first of equal draws first) go to
    chemical type 1 for the first nint(c_1 ncells), then to type 2, and so on; cells left
    over are vacancies (a dilute alloy).  ``conc[ia]`` lists the concentrations of the
    site's types 1, 2, ....  Returns achtype over the full atom list (atom I0 + NA cell,
    0-based, cells x fastest): 1-based types, 0 for a vacancy.  Concentrations whose rounded
    counts exceed the cells (0.7 and 0.3 on 125 cells: 88 + 38) are refused; the
    reference's loop would index past its cell list.  (An exact 0.0 draw, 2^-32 per draw,
    would make the reference's maxloc pick an already taken cell; here every cell is taken
    once.)"""
    na = len(conc)
    if uniform is None:
        if seed is None:
            raise ValueError("random_chemistry needs the seed (tseed) or the uniform draws")
        uniform = mtprng_real2(seed, na * ncells)
    uniform = np.asarray(uniform, dtype=np.float64)
    if uniform.size < na * ncells:
        raise ValueError(f"need {na * ncells} uniform draws")
    achtype = np.zeros(na * ncells, dtype=np.int32)
    for ia in range(na):
        q = [_nint(float(c) * ncells) for c in conc[ia]]
        if sum(q) > ncells:
            raise ValueError(f"concentrations of site {ia + 1} exceed one")
        order = np.argsort(-uniform[ia * ncells:(ia + 1) * ncells], kind="stable")
        start = 0
        for ich, qq in enumerate(q, 1):
            achtype[order[start:start + qq] * na + ia] = ich
            start += qq
    return achtype


def from_tables(cell, ncell, bc, sites, jfile, sym: int = 0, dmfile=None, kfile=None, reduce: bool = False,
                maptype: int = 1, aunits: bool = False, posfiletype: str = "C", tensor: bool = False,
                chemistry=None, achtype=None, tseed: Optional[int] = None):
    """A Hamiltonian built from the reference's own input tables: the ``cell``, ``ncell``,
    ``BC`` and ``Sym`` keywords of inpsd.dat, the posfile and momfile rows (``sites``:
    per basis site ``(type, x, y, z, mom, ex, ey, ez)``, Cartesian, posfiletype 'C'),
    jfile rows ``(isite, jsite, rx, ry, rz, J)`` (Cartesian bond vectors, maptype 1, or
    cell offsets n1 n2 n3 from site isite to site jsite, maptype 2:
    r = Bas(jsite) - Bas(isite) + n1 C1 + n2 C2 + n3 C3, read_exchange_getNeighVec),
    optional dmfile rows ``(isite, jsite, rx, ry, rz, Dx, Dy, Dz)`` (Sym 0) and kfile rows
    ``(isite, type, K1, K2, ex, ey, ez, ratio)``; J, D and K in mRy, no chemical disorder.

    Shells follow read_exchange (Input/inputhandler_ext.f90:444-618): per atom type, one
    shell per distinct bond vector in file order, a repeated vector overwriting the
    coupling, the neighbour's type fixed by the jsite column; each shell is expanded by
    the lattice symmetry (``cubic_images`` for Sym 1).  Couplings are scaled by
    2 mRy/muB/(m_i m_j) (zero when m_i m_j < 1e-6), anisotropies by mRy/muB/m^2, m^4
    (uniaxial) or m^4, m^6 (cubic) (Hamiltonian/hamiltonianinit.f90:895-909, :1060-1068).
    ``reduce`` gives the reduced Hamiltonian (do_reduced 'Y'); ``aunits`` the atomic units of
    aunits 'Y' (mry = mub = 1, Input/inputhandler.f90:1685-1704); ``posfiletype`` 'D' reads
    the site positions in units of the cell vectors; ``tensor`` reads jfile rows with nine
    couplings J_xx J_xy ... J_zz (row by row, read_exchange_tensor_base,
    Input/inputhandler_ext.f90:658-741) into ``j_tens`` (do_jtensor = 1), scaled like ncoup.

    Random alloys (do_ralloy 1): ``chemistry`` maps each basis site (1-based) to its rows
    ``(ichem, conc, mom, ex, ey, ez)`` (the posfile's chemical columns and the momfile
    rows of that site); jfile rows are then ``(isite, jsite, ichem, jchem, rx, ry, rz, J)``
    and a shell's coupling is taken by the chemical types of both atoms, scaled by their
    moments (setup_neighbour_hamiltonian, Hamiltonian/hamiltonianinit.f90:1060-1068).  The
    types are ``achtype`` (1-based over the full atom list, 0 a vacancy) or drawn as the
    reference draws them from ``tseed`` (``random_chemistry``); vacancies leave the atom
    list and every neighbour list, the remaining atoms numbered in order
    (setup_chemicaldata's acellnumb).  ``Lattice.species`` holds the 0-based types.  DM
    rows gain the same two chemical columns, kfile rows one (``isite, ichem, type, ...``);
    the tensor and reduced forms are not read with chemistry.

    Returns the lattice and the momfile directions normalised per atom (Initmag 3)."""
    sites = [tuple(float(v) for v in s) for s in sites]
    na = len(sites)
    types = [int(s[0]) for s in sites]
    pos = [np.array(s[1:4]) for s in sites]
    if str(posfiletype).upper() == "D":
        pos = [np.asarray(cell, dtype=np.float64).T @ p for p in pos]
    moms = np.array([s[4] for s in sites])
    periodic = tuple(str(c).upper() == "P" for c in bc)
    if maptype not in (1, 2):
        raise ValueError("maptype 1 (Cartesian bond vectors) and 2 (cell offsets) are supported")
    if sym not in (0, 1):
        raise ValueError("Sym 0 (none) and 1 (cubic) are supported")
    expand = (lambda r: [np.asarray(r, dtype=np.float64)]) if sym == 0 else cubic_images

    chem = chemistry is not None
    if chem and (tensor or reduce):
        raise ValueError("random alloys: the tensor and reduced forms are not read")
    off = 4 if chem else 2  # (isite, jsite[, ichem, jchem]) before the vector

    def read_shells(rows, width):
        # values[t][k]: the shell's coupling, or with chemistry {(ichem, jchem): coupling}
        # (read_exchange, Input/inputhandler_ext.f90:484-530: a repeated vector overwrites
        # the coupling of its chemical pair)
        shells, values = {t: [] for t in set(types)}, {t: [] for t in set(types)}
        for row in rows:
            isite, jsite = int(row[0]), int(row[1])
            it, jt = types[isite - 1], types[jsite - 1]
            r = np.array([float(v) for v in row[off:off + 3]])
            if maptype == 2:
                r = pos[jsite - 1] - pos[isite - 1] + np.asarray(cell, dtype=np.float64).T @ r
            val = np.array([float(v) for v in row[off + 3:off + 3 + width]])
            key = (int(row[2]), int(row[3])) if chem else None
            for k, (r0, _) in enumerate(shells[it]):
                if np.sum((r - r0) ** 2) < 1.0e-5:
                    if chem:
                        values[it][k][key] = val
                    else:
                        values[it][k] = val
                    break
            else:
                shells[it].append((r, jt))
                values[it].append({key: val} if chem else val)
        return ({t: [(expand(r), jt) for r, jt in v] for t, v in shells.items()}, values)

    fc, fc2 = (1.0, 2.0) if aunits else (FC, FC2)
    ncells = int(np.prod(ncell))
    natom = na * ncells
    b_of = np.arange(natom) % na
    m_of = moms[b_of]
    if chem:
        rows_of = {int(s): sorted((tuple(float(v) for v in r) for r in rs), key=lambda r: r[0])
                   for s, rs in chemistry.items()}
        if sorted(rows_of) != list(range(1, na + 1)):
            raise ValueError("chemistry needs the rows of every basis site")
        if achtype is None:
            achtype = random_chemistry(ncells, [[r[1] for r in rows_of[s]] for s in range(1, na + 1)], seed=tseed)
        achtype = np.asarray(achtype, dtype=np.int32).reshape(-1)
        if achtype.size != natom or achtype.min() < 0:
            raise ValueError(f"achtype needs {natom} non-negative entries")
        # (site, type) -> its row (ichem, conc, mom, ex, ey, ez); type 0, a vacancy, all zero
        nch = max(int(achtype.max()), max(int(r[0]) for rs in rows_of.values() for r in rs))
        tab = np.zeros((na, nch + 1, 6))
        known = np.zeros((na, nch + 1), dtype=bool)
        known[:, 0] = True
        for s, rs in rows_of.items():
            for r in rs:
                tab[s - 1, int(r[0])] = r
                known[s - 1, int(r[0])] = True
        miss = ~known[b_of, achtype]
        if np.any(miss):
            i = int(np.nonzero(miss)[0][0])
            raise ValueError(f"chemical type {achtype[i]} has no row on site {b_of[i] + 1}")
        rec = tab[b_of, achtype]
        m_of = rec[:, 2].copy()

    def coupled(rows, width):
        shells, values = read_shells(rows, width)
        nl, ns, sh = _table_neighbours(cell, ncell, periodic, pos, types, shells)
        c = np.zeros(nl.shape + (width,))
        for i_b in range(na):
            t = types[i_b]
            for k, val in enumerate(values[t]):
                sel = (b_of[:, None] == i_b) & (sh == k)
                ii, ss = np.nonzero(sel)
                jj = nl[ii, ss] - 1
                mj = m_of[jj]
                mm = m_of[ii] * mj
                if chem:
                    # the coupling of this pair's chemical types, zero for a pair the file omits
                    v = np.zeros((ii.size, width))
                    for (ci, cj), vv in val.items():
                        v[(achtype[ii] == ci) & (achtype[jj] == cj)] = vv
                else:
                    v = val[None, :]
                c[ii, ss] = np.where((np.abs(mm) < 1.0e-6)[:, None], 0.0, v * fc2 / np.where(mm == 0, 1.0, mm)[:, None])
        return nl, ns, c

    nlist, nsize, c = coupled(jfile, 9 if tensor else 1)
    keep = achtype > 0 if chem else None
    newidx = np.cumsum(keep).astype(np.int32) if chem else None  # 1-based number of a kept atom

    def drop_vacancies(nl, ns, cc):
        """The lists without vacancies (the order of the rest kept), renumbered, and the
        vacancies' own rows removed (setup_nm and setup_chemicaldata's acellnumb)."""
        slot = np.arange(nl.shape[1])[None, :]
        live = (slot < ns[:, None]) & keep[np.maximum(nl, 1) - 1]
        order = np.argsort(~live, axis=1, kind="stable")
        nl = np.take_along_axis(nl, order, axis=1)
        cc = np.take_along_axis(cc, np.broadcast_to(order[..., None], cc.shape), axis=1)
        ns = live.sum(axis=1).astype(np.int32)
        inside = slot < ns[:, None]
        nl = np.where(inside, newidx[np.maximum(nl, 1) - 1], 0).astype(np.int32)
        cc = np.where(inside[..., None], cc, 0.0)
        return nl[keep], ns[keep], cc[keep]

    if chem:
        nlist, nsize, c = drop_vacancies(nlist, nsize, c)
    jt = None
    if tensor:
        jt = tensor_from_matrices(c.reshape(c.shape[:2] + (3, 3)))
        c = np.zeros(c.shape[:2] + (1,))
    n_out = int(keep.sum()) if chem else natom
    sel_out = keep if chem else slice(None)
    lat = Lattice(natom=n_out, mensemble=1, nlist=nlist, nlistsize=nsize, ncoup=np.ascontiguousarray(c[..., 0]),
                  j_tens=jt,
                  aham=np.arange(1, n_out + 1, dtype=np.int32), mmom=m_of[sel_out][None, :].copy(),
                  extfield=np.zeros((1, n_out, 3)), cells=tuple(int(n) for n in ncell), nbasis=na,
                  periodic=periodic, species=(achtype[keep] - 1).astype(np.int8) if chem else None,
                  meta={"types": types, "cell": np.asarray(cell, dtype=np.float64).tolist(),
                        "basis": np.asarray(pos).tolist()})
    if chem:
        lat.meta["achtype"] = achtype
        if n_out != natom:
            lat.cells, lat.nbasis = (0, 0, 0), 1  # no cell structure once atoms are missing
    if dmfile is not None and len(dmfile):
        if sym != 0:
            raise ValueError("DM tables are supported with Sym 0 only")
        dl, ds, dv = coupled(dmfile, 3)
        if chem:
            dl, ds, dv = drop_vacancies(dl, ds, dv)
        lat.dmlist, lat.dmlistsize, lat.dm_vect = dl, ds, np.ascontiguousarray(dv)
    if kfile is not None and len(kfile):
        # rows (isite, type, K1, K2, ex, ey, ez, ratio), with chemistry (isite, ichem, type,
        # ...) (read_anisotropy / read_anisotropy_alloy, Input/inputhandler_ext.f90:1046-1080);
        # scaled by the moment of the atom's site and type (hamiltonianinit.f90:895-960)
        kc = 1 if chem else 0
        kt = {(int(r[0]), int(r[1]) if chem else 0): [float(v) for v in r] for r in kfile}
        taniso = np.zeros(natom, dtype=np.int32)
        eaniso = np.zeros((natom, 3))
        kaniso = np.zeros((natom, 2))
        sb = np.zeros(natom)
        for (site, ich), r in kt.items():
            sel = (b_of == site - 1) & ((achtype == ich) if chem else True)
            if not np.any(sel):
                continue
            e = np.array(r[kc + 4:kc + 7])
            typ = int(r[kc + 1])
            taniso[sel] = typ
            eaniso[sel] = e / np.sqrt(e @ e + 1.0e-15)
            p1, p2 = (4, 6) if typ == 2 else (2, 4)
            mom = m_of[sel]
            kaniso[sel, 0] = fc * r[kc + 2] / mom ** p1
            kaniso[sel, 1] = fc * r[kc + 3] / mom ** p2
            sb[sel] = r[kc + 7] if len(r) > kc + 7 else 0.0
        lat.taniso, lat.eaniso, lat.kaniso, lat.sb = (taniso[sel_out], eaniso[sel_out], kaniso[sel_out],
                                                      sb[sel_out])
    if reduce:
        lat = reduced(lat)
    if chem:
        d = rec[keep][:, 3:6]
        d = d / np.sqrt(np.sum(d * d, axis=1))[:, None]
        return lat, np.ascontiguousarray(d[None, :, :])
    d = np.array([s[5:8] for s in sites])
    d = d / np.sqrt(np.sum(d * d, axis=1))[:, None]
    return lat, np.ascontiguousarray(d[b_of][None, :, :])


def tensor_from_matrices(mats) -> np.ndarray:
    """(nham, mnn, 3, 3) matrices J[ih, j, a, b] -> the Fortran memory image of j_tens."""
    return np.ascontiguousarray(np.swapaxes(np.asarray(mats, dtype=np.float64), -1, -2))


def with_isotropic_tensor(lat: Lattice) -> Lattice:
    """The tensor form of a scalar exchange, J_ab = ncoup * delta_ab per neighbour slot, as
    read_exchange_build_tensor (Input/inputhandler_ext.f90) builds it for calc_jtensor;
    the DMI list stays a separate term, as the reference's field keeps it."""
    out = Lattice(**{k: getattr(lat, k) for k in lat.__dataclass_fields__})
    eye = np.eye(3)
    out.j_tens = tensor_from_matrices(lat.ncoup[:, :, None, None] * eye)
    return out


def fold_dm_into_tensor(lat: Lattice) -> Lattice:
    """The block form of the reference's sparse path (setupSparseBlock,
    Hamiltonian/sparse.f90:122-268): per neighbour one 3x3 block with J on the diagonal and
    +-D off it, B_i += sum_j (J_ij I + [D_ij]) m_j with [D] m = m x D, so that the exchange
    tensor gather carries exchange and DMI together.  Every DM neighbour must be an
    exchange neighbour, in the same slot for all atoms of one Hamiltonian row.  The field
    and the dynamics are those of the separate terms; the energy is then the tensor's pair
    energy, as the reference computes it with do_jtensor."""
    if lat.dmlist is None:
        raise ValueError("no DM interaction to fold")
    if lat.j_tens is not None:
        mats = np.swapaxes(np.asarray(lat.j_tens, dtype=np.float64), -1, -2).copy()
    else:
        mats = lat.ncoup[:, :, None, None] * np.eye(3)
    ih_of = np.asarray(lat.aham) - 1
    slot = {}
    for i in range(lat.natom):
        ih = ih_of[i]
        row = lat.nlist[i, :lat.nlistsize[ih]]
        for sd in range(lat.dmlistsize[ih]):
            hit = np.nonzero(row == lat.dmlist[i, sd])[0]
            if hit.size == 0:
                raise ValueError(f"DM neighbour {lat.dmlist[i, sd]} of atom {i + 1} is not an exchange neighbour")
            if slot.setdefault((ih, sd), int(hit[0])) != int(hit[0]):
                raise ValueError("DM slots differ between atoms of one Hamiltonian row")
    for (ih, sd), s in slot.items():
        d0, d1, d2 = lat.dm_vect[ih, sd]
        mats[ih, s] += np.array([[0.0, d2, -d1], [-d2, 0.0, d0], [d1, -d0, 0.0]])
    out = Lattice(**{k: getattr(lat, k) for k in lat.__dataclass_fields__})
    out.j_tens = tensor_from_matrices(mats)
    out.dmlist = out.dmlistsize = out.dm_vect = None
    return out


def reduced(lat: Lattice) -> Lattice:
    """The reduced Hamiltonian (do_reduced = 'Y'): one coupling row per basis atom,
    aHam(i) = anumb(i) (Hamiltonian/hamiltonianinit.f90:818-838, nHam = NA at :185).
    Valid for translation-invariant lattices, whose rows of one basis atom coincide;
    raises otherwise.  Neighbour lists, anisotropy and fields stay per atom."""
    nb = lat.nbasis
    if lat.cells[0] <= 0 or lat.nham != lat.natom:
        raise ValueError("reduced() needs a full (nham == natom) lattice with a cell structure")
    b = np.arange(lat.natom) % nb
    out = Lattice(**{k: getattr(lat, k) for k in lat.__dataclass_fields__})
    for name in ("ncoup", "nlistsize", "dmlistsize", "dm_vect", "j_tens"):
        a = getattr(lat, name)
        if a is None:
            continue
        if not np.array_equal(a, a[:nb][b]):
            raise ValueError(f"{name} is not translation invariant; the Hamiltonian does not reduce")
        setattr(out, name, np.ascontiguousarray(a[:nb]))
    out.aham = (b + 1).astype(np.int32)
    return out


_KAGOME_BASIS = np.array([[0.0, 0.0], [0.5, 0.0], [0.0, 0.5]])
_KAGOME_STENCIL = [
    [(0, 0, 0, 1, 1), (-1, 0, 0, 1, 1), (0, 0, 0, 2, 1), (0, -1, 0, 2, 1)],
    [(0, 0, 0, 0, 1), (1, 0, 0, 0, 1), (0, 0, 0, 2, 1), (1, -1, 0, 2, 1)],
    [(0, 0, 0, 0, 1), (0, 1, 0, 0, 1), (0, 0, 0, 1, 1), (-1, 1, 0, 1, 1)],
]


def kagome(L: int, j_mry: float = -1.0, d_mry: float = 0.1, g_mry: float = 0.05, mom: float = 1.0,
           bz: float = 0.0) -> Lattice:
    """Kagome monolayer (triangular cell a1 = (1, 0), a2 = (1/2, sqrt(3)/2), three sites at
    (0, 0), (1/2, 0), (0, 1/2) in cell units), L x L cells, periodic, nearest neighbours
    only, with a full exchange tensor per bond (do_jtensor = 1):

        J_ij = j I + g e e^T + [D]_x,   D = d (z x e),   e = unit bond vector i -> j,

    [D]_x the antisymmetric matrix with m_i . [D]_x m_j = D . (m_i x m_j).  J_ji = J_ij^T,
    so the energy -1/2 sum m_i J_ij m_j is a proper pair sum.  Scaled like ncoup."""
    natom = 3 * L * L
    nlist, nsize, _ = _build_from_stencil((L, L, 1), 3, (True, True, False), _KAGOME_STENCIL,
                                          lambda i, j, sh: np.zeros(i.shape), natom)
    a1, a2 = np.array([1.0, 0.0, 0.0]), np.array([0.5, np.sqrt(3.0) / 2.0, 0.0])
    z = np.array([0.0, 0.0, 1.0])
    mats = np.zeros((3, 4, 3, 3))
    for bi in range(3):
        for s, (dx, dy, dz, bj, sh) in enumerate(_KAGOME_STENCIL[bi]):
            dr = _KAGOME_BASIS[bj] + (dx, dy) - _KAGOME_BASIS[bi]
            e = dr[0] * a1 + dr[1] * a2
            e = e / np.linalg.norm(e)
            D = d_mry * np.cross(z, e)
            A = np.array([[0.0, D[2], -D[1]], [-D[2], 0.0, D[0]], [D[1], -D[0], 0.0]])
            mats[bi, s] = (j_mry * np.eye(3) + g_mry * np.outer(e, e) + A) * FC2 / mom / mom
    jt = tensor_from_matrices(mats[np.arange(natom) % 3])
    ext = np.zeros((1, natom, 3))
    ext[..., 2] = bz
    return Lattice(natom=natom, mensemble=1, nlist=nlist, nlistsize=nsize,
                   ncoup=np.zeros((natom, 4)), aham=np.arange(1, natom + 1, dtype=np.int32),
                   mmom=np.full((1, natom), mom), extfield=ext, j_tens=jt,
                   cells=(L, L, 1), nbasis=3, periodic=(True, True, False),
                   stencil=np.array([[s[:4] for s in b] for b in _KAGOME_STENCIL], dtype=np.int32),
                   meta={"cell": [a1.tolist(), a2.tolist(), [0.0, 0.0, 1.0]],
                         "basis": [(f[0] * a1 + f[1] * a2).tolist() for f in _KAGOME_BASIS]})


def greedy_colouring(lat: Lattice):
    """Colour sites so that no two coupled sites (exchange or DMI) share a colour.

    Returns (colour_of_site, colour_sites, colour_start).  Tries the sublattices
    alone, then sublattice x cell parity (exact for the shipped lattices), verifying
    each; falls back to a greedy colouring of the coupling graph.
    """
    n = lat.natom
    nl = lat.nlist.astype(np.int64) - 1
    mask = np.arange(nl.shape[1])[None, :] < lat.nlistsize[lat.aham - 1][:, None]
    col = None
    if lat.cells[0] > 0:
        n1, n2, n3 = lat.cells
        idx = np.arange(n)
        b = idx % lat.nbasis
        c = idx // lat.nbasis
        x, y, z = c % n1, (c // n1) % n2, c // (n1 * n2)
        # the sublattices alone, then sublattice x cell parity (the library's order)
        if lat.nbasis > 1 and _colouring_ok(b.astype(np.int32), nl, mask, lat):
            col = b.astype(np.int32)
        else:
            cand = (b * 2 + ((x + y + z) % 2)).astype(np.int32)
            if _colouring_ok(cand, nl, mask, lat):
                col = cand
    if col is None:
        col = np.full(n, -1, dtype=np.int32)
        for i in range(n):
            used = set(col[nl[i][mask[i]]].tolist())
            if lat.dmlist is not None:
                dm = lat.dmlist[i][: lat.dmlistsize[lat.aham[i] - 1]] - 1
                used |= set(col[dm].tolist())
            cc = 0
            while cc in used:
                cc += 1
            col[i] = cc
        assert _colouring_ok(col, nl, mask, lat)
    # compact colour ids
    uniq = np.unique(col)
    remap = {u: k for k, u in enumerate(uniq)}
    col = np.array([remap[u] for u in col], dtype=np.int32) if len(uniq) < col.max() + 1 else col
    order = np.argsort(col, kind="stable").astype(np.int32)
    start = np.zeros(len(uniq) + 1, dtype=np.int32)
    start[1:] = np.cumsum(np.bincount(col, minlength=len(uniq)))
    return col, order, start


def _colouring_ok(col, nl, mask, lat) -> bool:
    same = (col[nl] == col[:, None]) & mask
    if same.any():
        return False
    if lat.dmlist is not None:
        dl = lat.dmlist.astype(np.int64) - 1
        dmask = np.arange(dl.shape[1])[None, :] < lat.dmlistsize[lat.aham - 1][:, None]
        if ((col[dl] == col[:, None]) & dmask).any():
            return False
    return True
