"""Random alloys from the reference's input tables (do_ralloy 1), on the CPU:

* ``lattice.mtprng_real2`` gives the oracle's restatement of the reference's Mersenne
  twister (RNG/mtprng.f90) draw for draw, across several regenerations;
* ``lattice.random_chemistry`` assigns the chemical types as setup_chemicaldata's loop
  does (System/geometry.f90:231-279), checked against a literal restatement of that loop
  (maxloc over the draws, the taken draw zeroed) on the same stream, dilute case included;
* ``lattice.from_tables`` with chemistry couples every pair by the chemical types of both
  atoms and their moments, checked against a brute-force search by distance on the
  reference's RandomAlloy example tables (examples/Mappings/RandomAlloy: bcc as a cubic
  cell with two sites, 80/20 and 20/80, two shells), and a dilute alloy drops its
  vacancies from the atom and neighbour lists with every other coupling unchanged;
  anisotropy and DM rows with chemical columns follow each atom's (site, type)."""
import numpy as np
import pytest

from oracle import pyoracle as po
from uppasd_gb300 import lattice

SITES = [(1, 0.0, 0.0, 0.0, 1.0, 1.0, 0.0, 0.0), (1, 0.5, 0.5, 0.5, 1.0, 1.0, 0.0, 0.0)]
MOM = {1: 2.23, 2: 1.80}
JTAB = {(1, 1): (1.0, 0.2), (2, 1): (0.5, 0.02), (1, 2): (0.5, 0.02), (2, 2): (-0.8, 0.2)}
JFILE = [(1, 1, ci, cj, *r, JTAB[(ci, cj)][k]) for (ci, cj) in JTAB
         for k, r in enumerate(((0.5, 0.5, 0.5), (1.0, 0.0, 0.0)))]


def _chemistry(c1=(0.8, 0.2), c2=(0.2, 0.8)):
    return {1: [(1, c1[0], MOM[1], 1.0, 0.0, 0.0), (2, c1[1], MOM[2], 1.0, 0.0, 0.0)],
            2: [(1, c2[0], MOM[1], 0.0, 0.0, 1.0), (2, c2[1], MOM[2], 0.0, 0.0, 1.0)]}


@pytest.mark.parametrize("seed", [1, 5489, 2024, -3])
def test_mtprng_matches_the_oracle_stream(seed):
    assert np.array_equal(lattice.mtprng_real2(seed, 2500), po.mt_stream(seed, 2500, "real2"))


def test_initmag_random_matches_the_oracle():
    """Initmag 1 against the oracle's restatement (which the HeisStripe, HeisChainAF and
    SCsurf pins fix), in chunks that split the stream, and the stream left where the
    oracle's is."""
    lat = lattice.bcc(5, [1.0], 2.0).with_ensembles(2)
    o = po.Oracle(lat)
    o.init_random(7)
    s = lattice.MtprngStream(7)
    u = lattice.initmag_random(lat.natom, s, chunk=37)
    assert np.array_equal(u, o.emom[0]) and np.array_equal(u, o.emom[1])
    nxt = [o.lib.orc_mt_real2(po.C.byref(o.mt)) for _ in range(5)]
    assert np.array_equal(s.real2(5), nxt)


def _fortran_assignment(ncells, conc, rn_all):
    """setup_chemicaldata's loop as written: per site, maxloc over the draws, the taken
    draw set to zero; the first nint(c ncells) taken cells get type 1, and so on."""
    na = len(conc)
    ach = np.zeros(na * ncells, dtype=np.int32)
    for ia in range(na):
        rn = rn_all[ia * ncells:(ia + 1) * ncells].copy()
        q = [int(np.floor(c * ncells + 0.5)) for c in conc[ia]]
        atoms = []
        for _ in range(ncells):
            k = int(np.argmax(rn))  # the first maximum, as maxloc
            atoms.append(k)
            rn[k] = 0.0
        start = 0
        for ich, qq in enumerate(q, 1):
            for i in range(start, start + qq):
                ach[atoms[i] * na + ia] = ich
            start += qq
    return ach


@pytest.mark.parametrize("conc", [[(0.8, 0.2), (0.2, 0.8)], [(0.5, 0.3), (0.25, 0.25, 0.3)]])
def test_random_chemistry_follows_the_reference_loop(conc):
    ncells, seed = 125, 7
    rn = po.mt_stream(seed, len(conc) * ncells, "real2")
    ach = lattice.random_chemistry(ncells, conc, seed=seed)
    assert np.array_equal(ach, _fortran_assignment(ncells, conc, rn))
    for ia, cs in enumerate(conc):
        counts = np.bincount(ach[ia::len(conc)], minlength=len(cs) + 1)
        assert list(counts[1:]) == [int(np.floor(c * ncells + 0.5)) for c in cs]
    with pytest.raises(ValueError):
        lattice.random_chemistry(10, [(0.7, 0.4)], seed=1)


def _pairs_by_distance(lat, L):
    """{(i, j): shell} of every pair within the second shell, by minimum-image distance."""
    coords = np.array([[c % L, (c // L) % L, c // (L * L)] for c in range(L ** 3)], dtype=np.float64)
    pos = np.concatenate([coords[:, None, :] + np.array(s[1:4])[None, None, :] for s in SITES], axis=1).reshape(-1, 3)
    out = {}
    for i in range(pos.shape[0]):
        d = pos - pos[i]
        d -= L * np.rint(d / L)
        r = np.sqrt(np.sum(d * d, axis=1))
        for j in np.nonzero(np.abs(r - np.sqrt(0.75)) < 1e-9)[0]:
            out[(i, int(j))] = 0
        for j in np.nonzero(np.abs(r - 1.0) < 1e-9)[0]:
            out[(i, int(j))] = 1
    return out


def test_alloy_couplings_follow_the_chemical_pairs():
    L = 5
    lat, e0 = lattice.from_tables(np.eye(3), (L, L, L), "PPP", SITES, JFILE, sym=1, maptype=2,
                                  chemistry=_chemistry(), tseed=1)
    ach = lat.meta["achtype"]
    assert np.array_equal(lat.species, ach - 1)
    assert np.array_equal(lat.mmom[0], np.array([MOM[a] for a in ach]))
    pairs = _pairs_by_distance(lat, L)
    got = {}
    for i in range(lat.natom):
        for s in range(lat.nlistsize[i]):
            got[(i, int(lat.nlist[i, s]) - 1)] = lat.ncoup[i, s]
    assert set(got) == set(pairs)
    for (i, j), sh in pairs.items():
        want = JTAB[(int(ach[i]), int(ach[j]))][sh] * lattice.FC2 / (MOM[ach[i]] * MOM[ach[j]])
        assert got[(i, j)] == pytest.approx(want, rel=1e-14)
    # the momfile directions of each atom's (site, type)
    assert np.allclose(e0[0, 0::2], [1.0, 0.0, 0.0]) and np.allclose(e0[0, 1::2], [0.0, 0.0, 1.0])


def test_dilute_alloy_drops_its_vacancies():
    L = 5
    lat, _ = lattice.from_tables(np.eye(3), (L, L, L), "PPP", SITES, JFILE, sym=1, maptype=2,
                                 chemistry=_chemistry((0.7, 0.2), (0.2, 0.7)), tseed=3)
    ach = lat.meta["achtype"]
    keep = ach > 0
    assert 0 < (~keep).sum() and lat.natom == keep.sum() == lat.species.size
    # the same types with every vacancy filled: the full lattice's lists and couplings
    full_types = np.where(keep, ach, 1)
    full, _ = lattice.from_tables(np.eye(3), (L, L, L), "PPP", SITES, JFILE, sym=1, maptype=2,
                                  chemistry=_chemistry((0.7, 0.2), (0.2, 0.7)), achtype=full_types)
    new_of = np.cumsum(keep)  # 1-based number of a kept atom
    old_of = np.nonzero(keep)[0]
    for n, i in enumerate(old_of):
        row = full.nlist[i, :full.nlistsize[i]] - 1
        ok = keep[row]
        assert lat.nlistsize[n] == ok.sum()
        assert np.array_equal(lat.nlist[n, :lat.nlistsize[n]], new_of[row[ok]])
        assert np.array_equal(lat.ncoup[n, :lat.nlistsize[n]], full.ncoup[i, :full.nlistsize[i]][ok])
    assert lat.nlist.max() <= lat.natom and lat.cells == (0, 0, 0)


def test_chemistry_rejects_missing_rows_and_other_forms():
    with pytest.raises(ValueError):
        lattice.from_tables(np.eye(3), (2, 2, 2), "PPP", SITES, JFILE, sym=1, maptype=2,
                            chemistry={1: _chemistry()[1]}, tseed=1)
    with pytest.raises(ValueError):
        lattice.from_tables(np.eye(3), (2, 2, 2), "PPP", SITES, JFILE, sym=1, maptype=2, chemistry=_chemistry(),
                            tseed=1, tensor=True)


def test_alloy_anisotropy_and_dm_follow_the_types():
    """kfile rows (isite, ichem, type, K1, K2, e, ratio) and DM rows with two chemical
    columns: each atom's anisotropy is its (site, type) row scaled by its own moment, each DM
    pair's vector that of the two types scaled by both moments (Sym 0: one bond vector)."""
    L = 4
    kfile = [(1, 1, 1, 0.10, 0.00, 0.0, 0.0, 1.0, 0.0), (1, 2, 1, 0.30, 0.02, 0.0, 0.0, 1.0, 0.0),
             (2, 1, 2, 0.05, 0.01, 1.0, 0.0, 0.0, 0.5), (2, 2, 1, 0.20, 0.00, 0.0, 1.0, 0.0, 0.0)]
    dtab = {(1, 1): (0.1, 0.0, 0.0), (1, 2): (0.0, 0.2, 0.0), (2, 1): (0.0, 0.0, 0.3), (2, 2): (0.4, 0.1, 0.0)}
    jrows = [(1, 1, ci, cj, 0.5, 0.5, 0.5, JTAB[(ci, cj)][0]) for (ci, cj) in JTAB]
    drows = [(1, 1, ci, cj, 0.5, 0.5, 0.5, *dtab[(ci, cj)]) for (ci, cj) in dtab]
    lat, _ = lattice.from_tables(np.eye(3), (L, L, L), "PPP", SITES, jrows, sym=0, maptype=2,
                                 chemistry=_chemistry(), tseed=5, kfile=kfile, dmfile=drows)
    ach = lat.meta["achtype"]
    rows = {(r[0], r[1]): r for r in kfile}
    for i in range(lat.natom):
        r = rows[(i % 2 + 1, int(ach[i]))]
        m = MOM[int(ach[i])]
        p1, p2 = (4, 6) if r[2] == 2 else (2, 4)
        assert lat.taniso[i] == r[2] and lat.sb[i] == r[8]
        assert lat.kaniso[i, 0] == pytest.approx(lattice.FC * r[3] / m ** p1, rel=1e-14)
        assert lat.kaniso[i, 1] == pytest.approx(lattice.FC * r[4] / m ** p2, rel=1e-14)
        assert np.allclose(lat.eaniso[i], np.array(r[5:8]) / np.linalg.norm(r[5:8]))
        assert lat.dmlistsize[i] == 1
        j = int(lat.dmlist[i, 0]) - 1
        want = np.array(dtab[(int(ach[i]), int(ach[j]))]) * lattice.FC2 / (m * MOM[int(ach[j])])
        assert np.allclose(lat.dm_vect[i, 0], want, rtol=1e-14, atol=0.0)
