"""The C ABI from plain C: tests/c_harness.c, compiled as C99 with -Wall -Wextra -pedantic
-Werror against include/uppasd_gpu.h, plays the Fortran driver (Fortran-layout arrays,
status checks).  On CPU it must compile, link and see its malformed init refused; on the
GPU its Depondt run at 100 K and its heat-bath sweeps must equal the oracle's (1e-9 for the
LLG trajectory, 1e-12 per spin for the sweeps, as the Python-driven parity tests)."""
import os
import subprocess

import numpy as np
import pytest

from oracle import pyoracle as po
from uppasd_gb300 import lattice

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
L, M = 8, 2


@pytest.fixture(scope="module")
def harness(tmp_path_factory):
    from uppasd_gb300 import build as b
    b.build()
    exe = str(tmp_path_factory.mktemp("harness") / "c_harness")
    libdir = os.path.join(ROOT, "uppasd_gb300")
    subprocess.run(["gcc", "-std=c99", "-O1", "-Wall", "-Wextra", "-pedantic", "-Werror",
                    os.path.join(ROOT, "tests", "c_harness.c"), "-o", exe, "-L" + libdir, "-luppasd_gb300",
                    "-Wl,-rpath," + libdir, "-lm"], check=True)
    return exe


def test_compiles_as_c99_and_rejects_bad_input(harness):
    out = subprocess.run([harness, "reject"], capture_output=True, text=True)
    assert out.returncode == 0, out.stdout + out.stderr
    assert out.stdout.startswith("-1 ") and "nlist" in out.stdout


def _lattice():
    lat, _ = lattice.from_tables(np.eye(3), (L, L, L), "PPP", [(1, 0.0, 0.0, 0.0, 2.0, 0.0, 0.0, 1.0)],
                                 [(1, 1, 0.0, 0.0, 1.0, 1.0)], sym=1, kfile=[(1, 1, 0.1, 0.0, 0.0, 0.0, 1.0, 0.0)])
    lat = lat.with_ensembles(M)
    lat.extfield[..., 2] = 0.5
    return lat


def _start():
    i = np.arange(L ** 3)
    e = np.zeros((M, L ** 3, 3))
    for k in range(M):
        e[k, :, 0] = np.sin(0.37 * i + 1.1 * k)
        e[k, :, 1] = np.cos(0.23 * i)
        e[k, :, 2] = 0.4 + 0.1 * k
    return e / np.sqrt(np.sum(e * e, axis=-1))[..., None]


@pytest.mark.gpu
def test_run_matches_oracle(harness, tmp_path):
    nsteps = 100
    out = tmp_path / "out.bin"
    r = subprocess.run([harness, "run", str(nsteps), str(out)], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    d = np.fromfile(out, dtype=np.float64)
    n3 = 3 * L ** 3 * M
    emom, mvec, mabs, en, emom_mc = np.split(d, [n3, n3 + 3 * M, n3 + 4 * M, n3 + 5 * M])
    lat = _lattice()
    o = po.Oracle(lat)
    o.set_moments(_start())
    o.make_llg(5, 1e-16, 0.1, 100.0, 1.0, noise_mode=po.NOISE_PHILOX, seed=7)
    for _ in range(nsteps):
        o.sd_step()
    assert np.max(np.abs(emom.reshape(M, -1, 3) - o.emom)) <= 1e-9
    mv, ma = o.mavg()
    assert np.allclose(mvec.reshape(M, 3), mv, rtol=1e-9, atol=1e-12)   # total moment, as calc_mavrg sums it
    assert np.allclose(mabs, ma, rtol=1e-9, atol=1e-12)
    assert np.allclose(en, o.energy()["total"], rtol=1e-9, atol=1e-12)
    o.set_moments(emom.reshape(M, -1, 3))
    _, order, start = lattice.greedy_colouring(lat)
    for sw in range(3):
        o.mc_sweep_checkerboard("H", 50.0, order, start, 7, sw)
    assert np.max(np.abs(emom_mc.reshape(M, -1, 3) - o.emom)) <= 1e-12
