"""A replica table split over processes and merged on the host (one process per GPU
on a multi-GPU machine; here two gloo ranks on the CPU, rendezvous on 127.0.0.1).

Each rank takes its contiguous share of the table (``replicas.partition``, balanced
by atom count) and advances its replicas' chains; here the chain is the oracle's
checkerboard heat bath, whose Philox draws are keyed by the replica's id in the
whole table, as the GPU batch's are after ``set_replica_ids``.  The per-replica
accumulators (n, E, E^2, |M|, M^2, M^4, M vector, |M|^3) and (E, |M|) series are
gathered with ``replicas.gather_rows``; the merged cumulants, tau_int and the
table's independent samples/s must equal a one-process run of the same table
bit for bit.  bench.py's timing helpers (barrier, max over ranks) are checked too.
"""
import os
import socket

import numpy as np
import pytest
import torch.multiprocessing as mp

L_TABLE = [4, 4, 6, 4, 6, 4, 4]
T_TABLE = [600.0, 900.0, 1100.0, 1200.0, 1300.0, 1400.0, 1500.0]
SEED, NSWEEP = 77, 40


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _replica_chain(g):
    """Replica g of the table: accumulators (10,) and the (E, |M|) series of NSWEEP
    heat-bath sweeps of the oracle's checkerboard chain with replica id g."""
    from oracle import pyoracle as po
    from uppasd_gb300 import lattice

    L, T = L_TABLE[g], T_TABLE[g]
    lat = lattice.bcc(L, [1.3, 0.7], 2.2).with_ensembles(g + 1)   # ensemble g carries id g
    rng = np.random.default_rng(1000 + g)
    e0 = rng.normal(size=(1, lat.natom, 3))
    e0 /= np.linalg.norm(e0, axis=-1, keepdims=True)
    o = po.Oracle(lat, threads=1)
    o.set_moments(np.broadcast_to(e0, (g + 1, lat.natom, 3)))
    _, order, start = lattice.greedy_colouring(lat)
    ser = np.zeros((NSWEEP, 2))
    acc = np.zeros(10)
    for sw in range(NSWEEP):
        o.mc_sweep_checkerboard("H", T, order, start, SEED, sw)
        E = o.energy()["total"][g]
        mv, ma = o.mavg()
        M = ma[g]
        ser[sw] = (E, M)
        acc += [1.0, E, E * E, M, M * M, M ** 4, mv[g, 0], mv[g, 1], mv[g, 2], M ** 3]
    return acc, ser


def _table_results(acc, ser, sweeps_per_s):
    from uppasd_gb300 import replicas

    natoms = 2 * np.asarray(L_TABLE) ** 3
    st = replicas.merged_statistics(acc, natoms, T_TABLE)
    tau = replicas.tau_of_series(ser)
    return st, tau, replicas.independent_samples_per_s(sweeps_per_s, tau)


def _worker(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    import bench
    from uppasd_gb300 import replicas

    w, r = bench.dist_setup()
    assert (w, r) == (world, rank)
    natoms = 2 * np.asarray(L_TABLE) ** 3
    s0, s1 = replicas.share_of(natoms, world, rank)
    loc = [_replica_chain(g) for g in range(s0, s1)]
    acc = replicas.gather_rows(np.array([a for a, _ in loc]), (s0, s1), len(L_TABLE), world)
    ser = replicas.gather_rows(np.array([s for _, s in loc]), (s0, s1), len(L_TABLE), world)
    bench.dist_barrier(w)
    # the table's sweep rate is set by the slowest rank
    rate = bench.dist_max(100.0 + 5 * rank, w)
    st, tau, indep = _table_results(acc, ser, 1.0 / rate)
    out[rank] = (acc, ser, st["binder"], st["chi"], tau, indep, (s0, s1), rate)
    import torch.distributed as dist
    dist.destroy_process_group()


def test_partition_is_contiguous_and_balanced():
    from uppasd_gb300 import replicas

    natoms = 2 * np.array([16] * 16 + [24] * 16 + [32] * 16 + [48] * 16) ** 3
    for world in (1, 2, 3, 4, 8):
        sh = replicas.partition(natoms, world)
        assert sh[0][0] == 0 and sh[-1][1] == natoms.size
        assert all(a[1] == b[0] for a, b in zip(sh, sh[1:]))
        assert all(b > a for a, b in sh)
        work = np.array([natoms[a:b].sum() for a, b in sh])
        # no share exceeds the ideal by more than its largest replica
        assert work.max() <= natoms.sum() / world + natoms.max()
    with pytest.raises(ValueError):
        replicas.partition([10, 10], 3)


def test_split_table_merges_to_the_one_process_result():
    world = 2
    port = _free_port()
    mgr = mp.get_context("spawn").Manager()
    out = mgr.dict()
    mp.start_processes(_worker, args=(world, port, out), nprocs=world, start_method="spawn", join=True)
    # one process, the whole table
    full = [_replica_chain(g) for g in range(len(L_TABLE))]
    acc1 = np.array([a for a, _ in full])
    ser1 = np.array([s for _, s in full])
    st1, tau1, indep1 = _table_results(acc1, ser1, 1.0 / 105.0)
    shares = [out[r][6] for r in range(world)]
    assert shares[0][1] == shares[1][0] and shares[0][0] == 0 and shares[1][1] == len(L_TABLE)
    for r in range(world):
        acc, ser, binder, chi, tau, indep, _, rate = out[r]
        assert rate == 105.0
        assert np.array_equal(acc, acc1) and np.array_equal(ser, ser1)
        assert np.array_equal(binder, st1["binder"]) and np.array_equal(chi, st1["chi"])
        assert np.array_equal(tau, tau1) and indep == indep1
