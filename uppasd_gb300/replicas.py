"""Replica tables split over GPUs (one process per GPU) and merged on the host.

The reference runs its replicas one system at a time in one process
(mc_mphase per temperature, MonteCarlo/mc_driver.f90:234-420; the replica loop
of MonteCarlo/pt_driver.f90:58-367); there is no communication layer.  Replicas
are independent Markov chains, so a table of them shards without any data-path
exchange: rank r runs a contiguous share of the replicas, balanced by atom count,
as one ``ReplicaBatch`` whose replica ids start at the share's first index (its
Philox draws are then those of the whole table, whichever rank runs it), and the
per-replica accumulators are gathered on the host afterwards.  The merged
statistics are the reference's cumulants (``analysis.cumulants``) per replica.

The collectives here are host-side (``torch.distributed`` with any backend that
moves CPU tensors, gloo on a CPU-only box); nothing crosses between GPUs while the
chains run.
"""
from __future__ import annotations

import numpy as np

from .analysis import cumulants, tau_int

# per-replica accumulator columns of uppasd_gpu_mcbatch_stats
ACC_COLUMNS = ("n", "E", "E2", "M", "M2", "M4", "Mx", "My", "Mz", "M3")


def partition(natoms, world: int):
    """Contiguous shares [(start, stop)] of the replica list, one per rank, balanced by
    atom count (the work of a sweep): share r ends where the running atom count first
    reaches (r + 1) / world of the total.  Every rank gets at least one replica when
    there are at least `world` replicas."""
    natoms = np.asarray(natoms, dtype=np.float64)
    n = natoms.size
    if world < 1 or n < world:
        raise ValueError(f"cannot split {n} replicas over {world} ranks")
    cum = np.concatenate([[0.0], np.cumsum(natoms)])
    total = cum[-1]
    cuts = [0]
    for r in range(1, world):
        target = total * r / world
        # the boundary nearest to the target that leaves one replica for each later rank
        k = int(np.argmin(np.abs(cum - target)))
        k = max(k, cuts[-1] + 1)
        k = min(k, n - (world - r))
        cuts.append(k)
    cuts.append(n)
    return [(cuts[r], cuts[r + 1]) for r in range(world)]


def share_of(natoms, world: int, rank: int):
    return partition(natoms, world)[rank]


def gather_rows(local, share, nrep: int, world: int):
    """All-gather of per-replica rows: `local` holds the rows of replicas
    share[0]:share[1]; returns the (nrep, ...) array in replica order on every rank.
    With world == 1 it is `local` itself."""
    local = np.ascontiguousarray(local, dtype=np.float64)
    if world == 1:
        return local.copy()
    import torch
    import torch.distributed as dist

    tail = local.shape[1:]
    width = int(np.prod(tail)) if tail else 1
    # fixed-size slots: the largest share, padded; each slot carries its start and count
    cnt = torch.tensor([local.shape[0]], dtype=torch.int64)
    counts = [torch.zeros(1, dtype=torch.int64) for _ in range(world)]
    dist.all_gather(counts, cnt)
    cap = int(max(c.item() for c in counts))
    buf = torch.zeros((cap * width + 2,), dtype=torch.float64)
    buf[0], buf[1] = float(share[0]), float(local.shape[0])
    buf[2:2 + local.size] = torch.from_numpy(local.reshape(-1))
    bufs = [torch.zeros_like(buf) for _ in range(world)]
    dist.all_gather(bufs, buf)
    out = np.zeros((nrep,) + tail)
    for b in bufs:
        s0, k = int(b[0].item()), int(b[1].item())
        out[s0:s0 + k] = b[2:2 + k * width].numpy().reshape((k,) + tail)
    return out


def merged_statistics(acc, natoms, temperature):
    """Cumulants of every replica of the table from the gathered accumulators
    (nrep, 10): <M>, <M^2>, <M^4>, U_L, chi and C_v as calc_and_print_cumulant forms them."""
    acc = np.asarray(acc, dtype=np.float64)
    out = cumulants(acc[:, 0], acc[:, 1], acc[:, 2], acc[:, 3], acc[:, 4], acc[:, 5],
                    np.asarray(natoms, dtype=np.float64), np.asarray(temperature, dtype=np.float64))
    out["n"] = acc[:, 0]
    return out


def tau_of_series(series, c: float = 6.0):
    """Per replica the larger of tau_int(E) and tau_int(|M|) from a (k, n, 2) series."""
    return np.array([max(tau_int(s[:, 0], c)[0], tau_int(s[:, 1], c)[0]) for s in np.asarray(series)])


def independent_samples_per_s(sweeps_per_s: float, tau):
    """sum_r sweeps/s / (2 tau_r) over the whole table."""
    return float(np.sum(sweeps_per_s / (2.0 * np.asarray(tau, dtype=np.float64))))
