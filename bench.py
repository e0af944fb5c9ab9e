"""Benchmark of the GB300 LLG hot path (one JSON line on stdout).

Workload (default): the large plain + batched LLG configuration -- random
binary alloy on bcc 100x100x100 conventional cells (2,000,000 atoms), A/B
50/50 from a seed, four exchange shells J_AA/AB/BB = 1.3/1.8/0.9 mRy decaying
0.5x per shell, moments 2.2/1.6 muB, Depondt solver, T = 300 K, 8 ensembles
advanced together (16 M spins).  Inputs are synthetic (generated from seeds);
the spin state (>= 384 MB) is larger than the 129 MB L2, so no L2 flush is
needed between timed steps.

A "step" is one full LLG step (field, predictor, field, corrector, moment
update) of all 16 M spins.  `value` is atom-steps/s with the state resident in
HBM; `e2e` is the same metric through the C ABI with the spin state copied
from pinned host memory before, and back after, each block of `--e2e-inner`
steps (the drop-in's measurement interval).

The same JSON line carries an "mc" object for the batched Monte Carlo
temperature sweep: 64 bcc J1/J2 replicas (16 temperatures 600-1400 K x L = 16,
24, 32, 48 cells; 8,192 to 221,184 atoms each, 5,160,960 spins), checkerboard
heat bath, 10^4 thermalisation + 10^5 measured sweeps in one persistent launch
per 250 sweeps replayed from a CUDA graph, autotuned schedule.  Its headline is
independent samples/s = sum_r (sweeps/s) / (2 tau_int,r), tau_int the larger of
the Sokal-windowed times of E and |M| per replica, against the plain GPU heat
bath (one launch per colour per replica, the same Markov chain and so the same
tau_int) timed on the same sizes.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

WORKLOADS = {
    "alloy2m": dict(kind="alloy", L=100, ens=8, solver=5, dt=1e-16, damping=0.1, temp=300.0,
                    desc="bcc random binary alloy 100^3 cells (2,000,000 atoms) x 8 ensembles, 4 shells (50 nbrs), "
                         "Depondt, T=300 K"),
    # same Hamiltonian on 64^3 cells (524,288 atoms x 8 = 4.2 M spins, ~0.3 GB of state):
    # the profiling case (still larger than L2, a few hundred MB on the device)
    "alloy64": dict(kind="alloy", L=64, ens=8, solver=5, dt=1e-16, damping=0.1, temp=300.0,
                    desc="bcc random binary alloy 64^3 cells (524,288 atoms) x 8 ensembles, 4 shells, Depondt, "
                         "T=300 K"),
    "bcc16k": dict(kind="bcc", L=20, ens=1, solver=5, dt=1e-16, damping=0.1, temp=300.0,
                   desc="bcc ferromagnet 20^3 cells (16,000 atoms), J1=1.3 J2=0.7 mRy, Depondt, T=300 K"),
    "square256": dict(kind="square", L=256, ens=1, solver=1, dt=1e-16, damping=0.05, temp=50.0,
                      desc="square monolayer 256^2, J=1.0, interfacial D=0.3, Kz=-0.05 mRy, Bz=0.5 T, midpoint, "
                           "T=50 K"),
    # the square DMI Hamiltonian at a size where the GPU is filled: the general-Hamiltonian
    # variant line (FP64 path against the FP32-gather / FP64-master path)
    "square1024x4": dict(kind="square", L=1024, ens=4, solver=1, dt=1e-16, damping=0.05, temp=50.0,
                         desc="square monolayer 1024^2 x 4 ensembles, J=1.0, interfacial D=0.3, Kz=-0.05 mRy, "
                              "Bz=0.5 T, midpoint, T=50 K"),
}


def build_lattice(w):
    from uppasd_gb300 import lattice

    if w["kind"] == "alloy":
        lat = lattice.bcc_alloy(w["L"], seed=2024)
    elif w["kind"] == "bcc":
        lat = lattice.bcc(w["L"], [1.3, 0.7], 2.2)
    else:
        lat = lattice.square_dmi(w["L"], 1.0, 0.3, -0.05, 0.5, 1.0)
    return lat.with_ensembles(w["ens"])


def random_state(n_ens, natom, seed=7):
    rng = np.random.default_rng(seed)
    e = rng.normal(size=(n_ens, natom, 3))
    e /= np.linalg.norm(e, axis=-1, keepdims=True)
    return e


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.index = index
        self.proc = None
        self.lines = []
        self.first = 0

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.QUERY}",
                                          "--format=csv,noheader,nounits", "-lms", "50"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self._t = threading.Thread(target=self._read, daemon=True)
            self._t.start()
            # nvidia-smi takes a moment to start: let its first sample land before the
            # timed region begins, so that the region itself is sampled
            t0 = time.perf_counter()
            while not self.lines and time.perf_counter() - t0 < 3.0 and self.proc.poll() is None:
                time.sleep(0.01)
            self.first = len(self.lines)
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for ln in self.proc.stdout:
            self.lines.append(ln.strip())

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        # the samples taken once the region had begun (the one before it when there are none)
        for ln in self.lines[self.first:] or self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


def bf16_peak():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        return float(json.load(open(p)).get("bf16_tflops", 1900.0))
    return 1900.0


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return d.get("hbm_gbs", 6800.0), "measured"
    return 6800.0, "fallback"


# DRAM read + write bytes per launch of the dominant kernels (ncu dram__bytes_read.sum +
# dram__bytes_write.sum, one capture each, not measured by this run): (bytes, how the
# figure was obtained).  A kernel that has none reports traffic null.
PROFILED_TRAFFIC = {
    "stencil_tma_correct:alloy2m:p2": (1.421e9, "ncu capture at the benchmark size (100^3 x 8 ensembles, one pass)"),
    "stencil_tma_predict:alloy2m:p2": (0.757e9, "ncu capture at the benchmark size (100^3 x 8 ensembles, one pass)"),
    "mb_sweeps:mc64": (12.8e9, "ncu capture of a 40-sweep launch of the 64-replica table, scaled x 250/40"),
}


def profiled_traffic(name):
    """(per-launch DRAM bytes, source) of a dominant kernel from a committed ncu capture."""
    return PROFILED_TRAFFIC.get(name, (None, None))


def cpu_baseline(w, lat, e0, threads, target_s=12.0):
    """The oracle (C restatement of the reference's Fortran) on a bounded sample:
    one ensemble of the same lattice, steps until ~target_s of CPU work."""
    from oracle import pyoracle as po

    o = po.Oracle(lat, threads=threads, fast=True)
    o.set_moments(e0)
    o.make_llg(w["solver"], w["dt"], w["damping"], w["temp"], 1.0, noise_mode=po.NOISE_PHILOX, seed=5)
    t0 = time.perf_counter()
    o.sd_step()
    one = time.perf_counter() - t0
    n = max(1, min(2000, int(target_s / max(one, 1e-6))))
    t0 = time.perf_counter()
    for _ in range(n):
        o.sd_step()
    dt = time.perf_counter() - t0
    nspin = lat.natom * lat.mensemble
    return {"value": nspin * n / dt, "unit": "atom-steps/s", "cores": o.lib.orc_get_threads(),
            "kind": "port",
            "sample": f"{n} steps of all {lat.mensemble} ensembles ({nspin} spins), same Hamiltonian; "
                      "oracle built -O3 (liboracle_fast.so), OpenMP over sites"}


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("gloo")
    return world, rank


def dist_max(x, world):
    if world == 1:
        return x
    import torch
    import torch.distributed as dist

    t = torch.tensor([x], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def dist_barrier(world):
    if world > 1:
        import torch.distributed as dist

        dist.barrier()


def run_reference(args, w):
    world, rank = dist_setup()
    if rank != 0:
        return
    lat = build_lattice(w)
    e0 = random_state(lat.mensemble, lat.natom)
    threads = os.cpu_count() or 1
    from oracle import pyoracle as po

    po.build()
    o = po.Oracle(lat, threads=threads, fast=True)
    o.set_moments(e0)
    o.make_llg(w["solver"], w["dt"], w["damping"], w["temp"], 1.0, noise_mode=po.NOISE_PHILOX, seed=5)
    for _ in range(args.warmup):
        o.sd_step()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        o.sd_step()
    dt = time.perf_counter() - t0
    nspin = lat.natom * lat.mensemble
    v = nspin * args.steps / dt
    line = {"impl": "reference", "metric": "LLG atom-steps/s", "value": v, "unit": "atom-steps/s",
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup, "ms_per_step": dt / args.steps * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded lattice, species and spins)",
            "config": {"workload": args.workload, "description": w["desc"], "natom": lat.natom,
                       "ensembles": lat.mensemble, "spins": nspin},
            "cpu_baseline": {"value": v, "unit": "atom-steps/s", "cores": threads, "kind": "port",
                             "sample": f"{args.steps} steps of all {lat.mensemble} ensembles ({nspin} spins) "
                                       "per run, the oracle's C restatement of the Fortran built -O3 with "
                                       "OpenMP over sites (no Fortran compiler exists on either machine)"},
            "e2e": {"value": v, "unit": "atom-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    if not args.no_mc:
        line["mc"] = {"cpu_baseline": mc_cpu_baseline()}
    print(json.dumps(line), flush=True)


MC_LS = (16, 24, 32, 48)
MC_T = (600.0, 1400.0, 16)
MC_J = (1.3, 0.7)


def mc_table():
    Ts = np.linspace(*MC_T)
    return [l for l in MC_LS for _ in Ts], [float(t) for _ in MC_LS for t in Ts]


def _mc_cpu_worker(job):
    """One replica of the reference chain (random-permutation heat bath, mtprng +
    ziggurat) on one core for about `seconds`: spin updates per second."""
    L, T, seconds, seed = job
    from oracle import pyoracle as po
    from uppasd_gb300 import lattice

    lat = lattice.bcc(L, list(MC_J), 2.2)
    o = po.Oracle(lat, threads=1)
    rng = np.random.default_rng(seed)
    e0 = rng.normal(size=(1, lat.natom, 3))
    e0 /= np.linalg.norm(e0, axis=-1, keepdims=True)
    o.set_moments(e0)
    import ctypes as C

    o.mt = po.OrcMT()
    o.lib.orc_mt_init(C.byref(o.mt), seed)
    o.setup_ziggurat(seed)
    iflip = o.choose_random_atom_x()
    n, t0 = 0, time.perf_counter()
    while True:
        o.mc_sweep_ref("H", T, iflip)
        n += 1
        dt = time.perf_counter() - t0
        if dt >= seconds:
            break
    return lat.natom * n / dt, n


def mc_cpu_baseline(seconds=10.0):
    """The reference's MC path restated (oracle) on the host cores: one process per
    core, each sweeping one replica of the table (the reference runs one
    replica per thread; its OpenMP site loop is racy)."""
    import multiprocessing as mp

    L, T = mc_table()
    ncores = os.cpu_count() or 1
    jobs = [(L[i * len(L) // ncores], T[i * len(L) // ncores], seconds, 11 + i) for i in range(ncores)]
    with mp.get_context("spawn").Pool(ncores) as pool:
        res = pool.map(_mc_cpu_worker, jobs)
    return {"value": float(sum(r[0] for r in res)), "unit": "spin-updates/s", "cores": ncores, "kind": "port",
            "sample": f"{ncores} replicas of the table (one per core), {seconds:.0f} s of heat-bath sweeps each"}


def _mc_table_run(args, world, rank, heatbath, stream, spl=250):
    """The replica table in one mode (heat bath or Metropolis), split over the ranks by
    atom count (each rank one contiguous share, replica ids continuing across shares):
    autotune, thermalise, then the timed measured sweeps.  Returns the merged per-replica
    accumulators and tau_int, the max-over-ranks time and the schedule."""
    import torch

    from uppasd_gb300 import replicas
    from uppasd_gb300.batch import DEFAULT_CACHE, ReplicaBatch

    L, T = mc_table()
    natoms = 2 * np.asarray(L, dtype=np.int64) ** 3
    s0, s1 = replicas.share_of(natoms, world, rank)
    b = ReplicaBatch(L[s0:s1], T[s0:s1], heatbath=1 if heatbath else 0, j_shells_mry=MC_J, seed=31,
                     series_len=args.mc_meas, max_sweeps_per_launch=spl, first_id=s0)
    tuned = b.autotune(20, cache=DEFAULT_CACHE)
    bld, thr, ctas = b.schedule()
    b.run(args.mc_therm, spl)
    b.set_stream(stream.cuda_stream)
    b.run(0, spl, measure=True)  # sets the measuring flag before the timed region
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    dist_barrier(world)
    torch.cuda.synchronize()
    ev0.record(stream)
    b.enqueue(args.mc_meas, spl, measure=True)
    ev1.record(stream)
    torch.cuda.synchronize()
    b.check()
    dist_barrier(world)
    ms = dist_max(ev0.elapsed_time(ev1), world)
    acc, _, _ = b.raw_stats()
    tau_loc = b.tau_int()
    b.close()
    acc = replicas.gather_rows(acc, (s0, s1), len(L), world)
    tau = replicas.gather_rows(tau_loc, (s0, s1), len(L), world)
    return {"acc": acc, "tau": tau, "ms": ms, "schedule": (bld, thr, ctas, tuned), "share": (s0, s1),
            "natoms": natoms, "L": L, "T": T}


def _plain_tau(Lv, T, nsweeps, stream, seed=3):
    """tau_int of the plain FP64 heat bath (the simulation's checkerboard sweeps, one
    temperature per ensemble) for the replicas of size Lv: E and |M| every sweep."""
    from uppasd_gb300 import lattice, replicas
    from uppasd_gb300.simulation import GpuSimulation

    lat = lattice.bcc(Lv, list(MC_J), 2.2).with_ensembles(len(T))
    sim = GpuSimulation(lat, emom=random_state(len(T), lat.natom, seed=seed), seed=seed + 1)
    sim.set_stream(stream.cuda_stream)
    sim.relax_temps("H", T, 2000)
    ser = np.zeros((len(T), nsweeps, 2))
    for k in range(nsweeps):
        sim.relax_temps("H", T, 1)
        ob = sim.observables()
        ser[:, k, 0] = ob["energy"]
        ser[:, k, 1] = ob["mabs"]
    sim.close()
    return replicas.tau_of_series(ser)


def run_mc(args, world, rank, peak, peak_kind):
    """Batched replica MC (heat bath and Metropolis tables) against the plain GPU heat
    bath (see the module docstring)."""
    import torch

    from uppasd_gb300 import lattice, replicas
    from uppasd_gb300.simulation import GpuSimulation

    spl = 250
    stream = torch.cuda.Stream()
    runs = {"heat_bath": _mc_table_run(args, world, rank, True, stream, spl)}
    if not args.no_metropolis:
        runs["metropolis"] = _mc_table_run(args, world, rank, False, stream, spl)
    hb = runs["heat_bath"]
    L, T, natoms = hb["L"], hb["T"], hb["natoms"]
    nlaunch = -(-args.mc_meas // spl)

    def summary(r, name):
        sweeps_s = args.mc_meas / (r["ms"] * 1e-3)
        st = replicas.merged_statistics(r["acc"], natoms, T)
        bld, thr, ctas, tuned = r["schedule"]
        return {
            "mode": name, "value": replicas.independent_samples_per_s(sweeps_s, r["tau"]), "unit": "samples/s",
            "spin_updates_per_s": float(natoms.sum()) * sweeps_s, "sweeps_per_s_per_replica": sweeps_s,
            "ms_per_sweep": r["ms"] / args.mc_meas,
            "tau_int": {"min": float(r["tau"].min()), "max": float(r["tau"].max()),
                        "median": float(np.median(r["tau"]))},
            "schedule_rank0": {"register_build": bld, "threads": thr, "ctas": int(np.sum(ctas)),
                               "tuned_ms_per_sweep": tuned, "replicas": list(r["share"])},
            "observables": {f"L{l}": {"T": [round(t, 1) for t in T[i * 16:(i + 1) * 16]],
                                      "binder": [round(float(u), 5) for u in st["binder"][i * 16:(i + 1) * 16]],
                                      "chi": [float(c) for c in st["chi"][i * 16:(i + 1) * 16]],
                                      "M": [round(float(m), 5) for m in st["M"][i * 16:(i + 1) * 16]],
                                      "E": [round(float(e), 5) for e in st["E"][i * 16:(i + 1) * 16]]}
                            for i, l in enumerate(MC_LS)}}

    hb_sum = summary(hb, "heat bath")
    # plain GPU heat bath: the FP64 checkerboard chain of the simulation path, one
    # replica at a time (the reference's mc_mphase runs one system per temperature)
    plain_sweeps_s = {}
    for Lv in MC_LS:
        lat = lattice.bcc(Lv, list(MC_J), 2.2)
        sim = GpuSimulation(lat, emom=random_state(1, lat.natom, seed=3), seed=5)
        sim.set_stream(stream.cuda_stream)
        sim.relax("H", 1000.0, 20)
        n = 200
        torch.cuda.synchronize()
        e0v, e1v = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0v.record(stream)
        sim.relax("H", 1000.0, n)
        e1v.record(stream)
        torch.cuda.synchronize()
        plain_sweeps_s[Lv] = n / (e0v.elapsed_time(e1v) * 1e-3)
        sim.close()
    # a sweep of the whole table costs sum_r 1 / rate_r on the plain path, and each
    # replica advances one sweep per table sweep
    table_sweep_s = float(np.sum([1.0 / plain_sweeps_s[l] for l in L]))
    # the plain chain's own tau_int, measured on the two smaller sizes (all 16 T each);
    # the two larger sizes take the batched chain's tau (the same algorithm, FP32 draws)
    plain_tau = hb["tau"].copy()
    tau_cmp = {}
    if not args.no_plain_tau:
        for i, Lv in enumerate(MC_LS[:2]):
            sl = slice(i * 16, (i + 1) * 16)
            pt = _plain_tau(Lv, T[sl], args.plain_tau_sweeps, stream)
            plain_tau[sl] = pt
            tau_cmp[f"L{Lv}"] = {"plain_fp64": [round(float(x), 2) for x in pt],
                                 "batched_fp32": [round(float(x), 2) for x in hb["tau"][sl]]}
    plain_indep = float(np.sum((1.0 / table_sweep_s) / (2.0 * plain_tau))) * world
    # algorithmic bytes: 6 s per spin update (read and write 3 FP32 components)
    per_launch_bytes = 24.0 * natoms.sum() * spl / world
    ms_launch = hb["ms"] / nlaunch
    achieved = per_launch_bytes / (ms_launch * 1e-3) / 1e9 * world
    tr, tr_src = profiled_traffic("mb_sweeps:mc64")
    out = dict(hb_sum)
    out.update({
        "metric": "MC independent samples/s (batched heat bath)",
        "plain_gpu_heat_bath": plain_indep, "speedup_vs_plain": hb_sum["value"] / plain_indep,
        "plain_sweeps_per_s": {str(k): v for k, v in plain_sweeps_s.items()},
        "plain_table_sweep_ms": table_sweep_s * 1e3,
        "plain_tau_measured": tau_cmp,
        "plain_tau_note": "plain FP64 chain's tau_int measured for L=16, 24 (every T); L=32, 48 use the batched "
                          "chain's tau (same Markov chain, FP32 draws)",
        "workload": "bcc J1=1.3 J2=0.7 mRy, 64 replicas: 16 T in 600-1400 K x L=16,24,32,48 (5,160,960 spins), "
                    "checkerboard heat bath and Metropolis tables",
        "thermalisation_sweeps": args.mc_therm, "measured_sweeps": args.mc_meas, "sweeps_per_launch": spl,
        "ranks": world, "replica_split": "contiguous shares balanced by atoms, merged on the host",
        "gpu_launches": 3 * nlaunch * len(runs),
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "traffic": tr, "traffic_source": tr_src, "kernel": "mb_sweeps",
                     "peak_source": peak_kind, "algorithmic_bytes_per_launch": per_launch_bytes,
                     "note": "24 B per spin update; the 83 MB spin pool is L2-resident"},
    })
    if "metropolis" in runs:
        out["metropolis"] = summary(runs["metropolis"], "Metropolis")
    return out


# Learned-proposal workload: 128^2 square DMI lattice (J = 1 mRy, D/J = 0.3), a grid of
# 19 temperatures 5-30 K x 8 chains (152 chains: 38,912 patch rows per colour, 304
# tensor-core row tiles = two full waves on 152 SMs), the field chosen by a scan for the
# largest skyrmion density.
C3 = dict(L=128, temps=(5.0, 30.0, 19), copies=8, J=1.0, D=0.3,
          bz_scan=(5.0, 10.0, 15.0, 20.0, 25.0, 30.0, 35.0, 40.0, 50.0, 60.0),
          scan_chains=16, eta_scale=16.0, therm=20000, snapshots=96, snap_every=50, train_steps=3000,
          train_rows=16384, lr=1e-3)


def _c3_temps():
    c = C3
    Ts = np.linspace(*c["temps"])
    return np.repeat(Ts, c["copies"]), Ts


def _bz_scan(seed=1):
    """Field scan at the grid's lowest temperature: each field's chains are field-cooled by
    the heat bath (2000 sweeps at 30 K, 4000 at 5 K) from a random start; reported per
    field: mean |Q| (skyrmion number) and m_z per spin.  The skyrmion-lattice window is
    where |Q| is large and m_z below saturation."""
    from uppasd_gb300 import analysis, lattice
    from uppasd_gb300.simulation import GpuSimulation

    c = C3
    out = []
    for bz in c["bz_scan"]:
        lat = lattice.square_dmi(c["L"], c["J"], c["D"], 0.0, bz, 1.0).with_ensembles(c["scan_chains"])
        sim = GpuSimulation(lat, emom=random_state(c["scan_chains"], lat.natom, seed=seed), seed=seed + 1)
        sim.relax("H", 30.0, 2000, structured=True)
        sim.relax("H", c["temps"][0], 4000, structured=True)
        e = sim.get_moments()
        sim.close()
        q = analysis.topological_charge(e, c["L"])
        out.append({"bz": bz, "abs_Q_mean": float(np.mean(np.abs(q))), "Q": [round(float(v), 2) for v in q],
                    "mz": float(np.mean(e[..., 2]))})
    best = max(out, key=lambda r: r["abs_Q_mean"])
    return out, best["bz"]


def _tau_modes(sim, prop, snap, temps, Ts, modes, structured_ms, learned_ms, plain_ms):
    """Run each (name, hb sweeps, learned sweeps, cycles, plain) mode from the same snapshot;
    per temperature of the grid: tau_int of E and |M| (median over the copies), cost per
    cycle, independent samples/s, E and |M| with their errors over the copies."""
    from uppasd_gb300 import analysis

    out = {}
    ncopy = C3["copies"]
    for name, k_hb, k_l, n, plain in modes:
        sim.put_moments(snap)
        es, ms = [], []
        acc = prop_n = 0
        for _ in range(n):
            if plain:
                sim.relax_temps("H", temps, 1)
            elif k_l:
                a, p_, _ = prop.mix_temps(temps, 1, k_hb)
                acc += a
                prop_n += p_
            else:
                sim.relax_temps_square(temps, k_hb)
            ob = sim.observables()
            es.append(ob["energy"].copy())
            ms.append(ob["mabs"].copy())
        es, ms = np.array(es), np.array(ms)
        cost = plain_ms if plain else k_hb * structured_ms + k_l * learned_ms
        per_t = []
        for it, T in enumerate(Ts):
            cols = range(it * ncopy, (it + 1) * ncopy)
            te = float(np.median([analysis.tau_int(es[:, k])[0] for k in cols]))
            tm = float(np.median([analysis.tau_int(ms[:, k])[0] for k in cols]))
            ec, mc = es[:, list(cols)].mean(axis=0), ms[:, list(cols)].mean(axis=0)
            per_t.append({"T": round(float(T), 3), "tau_E": te, "tau_M": tm,
                          "indep_samples_per_s": ncopy / (2.0 * max(te, tm) * cost * 1e-3),
                          "E": [float(ec.mean()), float(ec.std(ddof=1) / np.sqrt(ncopy))],
                          "M": [float(mc.mean()), float(mc.std(ddof=1) / np.sqrt(ncopy))]})
        out[name] = {"heat_bath_sweeps_per_cycle": k_hb, "learned_sweeps_per_cycle": k_l, "cycles": n,
                     "ms_per_cycle": cost, "acceptance": acc / prop_n if prop_n else None,
                     "indep_samples_per_s": float(sum(r["indep_samples_per_s"] for r in per_t)), "per_T": per_t}
    return out


def run_c3(args, peak_tf):
    """Learned-proposal MC on the square DMI lattice over the temperature grid, against the
    batched heat bath alone and the plain FP64 heat bath."""
    import torch

    from uppasd_gb300 import lattice
    from uppasd_gb300.learned import LearnedProposal
    from uppasd_gb300.simulation import GpuSimulation

    c = C3
    scan, bz = _bz_scan()
    temps, Ts = _c3_temps()
    chains = temps.size
    lat = lattice.square_dmi(c["L"], c["J"], c["D"], 0.0, bz, 1.0).with_ensembles(chains)
    e0 = random_state(chains, lat.natom, seed=1)
    sim = GpuSimulation(lat, emom=e0, seed=2)
    sim.relax_temps_square(np.full(chains, 30.0), 2000)      # field-cooled start, as in the scan
    sim.relax_temps_square(temps, c["therm"])
    prop = LearnedProposal(sim, c["L"], eta_scale=c["eta_scale"],
                           data_capacity=chains * 1024 * c["snapshots"], seed=3)
    untrained = prop.mix_temps(temps, 2, 0)
    for _ in range(c["snapshots"]):
        sim.relax_temps_square(temps, c["snap_every"])
        prop.collect()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    losses = prop.train(c["train_steps"], rows=c["train_rows"], lr=c["lr"])
    torch.cuda.synchronize()
    t_train = time.perf_counter() - t0
    snap = sim.get_moments()

    def timed(fn, n):
        torch.cuda.synchronize()
        t = time.perf_counter()
        fn(n)
        torch.cuda.synchronize()
        return (time.perf_counter() - t) / n * 1e3

    learned_ms = timed(lambda n: prop.mix_temps(temps, n, 0), 50)
    structured_ms = timed(lambda n: sim.relax_temps_square(temps, n), 1000)
    plain_ms = timed(lambda n: sim.relax_temps("H", temps, n), 50)
    modes = [("plain_fp64_heat_bath", 1, 0, 4000, True), ("batched_heat_bath", 1, 0, 24000, False),
             ("learned", 0, 1, 6000, False), ("batched_heat_bath_x8+learned", 8, 1, 3000, False)]
    res = _tau_modes(sim, prop, snap, temps, Ts, modes, structured_ms, learned_ms, plain_ms)
    rows = chains * (c["L"] // 8) ** 2
    flop_pass = 2.0 * rows * (192 * 256 + 2 * 256 * 256 + 256 * 64)
    flops_sweep = 4 * 4 * flop_pass  # 4 colours x 4 passes
    achieved_tf = flops_sweep / (learned_ms * 1e-3) / 1e12
    hb, mix = res["batched_heat_bath"], res["batched_heat_bath_x8+learned"]
    gain_per_T = [{"T": a["T"], "mix_over_heat_bath": b["indep_samples_per_s"] / a["indep_samples_per_s"]}
                  for a, b in zip(hb["per_T"], mix["per_T"])]
    plain = res["plain_fp64_heat_bath"]["indep_samples_per_s"]
    prop.close()
    sim.close()
    return {
        "metric": "MC independent samples/s, learned + batched vs batched heat bath alone and plain FP64 heat bath",
        "workload": f"square {c['L']}x{c['L']} J={c['J']} mRy, D/J={c['D']/c['J']}, Bz={bz} T (scan below), "
                    f"T grid {Ts[0]}-{Ts[-1]} K x {len(Ts)} x {c['copies']} chains; MADE 4x4-patch proposal "
                    "(3x8x8 input, 3x256 tanh, vMF per spin), one network for the whole grid",
        "value": mix["indep_samples_per_s"], "unit": "samples/s",
        "speedup_vs_plain": mix["indep_samples_per_s"] / plain,
        "learned_plus_batched_vs_batched_alone": mix["indep_samples_per_s"] / hb["indep_samples_per_s"],
        "learned_only_vs_batched_alone": res["learned"]["indep_samples_per_s"] / hb["indep_samples_per_s"],
        "batched_heat_bath_vs_plain": hb["indep_samples_per_s"] / plain,
        "gain_per_T": gain_per_T,
        "max_gain_over_grid": max(g["mix_over_heat_bath"] for g in gain_per_T),
        "bz_scan": scan, "bz": bz,
        "acceptance_untrained": untrained[0] / max(untrained[1], 1),
        "modes": res,
        "ms_per_sweep": {"plain_fp64_heat_bath": plain_ms, "batched_heat_bath": structured_ms,
                         "learned": learned_ms},
        "training": {"configurations": int(chains * c["snapshots"]),
                     "windows": int(chains * 1024 * c["snapshots"]), "steps": c["train_steps"],
                     "rows_per_step": c["train_rows"], "window_samples": c["train_steps"] * c["train_rows"],
                     "seconds": t_train, "loss_first": float(losses[0]),
                     "loss_last100": float(np.mean(losses[-100:]))},
        "roofline": {"bound": "tensor", "achieved": achieved_tf, "peak": peak_tf, "unit": "TFLOP/s",
                     "frac": achieved_tf / peak_tf, "traffic": None, "kernel": "learned sweep (all kernels)",
                     "flop_per_sweep": flops_sweep,
                     "note": "network FLOPs of a learned sweep over its whole duration (GEMMs plus sampling "
                             "and acceptance kernels)"},
    }


def run_mc_only(args):
    """The Monte Carlo section alone (profiling and quick checks)."""
    import torch

    world, rank = dist_setup()
    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    from uppasd_gb300 import build as b

    b.build()
    peak, peak_kind = measured_peaks()
    with ClockSampler(int(os.environ.get("LOCAL_RANK", "0"))) as clk:
        mc = run_mc(args, world, rank, peak, peak_kind)
    if rank == 0:
        if not args.no_cpu_baseline:
            mc["cpu_baseline"] = mc_cpu_baseline()
        mc["clocks"] = clk.summary()
        print(json.dumps(mc), flush=True)


def _make_sim(lat, w, prec, seed, e0):
    from uppasd_gb300.simulation import GpuSimulation

    return GpuSimulation(lat, sdealgh=w["solver"], delta_t=w["dt"], damping=w["damping"], temperature=w["temp"],
                         seed=seed, emom=e0, precision=prec)


def _time_steps(sim, stream, steps, warmup, world):
    import torch

    sim.evolve(max(warmup, 1))  # warm-up; also captures and instantiates the step graph
    torch.cuda.synchronize()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    dist_barrier(world)
    torch.cuda.synchronize()
    ev0.record(stream)
    sim.evolve(steps)
    ev1.record(stream)
    torch.cuda.synchronize()
    dist_barrier(world)
    return dist_max(ev0.elapsed_time(ev1), world)


def _roofline(kt, nspin, s_bytes, ms_step, peak, peak_kind, traffic, traffic_source=None):
    bytes_pred = 6 * s_bytes * nspin
    bytes_corr = 9 * s_bytes * nspin
    if kt["correct_ms"] >= kt["predict_ms"]:
        dom, dom_ms, dom_bytes = "correct", kt["correct_ms"], bytes_corr
    else:
        dom, dom_ms, dom_bytes = "predict", kt["predict_ms"], bytes_pred
    achieved = dom_bytes / (dom_ms * 1e-3) / 1e9
    return {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
            "traffic": traffic, "traffic_source": traffic_source, "kernel": dom, "peak_source": peak_kind,
            "algorithmic_bytes_per_launch": dom_bytes,
            "step": {"achieved_GBs": (bytes_pred + bytes_corr) / (ms_step * 1e-3) / 1e9,
                     "frac": (bytes_pred + bytes_corr) / (ms_step * 1e-3) / 1e9 / peak,
                     "bytes_per_spin_step": 15 * s_bytes}}


PREC_NAMES = {0: "fp64-generic", 1: "fp32-gather/fp64-master", 2: "fp32-gather/double-single-master",
              3: "fp32-gather-lists/fp64-master", 4: "fp32-gather-lists/double-single-master"}
KERNEL_NAMES = {0: ("llg_predict", "llg_correct"), 1: ("stencil_tma_predict", "stencil_tma_correct"),
                2: ("stencil_tma_predict", "stencil_tma_correct"), 3: ("mixed_predict", "mixed_correct"),
                4: ("mixed_predict", "mixed_correct")}


def oracle_error(lat, w, prec, e0, stream, nsteps=20, seed=5):
    """Error of the timed path against the FP64 oracle on the benchmarked lattice: the
    same start, Philox seed and step count on the GPU (all ensembles) and in the
    oracle's parity build (ensemble 0, whose chain equals the GPU's ensemble 0);
    max and RMS per spin component after `nsteps` steps."""
    from oracle import pyoracle as po

    sim = _make_sim(lat, w, prec, seed, e0)
    sim.set_stream(stream.cuda_stream)
    sim.evolve(nsteps)
    g = sim.get_moments()[0]
    sim.close()
    o = po.Oracle(lat.with_ensembles(1), threads=os.cpu_count() or 1)
    o.set_moments(e0[:1])
    o.make_llg(w["solver"], w["dt"], w["damping"], w["temp"], 1.0, noise_mode=po.NOISE_PHILOX, seed=seed)
    for _ in range(nsteps):
        o.sd_step()
    d = g - o.emom[0]
    return {"steps": nsteps, "ensemble": 0, "max_abs": float(np.max(np.abs(d))),
            "rms": float(np.sqrt(np.mean(d * d))),
            "norm_dev_max": float(np.max(np.abs(np.linalg.norm(g, axis=-1) - 1.0))),
            "against": "oracle parity build (FP64, the Fortran's evaluation order), same start and Philox stream"}


# The configured FP64 runs benchmarked beside the headline: (workload, [(temperature, steps)])
FP64_CONFIGS = {
    "bcc16k": [(0.0, 1000), (300.0, 1000)],
    "square256": [(0.0, 20000), (50.0, 20000)],
}


def run_fp64_config(key, world, rank, stream, peak, peak_kind, cpu):
    """A configured FP64 run on the generic neighbour-list path: every phase of the
    configuration timed with CUDA events on the library's stream (device rate), then
    the same phases end to end through the C ABI with the state copied from and to
    pinned host memory, and the oracle's -O3 build timed on a sample of steps."""
    import torch

    w = WORKLOADS[key]
    lat = build_lattice(w)
    e0 = random_state(lat.mensemble, lat.natom, seed=17 + rank)
    nspin = lat.natom * lat.mensemble
    phases = FP64_CONFIGS[key]
    total = sum(n for _, n in phases)
    sim = _make_sim(lat, dict(w, temp=phases[0][0]), 0, 500 + rank, e0)
    sim.set_stream(stream.cuda_stream)
    sim.evolve(16)   # warm-up: step graph captured
    sim.put_moments(e0)
    torch.cuda.synchronize()
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
    dist_barrier(world)
    ev[0].record(stream)
    for T, n in phases:
        sim.set_temperature(T)
        sim.evolve(n)
    ev[1].record(stream)
    torch.cuda.synchronize()
    dist_barrier(world)
    ms = dist_max(ev[0].elapsed_time(ev[1]), world)
    kt = sim.time_kernels(20)
    # e2e: the whole configured run as one call sequence from pinned host memory
    host = torch.empty((lat.mensemble, lat.natom, 3), dtype=torch.float64, pin_memory=True).numpy()
    out = torch.empty((lat.mensemble, lat.natom, 3), dtype=torch.float64, pin_memory=True).numpy()
    host[...] = e0
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    sim.put_moments(host)
    for T, n in phases:
        sim.set_temperature(T)
        sim.evolve(n)
    sim.get_moments(out=out)
    torch.cuda.synchronize()
    e2e_s = dist_max(time.perf_counter() - t0, world)
    sim.close()
    value = nspin * total * world / (ms * 1e-3)
    roof = _roofline(kt, nspin, 8, ms / total, peak, peak_kind, None, None)
    roof["kernel"] = KERNEL_NAMES[0][1 if kt["correct_ms"] >= kt["predict_ms"] else 0]
    roof["note"] = (f"state {nspin * 24 * 4 / 1e6:.1f} MB: L2-resident (129 MB L2), so the fraction of the HBM "
                    "peak is a lower bound on the on-chip rate, not a DRAM figure")
    res = {"workload": key, "description": w["desc"], "spins": nspin, "phases": [list(p) for p in phases],
           "steps": total, "value": value, "unit": "atom-steps/s", "ms_per_step": ms / total, "dtype": "f64",
           "precision_path": PREC_NAMES[0], "l2_resident": True, "kernel_ms": kt, "roofline": roof,
           "e2e": {"value": nspin * total * world / e2e_s, "unit": "atom-steps/s",
                   "h2d_bytes_per_step": host.nbytes / total, "d2h_bytes_per_step": host.nbytes / total,
                   "note": "put_moments(pinned) + every phase (set_temperature, sd_run) + get_moments(pinned)"},
           "gpu_launches": total * 2 + -(-total // 16)}
    if cpu and rank == 0:
        res["cpu_baseline"] = cpu_baseline(dict(w, temp=phases[-1][0]), lat, e0, os.cpu_count() or 1, target_s=8.0)
    return res


# LLG with the dipole-dipole field on the FP64 path: (bcc cells per axis, do_dip)
DIPOLE_CASES = [(20, 1), (20, 3), (64, 3), (100, 3)]
DIPOLE_ALAT = 2.87e-10


def run_dipole(world, rank, stream, cpu):
    """Depondt steps (bcc ferromagnet J1=1.3 J2=0.7 mRy, 300 K, one ensemble) without and with
    the dipolar field, timed with CUDA events on the library's stream; the difference over
    two field evaluations per step is the field's cost.  The field of the 20^3 lattice is
    checked against the oracle's brute-force sum, which is also timed as the CPU figure."""
    import torch
    from uppasd_gb300 import lattice

    w = dict(solver=5, dt=1e-16, damping=0.1, temp=300.0)
    cases = []
    field_err = {}
    for L, mode in DIPOLE_CASES:
        lat = lattice.bcc(L, [1.3, 0.7], 2.2)
        e0 = random_state(1, lat.natom, seed=31)
        sim = _make_sim(lat, w, 0, 900 + rank, e0)
        sim.set_stream(stream.cuda_stream)
        n = 32 if lat.natom <= 20000 else 16
        ms0 = _time_steps(sim, stream, n, 3, world)
        sim.put_moments(e0)
        sim.set_dipole(mode, DIPOLE_ALAT)
        if L == 20:
            b = sim.get_fields()
            field_err[mode] = b
        ms1 = _time_steps(sim, stream, n, 3, world)
        sim.close()
        torch.cuda.synchronize()
        field_ms = (ms1 - ms0) / n / 2
        cases.append({"cells": L, "atoms": lat.natom, "do_dip": mode, "steps": n,
                      "ms_per_step_without": ms0 / n, "ms_per_step_with": ms1 / n,
                      "field_ms_per_evaluation": field_ms,
                      "atom_steps_per_s_with": lat.natom * n * world / (ms1 * 1e-3),
                      "field_evaluations_per_s": 1e3 / field_ms if field_ms > 0 else None})
    res = {"workload": "bcc ferromagnet with the dipole-dipole field (alat 2.87 A), FP64 path, Depondt, 300 K",
           "cases": cases, "launches_per_field": {"1": 1, "3": "memset + pad + 2 cuFFT + multiply + unpad"}}
    if rank == 0:
        from oracle import pyoracle as po

        lat = lattice.bcc(20, [1.3, 0.7], 2.2)
        e0 = random_state(1, lat.natom, seed=31)
        o = po.Oracle(lat, threads=os.cpu_count() or 1, fast=True, dipole_alat=DIPOLE_ALAT)
        o.set_moments(e0)
        ref_b, _ = o.field()
        # relative to the largest dipolar field component (the exchange field is ~100x larger)
        scale = float(np.max(np.abs(o.dipole_field())))
        res["field_error_vs_oracle"] = {str(m): float(np.max(np.abs(b - ref_b)) / scale) for m, b in field_err.items()}
        res["field_error_note"] = "max |B_gpu - B_oracle| over the full field / max |B_dip|, 20^3 bcc"
        if cpu:
            t0 = time.perf_counter()
            o.dipole_field()
            dt = time.perf_counter() - t0
            res["cpu_baseline"] = {"value": 1.0 / dt, "unit": "field evaluations/s", "cores": o.lib.orc_get_threads(),
                                   "kind": "port",
                                   "sample": "one brute-force dipolar field of the 20^3 bcc lattice (16,000 atoms), "
                                             "oracle built -O3, OpenMP over sites"}
    return res


def run_gb300(args, w):
    import torch

    world, rank = dist_setup()
    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    from uppasd_gb300 import build as b

    b.build()
    lat = build_lattice(w)
    e0 = random_state(lat.mensemble, lat.natom, seed=7 + rank)
    nspin = lat.natom * lat.mensemble
    # default: the double-single master (FP32 gather; the master and its renormalisation
    # in hi + lo FP32 pairs, ~48-bit), whose error against the FP64 oracle on this lattice
    # equals the FP64 master's (both ~1e-7 after 20 steps at T = 0, ~4e-6 at 300 K: the
    # FP32 gather sets it); the FP64 master is timed as a variant
    order = [int(args.precision)] if args.precision != "auto" else [2, 1, 0]
    sim, prec = None, None
    for p in order:
        try:
            sim = _make_sim(lat, w, p, 1000 + rank, e0)
            prec = p
            break
        except Exception as exc:
            print(f"# precision {p} unavailable ({exc})", file=sys.stderr)
    if sim is None:
        raise SystemExit("no GPU path could be set up")
    # a dedicated (non-default) stream: the library issues all work on it and the
    # CUDA events are recorded on the same stream
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    sim.set_stream(stream.cuda_stream)
    with ClockSampler(int(os.environ.get("LOCAL_RANK", "0"))) as clk:
        ms = _time_steps(sim, stream, args.steps, args.warmup, world)
    value = nspin * args.steps * world / (ms * 1e-3)
    graphs, rem = divmod(args.steps, 16)
    # a captured 16-step graph: predictor and corrector per step, on the structured path once
    # per ensemble half (two chains), and the step-counter kernel; the remaining steps the same
    chains = 2 if prec in (1, 2) and lat.mensemble >= 2 else 1
    launches = graphs * (16 * 2 * chains + 1) + rem * 2 * chains + (1 if rem else 0)
    kt = sim.time_kernels(3)
    peak, peak_kind = measured_peaks()
    kname = KERNEL_NAMES[prec][1 if kt["correct_ms"] >= kt["predict_ms"] else 0]
    tr, tr_src = profiled_traffic(f"{kname}:{args.workload}:p{prec}")
    roof = _roofline(kt, nspin, 8, ms / args.steps, peak, peak_kind, tr, tr_src)
    roof["kernel"] = kname
    # e2e through the C ABI with pinned host buffers
    inner = args.e2e_inner
    host = torch.empty((lat.mensemble, lat.natom, 3), dtype=torch.float64, pin_memory=True).numpy()
    host_out = torch.empty((lat.mensemble, lat.natom, 3), dtype=torch.float64, pin_memory=True).numpy()
    host[...] = e0
    # one sd_run_io call per block: the block's input copied in, `inner` steps, the result
    # copied out; on the structured path the ensemble groups' copies overlap the other
    # groups' steps
    rounds = max(1, args.e2e_rounds)

    def timed_blocks(block, reps=3):
        # three warm-up blocks, then the median of `reps` timings of `rounds` blocks each (a
        # single timing picks up the host's occasional multi-millisecond stalls)
        for _ in range(3):
            block()
        torch.cuda.synchronize()
        ts = []
        for _ in range(reps):
            t0 = time.perf_counter()
            for _ in range(rounds):
                block()
            torch.cuda.synchronize()
            ts.append(dist_max(time.perf_counter() - t0, world))
        return statistics.median(ts), ts

    e2e_s, e2e_reps = timed_blocks(lambda: sim.run_io(host, inner, host_out))
    e2e_val = nspin * inner * rounds * world / e2e_s
    # the same blocks as three calls in turn (put_moments, sd_run, get_moments)

    def seq_block():
        sim.put_moments(host)
        sim.evolve(inner)
        sim.get_moments(out=host_out)

    seq_s, seq_reps = timed_blocks(seq_block)
    e2e_seq = nspin * inner * rounds * world / seq_s
    variants = {}
    if not args.no_variants:
        # the same blocks of `inner` steps with the state handed to the host after each
        # block through sd_run_measured, whose copies overlap the next block
        blocks = max(1, args.e2e_rounds)
        got = []
        sim.sd_run_measured(inner, inner, lambda st, e, m: got.append(st))
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        sim.sd_run_measured(inner * blocks, inner, lambda st, e, m: None)
        torch.cuda.synchronize()
        meas_s = dist_max(time.perf_counter() - t0, world)
        variants["measured_run"] = {
            "value": nspin * inner * blocks * world / meas_s, "unit": "atom-steps/s",
            "steps_per_measurement": inner, "measurements": blocks,
            "d2h_bytes_per_measurement": 2 * host.nbytes,
            "note": "sd_run_measured: emom and emomM to the host after every block, copied on a second "
                    "stream while the next block runs; the host callback (here empty) runs while the "
                    "GPU works on the following block"}
    sim.close()
    if not args.no_variants and prec in (1, 2):
        other = 1 if prec == 2 else 2
        vname = "fp64_master" if other == 1 else "double_single_master"
        try:
            alt = _make_sim(lat, w, other, 1000 + rank, e0)
            alt.set_stream(stream.cuda_stream)
            ms2 = _time_steps(alt, stream, args.steps, args.warmup, world)
            kt2 = alt.time_kernels(3)
            alt.close()
            variants[vname] = {
                "value": nspin * args.steps * world / (ms2 * 1e-3), "ms_per_step": ms2 / args.steps,
                "kernel_ms": kt2, "roofline": _roofline(kt2, nspin, 8, ms2 / args.steps, peak, peak_kind, None)}
        except Exception as exc:
            variants[vname] = {"error": str(exc)}
        # the same lattice through the general neighbour-list path (precision 4: FP32 gather,
        # double-single master), with the chemical site classes the alloy's types allow
        try:
            gp = _make_sim(lat, w, 4, 1000 + rank, e0)
            gp.set_stream(stream.cuda_stream)
            info = gp.path_info()
            msg = _time_steps(gp, stream, 16, 4, world)
            ktg = gp.time_kernels(3)
            gp.close()
            variants["general_path_same_lattice"] = {
                "value": nspin * 16 * world / (msg * 1e-3), "ms_per_step": msg / 16, "kernel_ms": ktg,
                "site_classes": info["site_classes"], "chemical_types": info["chemical_types"],
                "note": "precision 4 over the caller's neighbour lists (no stencil, no shared-memory planes)"}
        except Exception as exc:
            variants["general_path_same_lattice"] = {"error": str(exc)}
        # general Hamiltonians (neighbour lists, DMI, anisotropy): FP64 path and FP32 gather
        # with the FP64 state (precision 3) or a double-single pair (precision 4) as master,
        # on the same lattice
        try:
            wg = WORKLOADS["square1024x4"]
            lg = build_lattice(wg)
            eg = random_state(lg.mensemble, lg.natom, seed=11 + rank)
            gen = {"workload": "square1024x4", "description": wg["desc"], "spins": lg.natom * lg.mensemble}
            for pg, key in ((0, "fp64"), (3, "fp32_gather_fp64_master"), (4, "fp32_gather_double_single_master")):
                sg = _make_sim(lg, wg, pg, 3000 + rank, eg)
                sg.set_stream(stream.cuda_stream)
                msg = _time_steps(sg, stream, 16, 4, world)
                # heat-bath sweeps of the same simulation (mc_run 'H')
                sg.relax("H", wg["temp"], 2)
                torch.cuda.synchronize()
                ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                ev0.record(stream)
                sg.relax("H", wg["temp"], 8)
                ev1.record(stream)
                torch.cuda.synchronize()
                msw = ev0.elapsed_time(ev1) / 8
                # Metropolis sweeps (mc_run 'M')
                sg.relax("M", wg["temp"], 2)
                torch.cuda.synchronize()
                ev0.record(stream)
                sg.relax("M", wg["temp"], 8)
                ev1.record(stream)
                torch.cuda.synchronize()
                mswm = ev0.elapsed_time(ev1) / 8
                sg.close()
                gen[key] = {"ms_per_step": msg / 16, "value": lg.natom * lg.mensemble * 16 * world / (msg * 1e-3),
                            "heat_bath_ms_per_sweep": msw, "metropolis_ms_per_sweep": mswm}
            variants["general_hamiltonian"] = gen
        except Exception as exc:
            variants["general_hamiltonian"] = {"error": str(exc)}
    oracle_err = None
    if not args.no_oracle_error:
        oracle_err = oracle_error(lat, w, prec, e0, stream)
    configs = {}
    if not args.no_configs:
        for key in FP64_CONFIGS:
            configs[key] = run_fp64_config(key, world, rank, stream, peak, peak_kind, not args.no_cpu_baseline)
    dipole = None
    if not args.no_dipole:
        dipole = run_dipole(world, rank, stream, not args.no_cpu_baseline)
    mc = None
    if not args.no_mc:
        mc = run_mc(args, world, rank, peak, peak_kind)
    c3 = None
    if not args.no_mc:
        c3 = run_c3(args, bf16_peak())
    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        cpu = cpu_baseline(w, lat, e0, os.cpu_count() or 1)
        if mc is not None:
            mc["cpu_baseline"] = mc_cpu_baseline()
    if rank != 0:
        return
    line = {
        "metric": "LLG atom-steps/s", "value": value, "unit": "atom-steps/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": {0: "f64", 1: "f32-gather/f64-state", 2: "f32-gather/double-single-state", 3: "f32-gather/f64-state",
                  4: "f32-gather/double-single-state"}[prec],
        "data": "synthetic (seeded lattice, species and spins)",
        "config": {"workload": args.workload, "description": w["desc"], "natom": lat.natom,
                   "ensembles": lat.mensemble, "spins": nspin,
                   "solver": "Depondt" if w["solver"] == 5 else "midpoint", "precision_path": PREC_NAMES[prec],
                   "l2": "inputs larger than L2 (no flush)", "parallelism": f"replicas x{world}"},
        "roofline": roof,
        "cpu_baseline": cpu,
        "e2e": {"value": e2e_val, "unit": "atom-steps/s", "h2d_bytes_per_step": host.nbytes / inner,
                "d2h_bytes_per_step": host.nbytes / inner, "inner_steps_per_call": inner,
                "bytes_per_call": {"h2d": host.nbytes, "d2h": host.nbytes},
                "note": "one sd_run_io call per block (emom in from pinned host memory, inner steps, emom out "
                        "to pinned host memory; the ensemble groups' copies overlap the other groups' steps); "
                        "the per-step bytes are one call's copies over its steps; after 3 warm-up blocks, the "
                        "median of 3 timings of e2e_rounds blocks each (all three in rep_seconds)",
                "blocks_per_timing": rounds, "rep_seconds": e2e_reps,
                "sequential_calls": {"value": e2e_seq, "unit": "atom-steps/s", "rep_seconds": seq_reps,
                                     "note": "put_moments + sd_run + get_moments in turn, same blocks, bytes "
                                             "and timing"}},
        "oracle_error": oracle_err,
        "configs": configs,
        "clocks": clk.summary(),
        "gpu_launches": launches + (mc["gpu_launches"] if mc else 0),
        "kernel_ms": kt,
        "variants": variants,
        "mc": mc,
        "mc_learned": c3,
        "dipole": dipole,
    }
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=40)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="alloy2m", choices=sorted(WORKLOADS))
    ap.add_argument("--precision", default="auto", choices=["auto", "0", "1", "2", "3", "4"])
    ap.add_argument("--e2e-inner", type=int, default=10)
    ap.add_argument("--e2e-rounds", type=int, default=10)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-variants", action="store_true",
                    help="skip the double-single master and general-Hamiltonian variant timings")
    ap.add_argument("--no-mc", action="store_true", help="skip the batched Monte Carlo section")
    ap.add_argument("--no-configs", action="store_true", help="skip the configured FP64 runs (bcc16k, square256)")
    ap.add_argument("--no-oracle-error", action="store_true", help="skip the FP64-oracle error of the headline")
    ap.add_argument("--no-dipole", action="store_true", help="skip the dipole-dipole field runs")
    ap.add_argument("--dipole-only", action="store_true", help="only the dipole-dipole field runs")
    ap.add_argument("--mc-only", action="store_true", help="only the batched Monte Carlo section")
    ap.add_argument("--c3-only", action="store_true", help="only the learned-proposal Monte Carlo section")
    ap.add_argument("--c3-profile", action="store_true",
                    help="two learned sweeps of the learned-proposal workload (kernel profiling)")
    ap.add_argument("--no-metropolis", action="store_true", help="skip the Metropolis replica table")
    ap.add_argument("--no-plain-tau", action="store_true", help="skip measuring the plain chain's tau_int")
    ap.add_argument("--plain-tau-sweeps", type=int, default=20000)
    ap.add_argument("--mc-therm", type=int, default=10000)
    ap.add_argument("--mc-meas", type=int, default=100000)
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    w = WORKLOADS[args.workload]
    if args.impl == "reference":
        run_reference(args, w)
    elif args.mc_only:
        run_mc_only(args)
    elif args.c3_profile:
        from uppasd_gb300 import build as b
        from uppasd_gb300 import lattice
        from uppasd_gb300.learned import LearnedProposal
        from uppasd_gb300.simulation import GpuSimulation

        b.build()
        c = C3
        temps, _ = _c3_temps()
        lat = lattice.square_dmi(c["L"], c["J"], c["D"], 0.0, 15.0, 1.0).with_ensembles(temps.size)
        sim = GpuSimulation(lat, emom=random_state(temps.size, lat.natom, seed=1), seed=2)
        prop = LearnedProposal(sim, c["L"], eta_scale=c["eta_scale"], seed=3)
        print(json.dumps({"learned_sweeps": 2, "accepted_proposed": prop.mix_temps(temps, 2, 0)[:2]}), flush=True)
    elif args.c3_only:
        import torch

        torch.cuda.set_device(0)
        from uppasd_gb300 import build as b

        b.build()
        print(json.dumps(run_c3(args, bf16_peak())), flush=True)
    elif args.dipole_only:
        import torch

        torch.cuda.set_device(0)
        from uppasd_gb300 import build as b

        b.build()
        stream = torch.cuda.Stream()
        print(json.dumps(run_dipole(1, 0, stream, not args.no_cpu_baseline)), flush=True)
    else:
        run_gb300(args, w)


if __name__ == "__main__":
    main()
