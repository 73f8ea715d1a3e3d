"""Benchmark of the GB300 event-time engine: events/s of batched Lennard-Jones ECMC chains.

Workload (one step = every chain advances ``--events`` events):
    4096 independent chains of N = 1024 Lennard-Jones atoms (epsilon = sigma = 1, density 0.8, beta = 1/1.2),
    periodic cube L = (1024 / 0.8)^(1/3), 12^3 cells with 3 neighbour layers (nearby cells cover 2.5 sigma),
    far field by the cell-bounding potential (InnerPointEstimator bounds, prefactor 1.5, 10 points per side),
    chain time 2 sigma with directions +x -> +y -> +z, seeded simple-cubic lattice plus +-0.05 sigma jitter.
    Mixed precision: FP32 screening of every candidate, FP64 re-solve of the near-winners (the event times are the
    FP64 ones).  The working set (positions, FP32 mirror, occupancy: ~210 MB) is larger than the 126 MB L2.

Arms:
    default            the GPU engine (value = device-timed events/s; e2e = through ChainBatch with host buffers)
    --impl reference   the CPU oracle (a C restatement of the reference's event loop) on all host threads

Other workloads (parity configurations measured beside the headline, not the headline):
    ``--workload coulomb``: 1024 replicas of 32 point charges (16 of each sign) with a hard core of radius 0.05 in the
    unit cube, beta = 1, merged-image Coulomb bounded by the inverse-power bound, cell veto on 8^3 cells.
    ``--workload water``:
    512 independent chains of 64 flexible water molecules (12.42 A box, 300 K, O-H and H-H harmonic bonds,
    Lennard-Jones on oxygen, merged-image Coulomb between molecules, inside-first lifting) with the molecular cells of
    the reference's water cell-veto configuration: root units in 8^3 cells with two neighbour layers, the
    summed-bounding Coulomb factor with the molecules of the nearby cells and the surplus molecules, the molecular
    cell veto (the reference's dipole Monte Carlo bound tables of this geometry, recorded with the trajectory
    tests/golden/water_n64_cell_veto.npz) and the cell-boundary events of the active root unit; mixed precision
    (FP32 screen of the Coulomb candidates and of the thinning, FP64 re-solve), one block per chain; seeded lattices
    of molecules in random orientations.
    ``--workload water_all_pairs``: the same water with a Coulomb factor for every pair of molecules.

Multi-GPU: one process per GPU under torchrun; every rank runs its own 4096 chains (independent replicas, no
collective on the data path), value = all ranks' events / max-over-ranks time.
"""
import argparse
import json
import math
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "events/s on 1 GB300, batched mixed-precision vs plain FP64 at <=1e-9 rel err"
from jellyfysh_gb300 import workloads as _workloads  # noqa: E402

WORKLOAD = _workloads.LENNARD_JONES
COULOMB_WORKLOAD = _workloads.COULOMB
WATER_ALL_PAIRS_WORKLOAD = dict(workload="water_chains_512x64_molecular_coulomb", chains=512, molecules=64,
                                system_length=12.42, temperature_kelvin=300.0, chain_time=2.0, lifting="inside_first",
                                coulomb="a summed-bounding factor for every pair of molecules")
WATER_WORKLOAD = dict(WATER_ALL_PAIRS_WORKLOAD, workload="water_chains_512x64_molecular_cell_veto", cells_per_side=8,
                      neighbor_layers=2,
                      coulomb="molecular cells: nearby and surplus factors, molecular cell veto, cell boundaries",
                      bound_tables="the reference's DipoleMonteCarloEstimator tables of this geometry (dipole "
                                   "separation 0.5, charge 0.82, prefactor 1.5, 1000 trials, empirical bound 30)")
WATER_BOUNDS = os.path.join(ROOT, "tests", "golden", "water_n64_cell_veto.npz")
NEAR_CELLS = (2 * WORKLOAD["neighbor_layers"] + 1) ** 3  # cells scanned for pair candidates per event
CPU_SECONDS = 10.0  # wall time of the CPU baseline sample
TIMING_STRIDE = 16  # event rounds between two rounds bracketed by per-kernel CUDA events
# DRAM traffic of the dominant kernel per event, from the ncu captures summarised under profiles/: the screening
# kernel of the Lennard-Jones workload in steady state (one-pass metrics with the caches left warm, mean of 20
# launches: 7.46 MB read + 3.26 MB written per launch of 4096 events), with the issue and pipe fractions of its full
# capture; the hard-sphere screening kernel (a cold-cache capture: 34.03 MB + 0.01 MB per launch of 4096 events); the
# Coulomb replica kernel (2.45 MB + 0.02 MB per launch of 1024 chains x 8 events) with its FP64 pipe's busy fraction
NCU = {
    "lennard_jones": {"traffic_per_event": (7.458240e6 + 3.261158e6) / 4096, "traffic_caches": "warm",
                      "issue_active": 0.524, "fma_pipe_active": 0.199, "alu_pipe_active": 0.411,
                      "fp64_pipe_active": 0.052},
    "hard_spheres": {"traffic_per_event": (34.032640e6 + 0.005888e6) / 4096, "traffic_caches": "cold",
                     "issue_active": 0.258, "fma_pipe_active": 0.076, "alu_pipe_active": 0.158},
    "coulomb": {"traffic_per_event": (2.450944e6 + 0.024576e6) / (1024 * 8), "traffic_caches": "cold",
                "issue_active": 0.102, "fp64_pipe_active": 0.356},
}
# the all-pairs water kernel (2.83 MB + 0.22 MB over 512 chains x 32 events) with the FP64 pipe's busy fraction of
# its capture; the water kernel with molecular cells in steady state (one-pass metrics with the caches left warm, mean
# of 3 launches of 512 chains x 32 events) with the FP64 pipe's busy fraction and the issue fraction of its full capture
WATER_NCU = {"water_all_pairs": {"traffic_per_event": (2.830080e6 + 0.221952e6) / (512 * 32),
                                 "fp64_pipe_active": 0.501},
             "water": {"traffic_per_event": (0.044800e6 + 0.059819e6) / (512 * 32), "traffic_caches": "warm",
                       "fp64_pipe_active": 0.223, "issue_active": 0.079}}
WATER_METRICS = {"water": "events/s on 1 GB300, batched water chains with the molecular cell veto",
                 "water_all_pairs": "events/s on 1 GB300, batched water chains, Coulomb factors of all pairs"}


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=100)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    p.add_argument("--events", type=int, default=128, help="events per chain and step")
    p.add_argument("--chains", type=int, default=WORKLOAD["chains"])
    p.add_argument("--block-warps", type=int, default=None, help="warps per screening block (0 = autotune)")
    p.add_argument("--groups", type=int, default=None, help="chain groups on streams of their own (0 = autotune)")
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--no-fp64", action="store_true")
    p.add_argument("--no-parity", action="store_true")
    p.add_argument("--fp64-events", type=int, default=16, help="events per chain of the batched FP64 comparison")
    p.add_argument("--workload", default="lennard_jones",
                   choices=["lennard_jones", "coulomb", "water", "water_all_pairs", "hard_spheres",
                            "hard_spheres_n64"])
    args = p.parse_args()
    if args.workload in ("hard_spheres", "hard_spheres_n64") and "--chains" not in sys.argv:
        args.chains = _workloads.BUILDERS[args.workload][0]["chains"]
    # launch shape: the batched hard-sphere workloads are tuned by the package's autotuner, the others take the
    # shape measured best for them (4 warps per block, one chain group)
    tuned_default = 0 if args.workload in ("hard_spheres", "hard_spheres_n64") else None
    if args.block_warps is None:
        args.block_warps = 4 if tuned_default is None else tuned_default
    if args.groups is None:
        args.groups = 1 if tuned_default is None else tuned_default
    if args.workload.startswith("water") and "--chains" not in sys.argv:
        args.chains = WATER_WORKLOAD["chains"]
    if args.workload == "water_all_pairs" and "--events" not in sys.argv:
        args.events = 32
    if args.workload == "water" and "--events" not in sys.argv:
        args.events = 128
    if args.workload == "coulomb" and "--chains" not in sys.argv:
        args.chains = COULOMB_WORKLOAD["chains"]
    return args


def workload_of(args):
    return _workloads.BUILDERS[args.workload][0]


METRICS = {"lennard_jones": METRIC, "coulomb": "events/s on 1 GB300, batched Coulomb replicas",
           "hard_spheres": "events/s on 1 GB300, batched hard-sphere chains of uneven N and density",
           "hard_spheres_n64": "events/s on 1 GB300, hard-sphere chains N=64"}
DATA = {"lennard_jones": "synthetic: seeded simple-cubic lattice + uniform jitter",
        "coulomb": "synthetic: seeded random sequential addition of +-1 charges with a hard core",
        "hard_spheres": "synthetic: seeded random sequential addition below packing fraction 0.35, jittered fcc "
                        "lattice above",
        "hard_spheres_n64": "synthetic: seeded random sequential addition"}
KERNELS = {"lennard_jones": "jf::screen_kernel<1, 2>", "hard_spheres": "jf::screen_kernel<0, 0>",
           "hard_spheres_n64": "jf::screen_kernel<0, 0>", "coulomb": "jf::coulomb_group_kernel<32>"}


def metric_of(args):
    return METRICS[args.workload]


def data_of(args):
    return DATA[args.workload]


def build_workload(args, chains, seed_offset=0):
    """(specs, positions, charges or None, box length) of the selected atomic workload."""
    from jellyfysh_gb300 import workloads
    return workloads.BUILDERS[args.workload][1](chains, seed_offset)


class ClockSampler:
    """nvidia-smi samples of the SM clock and throttle reasons during the timed region."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.QUERY,
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, sm_max, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                sm_max = max(sm_max, float(parts[2]))
            except ValueError:
                continue
            for name, flag in zip(names, parts[5:9]):
                if flag.lower() == "active":
                    reasons.add(name)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": sm_max, "reasons": sorted(reasons),
                "samples": len(sm)}


def measured_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as handle:
            data = json.load(handle)
        return float(data["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def cpu_chains(threads, pool, seed_offset=99, args=None):
    """One oracle chain (C restatement of the reference's event loop) of the workload per host thread."""
    import oracle
    specs, positions, charges, _ = build_workload(args, threads, seed_offset=seed_offset)
    potentials = {"hard_sphere": oracle.POT_HARD_SPHERE, "lennard_jones": oracle.POT_LENNARD_JONES,
                  "coulomb": oracle.POT_COULOMB}
    fars = {"none": oracle.FAR_NONE, "cell_veto": oracle.FAR_CELL_VETO, "cell_bounding": oracle.FAR_CELL_BOUNDING}
    systems = []
    for c, spec in enumerate(specs):
        systems.append(oracle.make_system(
            n=spec.n, system_length=spec.system_length, cells_per_side=spec.cells_per_side,
            neighbor_layers=spec.neighbor_layers, max_occupants=1, beta=spec.beta, chain_time=spec.chain_time,
            initial_active=spec.initial_active, initial_direction=spec.initial_direction,
            potential=potentials[spec.potential], far=fars[spec.far], hs_radius=spec.hs_radius,
            lj_prefactor=spec.lj_prefactor, lj_sigma=spec.lj_sigma, coulomb_prefactor=spec.coulomb_prefactor,
            bound_prefactor=spec.bound_prefactor, ewald_alpha=spec.ewald_alpha, fourier_cutoff=spec.fourier_cutoff,
            position_cutoff=spec.position_cutoff, estimator_points=spec.estimator_points,
            estimator_prefactor=spec.estimator_prefactor, rng_key=oracle.chain_key(99, c)))
    return list(pool.map(lambda i: oracle.Chain(systems[i], positions[i], None if charges is None else charges[i]),
                         range(len(systems))))


def cpu_run(pool, chains, seconds, chunk=500):
    """Every thread advances its chain in chunks of events until `seconds` have passed; returns (events, wall s)."""
    def work(chain):
        done, start = 0, time.perf_counter()
        while time.perf_counter() - start < seconds:
            done += chain.run(chunk, record=False)
        return done
    start = time.perf_counter()
    done = sum(pool.map(work, chains))
    return done, time.perf_counter() - start


PARITY_CHAINS = 16  # chains of the benchmarked batch replayed in the FP64 path
PARITY_ORACLE_EVENTS = 1000  # events per chain compared with the oracle


def time_exact(batch, stream, device, events, first, count, per_chain=False):
    """events/s of the plain FP64 path (mode "exact") on chains [first, first + count) of the batch, all in one
    launch or one launch per chain, device-timed with CUDA events on the launching stream."""
    import torch
    torch.cuda.synchronize(device)
    before = batch.state()
    begin = torch.cuda.Event(enable_timing=True)
    end = torch.cuda.Event(enable_timing=True)
    begin.record(stream)
    if per_chain:
        for c in range(first, first + count):
            batch.run(events, mode="exact", first=c, count=1, sync=False)
    else:
        batch.run(events, mode="exact", first=first, count=count, sync=False)
    end.record(stream)
    torch.cuda.synchronize(device)
    batch.check_status()
    ms = begin.elapsed_time(end)
    after = batch.state()
    done = int(after["events"][first:first + count].sum() - before["events"][first:first + count].sum())
    return {"value": done / (ms / 1000.0), "unit": "events/s", "events": done, "ms": ms,
            "sample": "%d chains x %d events, %s" % (count, events, "one launch per chain" if per_chain
                                                      else "one launch, one warp per chain")}


def parity_record(args, specs, positions, charges, batch, events, state, final_positions):
    """The first PARITY_CHAINS chains of the benchmarked batch, replayed from their initial state in the plain FP64
    path for the `events` events each ran in the mixed path: positions and chain states compared bit for bit.  Then
    the same chains' first PARITY_ORACLE_EVENTS events in the mixed path against the oracle (test infrastructure,
    the checker): discrete outcomes exactly, event times by their largest relative difference."""
    import concurrent.futures
    import dataclasses
    import oracle
    from jellyfysh_gb300 import ChainBatch
    p = min(PARITY_CHAINS, len(specs))
    sub_specs = [dataclasses.replace(specs[c], rng_key=batch.keys[c]) for c in range(p)]
    sub_charges = None if charges is None else charges[:p]
    replay = ChainBatch(sub_specs, positions[:p], sub_charges, device=str(batch.device))
    replay.run(events, mode="exact")
    replay.check_status()
    got = replay.state()
    fields = ("time_q", "time_r", "eoc_q", "eoc_r", "events", "active", "direction", "n_surplus", "occ_cell",
              "lift_sum", "liftings")
    state_equal = all(np.array_equal(got[f], state[f]) for f in fields)
    positions_equal = all(np.array_equal(replay.positions(c), final_positions[c]) for c in range(p))
    replay.close()
    # the mixed path against the oracle, event by event
    logged = ChainBatch(sub_specs, positions[:p], sub_charges, device=str(batch.device))
    n_log = PARITY_ORACLE_EVENTS
    logs = logged.run(n_log, mode="mixed", log_capacity=n_log)
    logged.check_status()
    logged.close()
    chains = cpu_chains_for(sub_specs, positions[:p], sub_charges)
    with concurrent.futures.ThreadPoolExecutor(max_workers=min(p, host_threads())) as pool:
        expected = list(pool.map(lambda chain: chain.run(n_log), chains))
    mismatches, max_rel = 0, 0.0
    for c in range(p):
        discrete = np.zeros(n_log, dtype=bool)
        for field in ("kind", "moved", "target", "new_active", "new_direction", "accepted"):
            discrete |= logs[c][field] != expected[c][field]
        mismatches += int(discrete.sum())
        t_gpu = logs[c]["time_q"] + logs[c]["time_r"]
        t_cpu = expected[c]["time_q"] + expected[c]["time_r"]
        max_rel = max(max_rel, float(np.max(np.abs(t_gpu - t_cpu) / np.maximum(np.abs(t_cpu), 1e-300))))
    return {"replayed_chains": p, "events_per_chain": events, "replay": "FP64 path from the initial state",
            "state_bitwise_equal": bool(state_equal), "positions_bitwise_equal": bool(positions_equal),
            "oracle_chains": p, "oracle_events_per_chain": n_log, "discrete_mismatches": mismatches,
            "max_rel_time_err": max_rel, "bound": 1e-9}


def cpu_chains_for(specs, positions, charges):
    """Oracle chains (the C restatement of the reference's event loop) of the given chain parameters."""
    import oracle
    potentials = {"hard_sphere": oracle.POT_HARD_SPHERE, "lennard_jones": oracle.POT_LENNARD_JONES,
                  "coulomb": oracle.POT_COULOMB}
    fars = {"none": oracle.FAR_NONE, "cell_veto": oracle.FAR_CELL_VETO, "cell_bounding": oracle.FAR_CELL_BOUNDING}
    chains = []
    for c, spec in enumerate(specs):
        system = oracle.make_system(
            n=spec.n, system_length=spec.system_length, cells_per_side=spec.cells_per_side,
            neighbor_layers=spec.neighbor_layers, max_occupants=spec.max_occupants, beta=spec.beta,
            chain_time=spec.chain_time, initial_active=spec.initial_active, initial_direction=spec.initial_direction,
            potential=potentials[spec.potential], far=fars[spec.far], hs_radius=spec.hs_radius,
            lj_prefactor=spec.lj_prefactor, lj_sigma=spec.lj_sigma, coulomb_prefactor=spec.coulomb_prefactor,
            bound_prefactor=spec.bound_prefactor, ewald_alpha=spec.ewald_alpha, fourier_cutoff=spec.fourier_cutoff,
            position_cutoff=spec.position_cutoff, estimator_points=spec.estimator_points,
            estimator_prefactor=spec.estimator_prefactor, rng_key=spec.rng_key)
        chains.append(oracle.Chain(system, positions[c], None if charges is None else charges[c]))
    return chains


def host_threads():
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:
        return os.cpu_count() or 1


def reference_arm(args):
    """The reference's CPU path on all host threads: the oracle's restatement of its event loop, one chain per
    thread (the reference is single-threaded), each step a bounded time sample of the same workload."""
    import concurrent.futures
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    threads = host_threads()
    # each step a bounded sample: the timed steps take about 90 s of wall time in total
    seconds = max(0.2, min(3.0, 90.0 / max(args.steps, 1)))
    with concurrent.futures.ThreadPoolExecutor(max_workers=threads) as pool:
        chains = cpu_chains(threads, pool, args=args)
        for _ in range(args.warmup):
            cpu_run(pool, chains, 0.5)
        total_events, total_time = 0, 0.0
        for _ in range(args.steps):
            done, elapsed = cpu_run(pool, chains, seconds)
            total_events += done
            total_time += elapsed
    value = total_events / total_time
    config = dict(workload_of(args))
    config["sample"] = "%d chains (one per host thread) x %.0f s of events per step" % (threads, seconds)
    line = {"impl": "reference", "metric": metric_of(args), "value": value, "unit": "events/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000.0 * total_time / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": data_of(args), "config": config,
            "cpu_baseline": {"value": value, "unit": "events/s", "cores": threads, "kind": "port",
                             "per_core": value / threads, "sample": config["sample"]},
            "e2e": {"value": value, "unit": "events/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def drop_in_costs(args, calls=200, pairs=30):
    """Wall time of one call of the drop-in layer from Python: a GpuLennardJonesPotential.displacement (one pair, one
    launch with its copies, as the reference's TwoLeafUnitEventHandler makes it per pair and event) and a
    GpuNeighbourhoodEventHandler solve of `pairs` pairs (one launch per event for the whole neighbourhood)."""
    from jellyfysh_gb300.plugin.potential._common import earliest
    from jellyfysh_gb300.plugin.potential.gpu_lennard_jones_potential import GpuLennardJonesPotential
    potential = GpuLennardJonesPotential(1.0, 1.0)
    rng = np.random.default_rng(5)
    separations = rng.uniform(-2.5, 2.5, (pairs, 3))
    separations = separations[np.linalg.norm(separations, axis=1) > 0.9]
    changes = rng.exponential(1.2, len(separations))
    for _ in range(10):
        potential.displacement([1.0, 0.0, 0.0], list(separations[0]), float(changes[0]))
        earliest(potential, [1.0, 0.0, 0.0], separations, None, changes)
    start = time.perf_counter()
    for k in range(calls):
        potential.displacement([1.0, 0.0, 0.0], list(separations[k % len(separations)]),
                               float(changes[k % len(separations)]))
    single = (time.perf_counter() - start) / calls
    start = time.perf_counter()
    for _ in range(calls):
        earliest(potential, [1.0, 0.0, 0.0], separations, None, changes)
    batched = (time.perf_counter() - start) / calls
    return {"potential_call_us": single * 1e6, "neighbourhood_call_us": batched * 1e6,
            "neighbourhood_pairs": int(len(separations)),
            "note": "wall time per call from Python, one GPU launch and its host copies each; the reference's "
                    "CPython LennardJonesPotential.displacement takes about 7 us a pair"}


def gpu_arm(args):
    import torch
    import torch.distributed as dist
    from jellyfysh_gb300 import ChainBatch, replicas
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    if world > 1:
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    device = torch.device("cuda", local)
    specs, positions, charges, length = build_workload(args, args.chains, seed_offset=rank)
    batch = ChainBatch(specs, positions, charges, seed=1000 + rank, device="cuda:%d" % local)
    stream = torch.cuda.current_stream(device)
    tuned = None
    if args.block_warps and args.groups:
        warps, groups = args.block_warps, args.groups
    else:
        from jellyfysh_gb300 import autotune
        (warps, groups), timings = autotune.tune(batch, 8, (args.block_warps,) if args.block_warps else autotune.WARPS,
                                                 (args.groups,) if args.groups else autotune.GROUPS)
        tuned = {"%dx%d" % shape: seconds * 1e6 for shape, seconds in timings.items()}
    batch.set_block_warps(warps)
    batch.set_groups(groups)
    # per-kernel CUDA events on the launching streams stay on through the warm-up and the timed region, around
    # every TIMING_STRIDE-th event round
    batch.set_timing(True, stride=TIMING_STRIDE)
    for _ in range(args.warmup):
        batch.run(args.events, mode="mixed")
    batch.check_status()
    batch.kernel_times(reset=True)
    state0 = batch.state()
    launches0 = batch.launch_count()
    if world > 1:
        dist.barrier()
    torch.cuda.synchronize(device)
    with ClockSampler(local) as clocks:
        begin = torch.cuda.Event(enable_timing=True)
        finish = torch.cuda.Event(enable_timing=True)
        begin.record(stream)
        for s in range(args.steps):
            batch.run(args.events, mode="mixed", sync=False)
        finish.record(stream)
        torch.cuda.synchronize(device)
    elapsed_ms = begin.elapsed_time(finish)
    launches = batch.launch_count() - launches0
    kernel_times = batch.kernel_times(reset=True)
    batch.set_timing(False)
    batch.check_status()
    state1 = batch.state()
    events_done = int(state1["events"].sum() - state0["events"].sum())
    candidates = int(state1["candidates"].sum() - state0["candidates"].sum())
    refined = int(state1["refined"].sum() - state0["refined"].sum())
    fallbacks = int(state1["refine_fallbacks"].sum() - state0["refine_fallbacks"].sum())
    lookups = int(state1["far_lookups"].sum() - state0["far_lookups"].sum())
    # whole job: events of all ranks over the longest rank's timed region
    _, total_ms, value = replicas.timed_throughput(events_done, elapsed_ms, device)
    # the state the parity record replays to: every chain has run (warmup + steps) x events events
    events_before_e2e = int(state1["events"][0])
    bench_state = state1[:PARITY_CHAINS].copy()
    bench_pos = [batch.positions(c) for c in range(min(PARITY_CHAINS, batch.n_chains))]

    # end to end through ChainBatch with host buffers: every step uploads the chain state from pinned host memory
    # (the FP32 mirror is rebuilt on the device from the uploaded positions), runs, and reads positions and chain
    # states back.  Double-buffered as a host pipeline would be: two batches of the same chains take the steps in
    # turn, each batch's copies on a stream of its own, so that one batch's copies overlap the other's run; the runs
    # themselves stay on one stream, one after the other, as in the device-timed region.
    pair = [batch, ChainBatch(specs, positions, charges, seed=1000 + rank, device="cuda:%d" % local)]
    pair[1].set_block_warps(warps)
    pair[1].set_groups(groups)
    pair[1].run(args.events, mode="mixed")  # captures its graphs outside the timed region
    pair[1].check_status()
    host = [t.cpu().pin_memory() for t in batch.input_tensors()]
    host_results = [[b.positions_dev.cpu().pin_memory(), b.state_dev.cpu().pin_memory()] for b in pair]
    h2d = sum(t.numel() * t.element_size() for t in host)
    d2h = sum(t.numel() * t.element_size() for t in host_results[0])
    e2e_steps = max(2, args.steps // 2)
    copy_streams = [torch.cuda.Stream(device), torch.cuda.Stream(device)]
    torch.cuda.synchronize(device)
    e_begin = torch.cuda.Event(enable_timing=True)
    e_end = torch.cuda.Event(enable_timing=True)
    e_begin.record(stream)
    for copy in copy_streams:
        copy.wait_event(e_begin)
    for step in range(e2e_steps):
        x = step % 2
        b, copy = pair[x], copy_streams[x]
        with torch.cuda.stream(copy):  # after this batch's previous read-back, in stream order
            for dst, src in zip(b.input_tensors(), host):
                dst.copy_(src, non_blocking=True)
        uploaded = torch.cuda.Event()
        uploaded.record(copy)
        stream.wait_event(uploaded)
        b.refresh_mirror()
        b.run(args.events, mode="mixed", sync=False)
        ran = torch.cuda.Event()
        ran.record(stream)
        copy.wait_event(ran)
        with torch.cuda.stream(copy):
            for dst, src in zip(host_results[x], (b.positions_dev, b.state_dev)):
                dst.copy_(src, non_blocking=True)
    for copy in copy_streams:
        done = torch.cuda.Event()
        done.record(copy)
        stream.wait_event(done)
    e_end.record(stream)
    torch.cuda.synchronize(device)
    for b in pair:
        b.check_status()
    e2e_ms = e_begin.elapsed_time(e_end)
    e2e_events = e2e_steps * sum(1 for _ in specs) * args.events
    e2e_value = e2e_events / (e2e_ms / 1000.0)
    pair[1].close()
    del pair

    # the precision comparison: the plain FP64 path over the same batch (every chain, one warp per chain, one
    # launch), and one chain per launch as the unbatched FP64 path; device-timed on the launching stream
    fp64 = fp64_batched = None
    if not args.no_fp64:
        fp64_batched = time_exact(batch, stream, device, events=args.fp64_events, first=0, count=batch.n_chains)
        fp64_batched["speedup_of_batched_mixed"] = value / fp64_batched["value"]
        fp64 = time_exact(batch, stream, device, events=16, first=0, count=64, per_chain=True)
        fp64["speedup_of_batched_mixed"] = value / fp64["value"]
        fp64["sample"] = "64 chains x 16 events, one launch per chain"

    # the drop-in layer's per-call cost, where the reference's own mediator calls it once per pair or per event
    drop_in = drop_in_costs(args) if args.workload == "lennard_jones" and not args.no_fp64 else None

    # parity of the benchmarked run: chains of the batch replayed from their initial state in the FP64 path for the
    # events they ran in the mixed path, bit for bit, and the event log of their first events against the oracle
    parity = None
    if not args.no_parity:
        parity = parity_record(args, specs, positions, charges, batch, events_before_e2e, bench_state, bench_pos)

    if rank != 0:
        if world > 1:
            dist.barrier()
            dist.destroy_process_group()
        return

    # roofline of the screening kernel, which reads the neighbourhood: algorithmic bytes per event (occupancy of the
    # nearby cells, FP32 position and identifier of every pair candidate, active position write, cell index and time)
    # times the events of one launch, over its mean CUDA-event duration on its stream in the timed region
    # (Coulomb replicas run the warp-per-chain FP64 kernel, one launch per step reading FP64 positions and charges)
    coulomb = args.workload == "coulomb"
    dominant = kernel_times["chains" if coulomb else "screen"]
    dominant_launches = max(dominant["launches"], 1)  # the timed launches
    # two kernels per event round and chain group (mixed rounds: screening and settle); one launch per step (FP64
    # kernel)
    events_per_launch = events_done / max(launches if coulomb else launches / 2, 1)
    nb = candidates / max(events_done, 1)
    # nearby cells scanned per event, averaged over the chains (each chain commits one event per round)
    near_cells = float(np.mean([_workloads.near_cells(spec) for spec in specs]))
    bytes_per_event = 4 * near_cells + (24 + 8 + 4) * nb + 32 if coulomb else 4 * near_cells + 12 * nb + 4 * nb + 32
    dominant_s = dominant["ms"] / dominant_launches / 1000.0
    achieved = bytes_per_event * events_per_launch / dominant_s / 1e9
    peak, peak_kind = measured_peaks()
    ncu = NCU.get(args.workload)
    traffic = ncu["traffic_per_event"] * events_per_launch if ncu else None
    total_kernel_ms = sum(v["ms"] for v in kernel_times.values()) or 1.0
    kernels = {name: {"launches": v["launches"], "ms_per_launch": v["ms"] / max(v["launches"], 1),
                      "share": v["ms"] / total_kernel_ms}
               for name, v in kernel_times.items() if v["launches"]}
    roofline = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                "traffic": traffic, "peak_source": peak_kind,
                "kernel": KERNELS[args.workload],
                "bytes_per_event": bytes_per_event, "events_per_launch": events_per_launch,
                "ms_per_launch": dominant_s * 1000.0, "neighbours_per_event": nb,
                "refined_per_event": refined / max(events_done, 1), "fallback_events": fallbacks,
                "far_lookups_per_event": lookups / max(events_done, 1),
                "kernels": kernels}
    if ncu:
        roofline["ncu"] = dict(ncu, source="profiles/ (committed ncu summaries of this kernel and workload)")
    cpu = None
    if not args.no_cpu_baseline and world == 1:
        import concurrent.futures
        threads = host_threads()
        with concurrent.futures.ThreadPoolExecutor(max_workers=threads) as pool:
            chains = cpu_chains(threads, pool, args=args)
            cpu_run(pool, chains, 0.5)
            done, elapsed = cpu_run(pool, chains, CPU_SECONDS)
        cpu = {"value": done / elapsed, "unit": "events/s", "cores": threads, "kind": "port",
               "per_core": done / elapsed / threads,
               "sample": "%d chains of the workload (one per host thread), %d events in %.1f s"
                         % (threads, done, elapsed)}
    config = dict(workload_of(args))
    config.update(chains=args.chains, events_per_chain_per_step=args.events, block_warps=warps, chain_groups=groups,
                  autotuned_us_per_round=tuned,
                  l2="inputs larger than L2 (working set %.0f MB)" % (sum(
                      t.numel() * t.element_size() for t in batch.state_tensors()) / 1e6),
                  parallelism="replicas" if world > 1 else "single GPU")
    line = {"metric": metric_of(args), "value": value, "unit": "events/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64",
            "data": data_of(args), "config": config,
            "e2e": {"value": e2e_value, "unit": "events/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                    "pipelining": "two batches take the steps in turn; each batch's copies overlap the other's run"},
            "roofline": roofline, "cpu_baseline": cpu, "gpu_launches": launches, "clocks": clocks.summary(),
            "fp64_batched": fp64_batched, "fp64_one_chain_per_launch": fp64, "parity": parity,
            "drop_in": drop_in}
    print(json.dumps(line))
    if world > 1:
        dist.barrier()
        dist.destroy_process_group()
    batch.close()


def water_model_and_positions(chains, seed):
    from jellyfysh_gb300 import water
    model = water.WaterModel(molecules=WATER_WORKLOAD["molecules"], system_length=WATER_WORKLOAD["system_length"],
                             chain_time=WATER_WORKLOAD["chain_time"], lifting=WATER_WORKLOAD["lifting"])
    return model, water.lattice_positions(model, chains, seed)


def water_cells(args):
    """The molecular cells of the water workload (None for the all-pairs water): 8^3 cells, two neighbour layers,
    the reference estimator's bound tables of this geometry."""
    if args.workload != "water":
        return None
    from jellyfysh_gb300 import water
    data = np.load(WATER_BOUNDS)
    return water.WaterCells(WATER_WORKLOAD["cells_per_side"], WATER_WORKLOAD["neighbor_layers"],
                            data["bounds_upper"], data["bounds_lower"])


def water_cpu_chains(threads, pool, cells, seed=99):
    """One oracle water chain of the water workload per host thread."""
    import oracle
    from jellyfysh_gb300 import systems
    model, positions = water_model_and_positions(threads, seed)
    spec = dict(vars(model))

    def make(c):
        extra = {}
        if cells is not None:
            roots = systems.water_roots(positions[c], model.system_length)
            extra["cells"] = (cells.cells_per_side, cells.neighbor_layers, roots, cells.bounds_upper,
                              cells.bounds_lower)
        return oracle.Water(oracle.make_water_system(spec, oracle.chain_key(seed, c)), positions[c], model.charges(),
                            **extra)
    return list(pool.map(make, range(threads)))


def water_state_tensors(batch):
    """The device tensors that hold a water batch's chains (uploaded and read back by the end-to-end steps)."""
    tensors = [batch.positions_dev, batch.state_dev]
    if batch.cells is not None:
        tensors += [batch.roots_dev, batch.occupancy_dev, batch.surplus_dev, batch.cell_state_dev]
    return tensors


def water_gpu_arm(args):
    """events/s of the water workload: device-timed, and end to end with host buffers."""
    import torch
    from jellyfysh_gb300 import replicas, water
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    device = torch.device("cuda", local)
    cells = water_cells(args)
    workload = WATER_WORKLOAD if cells is not None else WATER_ALL_PAIRS_WORKLOAD
    model, positions = water_model_and_positions(args.chains, 1000 + rank)
    batch = water.WaterBatch(model, positions, seed=1000 + rank, first_chain=0, cells=cells)
    stream = torch.cuda.current_stream(device)
    for _ in range(args.warmup):
        batch.run(args.events)
    batch.check_status()
    before = batch.states()
    if world > 1:
        dist.barrier()
    torch.cuda.synchronize(device)
    with ClockSampler(local) as clocks:
        begin = torch.cuda.Event(enable_timing=True)
        finish = torch.cuda.Event(enable_timing=True)
        begin.record(stream)
        for _ in range(args.steps):
            batch.run(args.events)
        finish.record(stream)
        torch.cuda.synchronize(device)
    elapsed_ms = begin.elapsed_time(finish)
    batch.check_status()
    after = batch.states()
    events_done = int(after["events"].sum() - before["events"].sum())
    _, total_ms, value = replicas.timed_throughput(events_done, elapsed_ms, device)
    # end to end: every step uploads positions and chain states from pinned host memory, runs, and reads both back;
    # double-buffered as for the atomic chains (two batches take the steps in turn, each batch's copies on a stream of
    # its own, the runs one after the other on one stream)
    pair = [batch, water.WaterBatch(model, positions, seed=1000 + rank, first_chain=0, cells=cells)]
    host_in = [t.cpu().pin_memory() for t in water_state_tensors(batch)]
    host_out = [[t.clone().pin_memory() for t in host_in] for _ in pair]
    h2d = sum(t.numel() * t.element_size() for t in host_in)
    e2e_steps = max(2, args.steps // 2)
    copy_streams = [torch.cuda.Stream(device), torch.cuda.Stream(device)]
    torch.cuda.synchronize(device)
    e_begin = torch.cuda.Event(enable_timing=True)
    e_end = torch.cuda.Event(enable_timing=True)
    e_begin.record(stream)
    for copy in copy_streams:
        copy.wait_event(e_begin)
    for step in range(e2e_steps):
        x = step % 2
        b, copy = pair[x], copy_streams[x]
        with torch.cuda.stream(copy):  # after this batch's previous read-back, in stream order
            for target, source in zip(water_state_tensors(b), host_in):
                target.copy_(source, non_blocking=True)
        uploaded = torch.cuda.Event()
        uploaded.record(copy)
        stream.wait_event(uploaded)
        b.run(args.events)
        ran = torch.cuda.Event()
        ran.record(stream)
        copy.wait_event(ran)
        with torch.cuda.stream(copy):
            for target, source in zip(host_out[x], water_state_tensors(b)):
                target.copy_(source, non_blocking=True)
    for copy in copy_streams:
        done = torch.cuda.Event()
        done.record(copy)
        stream.wait_event(done)
    e_end.record(stream)
    torch.cuda.synchronize(device)
    for b in pair:
        b.check_status()
    e2e_value = e2e_steps * args.chains * args.events / (e_begin.elapsed_time(e_end) / 1000.0)
    pair[1].close()
    del pair
    if rank != 0:
        if world > 1:
            dist.barrier()
            dist.destroy_process_group()
        return
    counts = {key: int(after[key].sum() - before[key].sum())
              for key in ("composite_events", "composite_accepted", "bond_events", "lj_events", "eoc_events",
                          "thinning_exact", "refined_items")}
    units = 3 * model.molecules
    if cells is None:
        # algorithmic bytes per event: every unit's position and charge read once (the candidates of all molecule
        # pairs), the active unit's position written, the chain state read and written
        bytes_per_event = units * (24 + 8) + 24 + 2 * 96
    else:
        cell_counts = batch.cell_states()
        counts.update(boundary_events=int(cell_counts["boundary_events"].sum()),
                      veto_events=int(cell_counts["veto_events"].sum()),
                      veto_targets=int(cell_counts["veto_targets"].sum()))
        # algorithmic bytes per event: the occupancy words of the nearby cells and the surplus words, the positions
        # and charges of the target molecules' units (the nearby cells hold 125/512 of the other molecules on
        # average), the oxygens and bond partners of the pair items (created at a third of the events: the active
        # unit is an oxygen a third of the time), the active leaf and root written, the chain and cell states read
        # and written
        n_near = (2 * cells.neighbor_layers + 1) ** 3
        targets = (model.molecules - 1) * n_near / cells.cells
        bytes_per_event = (4 * (n_near + model.molecules) + 3 * targets * (24 + 8) +
                           ((model.molecules - 1) / 3.0 + 2) * 24 + 2 * 24 + 2 * (96 + 128))
    step_s = elapsed_ms / args.steps / 1000.0
    achieved = bytes_per_event * args.chains * args.events / step_s / 1e9
    peak, peak_kind = measured_peaks()
    cpu = None
    if not args.no_cpu_baseline and world == 1:
        import concurrent.futures
        threads = host_threads()
        with concurrent.futures.ThreadPoolExecutor(max_workers=threads) as pool:
            chains = water_cpu_chains(threads, pool, cells)
            cpu_run(pool, chains, 0.5)
            done, seconds = cpu_run(pool, chains, CPU_SECONDS)
        cpu = {"value": done / seconds, "unit": "events/s", "cores": threads, "kind": "port",
               "per_core": done / seconds / threads,
               "sample": "%d water chains (one per host thread), %d events in %.1f s" % (threads, done, seconds)}
    config = dict(workload)
    config.update(chains=args.chains, events_per_chain_per_step=args.events, mode=model.mode,
                  l2="working set %.1f MB (in L2): the step is FP64-latency-bound, not HBM-bound" % (
                      sum(t.numel() * t.element_size() for t in water_state_tensors(batch)) / 1e6),
                  event_counts=counts, parallelism="replicas" if world > 1 else "single GPU")
    line = {"metric": WATER_METRICS[args.workload], "value": value, "unit": "events/s",
            "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": total_ms / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64",
            "data": "synthetic: seeded lattices of water molecules in random orientations", "config": config,
            "e2e": {"value": e2e_value, "unit": "events/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": h2d,
                    "pipelining": "two batches take the steps in turn; each batch's copies overlap the other's run"},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak,
                         "traffic": WATER_NCU[args.workload]["traffic_per_event"] * args.chains * args.events,
                         "peak_source": peak_kind,
                         "kernel": "jf::water_cells_kernel" if cells is not None else "jf::water_kernel",
                         "bytes_per_event": bytes_per_event,
                         "fp64_pipe_active": WATER_NCU[args.workload]["fp64_pipe_active"],
                         "ncu": WATER_NCU[args.workload]},
            "cpu_baseline": cpu, "gpu_launches": args.steps, "clocks": clocks.summary()}
    print(json.dumps(line))
    if world > 1:
        dist.barrier()
        dist.destroy_process_group()
    batch.close()


def water_reference_arm(args):
    """The oracle's water loop on all host threads, one chain per thread, bounded time samples."""
    import concurrent.futures
    if int(os.environ.get("RANK", "0")) != 0:
        return
    threads = host_threads()
    seconds = max(0.2, min(3.0, 90.0 / max(args.steps, 1)))
    cells = water_cells(args)
    with concurrent.futures.ThreadPoolExecutor(max_workers=threads) as pool:
        chains = water_cpu_chains(threads, pool, cells)
        for _ in range(args.warmup):
            cpu_run(pool, chains, 0.5)
        total_events, total_time = 0, 0.0
        for _ in range(args.steps):
            done, elapsed = cpu_run(pool, chains, seconds)
            total_events += done
            total_time += elapsed
    value = total_events / total_time
    config = dict(WATER_WORKLOAD if cells is not None else WATER_ALL_PAIRS_WORKLOAD)
    config["sample"] = "%d water chains (one per host thread) x %.0f s of events per step" % (threads, seconds)
    print(json.dumps({"impl": "reference", "metric": WATER_METRICS[args.workload],
                      "value": value, "unit": "events/s", "n_gpus": args.gpus, "steps": args.steps,
                      "warmup": args.warmup, "ms_per_step": 1000.0 * total_time / args.steps,
                      "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64",
                      "data": "synthetic: seeded lattices of water molecules in random orientations",
                      "config": config,
                      "cpu_baseline": {"value": value, "unit": "events/s", "cores": threads, "kind": "port",
                                       "per_core": value / threads, "sample": config["sample"]},
                      "e2e": {"value": value, "unit": "events/s", "h2d_bytes_per_step": 0,
                              "d2h_bytes_per_step": 0}}))


def main():
    args = parse()
    if args.workload.startswith("water"):
        if args.impl == "reference":
            water_reference_arm(args)
        else:
            water_gpu_arm(args)
    elif args.impl == "reference":
        reference_arm(args)
    else:
        gpu_arm(args)


if __name__ == "__main__":
    main()
