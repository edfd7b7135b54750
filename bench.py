"""Converged NDDO SCF solves/s on GB300.

Workload (one step): 256 replicas of a (H2O)32 cluster (96 atoms, 192 basis
functions, 128 doubly occupied MOs) under AM1, each replica displaced by
N(0, 0.05 A) per coordinate; every replica is SCF-solved to RMS density 1e-8
with density DIIS (the reference's SCF block: max_iter 500, damping 0,
5 DIIS vectors, start 0.1, end 0.0).  One step = integrals + SCF + energies +
Mulliken charges of all 256 molecules.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--precision fp64|mixed]
  python bench.py --impl reference ...      # the CPU restatement on the host cores

The headline line is the FP64 path (every eigensolve, Fock build, density,
DIIS and energy in FP64), as the workload specifies; the mixed-precision
path is measured on the same molecules and reported under the "mixed" key.

Prints one JSON line.  Under torchrun (N > 1) each rank solves its own 256
replicas (weak scaling) and rank 0 reports the max-over-ranks time.
"""
from __future__ import annotations

import argparse
import ctypes
import json
import math
import multiprocessing as mp
import os
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "converged SCF solves/s at |ΔE|≤1e-6 Eh, batched vs plain on GB300; p50/p99 latency"
SCF = dict(max_iter=500, rms_density=1e-8, damping_thresh=1.0, damping_weight=0.0, diis_num_error_vect=5,
           diis_start_error=0.1, diis_end_error=0.0)
N_MOL = 256


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--precision", default=None, choices=["fp64", "mixed"],
                    help="default: mixed for the uneven alkanes (their precision ramp), fp64 otherwise")
    ap.add_argument("--no-mixed", action="store_true", help="skip the mixed-precision measurement")
    ap.add_argument("--nmol", type=int, default=N_MOL)
    ap.add_argument("--dipole", default="on", choices=["on", "off"],
                    help="dipole moment after convergence (on: as the reference's DoSCF)")
    ap.add_argument("--cpu-sample", type=int, default=N_MOL,
                    help="molecules in the CPU-baseline sample (default: the whole step)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--plain-sample", type=int, default=16,
                    help="molecules solved one at a time on the plain FP64 path (0 = skip)")
    ap.add_argument("--workload", default="water32",
                    choices=["water32", "serving", "alkanes", "octane", "water512", "md"],
                    help="water32: 256 x (H2O)32 AM1 batched (the headline); serving: Poisson stream of PM3 "
                         "requests through the continuous-batching server; alkanes: uneven batch of random "
                         "alkanes with the precision ramp; octane: the plain one-molecule path")
    ap.add_argument("--rates", default="100,300,1000,3000,10000,20000", help="serving: arrival rates (req/s)")
    ap.add_argument("--requests", type=int, default=400, help="serving: requests per rate")
    ap.add_argument("--hbm-gb", type=float, default=96.0, help="serving: HBM budget of the server")
    ap.add_argument("--max-basis", type=int, default=1024, help="serving: largest basis accepted")
    ap.add_argument("--alkanes", type=int, default=4096, help="alkanes: molecules in the uneven batch")
    ap.add_argument("--repeats", type=int, default=200, help="octane: timed solves")
    ap.add_argument("--max-iter", type=int, default=500, help="water512: SCF iteration cap")
    a = ap.parse_args()
    if a.precision is None:
        a.precision = "mixed" if a.workload == "alkanes" else "fp64"
    return a


def workload(rank: int, nmol: int):
    from molds_gb300 import workloads as W
    base = W.water_cluster(shape=(4, 4, 2), spacing=2.9, jitter=0.2, seed=2)
    return W.water_replicas(base, nmol, sigma=0.05, seed0=1000 + rank * nmol)


# ---------------------------------------------------------------------------
# CPU restatement timed on the host cores (process pool, one thread each)
# ---------------------------------------------------------------------------
def _cpu_worker(args):
    Z, xyz = args
    from oracle import oracle as O
    mol = O.make_molecule("am1", Z, xyz)
    r = O.scf(mol, O.SCFParams(**SCF))
    return r.energy, r.iterations


def cpu_solve(mols, cores: int):
    os.environ.update(OMP_NUM_THREADS="1", OPENBLAS_NUM_THREADS="1", MKL_NUM_THREADS="1")
    from oracle import oracle as O
    O.build()
    ctx = mp.get_context("spawn")
    t0 = time.perf_counter()
    with ctx.Pool(cores) as pool:
        out = pool.map(_cpu_worker, [(m.Z, m.xyz) for m in mols], chunksize=1)
    dt = time.perf_counter() - t0
    return dt, out


def host_cores() -> int:
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:
        return os.cpu_count() or 1


def profiled_traffic(kernel_class: str):
    """DRAM bytes per launch of a kernel class from the committed ncu summaries
    (a line 'traffic_per_launch <class> <bytes> <workload>' in profiles/*.md)."""
    pdir = os.path.join(ROOT, "profiles")
    if not os.path.isdir(pdir):
        return None, None
    for fn in sorted(os.listdir(pdir)):
        if not fn.endswith(".md"):
            continue
        for line in open(os.path.join(pdir, fn)):
            f = line.strip().strip("`").split()
            if len(f) >= 3 and f[0] == "traffic_per_launch" and f[1] == kernel_class:
                return float(f[2]), "profiles/" + fn
    return None, None


def percentile(xs, q):
    xs = sorted(xs)
    if not xs:
        return None
    k = (len(xs) - 1) * q / 100.0
    lo, hi = int(math.floor(k)), int(math.ceil(k))
    return xs[lo] + (xs[hi] - xs[lo]) * (k - lo)


# ---------------------------------------------------------------------------
class Clocks:
    """nvidia-smi samples during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.lines = []
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                                          "-lms", "200", "-i", str(self.device)], stdout=subprocess.PIPE,
                                         stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except (FileNotFoundError, OSError):
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.t.join(timeout=2)
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        sm.sort()
        med = sm[len(sm) // 2] if sm else None
        return {"sm_mhz": med, "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sm)}


# ---------------------------------------------------------------------------
def dist_setup():
    """Rank, world size and local rank from the torchrun environment; the
    process group is NCCL on GPUs (gloo where CUDA is absent: the host-side
    sharding logic is tested that way on CPU)."""
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch
        import torch.distributed as dist
        if torch.cuda.is_available():
            torch.cuda.set_device(local)
            dist.init_process_group("nccl")
        else:
            dist.init_process_group("gloo")
        return rank, world, local, dist
    return rank, world, local, None


def barrier_sync(dist):
    import torch
    if dist is not None:
        dist.barrier()
    if torch.cuda.is_available():
        torch.cuda.synchronize()


def max_over_ranks(x, dist):
    if dist is None:
        return x
    import torch
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([x], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def aggregate_throughput(world: int, per_rank_units: int, max_ms_per_step: float) -> float:
    """Whole-job units/s: every rank's units over the slowest rank's step time."""
    return world * per_rank_units / (max_ms_per_step * 1e-3)


def run_reference(args):
    rank, world, local, dist = dist_setup()
    if rank != 0:
        if dist is not None:
            dist.barrier()
        return
    mols = workload(0, args.nmol)
    sample = mols[:args.cpu_sample]
    cores = host_cores()
    for _ in range(args.warmup):
        cpu_solve(sample[:max(1, min(len(sample), cores))], cores)
    total_t, total_n = 0.0, 0
    for _ in range(args.steps):
        dt, out = cpu_solve(sample, cores)
        total_t += dt
        total_n += len(sample)
    value = total_n / total_t
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": "solves/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * total_t / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic: seeded (H2O)32 replicas (no public dataset is named for this path)",
            "config": {"workload": f"{args.nmol} replicas of (H2O)32 per GPU, AM1, batched SCF to RMS 1e-8"
                                   if len(sample) == args.nmol else
                                   f"{len(sample)} of the {args.nmol} (H2O)32 AM1 replicas per step (bounded sample)",
                       "molecules_per_step": len(sample), "molecules_per_gpu": args.nmol, "atoms": 96,
                       "basis_functions": 192, "occupied": 128, "precision": "fp64", "theory": "AM1", "scf": SCF},
            "cpu_baseline": {"value": value, "unit": "solves/s", "cores": cores, "kind": "port",
                             "sample": f"{len(sample)} (H2O)32 AM1 replicas per step, spawn pool of {cores} "
                                       "single-thread processes (oracle: C integrals/Fock + LAPACK dsyevd/dsysv)"},
            "e2e": {"value": value, "unit": "solves/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    if dist is not None:
        dist.barrier()


def run_ours(args):
    rank, world, local, dist = dist_setup()
    import numpy as np
    import molds_gb300 as M
    from molds_gb300 import build
    build.build()
    import torch
    torch.cuda.set_device(local)
    ctx = M.Context(local)
    mols = workload(rank, args.nmol)
    params = M.SCFParams(**SCF, precision=args.precision, dipole=args.dipole == "on")
    batch = M.ResidentBatch("am1", mols, context=ctx)

    batch.profile(True)            # the per-class event pool is created during the warm-up
    for _ in range(args.warmup):
        batch.run(params)
    res_w, q_w = batch.results()

    # ---- timed region: K steps on device-resident inputs ------------------
    clocks = Clocks(local)
    batch.profile(True)            # resets the accumulated times, keeps the event pool
    l0 = batch.launch_count()
    barrier_sync(dist)
    clocks.start()
    batch.timer(0)
    for _ in range(args.steps):
        batch.run(params)
    batch.timer(1)
    ms = batch.timer(2)
    barrier_sync(dist)
    clk = clocks.stop()
    launches = batch.launch_count() - l0
    kt = batch.kernel_times()
    batch.profile(False)
    res, charges = batch.results()

    # ---- the same steps as the library runs them without the profiler:
    # each SCF iteration replayed from a captured CUDA graph --------------
    g0, gl0 = batch.graph_launch_count(), batch.launch_count()
    batch.run(params)                          # captures
    barrier_sync(dist)
    batch.timer(0)
    for _ in range(args.steps):
        batch.run(params)
    batch.timer(1)
    ms_graph = max_over_ranks(batch.timer(2), dist) / args.steps
    barrier_sync(dist)
    graphs = {"value": aggregate_throughput(world, args.nmol, ms_graph), "unit": "solves/s", "ms_per_step": ms_graph,
              "graph_launches_per_step": (batch.graph_launch_count() - g0) / (args.steps + 1),
              "kernels_per_step": (batch.launch_count() - gl0) / (args.steps + 1),
              "note": "profiler off: every SCF iteration of a molecule group is one replay of a captured CUDA graph; "
                      "the headline value above is measured with per-launch CUDA events (no graphs)"}
    ms_max = max_over_ranks(ms, dist)
    per_step_ms = ms_max / args.steps
    value = aggregate_throughput(world, args.nmol, per_step_ms)

    # ---- end to end through the public batched call (host buffers) --------
    e2e_steps = max(1, min(args.steps, 3))
    Z = np.concatenate([m.Z for m in mols])
    # the context keeps the batch between calls with the same molecules: after
    # the first call a step uploads the coordinates only
    h2d = int(Z.size * 3 * 8)
    d2h = int(args.nmol * ctypes.sizeof(M.ScfResultC) + Z.size * 8)
    M.batch_scf("am1", mols, params, context=ctx)       # warm-up: allocates the context's batch
    barrier_sync(dist)
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        r_e2e, q_e2e = M.batch_scf("am1", mols, params, context=ctx)
    e2e_s = max_over_ranks((time.perf_counter() - t0) / e2e_steps, dist)
    e2e_value = world * args.nmol / e2e_s

    its = [r["iterations"] for r in res]
    acc = {"all_converged": all(r["status"] == M.STATUS_CONVERGED for r in res),
           "iterations_min_max": [min(its), max(its)]}

    # ---- the mixed-precision path on the same molecules (untimed above) -----
    mixed = None
    if not args.no_mixed and args.precision == "fp64":
        nP = min(32, args.nmol)
        P64 = [batch.density(i, 192) for i in range(nP)]
        pm = M.SCFParams(**SCF, precision="mixed", dipole=args.dipole == "on")
        for _ in range(args.warmup):
            batch.run(pm)
        barrier_sync(dist)
        batch.timer(0)
        for _ in range(args.steps):
            batch.run(pm)
        batch.timer(1)
        ms_mixed = max_over_ranks(batch.timer(2), dist) / args.steps
        barrier_sync(dist)
        res_m, q_m = batch.results()
        de = np.array([abs(a["energy"] - b["energy"]) for a, b in zip(res_m, res)])
        dq = [float(np.max(np.abs(a - b))) for a, b in zip(q_m, charges)]
        dP = [float(np.max(np.abs(batch.density(i, 192) - P64[i]))) for i in range(nP)]
        its_m = [r["iterations"] for r in res_m]
        mixed = {"value": aggregate_throughput(world, args.nmol, ms_mixed), "unit": "solves/s",
                 "ms_per_step": ms_mixed, "dtype": "fp32+fp64",
                 "what": "FP32 phase (back-transformation of the density's eigenvectors on the CUDA cores in FP32, "
                         "density on the tensor cores, 3xTF32) until the DIIS error is below 1e-4, then FP64; "
                         "integrals, Fock build, eigensolve (tridiagonalisation, bisection, inverse iteration), DIIS, "
                         "core-core and energies always FP64",
                 "max_abs_dE_vs_fp64_gpu_Eh": float(de.max()),
                 "p50_abs_dE_vs_fp64_gpu_Eh": float(np.percentile(de, 50)),
                 "p99_abs_dE_vs_fp64_gpu_Eh": float(np.percentile(de, 99)),
                 "max_abs_dq_vs_fp64_gpu": max(dq),
                 "max_abs_dP_vs_fp64_gpu": max(dP), "dP_sample": nP,
                 "all_converged": all(r["status"] == M.STATUS_CONVERGED for r in res_m),
                 "iterations_min_max": [min(its_m), max(its_m)],
                 "vs_fp64": (ms_max / args.steps) / ms_mixed}

    # ---- plain path: one molecule at a time, FP64, ElectronicStructure ------
    plain = None
    if rank == 0 and args.plain_sample > 0:
        es = M.ElectronicStructure("am1", M.SCFParams(**SCF, precision="fp64", dipole=args.dipole == "on"),
                                   context=ctx)
        lat = []
        for i, m in enumerate(mols[:args.plain_sample] * 2):
            t0 = time.perf_counter()
            es.SetMolecule(m)
            es.DoSCF(True)
            es.GetMullikenCharges()
            if i >= args.plain_sample:          # first pass warms up
                lat.append(time.perf_counter() - t0)
        tot = sum(lat)
        plain = {"value": len(lat) / tot, "unit": "solves/s", "p50_ms": 1e3 * percentile(lat, 50),
                 "p99_ms": 1e3 * percentile(lat, 99), "sample": f"first {len(lat)} replicas, each SetMolecule + "
                 "DoSCF + Mulliken through ElectronicStructure (nddo_set_molecule / nddo_scf), FP64 throughout, "
                 "host wall clock"}

    # ---- roofline of the dominant kernel -----------------------------------
    # the roofline's kernel: the single kernel with the largest share of the
    # serialised device time (the ncu launch list under profiles/); on the
    # FP64 Householder path that is the tridiagonalisation, otherwise the
    # class with the most event time
    dom = max(kt, key=lambda k: kt[k]["ms"])
    if kt.get("tridiagonalisation", {}).get("launches", 0) > 0:
        dom = "tridiagonalisation"
    d = kt[dom]
    compute_bound = dom in ("jacobi_eigensolver", "warm_start_transform", "basis_orthonormalise", "density",
                            "fp64_refinement", "tridiagonalisation", "tridiagonal_eigenvectors")
    roof = None
    if rank == 0 and d["launches"] > 0 and d["ms"] > 0:
        avg_ms = d["ms"] / d["launches"]
        per_launch = d["work"] / d["launches"]
        if compute_bound:
            prec = "fp64" if (dom in ("fp64_refinement", "tridiagonalisation", "tridiagonal_eigenvectors")
                              or args.precision == "fp64") else "fp32"
            peak = ctx.fma_peak_tflops(prec)
            achieved = per_launch / (avg_ms * 1e-3) / 1e12
            traffic, tsrc = profiled_traffic(dom)
            work_note = {"tridiagonalisation": "work = (4/3) N^3 flops per molecule, the tridiagonalisation share "
                                               "of the (10/3) N^3 eigensolver convention",
                         "jacobi_eigensolver": "work by the (10/3) N^3 eigensolver convention"}.get(dom, "algorithmic flops")
            roof = {"bound": f"{prec}-cuda-core", "kernel": dom, "achieved": achieved, "peak": peak,
                    "unit": "TFLOP/s", "frac": achieved / peak, "traffic": traffic, "traffic_source": tsrc,
                    "peak_source": f"measured live: dependent-FMA loop on every SM ({prec}); MEASURED_PEAKS.json "
                                   "holds only HBM copy and bf16 tensor peaks",
                    "work_per_launch": per_launch, "avg_launch_ms": avg_ms, "launches": d["launches"],
                    "note": work_note + "; launch durations are CUDA events on each group's stream and overlap the "
                            "other groups' kernels, so achieved is a lower bound"}
        else:
            peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json"))) if os.path.exists(
                os.path.join(ROOT, "MEASURED_PEAKS.json")) else {"hbm_gbs": 6800.0}
            achieved = per_launch / (avg_ms * 1e-3) / 1e9
            traffic, tsrc = profiled_traffic(dom)
            roof = {"bound": "hbm", "kernel": dom, "achieved": achieved, "peak": peaks["hbm_gbs"], "unit": "GB/s",
                    "frac": achieved / peaks["hbm_gbs"], "traffic": traffic, "traffic_source": tsrc,
                    "peak_source": "MEASURED_PEAKS.json hbm_gbs",
                    "work_per_launch": per_launch, "avg_launch_ms": avg_ms, "launches": d["launches"]}

    # ---- CPU baseline: the oracle on the host cores, bounded sample --------
    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        sample = mols[:args.cpu_sample]
        cores = host_cores()
        dt, out = cpu_solve(sample, cores)
        cpu = {"value": len(sample) / dt, "unit": "solves/s", "cores": cores, "kind": "port",
               "sample": f"first {len(sample)} of the {args.nmol} replicas, spawn pool of {cores} single-thread "
                         "processes running the oracle (C integrals/Fock + LAPACK dsyevd/dsysv via scipy)"}
        acc["max_abs_dE_vs_cpu_oracle_Eh"] = max(abs(e - r["energy"]) for (e, _), r in zip(out, res))

    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": "solves/s", "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": per_step_ms, "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None,
                "dtype": "fp32+fp64" if args.precision == "mixed" else "f64",
                "data": "synthetic: seeded (H2O)32 replicas (no public dataset is named for this path)",
                "config": {"workload": f"{args.nmol} replicas of (H2O)32 per GPU, AM1, batched SCF to RMS 1e-8",
                           "molecules_per_gpu": args.nmol, "atoms": 96, "basis_functions": 192, "occupied": 128,
                           "precision": args.precision, "scf": SCF, "dipole": args.dipole == "on",
                           "l2": f"inputs larger than L2: {batch.device_bytes() / 1e9:.2f} GB resident per GPU",
                           "parallelism": f"replicas x{world} (molecules sharded, no collective)"},
                "e2e": {"value": e2e_value, "unit": "solves/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                        "call": "nddo_batch_scf with host arrays (coordinate upload, integrals, SCF, energies, "
                                "results and charges download); device arrays reused from the previous call"},
                "gpu_launches": launches,
                "latency_ms": {"batched_step": per_step_ms,
                               "note": "every molecule of a step completes within the step"},
                "plain_fp64_one_at_a_time": plain,
                "batched_vs_plain": (value / plain["value"]) if plain else None,
                "e2e_vs_plain": (e2e_value / plain["value"]) if plain else None,
                "roofline": roof,
                "kernels_ms": {k: round(v["ms"], 3) for k, v in kt.items()},
                "cpu_baseline": cpu,
                "clocks": clk,
                "accuracy": acc,
                "graphs": graphs,
                "mixed": mixed}
        print(json.dumps(line), flush=True)
    batch.close()
    if dist is not None:
        dist.barrier()
        dist.destroy_process_group()



# ---------------------------------------------------------------------------
# Uneven batch: random alkanes CnH2n+2, n uniform 3..60, PM3, precision ramp
# ---------------------------------------------------------------------------
def _gen_alkane(j):
    from molds_gb300 import workloads as W
    m = W.random_alkane(3_000_000 + j)
    return m.Z, m.xyz


def _cpu_worker_pm3(args):
    Z, xyz = args
    from oracle import oracle as O
    mol = O.make_molecule("pm3", Z, xyz)
    try:
        r = O.scf(mol, O.SCFParams(**SCF))
        return r.energy, r.iterations, True
    except O.NotConverged:
        return None, SCF["max_iter"], False


def run_alkanes(args):
    """All molecules of this rank in one device-resident batch; a step =
    integrals + SCF + energies of all of them.  The uneven workload's precision
    ramp is `--precision mixed` (FP32 back-transformation and density until the
    DIIS error drops below 1e-4, FP64 eigensolve throughout); each molecule's
    |dE| and max|dP| against the FP64 GPU path of the same batch.  Under
    torchrun the molecules are split over the ranks by predicted cost
    (molds_gb300/sharding.py)."""
    import numpy as np
    from molds_gb300.inputfile import Molecule
    from molds_gb300 import sharding
    from molds_gb300 import workloads as W
    os.environ.update(OMP_NUM_THREADS="1", OPENBLAS_NUM_THREADS="1")
    rank, world, local, dist = dist_setup()
    # every rank computes the same cost-based assignment (N^3 per molecule,
    # longest first onto the least-loaded rank) and builds its own share
    n_all = np.array([6 * W.alkane_carbons(3_000_000 + j) + 2 for j in range(args.alkanes)])
    shards = sharding.shard_by_cost(sharding.predicted_cost(n_all), world)
    mine = shards[rank]
    cores = host_cores()
    t0 = time.perf_counter()
    with mp.get_context("spawn").Pool(cores) as pool:      # before any CUDA call
        gen = pool.map(_gen_alkane, mine, chunksize=16)
    t_gen = time.perf_counter() - t0
    mols = [Molecule(Z, xyz) for Z, xyz in gen]
    import molds_gb300 as M
    from molds_gb300 import build
    build.build()
    if world > 1:
        import torch
        torch.cuda.set_device(local)
    ctx = M.Context(local)
    nao = np.array([int(sum(4 if z > 1 else 1 for z in m.Z)) for m in mols])
    steps = args.steps if args.steps != 10 else 2
    warm = args.warmup if args.warmup != 3 else 1
    params = M.SCFParams(**SCF, precision=args.precision, dipole=args.dipole == "on")
    batch = M.ResidentBatch("pm3", mols, context=ctx)
    batch.profile(True)
    for _ in range(warm):
        batch.run(params)
    clocks = Clocks(0)
    clocks.start()
    batch.profile(True)
    l0 = batch.launch_count()
    barrier_sync(dist)
    batch.timer(0)
    for _ in range(steps):
        batch.run(params)
    batch.timer(1)
    ms = max_over_ranks(batch.timer(2) / steps, dist)
    barrier_sync(dist)
    clk = clocks.stop()
    launches = (batch.launch_count() - l0) // steps
    kt = batch.kernel_times()
    batch.profile(False)
    res, q = batch.results()
    ref = M.ResidentBatch("pm3", mols, context=ctx)
    ref.run(M.SCFParams(**SCF, precision="fp64"))
    res64, q64 = ref.results()
    conv = np.array([r["status"] == M.STATUS_CONVERGED for r in res])
    conv64 = np.array([r["status"] == M.STATUS_CONVERGED for r in res64])
    both = np.nonzero(conv & conv64)[0]
    de = np.array([abs(res[i]["energy"] - res64[i]["energy"]) for i in both])
    rng = np.random.default_rng(0)
    samp = rng.choice(both, size=min(256, both.size), replace=False) if both.size else []
    dp = np.array([float(np.max(np.abs(batch.density(i, nao[i]) - ref.density(i, nao[i])))) for i in samp])
    its = np.array([r["iterations"] for r in res])
    n_conv = int(conv.sum())
    if dist is not None:                     # converged solves of the whole job over the slowest rank's time
        import torch
        t = torch.tensor([n_conv], dtype=torch.float64, device="cuda")
        dist.all_reduce(t)
        n_conv = int(t.item())
    value = n_conv / (ms * 1e-3)
    # CPU baseline: the oracle on a bounded sample, all host cores
    cpu = None
    if not args.no_cpu_baseline:
        sample = mols[:min(args.cpu_sample, 32)]
        t1 = time.perf_counter()
        with mp.get_context("spawn").Pool(cores) as pool:
            out = pool.map(_cpu_worker_pm3, [(m.Z, m.xyz) for m in sample], chunksize=1)
        dt = time.perf_counter() - t1
        ok = sum(1 for o in out if o[2])
        cpu = {"value": ok / dt, "unit": "converged solves/s", "cores": cores, "kind": "port",
               "sample": f"first {len(sample)} alkanes, spawn pool of {cores} single-thread processes running the "
                         f"oracle; {ok} converged in {dt:.1f} s",
               "max_abs_dE_gpu_vs_cpu_Eh": max((abs(o[0] - res[i]["energy"]) for i, o in enumerate(out)
                                                if o[2] and res[i]["status"] == M.STATUS_CONVERGED), default=None)}
    line = {"metric": "converged SCF solves/s, uneven batch of random alkanes with the precision ramp",
            "value": value, "unit": "solves/s", "n_gpus": world, "steps": steps, "warmup": warm, "ms_per_step": ms,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "fp32+fp64" if args.precision == "mixed" else "f64",
            "data": f"synthetic: {args.alkanes} seeded random alkanes (seed 3e6 + j), generated in {t_gen:.1f} s",
            "config": {"workload": f"{args.alkanes} alkanes CnH2n+2, n uniform 3..60, PM3, one batch",
                       "basis_min_median_max": [int(nao.min()), int(np.median(nao)), int(nao.max())],
                       "precision": args.precision, "scf": SCF, "dipole": args.dipole == "on",
                       "l2": f"inputs larger than L2: {batch.device_bytes() / 1e9:.2f} GB resident"},
            "gpu_launches": launches, "kernels_ms": {k: round(v["ms"] / steps, 3) for k, v in kt.items()},
            "convergence": {"converged": int(conv.sum()), "fp64_converged": int(conv64.sum()),
                            "not_converged_both": int((~conv & ~conv64).sum()),
                            "iterations_median": float(np.median(its)), "iterations_max": int(its.max())},
            "accuracy": {"molecules_compared": int(both.size),
                         "max_abs_dE_vs_fp64_gpu_Eh": float(de.max()) if de.size else None,
                         "abs_dE_percentiles_Eh": {str(q): float(np.percentile(de, q)) for q in (50, 90, 99, 100)}
                         if de.size else None,
                         "abs_dE_histogram_log10_Eh": {f"<=1e{e}": int(np.sum(de <= 10.0 ** e))
                                                       for e in (-14, -12, -10, -8, -6)} if de.size else None,
                         "max_abs_dP_sample": float(dp.max()) if dp.size else None,
                         "abs_dP_percentiles": {str(q): float(np.percentile(dp, q)) for q in (50, 90, 99, 100)}
                         if dp.size else None, "dP_sample": int(dp.size)},
            "sharding": {"ranks": world, "molecules_this_rank": len(mine),
                         "predicted_cost_imbalance": float(sharding.shard_loads(sharding.predicted_cost(n_all), shards).max()
                                                           / max(1e-30, sharding.predicted_cost(n_all).sum() / world))},
            "cpu_baseline": cpu, "clocks": clk}
    if rank == 0:
        print(json.dumps(line), flush=True)
    batch.close()
    ref.close()
    if dist is not None:
        dist.barrier()
        dist.destroy_process_group()


# ---------------------------------------------------------------------------
# Plain path: one PM3 n-octane solve at a time, FP64
# ---------------------------------------------------------------------------
def run_octane(args):
    import numpy as np
    import molds_gb300 as M
    from molds_gb300 import build, workloads as W
    build.build()
    ctx = M.Context(0)
    mol = W.octane()
    es = M.ElectronicStructure("pm3", M.SCFParams(**SCF, precision="fp64"), context=ctx)
    for _ in range(5):
        es.SetMolecule(mol)
        es.DoSCF()
    lat = []
    for _ in range(args.repeats):
        t0 = time.perf_counter()
        es.SetMolecule(mol)
        es.DoSCF()
        q = es.GetMullikenCharges()
        lat.append(time.perf_counter() - t0)
    e = es.GetElectronicEnergy()
    its = es.GetIterations()
    cpu = None
    if not args.no_cpu_baseline:
        from oracle import oracle as O
        O.build()
        om = O.make_molecule("pm3", mol.Z, mol.xyz)
        O.scf(om, O.SCFParams(**SCF))
        tl = []
        for _ in range(20):
            t0 = time.perf_counter()
            r = O.scf(om, O.SCFParams(**SCF))
            tl.append(time.perf_counter() - t0)
        cpu = {"value": 1.0 / float(np.median(tl)), "unit": "solves/s", "cores": 1, "kind": "port",
               "sample": "20 octane solves, one process (oracle: C integrals/Fock + LAPACK dsyevd/dsysv)",
               "p50_ms": 1e3 * float(np.median(tl)), "abs_dE_gpu_vs_cpu_Eh": abs(r.energy - e)}
    line = {"metric": "plain one-molecule PM3 SCF (n-octane), latency", "value": 1.0 / float(np.median(lat)),
            "unit": "solves/s", "n_gpus": 1, "steps": args.repeats, "warmup": 5,
            "ms_per_step": 1e3 * float(np.median(lat)), "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic: ideal all-trans n-octane",
            "config": {"workload": "C8H18 PM3, 26 atoms, 50 basis functions, FP64", "scf": SCF},
            "latency_ms": {"p50": 1e3 * percentile(lat, 50), "p99": 1e3 * percentile(lat, 99)},
            "e2e": {"value": 1.0 / float(np.mean(lat)), "unit": "solves/s",
                    "call": "SetMolecule + DoSCF + GetMullikenCharges (host arrays)"},
            "energy_Eh": e, "iterations": its, "cpu_baseline": cpu}
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------------------
# Moving molecules: warm-started SCF steps (the MD / RPMD pattern)
# ---------------------------------------------------------------------------
def run_md(args):
    """The (H2O)32 replicas take random-walk steps (0.01 A per coordinate and
    step); after each step the resident batch is re-solved from the previous
    densities (DoSCF(false), as MolDS's MD loop, src/md/MD.cpp:108, and RPMD
    beads, src/rpmd/RPMD.cpp:78-84).  Timed: the coordinate upload, integrals,
    SCF and properties of every step; a cold (guess) solve of the last
    geometry checks the warm results and gives the iteration count it saves."""
    import numpy as np
    import molds_gb300 as M
    from molds_gb300 import build
    build.build()
    ctx = M.Context(0)
    mols = workload(0, args.nmol)
    params = M.SCFParams(**SCF, precision=args.precision, dipole=args.dipole == "on")
    b = M.ResidentBatch("am1", mols, context=ctx)
    rng = np.random.default_rng(7)
    x = np.concatenate([m.xyz for m in mols])
    steps = [x]
    for _ in range(args.warmup + args.steps):
        steps.append(steps[-1] + rng.normal(scale=0.01 * M.ANG2AU, size=x.shape))
    b.run(params)                                   # first step from the guess
    for k in range(1, args.warmup + 1):
        b.set_coordinates(steps[k])
        b.run(params, requires_guess=False)
    clocks = Clocks(0)
    clocks.start()
    t0 = time.perf_counter()
    its = []
    for k in range(args.warmup + 1, args.warmup + 1 + args.steps):
        b.set_coordinates(steps[k])
        b.run(params, requires_guess=False)
        res, _ = b.results()
        its.append(float(np.mean([r["iterations"] for r in res])))
    wall = time.perf_counter() - t0
    clk = clocks.stop()
    warm_e = np.array([r["energy"] for r in res])
    ok = all(r["status"] == M.STATUS_CONVERGED for r in res)
    t1 = time.perf_counter()
    b.run(params)                                   # the same geometry from the guess
    cold_s = time.perf_counter() - t1
    cold, _ = b.results()
    cold_e = np.array([r["energy"] for r in cold])
    value = args.nmol * args.steps / wall
    line = {"metric": "warm-started SCF solves/s (MD / RPMD steps of resident molecules)", "value": value,
            "unit": "solves/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1e3 * wall / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "fp32+fp64" if args.precision == "mixed" else "f64",
            "data": "synthetic: seeded (H2O)32 replicas on a random walk",
            "config": {"workload": f"{args.nmol} replicas of (H2O)32, AM1, 0.01 A random-walk step, "
                                   "SCF from the previous density", "precision": args.precision,
                       "scf": SCF, "dipole": args.dipole == "on"},
            "e2e": {"value": value, "unit": "solves/s",
                    "h2d_bytes_per_step": int(x.size * 8), "d2h_bytes_per_step": int(args.nmol * ctypes.sizeof(M.ScfResultC)),
                    "call": "nddo_batch_set_coordinates + nddo_batch_run_ex(requires_guess = 0) + nddo_batch_results, "
                            "host wall clock"},
            "iterations": {"warm_mean": float(np.mean(its)), "cold_mean": float(np.mean([r["iterations"] for r in cold]))},
            "cold_step_ms": 1e3 * cold_s, "all_converged": ok,
            "accuracy": {"max_abs_dE_warm_vs_cold_Eh": float(np.max(np.abs(warm_e - cold_e)))},
            "clocks": clk}
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------------------
# Large single molecule: (H2O)512 MNDO, N = 3072
# ---------------------------------------------------------------------------
def run_water512(args):
    """One SCF of a 512-water cluster (8x8x8 jittered lattice, seed 4) under
    MNDO through the plain ElectronicStructure path (N = 3072: the whole-GPU
    Householder eigensolver), FP64 and then mixed precision, with the RMS /
    DIIS-error trace.  The reference's algorithm does not converge on this
    cluster with the benchmark's SCF block (density DIIS falls into an
    occupation-swapping 2-cycle, in the oracle as here), so the line reports
    seconds per SCF iteration over --max-iter iterations."""
    import numpy as np
    import molds_gb300 as M
    from molds_gb300 import build, workloads as W
    build.build()
    ctx = M.Context(0)
    mol = W.water_cluster(shape=(8, 8, 8), spacing=2.9, jitter=0.2, seed=4)
    scf = dict(SCF, max_iter=args.max_iter)
    out = {}
    clocks = Clocks(0)
    clocks.start()
    precs = [args.precision] + (["mixed"] if args.precision == "fp64" and not args.no_mixed else [])
    for prec in precs:
        es = M.ElectronicStructure("mndo", M.SCFParams(**scf, precision=prec), context=ctx)
        t0 = time.perf_counter()
        es.SetMolecule(mol)
        t1 = time.perf_counter()
        try:
            es.DoSCF()
            status = "converged"
        except M.SCFNotConverged:
            status = "not converged"
        t2 = time.perf_counter()
        tr = es.GetTrace()
        its = es.GetIterations()
        out[prec] = {"status": status, "iterations": its, "set_molecule_s": t1 - t0, "scf_s": t2 - t1,
                     "s_per_iteration": (t2 - t1) / max(1, its), "energy_Eh": es.GetElectronicEnergy(),
                     "rms_trace": [float(f"{t[1]:.3e}") for t in tr[:its]],
                     "diis_error_trace": [float(f"{t[2]:.3e}") for t in tr[:its]]}
    clk = clocks.stop()
    first = next(iter(out.values()))
    line = {"metric": "large single SCF: (H2O)512 MNDO, seconds per SCF iteration", "value": first["s_per_iteration"],
            "unit": "s/iteration", "n_gpus": 1, "steps": 1, "warmup": 0, "ms_per_step": 1e3 * first["scf_s"],
            "higher_is_better": False, "scaling": "replicas only", "vs_baseline": None,
            "dtype": "f64" if precs[0] == "fp64" else "fp32+fp64",
            "data": "synthetic: (H2O)512 on a jittered 8x8x8 lattice, seed 4",
            "config": {"workload": "(H2O)512 MNDO, 1536 atoms, 3072 basis functions, 2048 occupied", "scf": scf},
            "runs": out, "clocks": clk}
    print(json.dumps(line), flush=True)

# ---------------------------------------------------------------------------
# Serving: Poisson stream of PM3 single-point requests (energy + Mulliken)
# ---------------------------------------------------------------------------
def run_serving(args):
    """Open-loop arrivals at each rate through the continuous-batching server.
    The same request list (sizes log-uniform in 5..500 atoms, half alkanes,
    half water clusters, seed 5) is replayed at every rate with its arrival
    times scaled; latency = completion time - scheduled arrival time."""
    import numpy as np
    import molds_gb300 as M
    from molds_gb300 import build, workloads as W
    build.build()
    rates = [float(r) for r in args.rates.split(",")]
    stream = W.serving_stream(1.0, args.requests, seed=5)
    base_t = np.array([t for t, _ in stream])
    mols = [m for _, m in stream]
    nao = [int(sum(4 if z > 1 else 1 for z in m.Z)) for m in mols]
    ctx = M.Context(0)
    params = M.SCFParams(**SCF, precision=args.precision, dipole=args.dipole == "on")
    srv = M.Server(params, hbm_budget_bytes=int(args.hbm_gb * (1 << 30)), max_basis=args.max_basis, context=ctx)
    # warm-up: one small and one large request
    srv.submit("pm3", W.water_cluster_k(8, 1))
    srv.submit("pm3", W.water_cluster_k(40, 2))
    srv.drain()
    per_rate = []
    energies = {}
    clocks = Clocks(0)
    clocks.start()
    for rate in rates:
        arr = base_t / rate
        t0 = srv.clock()
        sched, done = {}, {}
        i = 0
        n = len(mols)
        while len(done) < n:
            now = srv.clock() - t0
            while i < n and arr[i] <= now:
                tk = srv.submit("pm3", mols[i])
                sched[tk] = (i, t0 + arr[i])
                i += 1
            wait = 2000 if i >= n else int(max(0.0, min(2000.0, (arr[i] - (srv.clock() - t0)) * 1e6)))
            for r in srv.poll(wait):
                done[r["ticket"]] = r
        lat = sorted(done[t]["t_done"] - sched[t][1] for t in done)
        # requests that the reference's SCF also fails on run to max_iter and
        # set the tail of `lat`; the converged requests' latencies separately
        lat_c = sorted(done[t]["t_done"] - sched[t][1] for t in done if done[t]["status"] == M.STATUS_CONVERGED)
        t_end = max(done[t]["t_done"] for t in done)
        its = [done[t]["iterations"] for t in done]
        for t in done:
            if done[t]["status"] == M.STATUS_CONVERGED:
                energies.setdefault(sched[t][0], done[t]["energy"])
        conv = sum(done[t]["status"] == M.STATUS_CONVERGED for t in done)
        lanes = {}
        for t in done:
            lanes.setdefault(done[t]["lane"], []).append(done[t])
        lane_stats = {str(k): {"requests": len(v), "converged": sum(r["status"] == M.STATUS_CONVERGED for r in v),
                               "mean_iterations": float(np.mean([r["iterations"] for r in v])),
                               "p50_ms": 1e3 * percentile([r["t_done"] - r["t_submit"] for r in v], 50),
                               "p99_ms": 1e3 * percentile([r["t_done"] - r["t_submit"] for r in v], 99)}
                      for k, v in sorted(lanes.items())}
        per_rate.append({"offered_req_s": rate, "requests": n, "converged": conv,
                         "solves_s": n / (t_end - t0), "converged_solves_s": conv / (t_end - t0),
                         "p50_ms": 1e3 * percentile(lat, 50), "p99_ms": 1e3 * percentile(lat, 99),
                         "converged_p50_ms": 1e3 * percentile(lat_c, 50) if lat_c else None,
                         "converged_p99_ms": 1e3 * percentile(lat_c, 99) if lat_c else None,
                         "max_ms": 1e3 * lat[-1], "mean_iterations": float(np.mean(its)), "span_s": t_end - t0,
                         "lanes": lane_stats})
        print(json.dumps({"rate": rate, **per_rate[-1]}), file=sys.stderr, flush=True)
    clk = clocks.stop()
    srv.close()
    # accuracy of the served (mixed-precision) energies against the FP64 path
    acc = None
    sample = list(range(0, len(mols), max(1, len(mols) // 48)))[:48]
    sample = [k for k in sample if k in energies]
    ref, _ = M.batch_scf("pm3", [mols[k] for k in sample], M.SCFParams(**SCF, precision="fp64"), context=ctx)
    both = [(k, r) for k, r in zip(sample, ref) if r["status"] == M.STATUS_CONVERGED]
    acc = {"sample": len(sample), "both_converged": len(both),
           "max_abs_dE_vs_fp64_gpu_Eh": max((abs(energies[k] - r["energy"]) for k, r in both), default=None)}
    best = max(per_rate, key=lambda r: r["converged_solves_s"])
    line = {"metric": "serving: p50/p99 latency and converged solves/s of a Poisson stream of PM3 single-point "
                      "requests",
            "value": best["converged_solves_s"], "unit": "solves/s", "n_gpus": 1, "steps": len(rates), "warmup": 1,
            "ms_per_step": None, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "fp32+fp64" if args.precision == "mixed" else "f64",
            "data": "synthetic: seeded serving stream (sizes log-uniform 5..500 atoms; alkanes n <= 60, "
                    "water clusters)",
            "config": {"workload": f"{len(mols)} PM3 requests per rate, Poisson arrivals, rates {rates}",
                       "hbm_budget_gb": args.hbm_gb, "max_basis": args.max_basis,
                       "basis_min_median_max": [min(nao), int(np.median(nao)), max(nao)],
                       "frac_basis_above_194": float(np.mean(np.array(nao) > 194)), "scf": SCF},
            "rates": per_rate, "accuracy": acc, "clocks": clk}
    print(json.dumps(line), flush=True)


if __name__ == "__main__":
    a = parse()
    if a.impl == "reference":
        run_reference(a)
    elif a.workload == "serving":
        run_serving(a)
    elif a.workload == "water32":
        run_ours(a)
    elif a.workload == "alkanes":
        run_alkanes(a)
    elif a.workload == "water512":
        run_water512(a)
    elif a.workload == "md":
        run_md(a)
    else:
        run_octane(a)
