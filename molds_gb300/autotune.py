"""Autotuner of the batched SCF's launch shapes; writes molds_gb300/tuning.txt.

Sweeps, on the GPU it runs on (one process per candidate table, named through
MOLDS_GB300_TUNING, so each candidate is read fresh by the library):

  * tridiag_threads -- the CTA size (256, 512, 1024) of the FP64
    tridiagonalisation, per basis-size class (a batch of 64 molecules of each
    size: (H2O)_k clusters and random alkanes);
  * vec_smem        -- whether the tridiagonal eigenvector kernel keeps its
    inverse-iteration factors in shared memory (fewer, larger CTAs per SM) or
    in the global workspace (up to 32 one-warp CTAs per SM), per basis-size
    class, in batches run as concurrent molecule groups;
  * groups          -- the number of concurrent molecule groups of a fixed
    batch (1, 2, 3, 4, 6), for batches of 64 and 256 (H2O)32;
  * check_block     -- SCF iterations enqueued per convergence check (1, 2, 4).

Each candidate is timed as the median of `--repeats` full batched FP64 SCF
solves (nddo_batch_scf, device arrays reused) after one warm-up; the fastest
wins.  Results do not depend on the launch shapes (every kernel works per
molecule), so only time is compared.

    python -m molds_gb300.autotune [--out molds_gb300/tuning.txt] [--repeats 3]
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import tempfile

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
SCF = dict(max_iter=500, rms_density=1e-8, damping_thresh=1.0, damping_weight=0.0, diis_num_error_vect=5,
           diis_start_error=0.1, diis_end_error=0.0)

_CHILD = r"""
import json, sys, time
sys.path.insert(0, {root!r})
import numpy as np
import molds_gb300 as M
from molds_gb300 import workloads as W
spec = json.loads({spec!r})
kind, nmol = spec["kind"], spec["nmol"]
if kind == "water32":
    base = W.water_cluster(shape=(4, 4, 2), spacing=2.9, jitter=0.2, seed=2)
    mols = W.water_replicas(base, nmol, sigma=0.05, seed0=1000)
    theory = "am1"
elif kind == "water":
    mols = [W.water_cluster_k(spec["k"], 11 + i) for i in range(nmol)]
    theory = "am1"
else:
    mols = [W.random_alkane(3100000 + i, n=spec["n"]) for i in range(nmol)]
    theory = "pm3"
p = M.SCFParams(**json.loads({scf!r}))
ctx = M.Context(0)
M.batch_scf(theory, mols, p, context=ctx)
ts = []
for _ in range(spec["repeats"]):
    t = time.perf_counter()
    M.batch_scf(theory, mols, p, context=ctx)
    ts.append(time.perf_counter() - t)
print(json.dumps(sorted(ts)[len(ts) // 2]))
"""


def _time(table_lines, spec, env=None):
    with tempfile.NamedTemporaryFile("w", suffix=".txt", delete=False) as f:
        f.write("\n".join(table_lines) + "\n")
        path = f.name
    try:
        e = dict(os.environ, MOLDS_GB300_TUNING=path, **(env or {}))
        code = _CHILD.format(root=ROOT, spec=json.dumps(spec), scf=json.dumps(SCF))
        r = subprocess.run([sys.executable, "-c", code], env=e, capture_output=True, text=True, timeout=900)
        if r.returncode != 0:
            raise RuntimeError(r.stderr[-2000:])
        return float(r.stdout.strip().splitlines()[-1])
    finally:
        os.unlink(path)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--out", default=os.path.join(HERE, "tuning.txt"))
    ap.add_argument("--repeats", type=int, default=3)
    args = ap.parse_args()
    from molds_gb300 import build
    build.build()
    log = []

    # 1. tridiagonalisation CTA size per basis-size class (one group of 64)
    classes = [("alkane", {"n": 8}, 50), ("water", {"k": 16}, 96), ("water32", {}, 192),
               ("water", {"k": 40}, 240), ("alkane", {"n": 60}, 362)]
    threads_rows = []
    for kind, extra, nbasis in classes:
        best = None
        for t in (256, 512, 1024):
            spec = dict(kind=kind, nmol=64, repeats=args.repeats, **extra)
            dt = _time([f"tridiag_threads 1073741824 {t}", "groups 1 1"], spec)
            log.append({"sweep": "tridiag_threads", "basis": nbasis, "threads": t, "s": dt})
            print(f"tridiag_threads basis {nbasis:4d} threads {t:4d}: {dt * 1e3:8.1f} ms", flush=True)
            if best is None or dt < best[1]:
                best = (t, dt)
        threads_rows.append((nbasis, best[0]))
    # bases between the classes take the next larger class's choice
    tlines = [f"tridiag_threads {nb} {t}" for nb, t in threads_rows]
    tlines[-1] = f"tridiag_threads 1073741824 {threads_rows[-1][1]}"

    # 2. eigenvector-kernel factor storage per basis-size class, in batches
    #    split into concurrent groups (the kernel's footprint decides how well
    #    it shares the SMs with the other groups' kernels)
    default_groups = ["groups 1 1", "groups 64 3", "groups 256 4"]
    smem_rows = []
    for kind, extra, nbasis in classes:
        nmol = 256 if nbasis <= 192 else (128 if nbasis <= 240 else 64)
        best = None
        for v in (1, 0):
            spec = dict(kind=kind, nmol=nmol, repeats=args.repeats, **extra)
            dt = _time(tlines + default_groups + [f"vec_smem 1073741824 {v}"], spec)
            log.append({"sweep": "vec_smem", "basis": nbasis, "molecules": nmol, "smem": v, "s": dt})
            print(f"vec_smem basis {nbasis:4d} molecules {nmol:4d} smem {v}: {dt * 1e3:8.1f} ms", flush=True)
            if best is None or dt < best[1]:
                best = (v, dt)
        smem_rows.append((nbasis, best[0]))
    vlines = [f"vec_smem {nb} {v}" for nb, v in smem_rows]
    vlines[-1] = f"vec_smem 1073741824 {smem_rows[-1][1]}"
    tlines = tlines + vlines

    # 3. molecule groups per batch size
    group_rows = []
    for nmol in (64, 256):
        best = None
        for g in (1, 2, 3, 4, 6):
            spec = dict(kind="water32", nmol=nmol, repeats=args.repeats)
            dt = _time(tlines + [f"groups 1 {g}"], spec)
            log.append({"sweep": "groups", "molecules": nmol, "groups": g, "s": dt})
            print(f"groups molecules {nmol:4d} groups {g}: {dt * 1e3:8.1f} ms", flush=True)
            if best is None or dt < best[1]:
                best = (g, dt)
        group_rows.append((nmol, best[0]))
    glines = ["groups 1 1"] + [f"groups {nm} {g}" for nm, g in group_rows]

    # 4. iterations per convergence check
    best = None
    for b in (1, 2, 4):
        spec = dict(kind="water32", nmol=256, repeats=args.repeats)
        dt = _time(tlines + glines + [f"check_block {b}"], spec)
        log.append({"sweep": "check_block", "block": b, "s": dt})
        print(f"check_block {b}: {dt * 1e3:8.1f} ms", flush=True)
        if best is None or dt < best[1]:
            best = (b, dt)

    lines = ["# molds_gb300 launch shapes, written by python -m molds_gb300.autotune",
             "# (median of full batched FP64 SCF solves per candidate; see molds_gb300/autotune.py)"]
    lines += tlines + glines + [f"check_block {best[0]}"]
    with open(args.out, "w") as f:
        f.write("\n".join(lines) + "\n")
    with open(os.path.splitext(args.out)[0] + "_sweep.json", "w") as f:
        json.dump(log, f, indent=1)
    print("\n".join(lines))


if __name__ == "__main__":
    main()
