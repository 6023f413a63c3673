#!/usr/bin/env python3
"""CPU pair-evaluation rate of the reference path on the host cores
(TEST / BASELINE INFRASTRUCTURE ONLY; used by bench.py's cpu_baseline leg and
its --impl reference arm).

The workload is the torus problem of the benchmark (R=0.6, r=0.25 on an
N^3 grid over [-1,1]^3, tube 3h, Dirichlet, k).  At 256^3 the reference
cannot run its own solver (its dense cache would need 2 n^2 doubles), so a
step here is the reference's pair evaluation (omp_get_Ccomp,
large3Dexample2.c:4463-4564) plus the complex multiply-add of its product
loop (:3243-3244) over a bounded block of target rows against all n sources,
rows spread over the host threads.  With --impl port the same block runs
through the C restatement (ibim_oracle.c) instead.

Prints one JSON line: pairs/s per step, setup time, n, rows, threads.
"""
import argparse
import json
import os
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--impl", choices=["reference", "port", "auto"], default="auto")
    ap.add_argument("--N", type=int, default=256)
    ap.add_argument("--wave", type=float, default=20.0)
    ap.add_argument("--R", type=float, default=0.6)
    ap.add_argument("--r", type=float, default=0.25)
    ap.add_argument("--threads", type=int, default=os.cpu_count() or 1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=1)
    ap.add_argument("--step-seconds", type=float, default=2.0, help="target CPU time of one step")
    a = ap.parse_args()

    import oracle as O
    from helmholtz_3d_torrone_gb300 import geometry as G

    impl = a.impl
    if impl == "auto":
        impl = "reference" if os.path.exists(os.path.join(O.REF_DIR, "libref_dirichlet.so")) else "port"
    d = G.torus(a.N, R=a.R, r=a.r, int_l=-1.0, int_u=1.0)
    rng = np.random.default_rng(7)
    t0 = time.time()
    if impl == "reference":
        # the reference prints progress on stdout; keep our JSON line clean
        saved = os.dup(1)
        devnull = os.open(os.devnull, os.O_WRONLY)
        os.dup2(devnull, 1)
        ref = O.Reference("dirichlet")
        ref.setup(a.N, a.wave, d)
        n = len(ref.tube())
        v = rng.standard_normal(n) + 1j * rng.standard_normal(n)

        def run(r0, r1):
            return ref.rows_matvec(n, v, r0, r1, a.threads)
    else:
        orc = O.Oracle()
        p = O.make_params(a.N, a.wave)
        tp = orc.pipeline(p, d)
        n = len(tp["idx"])
        v = rng.standard_normal(n) + 1j * rng.standard_normal(n)

        def run(r0, r1):
            return orc.matvec(p, tp, v, r0=r0, r1=r1, nthreads=a.threads)
    run(0, 1)  # builds the reference's per-point arrays (first call)
    setup = time.time() - t0
    # calibrate the row block to about step-seconds of work
    rows = max(a.threads, 16)
    t1 = time.time()
    run(0, rows)
    dt = max(time.time() - t1, 1e-6)
    rows = int(max(a.threads, min(n, rows * a.step_seconds / dt)))
    rates = []
    for s in range(a.warmup + a.steps):
        r0 = (s * rows) % max(1, n - rows)
        t1 = time.time()
        run(r0, r0 + rows)
        dt = time.time() - t1
        if s >= a.warmup:
            rates.append(rows * n / dt)
    if impl == "reference":
        sys.stdout.flush()
        os.dup2(saved, 1)
    out = dict(impl=impl, n=n, N=a.N, wave=a.wave, rows=rows, threads=a.threads, setup_s=setup,
               pairs_per_s=rates, pairs_per_step=rows * n,
               seconds_per_step=[rows * n / r for r in rates])
    print(json.dumps(out))
    sys.stdout.flush()


if __name__ == "__main__":
    main()
