#!/usr/bin/env python3
"""Benchmark of the GB300 IBIM Helmholtz hot path.

Workload (the at-scale configuration of the reference's hot path): torus
R=0.6, r=0.25 sampled as its analytic signed distance on a 256^3 grid over
[-1,1]^3, tube |phi| <= 3h (n = 581,420 points), k = 20, Dirichlet
(double-layer) formulation with point-source data from (0.6, 0, 0).

The headline ``value`` is the wall time of one complete solve of that
system to an FP64 relative residual below 1e-6: FP32 inner GMRES(120)
solves (one FP32 pair sweep per iteration, tile-local origins, phase k rho
reduced with a split k/(2 pi) before the SFU sin/cos) inside FP64
iterative refinement whose residual b - A x comes from the FP64 pair
sweep.  It replaces the reference's
parallel_BiCGcomplex (large3Dexample2.c:2954-3514).  ``e2e`` is the same
solve through the public C ABI with host buffers (H2D of b, D2H of x inside
the timed region).

Beside it: the plain FP64 GPU solve with the same method (measured seconds
of one FP64 product x the product count of a complete FP64 GMRES(120)
solve of this workload, measured once with ``--solve --fp64-full`` and
recorded in FP64_SOLVE_ITERS), the roofline of the FP64 sweep (the kernel
that takes most of the solve's time: two FP64 residual products), and the
FP32 sweep's rate and roofline over ``--steps`` timed inner iterations (L2
flushed between them).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

``--impl reference`` measures the reference's own CPU pair evaluation
(omp_get_Ccomp + its complex multiply-add) on the host cores for the same
workload (oracle/cpu_rate.py) and prints a lower bound of its solve time,
FP64_SOLVE_ITERS x n^2 / rate: the FP64 product count of the GMRES solve
(the reference's BiCG needs two products per iteration); with several ranks
only rank 0 runs it.
"""
import argparse
import csv
import ctypes as C
import io
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

METRIC = "256³ solve time & Gpair/s: FP32+FP64-refine vs plain FP64 GPU at 1e-6 rel err"
FLOPS_PER_PAIR = 40  # reference pair formula, large3Dexample2.c:4471-4550
SOLVE_TOL = 1e-6     # FP64 relative residual of the timed solve
INNER_TOL = 1e-7     # tightest inner FP32 tolerance (the first step solves to SOLVE_TOL / 4)
RESTART = 120        # GMRES basis size (no restart within these solves)
# Products (iterations) of the complete plain-FP64 GMRES(120) solve of this
# workload to SOLVE_TOL: 67, measured on a GB300 with
# bench.py --solve --N 256 --tol 1e-6 1e-11 --method gmres bicg --restart 120
#          --fp64-full --fp64-tol 1e-6 --fp64-method gmres
# (1,708 s, FP64 residual 8.4e-7).
FP64_SOLVE_ITERS = 67
FP64_SOLVE_ITERS_WORKLOAD = (256, 20.0)  # (N, k) the count was measured on


def fp64_solve_products(N, wave):
    """The measured FP64 product count, for the workload it was measured on
    only (None for any other --N / --wave)."""
    return FP64_SOLVE_ITERS if (N, float(wave)) == FP64_SOLVE_ITERS_WORKLOAD else None


# DRAM bytes (read + write) per launch of the fused FP32 sweep at 256^3:
# 22.36 MB measured by ncu on the 128^3 torus (n = 145,272), scaled by n to
# n = 581,420.  The sweep reads every record once from DRAM and the tiles
# from L2, so traffic grows in proportion to n.
SWEEP32_TRAFFIC = 22.36e6 * 581420 / 145272
# The same for one A p launch of the FP32 sweep: 15.19 MB measured by ncu on
# the 128^3 torus, scaled by n.
SWEEP32_TRAFFIC_A = 15.19e6 * 581420 / 145272
SWEEP64_TRAFFIC = 16.5e6 * 581420 / 145272  # ncu DRAM read of the FP64 sweep at 128^3, scaled by n
FP64_OPS_PER_PAIR = 38.5  # FP64 instructions per pair of the A-mode FP64 sweep (ncu, 128^3 torus, scaled records)


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["gb300", "reference"], default="gb300")
    ap.add_argument("--N", type=int, default=256)
    ap.add_argument("--wave", type=float, default=20.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--cpu-seconds", type=float, default=6.0, help="CPU time of one cpu_baseline step")
    ap.add_argument("--solve", action="store_true",
                    help="instead of the step benchmark, time complete solves (FP32+FP64 refinement at each "
                         "--tol, FP64 BiCG iterations) and print one JSON line with solve times")
    ap.add_argument("--tol", type=float, nargs="*", default=[1e-6, 1e-8])
    ap.add_argument("--fp64-iters", type=int, default=1,
                    help="--solve: timed plain-FP64 BiCG iterations (the full FP64 solve time is this "
                         "per-iteration time x the iteration count; --fp64-full runs it to tolerance)")
    ap.add_argument("--fp64-full", action="store_true")
    ap.add_argument("--fp64-method", choices=["bicg", "gmres"], default="gmres",
                    help="--solve --fp64-full: method of the FP64 solve")
    ap.add_argument("--fp64-tol", type=float, default=0.0,
                    help="--solve --fp64-full: tolerance of the FP64 solve (default: the smallest --tol)")
    ap.add_argument("--fp64-solve-iters", type=int, default=0,
                    help="--solve: FP64 BiCG iteration count of a complete solve, for the extrapolated FP64 time")
    ap.add_argument("--method", choices=["bicg", "gmres"], nargs="*", default=["bicg", "gmres"],
                    help="--solve: inner Krylov method(s) of the refined solves")
    ap.add_argument("--restart", type=int, default=40, help="--solve: GMRES restart length")
    ap.add_argument("--phase", choices=["direct", "split"], default="split",
                    help="--solve: phase mode of the FP32 sweeps (hz_set_phase_mode; split is the library default)")
    ap.add_argument("--inner-tol", type=float, default=INNER_TOL,
                    help="--solve: tightest inner FP32 tolerance of the refined solves")
    ap.add_argument("--save", default="",
                    help="--solve: write the densities (refined and, with --fp64-full, FP64) as .npy into this folder")
    ap.add_argument("--shape", choices=["torus", "ellipsoid"], default="torus",
                    help="--solve: torus (the step workload) or the ellipsoid (0.7,0.5,0.4) level set "
                         "reinitialised on the device before the build")
    ap.add_argument("--reinit-iters", type=int, default=60, help="--solve --shape ellipsoid: TVD-RK2 steps")
    ap.add_argument("--combo", action="store_true",
                    help="instead of the step benchmark: the Combo formulation (sphere r = 1 in [-2,2]^3, annulus "
                         "[0.1 sqrt(h), sqrt(h)], exterior monopole Neumann data): FP64 and FP32 product rates, a "
                         "refined solve, and with --fp64-full the FP64 solve")
    ap.add_argument("--gradient", action="store_true",
                    help="instead of the step benchmark: misfit gradients on the bumpy sphere (dJ/dphi at every "
                         "grid node, dJ/dg, dJ/dk by adjoint solves) with central-difference checks")
    ap.add_argument("--products-only", action="store_true",
                    help="--plane-waves: time the multi right-hand-side products only, no solves")
    ap.add_argument("--multi-method", choices=["gmres", "bicgstab"], default="gmres",
                    help="--plane-waves: lockstep method of the multi right-hand-side solve")
    ap.add_argument("--single-waves", type=int, default=4,
                    help="--plane-waves: waves also solved one at a time (per method) for the comparison")
    ap.add_argument("--plane-waves", type=int, default=0,
                    help="instead of the step benchmark: solve this many incident plane waves (Fibonacci-sphere "
                         "directions) on the torus with the multi right-hand-side solver and report the times")
    ap.add_argument("--batch", type=int, default=0,
                    help="instead of the step benchmark: solve this many seeded ellipsoids (semi-axes U[0.2,0.7], "
                         "grids 64^3-192^3) as one batch and one after another, and report both times")
    ap.add_argument("--batch-grids", type=int, nargs="*", default=[64, 96, 128, 160, 192],
                    help="--batch: grid sizes drawn per surface")
    ap.add_argument("--batch-axes", type=float, nargs=2, default=[0.2, 0.7],
                    help="--batch: range of the seeded semi-axes")
    ap.add_argument("--product", choices=["f32", "f64", "pair32", "pair64"], default="",
                    help="instead of the step benchmark: build the torus operator at --N and run --steps products of "
                         "this kind (A p, or the fused A p + A^H pt), timed with CUDA events (short runs for "
                         "profilers)")
    ap.add_argument("--config1", action="store_true",
                    help="instead of the step benchmark: the 64^3 sphere (k = 5, point source at the origin) solved "
                         "to 1e-13 on the GPU (FP64 BiCG and FP32 + FP64-refinement GMRES) and by the reference "
                         "build on the host cores (its dense matrix and omp_CompBiCG), end to end, with the "
                         "densities compared")
    ap.add_argument("--sweep-variant", type=int, default=-1,
                    help="use this FP32 sweep variant instead of the autotuner's choice (profiling)")
    return ap.parse_args()


def dist_env():
    return int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")), int(
        os.environ.get("LOCAL_RANK", "0"))


def max_over_ranks(dist, seconds, device):
    """The job's time: the largest of every rank's time (dist None: one rank)."""
    if dist is None:
        return seconds
    import torch
    t = torch.tensor([seconds], device=device, dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_rate(pairs_per_step, steps, world, seconds):
    """Whole-job pair evaluations per second in Gpair/s: every rank (replica)
    evaluates pairs_per_step pairs per step."""
    return pairs_per_step * steps * world / seconds / 1e9


def workload_desc(N, wave, n):
    return {"workload": "torus R=0.6 r=0.25, phi = analytic signed distance on %d^3 over [-1,1]^3, tube "
                        "|phi|<=3h, k=%g, Dirichlet point source at (0.6,0,0)" % (N, wave),
            "N": N, "n_tube": n, "wave": wave, "formulation": "dirichlet, exterior"}


def solve_desc():
    return {"tol": SOLVE_TOL, "inner_tol_floor": INNER_TOL, "method": "gmres(%d)" % RESTART,
            "fp32_phase": "k rho reduced with a split k/(2 pi) (the library default)",
            "value": "seconds of one complete solve to FP64 relative residual < tol: FP32 inner GMRES (one FP32 "
                     "sweep A p per iteration) inside FP64 iterative refinement (residual b - A x from the FP64 "
                     "sweep); b resident in HBM, CUDA events on the operator's stream, run once after the step loop",
            "step": "one iteration of that inner GMRES (FP32 sweep over all n^2 pairs + FP64 Gram-Schmidt), L2 "
                    "flushed between steps by a 256 MB device write; the steps give the FP32 pair rate"}


def cpu_solve_seconds(pair_rate, n, N=256, wave=20.0):
    """Lower bound of the reference's FP64 solve time on the host cores:
    the measured FP64 product count x n^2 pair evaluations / the measured
    rate (its BiCG evaluates two products per iteration); None where no
    count was measured."""
    prods = fp64_solve_products(N, wave)
    if not prods or not pair_rate:
        return None
    return prods * 1.0 * n * n / pair_rate


def cpu_rate(N, wave, impl, steps, warmup, step_seconds, timeout=900):
    cmd = [sys.executable, os.path.join(ROOT, "oracle", "cpu_rate.py"), "--impl", impl, "--N", str(N), "--wave",
           str(wave), "--steps", str(steps), "--warmup", str(warmup), "--step-seconds", str(step_seconds)]
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=timeout)
    if r.returncode != 0:
        raise RuntimeError("cpu_rate failed: %s" % r.stderr[-2000:])
    line = [l for l in r.stdout.splitlines() if l.startswith("{")][-1]
    return json.loads(line)


class Clocks:
    """Sample SM clocks and throttle reasons with nvidia-smi during a region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.f = tempfile.NamedTemporaryFile(mode="w+", suffix=".csv", delete=False)
        self.p = None

    def start(self):
        try:
            self.p = subprocess.Popen(["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.Q,
                                       "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.f,
                                      stderr=subprocess.DEVNULL)
        except OSError:
            self.p = None

    def stop(self):
        if self.p is None:
            return None
        self.p.terminate()
        try:
            self.p.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.p.kill()
        self.f.flush()
        rows = list(csv.reader(io.StringIO(open(self.f.name).read())))
        os.unlink(self.f.name)
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            if len(r) < 9:
                continue
            try:
                sm.append(float(r[1]))
                mx.append(float(r[2]))
            except ValueError:
                continue
            for nm, v in zip(names, r[5:9]):
                if v.strip().lower() == "active":
                    reasons.add(nm)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


def run_reference(a, rank, world):
    if rank != 0:
        return 0
    per_step = max(1.0, min(6.0, 150.0 / max(1, a.steps + a.warmup)))
    r = cpu_rate(a.N, a.wave, "auto", a.steps, a.warmup, per_step)
    rates = r["pairs_per_s"]
    total_pairs = r["pairs_per_step"] * len(rates)
    total_s = sum(r["seconds_per_step"])
    rate = total_pairs / total_s
    n = r["n"]
    solve_s = cpu_solve_seconds(rate, n, a.N, a.wave)
    kind = "reference" if r["impl"] == "reference" else "port"
    sample = ("%d target rows x %d sources per step (one row block of an A p product, the reference's pair "
              "evaluation + complex MAC), %d steps after %d warm-up; setup %.1f s untimed"
              % (r["rows"], n, len(rates), a.warmup, r["setup_s"]))
    line = {
        "impl": "reference", "metric": METRIC, "value": solve_s, "unit": "s", "n_gpus": a.gpus,
        "steps": a.steps, "warmup": a.warmup, "ms_per_step": 1e3 * total_s / len(rates),
        "higher_is_better": False, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": dict(workload_desc(a.N, a.wave, n), tol=SOLVE_TOL, method="FP64 (the reference's pair formula)",
                       value="lower bound of the FP64 solve time on the host cores: %s products (of the complete "
                             "FP64 GMRES(%d) GPU solve of this workload; the reference's BiCG needs two per "
                             "iteration) x n^2 pairs / the measured pair rate"
                             % (fp64_solve_products(a.N, a.wave), RESTART),
                       step="reference pair evaluation + complex MAC over a bounded block of target rows x all n "
                            "sources"),
        "pair_rate_gpair_s": rate / 1e9,
        "cpu_baseline": {"value": solve_s, "unit": "s", "cores": r["threads"], "kind": kind, "sample": sample,
                         "pair_rate_gpair_s": rate / 1e9},
        "e2e": {"value": solve_s, "unit": "s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))
    sys.stdout.flush()
    return 0


def run_gb300(a, rank, world, local):
    import numpy as np
    import torch
    import helmholtz_3d_torrone_gb300 as hz
    from helmholtz_3d_torrone_gb300 import geometry as G

    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")

    def barrier():
        if dist is not None:
            dist.barrier()

    L = hz.load()
    N, wave = a.N, a.wave
    d = G.torus(N, R=0.6, r=0.25, int_l=-1.0, int_u=1.0)
    p = hz.params(N, wave, int_l=-1.0, int_u=1.0, factor=3.0, tau_factor=2.0, dirichlet=1)
    stream = torch.cuda.Stream()
    op = hz.Operator(p)
    op.set_stream(stream.cuda_stream)
    op.set_distance(d)
    n = op.build()
    if a.sweep_variant >= 0:
        op.set_sweep_config(a.sweep_variant)
        sweep_cfg = a.sweep_variant
    else:
        sweep_cfg, sweep_cfg_ms = op.autotune()  # untimed: picks the FP32 sweep variant for this tube
    b = op.rhs_point_source(np.array([0.6, 0.0, 0.0]), hz.RHS_POINT_DIRICHLET)
    fp32_peak, fp64_peak = hz.measure_fma_peaks()

    dev = torch.device("cuda", local)
    b_re = torch.from_numpy(np.ascontiguousarray(b.real)).to(dev)
    b_im = torch.from_numpy(np.ascontiguousarray(b.imag)).to(dev)
    x_re = torch.empty(n, dtype=torch.float64, device=dev)
    x_im = torch.empty(n, dtype=torch.float64, device=dev)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)
    step_opts = hz.solve_opts(method=hz.GMRES, precision=hz.PREC_F32, tol=1e-300, maxit=1, stagnation=0,
                              restart=RESTART)
    solve_opts = hz.solve_opts(method=hz.GMRES, precision=hz.PREC_F32_REFINED, tol=SOLVE_TOL, inner_tol=INNER_TOL,
                               maxit=2000, max_outer=8, restart=RESTART)
    info = hz.SolveInfo()

    def call(opts, where, br, bi, xr, xi):
        rc = L.hz_solve(op.h, C.byref(opts), br, bi, xr, xi, where, C.byref(info))
        if rc != 0:
            raise hz.HzError(rc, L.hz_last_error().decode())
        return info.as_dict()

    dptr = (b_re.data_ptr(), b_im.data_ptr(), x_re.data_ptr(), x_im.data_ptr())
    op.sweep_timing(1)
    for _ in range(a.warmup):
        with torch.cuda.stream(stream):
            flush.fill_(1.0)
        call(step_opts, hz.HZ_DEVICE, *dptr)
    torch.cuda.synchronize()
    clocks = Clocks(local)
    clocks.start()
    # ---------------- timed steps: inner BiCG iterations, device-resident b
    op.sweep_timing(1)  # reset the per-kernel totals (stays on: graphs keep their events)
    launches0 = hz.kernel_launches()
    barrier()
    torch.cuda.synchronize()
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    t0 = time.perf_counter()
    for _ in range(a.steps):
        with torch.cuda.stream(stream):
            flush.fill_(float(_))
        call(step_opts, hz.HZ_DEVICE, *dptr)
    ev1.record(stream)
    torch.cuda.synchronize()
    wall = time.perf_counter() - t0
    barrier()
    launches = hz.kernel_launches() - launches0
    dev_s = ev0.elapsed_time(ev1) / 1e3
    sweep_ms, sweep_launches = op.sweep_timing(-1)
    op.sweep_timing(0)
    elapsed = max_over_ranks(dist, max(dev_s, 1e-9), dev)
    pairs_step = n * n
    step_rate = job_rate(pairs_step, a.steps, world, elapsed)

    # ---------------- the metric: one complete refined solve, b resident in HBM
    with torch.cuda.stream(stream):
        flush.fill_(2.0)
    torch.cuda.synchronize()
    barrier()
    ev2 = torch.cuda.Event(enable_timing=True)
    ev3 = torch.cuda.Event(enable_timing=True)
    solve_launches0 = hz.kernel_launches()
    ev2.record(stream)
    t1 = time.perf_counter()
    sinfo = call(solve_opts, hz.HZ_DEVICE, *dptr)
    ev3.record(stream)
    solve_launches = hz.kernel_launches() - solve_launches0
    torch.cuda.synchronize()
    solve_wall = time.perf_counter() - t1
    solve_s = max_over_ranks(dist, ev2.elapsed_time(ev3) / 1e3, dev)
    clk = clocks.stop()

    # ---------------- e2e: the same solve through the C ABI with host buffers
    hb_re = torch.from_numpy(np.ascontiguousarray(b.real)).pin_memory()
    hb_im = torch.from_numpy(np.ascontiguousarray(b.imag)).pin_memory()
    hx_re = torch.empty(n, dtype=torch.float64).pin_memory()
    hx_im = torch.empty(n, dtype=torch.float64).pin_memory()
    hptr = (hb_re.data_ptr(), hb_im.data_ptr(), hx_re.data_ptr(), hx_im.data_ptr())
    with torch.cuda.stream(stream):
        flush.fill_(3.0)
    torch.cuda.synchronize()
    barrier()
    t2 = time.perf_counter()
    einfo = call(solve_opts, hz.HZ_HOST, *hptr)
    torch.cuda.synchronize()
    e2e_s = max_over_ranks(dist, time.perf_counter() - t2, dev)
    x_host = hx_re.numpy() + 1j * hx_im.numpy()
    x_dev = x_re.cpu().numpy() + 1j * x_im.cpu().numpy()
    e2e_vs_dev = float(np.max(np.abs(x_host - x_dev)) / np.max(np.abs(x_dev)))

    # ---------------- plain FP64 GPU comparator: one FP64 product (the FP64
    # sweep, CUDA events on the operator's stream), also the roofline of the
    # kernel that takes most of the refined solve's time
    f64 = None
    if a.fp64_iters > 0:
        y_re = torch.empty(n, dtype=torch.float64, device=dev)
        y_im = torch.empty(n, dtype=torch.float64, device=dev)
        ev4 = torch.cuda.Event(enable_timing=True)
        ev5 = torch.cuda.Event(enable_timing=True)
        ev4.record(stream)
        for _ in range(a.fp64_iters):
            rc = L.hz_matvec(op.h, hz.PREC_F64, 0, x_re.data_ptr(), x_im.data_ptr(), y_re.data_ptr(),
                             y_im.data_ptr(), hz.HZ_DEVICE)
            if rc != 0:
                raise hz.HzError(rc, L.hz_last_error().decode())
        ev5.record(stream)
        torch.cuda.synchronize()
        per_prod = ev4.elapsed_time(ev5) / 1e3 / a.fp64_iters
        f64 = {"seconds_per_product": per_prod, "products_timed": a.fp64_iters,
               "gpair_per_s": float(n) * n / per_prod / 1e9,
               "solve_products": fp64_solve_products(N, wave),
               "solve_s_extrapolated": (per_prod * fp64_solve_products(N, wave)
                                        if fp64_solve_products(N, wave) else None),
               "how": "measured seconds of one FP64 product (sweep64_kernel, CUDA events) x the product count of "
                      "a complete FP64 GMRES(%d) solve of this workload to the same tol, measured once (bench.py "
                      "--solve --fp64-full); GMRES adds only FP64 Gram-Schmidt (milliseconds) per product" % RESTART}
        if f64["solve_s_extrapolated"]:
            f64["speedup_refined_vs_f64"] = f64["solve_s_extrapolated"] / solve_s

    if rank != 0:
        op.close()
        return 0
    avg_sweep_s = (sweep_ms / sweep_launches) / 1e3 if sweep_launches else None
    achieved = pairs_step * FLOPS_PER_PAIR / avg_sweep_s / 1e12 if avg_sweep_s else None
    roof32 = {"bound": "fp32", "kernel": "sweep32_kernel (A p, the inner GMRES product)",
              "achieved": achieved, "peak": fp32_peak, "unit": "TFLOP/s",
              "frac": (achieved / fp32_peak) if achieved else None, "traffic": SWEEP32_TRAFFIC_A,
              "flops_per_pair": FLOPS_PER_PAIR, "pairs_per_launch": pairs_step,
              "avg_launch_ms": avg_sweep_s * 1e3 if avg_sweep_s else None,
              "launches_timed": sweep_launches,
              "peak_source": "FP32 FFMA chains measured live on this GPU (hz_measure_fma_peaks)",
              "share_of_solve": (sinfo["iterations"] * avg_sweep_s / solve_s) if avg_sweep_s else None}
    roof64 = None
    if f64:
        a64 = float(n) * n * FLOPS_PER_PAIR / f64["seconds_per_product"] / 1e12
        roof64 = {"bound": "fp64", "kernel": "sweep64_kernel (A x, the FP64 refinement residual)",
                  "achieved": a64, "peak": fp64_peak, "unit": "TFLOP/s", "frac": a64 / fp64_peak,
                  "fp64_ops_per_pair": FP64_OPS_PER_PAIR,
                  "pipe_frac": float(n) * n * FP64_OPS_PER_PAIR / f64["seconds_per_product"] / (fp64_peak * 0.5e12),
                  "note": "frac counts the reference formula's 40 flops per pair against the DFMA peak (2 flops per "
                          "instruction); pipe_frac counts the FP64 instructions the kernel executes (ncu) against "
                          "the pipe's instruction rate (peak / 2)",
                  "traffic": SWEEP64_TRAFFIC, "flops_per_pair": FLOPS_PER_PAIR, "pairs_per_launch": n * n,
                  "avg_launch_ms": f64["seconds_per_product"] * 1e3, "launches_timed": a.fp64_iters,
                  "peak_source": "FP64 DFMA chains measured live on this GPU (hz_measure_fma_peaks)",
                  "share_of_solve": sinfo["outer"] * f64["seconds_per_product"] / solve_s}
    # the roofline of the kernel that takes most of the timed solve
    if roof64 and (roof64["share_of_solve"] or 0) > (roof32["share_of_solve"] or 0):
        roof_main, roof_other_key, roof_other = roof64, "roofline_fp32", roof32
    else:
        roof_main, roof_other_key, roof_other = roof32, "roofline_fp64", roof64
    keep = ("iterations", "outer", "resid_f64", "converged", "pair_evals", "steps", "step_iters",
            "step_inner_tol", "step_resid")
    line = {
        "metric": METRIC, "value": solve_s, "unit": "s", "n_gpus": world, "steps": a.steps,
        "warmup": a.warmup, "ms_per_step": 1e3 * elapsed / a.steps, "higher_is_better": False,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64-refine", "data": "synthetic",
        "config": dict(workload_desc(N, wave, n), sweep_variant=sweep_cfg, **solve_desc(),
                       l2="steps: flushed between steps by a 256 MB device write; solve: flushed before it",
                       replicas=world),
        "solve": dict({k: sinfo[k] for k in keep}, seconds=solve_s, wall_s=solve_wall,
                      gpair_per_s=sinfo["pair_evals"] / solve_s / 1e9),
        "e2e": {"value": e2e_s, "unit": "s", "h2d_bytes_per_step": 2 * n * 8, "d2h_bytes_per_step": 2 * n * 8,
                "resid_f64": einfo["resid_f64"], "iterations": einfo["iterations"],
                "max_rel_diff_vs_device_solve": e2e_vs_dev,
                "how": "hz_solve with pinned host b and x (H2D of b, D2H of x inside the timed region), wall clock"},
        "fp64_gpu": f64,
        "step_rate": {"value": step_rate, "unit": "Gpair/s", "pairs_per_step": pairs_step, "wall_s": wall},
        "gpu_launches": solve_launches,
        "step_launches": launches,
        "roofline": roof_main,
        roof_other_key: roof_other,
        "clocks": clk,
    }
    op.close()
    if not a.no_cpu_baseline and world == 1:
        try:
            r = cpu_rate(N, wave, "auto", 2, 1, a.cpu_seconds)
            rate = sum(r["pairs_per_s"]) / len(r["pairs_per_s"])
            cs = cpu_solve_seconds(rate, n, N, wave)
            line["cpu_baseline"] = {"value": cs, "unit": "s", "cores": r["threads"],
                                    "kind": "reference" if r["impl"] == "reference" else "port",
                                    "pair_rate_gpair_s": rate / 1e9,
                                    "sample": "%d target rows x %d sources per step (%.2e pairs), 2 steps after 1 "
                                              "warm-up, same 256^3 torus operator; setup %.1f s untimed; value = "
                                              "lower bound of the reference's FP64 solve (%s products x n^2 / rate)"
                                              % (r["rows"], r["n"], r["pairs_per_step"], r["setup_s"],
                                                 fp64_solve_products(N, wave))}
        except Exception as e:  # report, do not hide the GPU number
            line["cpu_baseline"] = {"value": None, "unit": "s", "error": str(e)[:300]}
    print(json.dumps(line))
    sys.stdout.flush()
    if dist is not None:
        dist.destroy_process_group()
    return 0


def run_solve(a, local):
    """Complete solves on the benchmark workload: FP32 pair sweeps inside FP64
    iterative refinement (BiCG), against plain FP64 BiCG."""
    import numpy as np
    import helmholtz_3d_torrone_gb300 as hz
    from helmholtz_3d_torrone_gb300 import geometry as G

    N, wave = a.N, a.wave
    H = 2.0 / N
    t0 = time.perf_counter()
    if a.shape == "ellipsoid":
        # analytic non-distance level set of the ellipsoid, reinitialised on the
        # device; its error against the exact ellipsoid distance is reported
        phi = G.ellipsoid_levelset(N)
        d = hz.reinitialize(phi, N, H, a.reinit_iters)
        exact = G.ellipsoid(N)
        band = np.abs(exact) <= 3 * H
        reinit_err = float(np.max(np.abs(d - exact)[band]))
        src = np.array([0.1, 0.05, 0.0])
    else:
        d = G.torus(N, R=0.6, r=0.25, int_l=-1.0, int_u=1.0)
        src = np.array([0.6, 0.0, 0.0])
    p = hz.params(N, wave, int_l=-1.0, int_u=1.0, factor=3.0, tau_factor=2.0, dirichlet=1)
    out = {"mode": "solve", "config": workload_desc(N, wave, 0), "runs": []}
    with hz.Operator(p) as op:
        op.set_distance(d)
        n = op.build()
        out["build_s"] = time.perf_counter() - t0
        out["config"] = workload_desc(N, wave, n)
        if a.shape == "ellipsoid":
            out["config"]["workload"] = ("ellipsoid (0.7,0.5,0.4): level set 0.3(1-|x/a|) reinitialised by %d "
                                         "TVD-RK2 steps on the device, %d^3 over [-1,1]^3, tube |phi|<=3h, k=%g, "
                                         "Dirichlet point source at (0.1,0.05,0)" % (a.reinit_iters, N, wave))
            out["config"]["reinit_max_err_in_band"] = reinit_err
        out["config"]["sweep_variant"] = op.autotune()[0]
        op.set_phase_mode(hz.PHASE_SPLIT if a.phase == "split" else hz.PHASE_DIRECT)
        out["config"]["phase"] = a.phase
        out["config"]["inner_tol_floor"] = a.inner_tol
        b = op.rhs_point_source(src, hz.RHS_POINT_DIRICHLET)
        sols = {}
        for meth in a.method:
            mid = hz.GMRES if meth == "gmres" else hz.BICG
            for tol in a.tol:
                x, info = op.solve(b, method=mid, precision=hz.PREC_F32_REFINED, tol=tol, inner_tol=a.inner_tol,
                                   restart=a.restart, max_outer=8)
                info.update(precision="f32+f64-refine", method=meth, tol=tol,
                            gpair_per_s=info["pair_evals"] / info["seconds"] / 1e9,
                            history=[float("%.3e" % v) for v in op.residual_history()])
                out["runs"].append(info)
                sols[(meth, tol)] = x
        # plain FP64 BiCG: the whole solve with --fp64-full, else its per-iteration time
        if a.save:
            os.makedirs(a.save, exist_ok=True)
            for (meth, t), x in sols.items():
                np.save(os.path.join(a.save, "x_%s_%s_%g.npy" % (a.shape, meth, t)), x)
        if a.fp64_full:
            tol = a.fp64_tol or min(a.tol)
            fm = hz.GMRES if a.fp64_method == "gmres" else hz.BICG
            x64, info = op.solve(b, method=fm, precision=hz.PREC_F64, tol=tol, maxit=2000, restart=a.restart)
            info.update(precision="f64", method=a.fp64_method, tol=tol, gpair_per_s=info["pair_evals"] / info["seconds"] / 1e9,
                        history=[float("%.3e" % v) for v in op.residual_history()])
            out["runs"].append(info)
            out["f64_solve_iterations"] = info["iterations"]
            out["f64_solve_s"] = info["seconds"]
            if a.save:
                np.save(os.path.join(a.save, "x_%s_f64_%g.npy" % (a.shape, tol)), x64)
            sols[("f64 " + a.fp64_method, tol)] = x64
        # errors of every solution against the FP64 solve and against the
        # tightest refined solve (an FP64-accurate solution when its FP64
        # residual is far below the others' tolerances): density (max-norm
        # and 2-norm relative) and off-surface field at 100 seeded receivers
        # on the sphere r = 0.9
        refs = {}
        if a.fp64_full:
            refs["f64 %s %g" % (a.fp64_method, tol)] = x64
        tight = min(a.tol)
        if len(a.tol) > 1:
            for meth in a.method:
                refs["%s %g" % (meth, tight)] = sols[(meth, tight)]
        rx = G.random_sphere_points(100, 0.9, seed=7)
        for rname, xr in refs.items():
            ur = op.evaluate(rx, xr, hz.DOUBLE_LAYER)
            errs = {}
            for (meth, t), x in sols.items():
                key = "%s %g" % (meth, t)
                if key == rname:
                    continue
                u = op.evaluate(rx, x, hz.DOUBLE_LAYER)
                errs[key] = {"density_max": float(np.max(np.abs(x - xr)) / np.max(np.abs(xr))),
                             "density_2": float(np.linalg.norm(x - xr) / np.linalg.norm(xr)),
                             "field_max": float(np.max(np.abs(u - ur)) / np.max(np.abs(ur)))}
            out.setdefault("rel_err_vs", {})[rname] = errs
        if not a.fp64_full and a.fp64_iters > 0:
            x64, info = op.solve(b, method=hz.BICG, precision=hz.PREC_F64, tol=1e-300, maxit=a.fp64_iters,
                                 stagnation=0)
            per_it = info["seconds"] / max(1, info["iterations"])
            out["f64_per_iteration_s"] = per_it
            out["f64_gpair_per_s"] = info["pair_evals"] / info["seconds"] / 1e9
            if a.fp64_solve_iters:
                out["f64_solve_s_extrapolated"] = per_it * a.fp64_solve_iters
                out["f64_extrapolation"] = ("measured FP64 BiCG seconds per iteration x %d iterations (the FP64 "
                                            "BiCG iteration count passed in, measured on a complete FP64 solve)"
                                            % a.fp64_solve_iters)
        for r in out["runs"]:
            if r["precision"] != "f64" and "f64_solve_s_extrapolated" in out:
                r["speedup_vs_f64_extrapolated"] = out["f64_solve_s_extrapolated"] / r["seconds"]
            if r["precision"] != "f64" and "f64_solve_s" in out:
                r["speedup_vs_f64"] = out["f64_solve_s"] / r["seconds"]
    print(json.dumps(out))
    sys.stdout.flush()
    return 0


def run_plane_waves(a):
    """Many incident fields on one surface: one kernel evaluation per pair
    serves 8 right-hand sides (hz_solve_multi), against single solves."""
    import numpy as np
    import helmholtz_3d_torrone_gb300 as hz
    from helmholtz_3d_torrone_gb300 import geometry as G
    N, wave, R = a.N, a.wave, a.plane_waves
    d = G.torus(N, R=0.6, r=0.25, int_l=-1.0, int_u=1.0)
    p = hz.params(N, wave, int_l=-1.0, int_u=1.0, factor=3.0, tau_factor=2.0, dirichlet=1)
    out = {"mode": "plane_waves"}
    with hz.Operator(p) as op:
        op.set_distance(d)
        n = op.build()
        cfg = op.autotune()[0]
        dirs = G.fibonacci_sphere(R)
        B = op.rhs_plane_waves(dirs, hz.RHS_POINT_DIRICHLET)
        out["config"] = {"workload": "torus R=0.6 r=0.25 on %d^3 over [-1,1]^3, tube |phi|<=3h, k=%g, %d incident "
                                     "plane waves e^{ik d.x} (Dirichlet data), directions on a Fibonacci sphere"
                                     % (N, wave, R), "N": N, "n_tube": n, "wave": wave, "nrhs": R,
                         "sweep_variant": cfg,
                         "rhs_per_kernel_pass": "blocks of 32 (FP32) and 16 (FP64), the last block the smallest of "
                                                "8/16/32 that holds the remaining columns"}
        # products: R right-hand sides through the multi-RHS sweep vs R single FP32 products
        op.matvec_multi(B)  # warm-up: loads every block kernel the timed call uses
        t0 = time.perf_counter()
        op.matvec_multi(B)
        t_multi = time.perf_counter() - t0
        t0 = time.perf_counter()
        for r in range(min(R, 8)):
            op.matvec(B[r], precision=hz.PREC_F32)
        t_single = (time.perf_counter() - t0) / min(R, 8) * R
        out["products"] = {"multi_s": t_multi, "single_s_for_all": t_single, "speedup": t_single / t_multi,
                           "pairs_x_rhs_per_s_multi": float(n) * n * R / t_multi,
                           "note": "wall time incl. host<->device copies of the vectors"}
        if a.products_only:
            print(json.dumps(out))
            sys.stdout.flush()
            return 0
        # solves: all R in lockstep (FP32 + FP64 refinement) vs one refined BiCGSTAB solve per field
        mm = hz.GMRES if a.multi_method == "gmres" else hz.BICGSTAB
        X, info, res = op.solve_multi(B, method=mm, precision=hz.PREC_F32_REFINED, tol=a.tol[0], inner_tol=1e-5,
                                      restart=a.restart)
        out["multi_solve"] = dict(info, max_resid=float(np.max(res)), method=a.multi_method)
        nsingle = min(R, a.single_waves)
        for meth, name in ((hz.BICGSTAB, "bicgstab"), (hz.GMRES, "gmres")) if nsingle > 0 else ():
            t0 = time.perf_counter()
            errs = []
            for r in range(nsingle):
                x, i1 = op.solve(B[r], method=meth, precision=hz.PREC_F32_REFINED, tol=a.tol[0], inner_tol=1e-5,
                                 restart=a.restart)
                errs.append(float(np.max(np.abs(x - X[r])) / np.max(np.abs(x))))
            t_one = (time.perf_counter() - t0) / nsingle
            out["single_solves_" + name] = {"seconds_per_field": t_one, "fields_timed": nsingle,
                                            "seconds_for_all_extrapolated": t_one * R,
                                            "max_rel_diff_vs_multi": max(errs),
                                            "method": "refined %s, one wave at a time" % name}
            out["multi_solve_speedup_vs_single_%s_extrapolated" % name] = t_one * R / info["seconds"]
    print(json.dumps(out))
    sys.stdout.flush()
    return 0


def run_combo(a):
    """The Combo formulation at scale: FP64 and FP32 matrix-free products,
    an FP32 + FP64-refinement solve and (with --fp64-full) the plain FP64
    solve, and the field at (1.5, 0.3, 0.2) against the exact exterior
    monopole -e^{ikr}/(kr)."""
    import numpy as np
    import helmholtz_3d_torrone_gb300 as hz
    from helmholtz_3d_torrone_gb300 import geometry as G
    N, k, tol = a.N, a.wave, min(a.tol)
    H = 4.0 / N
    eps0 = np.sqrt(H)
    p = hz.params(N, k)  # [-2,2]^3, FACTOR 2, Neumann, exterior (the reference's defaults)
    o = hz.dense_opts(hz.DENSE_COMBO, p, delta0=0.1 * eps0, epsilon=eps0, wavenum=k, eta=-1.0)
    d = G.sphere(N, radius=1.0, center=(0.013, 0.021, 0.007), int_l=-2.0, int_u=2.0)
    out = {"mode": "combo"}
    t0 = time.perf_counter()
    with hz.Operator(p) as op:
        op.set_combo(o)
        op.set_distance(d)
        n = op.build()
        out["config"] = {"workload": "Combo formulation: sphere r = 1 centred near the origin on %d^3 over "
                                     "[-2,2]^3, annulus 0.1 sqrt(h) <= |d| <= sqrt(h), SineWeight, eta = -1, "
                                     "k = %g, exterior monopole Neumann data" % (N, k),
                         "N": N, "n_annulus": n, "wave": k, "build_s": time.perf_counter() - t0}
        rng = np.random.default_rng(1)
        v = rng.standard_normal(n) + 1j * rng.standard_normal(n)
        prod = {}
        for name, prec, reps in (("f32", hz.PREC_F32, 5), ("f64", hz.PREC_F64, 1)):
            op.matvec(v, precision=prec)
            t1 = time.perf_counter()
            for _ in range(reps):
                q = op.matvec(v, precision=prec)
            dt = (time.perf_counter() - t1) / reps
            prod[name] = {"seconds": dt, "gpair_per_s": float(n) * n / dt / 1e9}
            prod[name + "_q"] = q
        prod["f32_rel_err_vs_f64"] = float(np.linalg.norm(prod.pop("f32_q") - prod["f64_q"]) /
                                           np.linalg.norm(prod.pop("f64_q")))
        out["products"] = dict(prod, note="wall time of hz_matvec incl. host<->device copies")
        b = op.rhs_point_source(np.zeros(3), hz.RHS_MONOPOLE_NEUMANN)
        rx = np.array([[1.5, 0.3, 0.2]])
        r = float(np.linalg.norm(rx))
        ue = -np.exp(1j * k * r) / (k * r)
        x, info = op.solve(b, method=hz.GMRES, precision=hz.PREC_F32_REFINED, tol=tol, inner_tol=1e-5,
                           maxit=3000, restart=a.restart)
        u = op.evaluate(rx, x, hz.COMBO_LAYER)[0]
        out["refined_solve"] = dict(info, method="gmres(%d)" % a.restart, tol=tol,
                                    field_rel_err_vs_exact=float(abs(u - ue) / abs(ue)))
        if a.fp64_full:
            x64, i64 = op.solve(b, method=hz.GMRES, precision=hz.PREC_F64, tol=tol, maxit=3000, restart=a.restart)
            u64 = op.evaluate(rx, x64, hz.COMBO_LAYER)[0]
            out["f64_solve"] = dict(i64, method="gmres(%d)" % a.restart, tol=tol,
                                    field_rel_err_vs_exact=float(abs(u64 - ue) / abs(ue)))
            out["density_rel_err_refined_vs_f64"] = float(np.max(np.abs(x - x64)) / np.max(np.abs(x64)))
            out["speedup_refined_vs_f64"] = i64["seconds"] / info["seconds"]
    print(json.dumps(out))
    sys.stdout.flush()
    return 0


def run_gradient(a):
    """Misfit gradients by adjoint solves on the bumpy sphere
    r = 0.5 (1 + 0.08 cos 3theta sin 2phi), its level set reinitialised on the
    device: J = sum |u(x_m) - t_m|^2 over 64 receivers on r = 0.95, t the
    field of the unperturbed sphere on the same grid.  dJ/dphi at every grid
    node (hz_shape_gradient) and dJ/dg, dJ/dk (hz_misfit_gradient) are timed
    and checked against central differences (step 1e-6) of complete refined
    solves (FP32 sweeps, FP64 residuals, to --tol)."""
    import numpy as np
    import helmholtz_3d_torrone_gb300 as hz
    from helmholtz_3d_torrone_gb300 import geometry as G
    N, wave, tol = a.N, a.wave, min(a.tol)
    H = 2.0 / N
    eps = 3.0 * H
    src = np.array([0.05, 0.02, 0.01])
    rx = G.random_sphere_points(64, 0.95, seed=17)
    sk = dict(method=hz.BICGSTAB, precision=hz.PREC_F32_REFINED, tol=tol, inner_tol=1e-5, maxit=3000)
    step = 1e-6

    def params(k):
        return hz.params(N, k, int_l=-1.0, int_u=1.0, factor=3.0, tau_factor=2.0, dirichlet=1)

    def field(dist, k=wave, b=None):
        with hz.Operator(params(k)) as op:
            op.set_distance(dist)
            op.build()
            if b is None:
                b = op.rhs_point_source(src, hz.RHS_POINT_DIRICHLET)
            x, info = op.solve(b, **sk)
            return op.evaluate(rx, x, hz.DOUBLE_LAYER), info

    t0 = time.perf_counter()
    d = hz.reinitialize(G.bumpy_sphere_levelset(N), N, H, a.reinit_iters)
    target, _ = field(G.sphere(N, 0.5))
    setup_s = time.perf_counter() - t0

    def J_of(dist, k=wave, b=None):
        u, _ = field(dist, k, b)
        return float(np.sum(np.abs(u - target) ** 2))

    out = {"mode": "gradient", "config": {
        "workload": "bumpy sphere r = 0.5(1 + 0.08 cos3theta sin2phi), level set reinitialised by %d TVD-RK2 steps "
                    "on %d^3 over [-1,1]^3, tube |phi|<=3h, k=%g, Dirichlet point source at (0.05,0.02,0.01); "
                    "J = sum |u - t|^2 at 64 seeded receivers on r = 0.95, t from the sphere r = 0.5 on the same grid"
                    % (a.reinit_iters, N, wave),
        "N": N, "wave": wave, "tol": tol, "fd_step": step, "setup_s": setup_s}}
    with hz.Operator(params(wave)) as op:
        op.set_distance(d)
        n = op.build()
        out["config"]["n_tube"] = n
        op.autotune()
        b = op.rhs_point_source(src, hz.RHS_POINT_DIRICHLET)
        J, gphi, info = op.shape_gradient(src, rx, target, **sk)
        out["shape_gradient"] = dict(info, J=J)
        J2, gb, dk, gw, info2 = op.misfit_gradient(b, rx, target, **sk)
        out["misfit_gradient"] = dict(info2, J=J2, dJ_dk=dk)
    t0 = time.perf_counter()
    checks = []
    rng = np.random.default_rng(5)
    inner = np.argwhere(np.abs(d) < eps - 0.5 * H)

    def fd_phi(q, h):
        dp, dm = d.copy(), d.copy()
        dp[q] += h
        dm[q] -= h
        return (J_of(dp) - J_of(dm)) / (2 * h)

    for q in (tuple(int(v) for v in inner[i]) for i in rng.choice(len(inner), 8, replace=False)):
        fd, fd7 = fd_phi(q, step), fd_phi(q, 0.1 * step)
        # a jump of J inside [phi - h, phi + h] shows as quotients that
        # disagree between the two steps
        checks.append({"wrt": "phi%s" % (q,), "phi": float(d[q]), "adjoint": float(gphi[q]), "fd": fd,
                       "fd_step_1e-7": fd7, "smooth": bool(abs(fd - fd7) <= 1e-2 * abs(fd7))})
    fdk = (J_of(d, wave + step, b) - J_of(d, wave - step, b)) / (2 * step)
    checks.append({"wrt": "k", "adjoint": dk, "fd": fdk})
    for i in (int(rng.integers(n)),):
        for part, unit in (("re", 1.0), ("im", 1j)):
            e = np.zeros(n, dtype=complex)
            e[i] = unit * step
            fd = (J_of(d, wave, b + e) - J_of(d, wave, b - e)) / (2 * step)
            adj = gb[i].real if part == "re" else gb[i].imag
            checks.append({"wrt": "%s g[%d]" % (part, i), "adjoint": float(adj), "fd": fd})
    for c in checks:
        c["rel_diff"] = abs(c["adjoint"] - c["fd"]) / max(abs(c["fd"]), 1e-300)
        if "fd_step_1e-7" in c:
            c["rel_diff_step_1e-7"] = abs(c["adjoint"] - c["fd_step_1e-7"]) / max(abs(c["fd_step_1e-7"]), 1e-300)
    out["fd_checks"] = checks
    phi = [c for c in checks if "smooth" in c]
    sm = [c for c in phi if c["smooth"]]
    out["phi_nodes_smooth"] = "%d of %d" % (len(sm), len(phi))
    if sm:
        out["phi_max_rel_diff_smooth"] = max(c["rel_diff"] for c in sm)
    out["phi_max_rel_diff_step_1e-7"] = max(c["rel_diff_step_1e-7"] for c in phi)
    out["fd_seconds"] = time.perf_counter() - t0
    out["note"] = ("J is piecewise smooth in phi: a node whose step moves a pair across the near-field radius or "
                   "flips an upwind branch of the stencils shows the jump in its difference quotient")
    print(json.dumps(out))
    sys.stdout.flush()
    return 0


def run_batch(a):
    """An uneven batch of ellipsoids solved together (hz_batch_solve: one
    persistent FP32 launch per product over all surfaces) against the same
    solves one after another."""
    import numpy as np
    import helmholtz_3d_torrone_gb300 as hz
    from helmholtz_3d_torrone_gb300 import geometry as G
    rng = np.random.default_rng(2024)
    count, wave = a.batch, a.wave
    grids = list(a.batch_grids)
    alo, ahi = a.batch_axes
    ops, cases = [], []
    t0 = time.perf_counter()
    for i in range(count):
        axes = tuple(float(x) for x in rng.uniform(alo, ahi, 3))
        # the 3h tube must keep the WENO stencils off the medial surface:
        # h <= min axis / 7
        need = int(np.ceil(14.0 / min(axes) / 8.0)) * 8
        N = max(int(rng.choice(grids)), need)
        H = 2.0 / N
        phi = G.ellipsoid_levelset(N, axes=axes)
        d = hz.reinitialize(phi, N, H, 40)
        op = hz.Operator(hz.params(N, wave, int_l=-1.0, int_u=1.0, factor=3.0, tau_factor=2.0, dirichlet=1))
        op.set_distance(d)
        n = op.build()
        ops.append(op)
        cases.append({"axes": [round(x, 4) for x in axes], "N": N, "n_tube": n})
    build_s = time.perf_counter() - t0
    bs = [op.rhs_point_source(np.array([0.02, 0.01, 0.0]), hz.RHS_POINT_DIRICHLET) for op in ops]
    out = {"mode": "batch", "config": {"workload": "%d ellipsoids, semi-axes U[%g,%g] (seed 2024), level sets "
                                                 "reinitialised on the device, grids %s over [-1,1]^3, tube "
                                                 "|phi|<=3h, k=%g, Dirichlet point source at (0.02,0.01,0)"
                                                 % (count, alo, ahi, "/".join("%d^3" % g for g in grids), wave),
                                       "surfaces": cases, "wave": wave, "build_s": build_s}}
    with hz.Batch(ops) as b:
        out["config"]["batch_variant"] = b.autotune()[0]
        xs, info, res = b.solve(bs, precision=hz.PREC_F32_REFINED, tol=a.tol[0], inner_tol=1e-5)
        out["batch_solve"] = dict(info, max_resid=float(np.max(res)))
    for op in ops:
        op.autotune()
    t0 = time.perf_counter()
    errs, its, pairs = [], 0, 0
    for op, rhs, x in zip(ops, bs, xs):
        x1, i1 = op.solve(rhs, method=hz.BICGSTAB, precision=hz.PREC_F32_REFINED, tol=a.tol[0], inner_tol=1e-5)
        its += i1["iterations"]
        pairs += i1["pair_evals"]
        errs.append(float(np.max(np.abs(x1 - x)) / np.max(np.abs(x1))))
    out["sequential_solves"] = {"seconds": time.perf_counter() - t0, "iterations": its, "pair_evals": pairs,
                                "max_rel_diff_vs_batch": max(errs),
                                "note": "one refined BiCGSTAB solve per surface, each with its own autotuned "
                                        "sweep variant (autotune untimed, as the batch's)"}
    out["batch_speedup"] = out["sequential_solves"]["seconds"] / info["seconds"]
    for op in ops:
        op.close()
    print(json.dumps(out))
    sys.stdout.flush()
    return 0


def run_config1(a):
    """Configuration 1 end to end on both sides: the GPU library (build,
    FP64 BiCG and refined GMRES solves to 1e-13) and the reference build on
    the host cores (grids, tube, per-point set-up and its dense matrix, then
    its OpenMP omp_CompBiCG to 1e-13; oracle/ref_worker.py, timed as the CPU
    baseline)."""
    import numpy as np
    import helmholtz_3d_torrone_gb300 as hz
    from helmholtz_3d_torrone_gb300 import geometry as G
    from oracle.ref_worker import RefWorker
    N, k = 64, 5.0
    d = G.sphere(N, radius=0.5)
    out = {"mode": "config1", "config": {"workload": "sphere R=0.5 at the origin, exact signed distance on 64^3 over "
                                                     "[-1,1]^3, tube |phi|<=3h, k=5, Dirichlet point source at the "
                                                     "origin, solves to relative residual 1e-13", "N": N, "wave": k}}
    rx = G.random_sphere_points(100, 0.9, seed=2024)
    r = np.linalg.norm(rx, axis=1)
    ue = np.exp(1j * k * r) / (4 * np.pi * r)
    t0 = time.perf_counter()
    op = hz.Operator(hz.params(N, k, int_l=-1.0, int_u=1.0, factor=3.0, tau_factor=2.0, dirichlet=1))
    op.set_distance(d)
    n = op.build()
    t_build = time.perf_counter() - t0
    b = op.rhs_point_source(np.zeros(3), hz.RHS_POINT_DIRICHLET)
    op.solve(b, method=hz.GMRES, precision=hz.PREC_F32_REFINED, tol=1e-6, restart=120)  # loads the kernels
    gpu = {"n_tube": n, "build_s": t_build}
    xs = {}
    for name, kw in (("f64_bicg", dict(method=hz.BICG, precision=hz.PREC_F64, tol=1e-13, maxit=1000)),
                     ("refined_gmres", dict(method=hz.GMRES, precision=hz.PREC_F32_REFINED, tol=1e-13,
                                            restart=120))):
        t1 = time.perf_counter()
        x, info = op.solve(b, **kw)
        dt = time.perf_counter() - t1
        u = op.evaluate(rx, x, hz.DOUBLE_LAYER)
        xs[name] = x
        gpu[name] = {"seconds": dt, "iterations": info["iterations"], "resid": info["resid"],
                     "field_rel_err_vs_exact": float(np.max(np.abs(u - ue)) / np.max(np.abs(ue)))}
    op.close()
    t2 = time.perf_counter()
    with RefWorker("dirichlet", N, k, d, omp_chunk=16) as ref:
        t_setup = time.perf_counter() - t2
        t3 = time.perf_counter()
        xr = ref.solve(b)
        t_solve = time.perf_counter() - t3
    cpu = {"setup_and_dense_s": t_setup, "compbicg_s": t_solve, "total_s": t_setup + t_solve,
           "cores": os.cpu_count(), "kind": "reference",
           "what": "reference build: ASSIGN_GRADIENT, BothCurvs loop, tube, per-point set-up and the dense matrix "
                   "of omp_get_Ccomp entries (OpenMP), then omp_CompBiCG (OpenMP, chunk 16 as the driver's "
                   "DEFAULT_OMP_CACHE_CHUNKSIZE) to 1e-13 (DEFAULTACC of this build)"}
    for name, x in xs.items():
        gpu[name]["density_rel_err_vs_reference"] = float(np.max(np.abs(x - xr)) / np.max(np.abs(xr)))
    gpu_total = t_build + gpu["refined_gmres"]["seconds"]
    out.update(gpu=gpu, cpu_reference=cpu,
               speedup_end_to_end=cpu["total_s"] / gpu_total,
               note="GPU end to end = build + refined GMRES solve (kernels loaded beforehand); the reference's "
                    "end to end = its set-up with the dense matrix + CompBiCG, in a child process")
    print(json.dumps(out))
    sys.stdout.flush()
    return 0


def run_product(a):
    """--steps products of one kind on the torus at --N (after --warmup)."""
    import numpy as np
    import torch
    import helmholtz_3d_torrone_gb300 as hz
    from helmholtz_3d_torrone_gb300 import geometry as G
    d = G.torus(a.N, R=0.6, r=0.25, int_l=-1.0, int_u=1.0)
    p = hz.params(a.N, a.wave, int_l=-1.0, int_u=1.0, factor=3.0, tau_factor=2.0, dirichlet=1)
    with hz.Operator(p) as op:
        op.set_distance(d)
        n = op.build()
        if a.sweep_variant >= 0:
            op.set_sweep_config(a.sweep_variant)
        rng = np.random.default_rng(1)
        v = rng.standard_normal(n) + 1j * rng.standard_normal(n)
        prec = hz.PREC_F64 if a.product.endswith("64") else hz.PREC_F32

        def one():
            if a.product.startswith("pair"):
                return op.matvec_pair(v, v, precision=prec)[0]
            return op.matvec(v, precision=prec)
        for _ in range(a.warmup):
            one()
        t0 = time.perf_counter()
        for _ in range(a.steps):
            q = one()
        dt = (time.perf_counter() - t0) / max(1, a.steps)
        print(json.dumps({"mode": "product", "product": a.product, "N": a.N, "n": n, "wave": a.wave,
                          "seconds_per_product": dt, "gpair_per_s": float(n) * n / dt / 1e9,
                          "note": "wall time of hz_matvec / hz_matvec_pair incl. host<->device copies",
                          "q0": [float(q[0].real), float(q[0].imag)]}))
    return 0


def main():
    a = parse()
    rank, world, local = dist_env()
    if a.impl == "reference":
        return run_reference(a, rank, world)
    if a.config1:
        # the reference worker's child processes start with spawn, which is
        # safe after this process has initialised CUDA
        import torch
        torch.cuda.set_device(local)
        return run_config1(a)
    if a.solve or a.plane_waves or a.batch or a.gradient or a.combo or a.product:
        import torch
        torch.cuda.set_device(local)
        if a.product:
            return run_product(a)
        if a.gradient:
            return run_gradient(a)
        if a.combo:
            return run_combo(a)
        if a.plane_waves:
            return run_plane_waves(a)
        if a.batch:
            return run_batch(a)
        return run_solve(a, local)
    return run_gb300(a, rank, world, local)


if __name__ == "__main__":
    sys.exit(main())
