"""Compile the sm_103a library ``libhzgb300.so`` in-tree with nvcc.

Translation units are compiled in parallel, one ``-gencode`` each.  The
stencil and tube units use ``-fmad=false`` so the level-set preprocessing
keeps the reference's unfused FP64 operation order (bit-identical grids;
the stencil unit's host code, the per-node entry points, is built with
``-ffp-contract=off`` for the same reason);
the pair sweeps and solvers use fused multiply-adds.
"""
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libhzgb300.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-lineinfo", "-std=c++17", "--extended-lambda", "-Xcompiler", "-fPIC",
          "-Xcompiler", "-fvisibility=hidden", "-I", CSRC]
UNITS = {
    "stencils.cu": ["-fmad=false", "-Xcompiler", "-ffp-contract=off"],
    "tube.cu": ["-fmad=false"],
    "dense.cu": ["-fmad=false"],
    "sweep_f64.cu": [],
    "sweep_f32.cu": ["-ftz=true"],
    "sweep_multi.cu": ["-ftz=true"],
    "sweep_combo32.cu": ["-ftz=true"],
    "krylov_multi.cu": [],
    "krylov.cu": [],
    "gmres.cu": [],
    "gmres_multi.cu": [],
    "evaluate.cu": [],
    "adjoint.cu": [],
    "combo.cu": [],
    "batch.cu": [],
    "shape_grad.cu": [],
    "capi.cu": [],
    "peaks.cu": [],
    "noalloc.cu": [],
    "ref_api.cu": [],
    "textio.cpp": [],
}


def nvcc():
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _newer(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose=False, extra=()):
    os.makedirs(BUILD, exist_ok=True)
    nv = nvcc()
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    headers += [os.path.join(HERE, "..", "include", f) for f in ("helmholtz_gb300.h", "helmholtz_ref_api.h")]
    headers = [h for h in headers if os.path.exists(h)]
    units = [u for u in UNITS if os.path.exists(os.path.join(CSRC, u))]

    def one(unit):
        src = os.path.join(CSRC, unit)
        obj = os.path.join(BUILD, unit + ".o")
        if _newer(obj, [src] + headers):
            cmd = [nv] + ARCH + COMMON + UNITS[unit] + list(extra) + ["-c", src, "-o", obj]
            r = subprocess.run(cmd, capture_output=True, text=True)
            if r.returncode != 0:
                raise RuntimeError("nvcc failed for %s:\n%s\n%s" % (unit, r.stdout, r.stderr))
            if verbose and (r.stdout or r.stderr):
                print(r.stdout + r.stderr, file=sys.stderr)
        return obj

    with ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 4)) as ex:
        objs = list(ex.map(one, units))
    if _newer(LIB, objs):
        cmd = [nv] + ARCH + ["-shared", "-o", LIB] + objs + ["-lcudart"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("link failed:\n%s\n%s" % (r.stdout, r.stderr))
    return LIB


if __name__ == "__main__":
    print(build(verbose=True, extra=sys.argv[1:]))
