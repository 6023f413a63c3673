#!/usr/bin/env python3
"""Build the reference's own C code as a test oracle (TEST INFRASTRUCTURE ONLY).

Recipe: copy the reference sources from REF_DIR into oracle/_ref/src/ (a
git-ignored build directory; nothing from the reference is committed), apply
the defect patches and the config hooks listed below, and compile them with
oracle/ref_harness.cpp into oracle/_ref/libref_<variant>.so.  The reference's
own Makefile is not used; this is a direct g++ call over its 10 source files.

Patches (each must match exactly the stated number of times):
  D1  large3Dexample2.c:4172-4175 and :4527-4530 read regfactor[j] /
      regfactor[i] with i, j uninitialised (segfaults); use regfactor[pj] /
      regfactor[pi], the target/source the entry belongs to.
  D2  large3Dexample2.c:4017 passes tstarz as the x coordinate; use tstarx.
  D3  large3Dexample2.c:2641,3121 read b[size+counter]; use bimg[counter].
  D4  errornorm is read before it is set (BICGSTAB.c:35,376,
      large3Dexample2.c:2514,2984); start it at 1.0.
  cfg the config macros of frame.h / PDE.h / BICGSTAB.h get #ifndef guards so
      each variant can set them with -D (the reference hard-codes them).

Variants:
  neumann   : the reference defaults ([-2,2]^3, FACTOR 2, TAU_FACTOR 2,
              Neumann, exterior); BiCG tolerance 1e-13.
  dirichlet : [-1,1]^3, FACTOR 3, TAU_FACTOR 2, Dirichlet, exterior;
              BiCG tolerance 1e-13.

Usage: python oracle/build_ref.py [--ref DIR] [--stage-only | --from-stage | --auto]
DIR is the reference tree: --ref, else the HZ_REFERENCE_DIR environment
variable, else DEFAULT_REF below (where this container mounts it).  The
staged sources stay in oracle/_ref/src so that a machine without the
reference tree (the GPU host) can still compile the variants
(python oracle/build_ref.py --from-stage).  --auto builds from the tree when
it exists, else from the staged sources, else does nothing.
"""
import argparse
import os
import re
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
DEFAULT_REF = "/root/reference"
OUT = os.path.join(HERE, "_ref")
SRC = os.path.join(OUT, "src")

SOURCES = ["distance_application3D.c", "finite_difference3D.c", "interpolate3D.c", "tools.c",
           "BICGSTAB.c", "functions.c", "HelmholtzKernel.c", "printslice.c", "weno.c",
           "large3Dexample2.c"]
HEADERS = ["distance_application3D.h", "finite_difference3D.h", "interpolate3D.h", "tools.h",
           "BICGSTAB.h", "functions.h", "HelmholtzKernel.h", "printslice.h", "weno.h", "frame.h",
           "PDE.h", "constants.h"]

GUARDED = {"frame.h": ["INT_U", "INT_L"],
           "PDE.h": ["DIRICHLET", "INTERIOR_MODE", "INCIDENTALWAVE", "FACTOR", "TAU_FACTOR"],
           "BICGSTAB.h": ["DEFAULTACC"]}

VARIANTS = {
    "neumann": ["-DDEFAULTACC=1e-13"],
    "dirichlet": ["-DINT_U=1.0", "-DINT_L=-1.0", "-DFACTOR=3.0", "-DDIRICHLET=1",
                  "-DINCIDENTALWAVE=0", "-DDEFAULTACC=1e-13"],
}

D1_OLD = ("\t\tif (DIRICHLET == 1)\n\t\t\tpartial = regfactor[j];\n"
          "\t\telse\n\t\t\tpartial = regfactor[i];\n")
D1_NEW = ("\t\tif (DIRICHLET == 1)\n\t\t\tpartial = regfactor[pj];\n"
          "\t\telse\n\t\t\tpartial = regfactor[pi];\n")

PATCHES = {
    "large3Dexample2.c": [
        (D1_OLD, D1_NEW, 2),
        ("cal_interpgrad(N,H,tstarz, tstary, tstarz,", "cal_interpgrad(N,H,tstarx, tstary, tstarz,", 1),
        ("(b[size+counter]!=b[size+counter])", "(bimg[counter]!=bimg[counter])", 2),
        ("\tdouble errornorm, preerrornorm;\n", "\tdouble errornorm = 1.0, preerrornorm;\n", 2),
    ],
    "BICGSTAB.c": [
        ("\tdouble errornorm, preerrornorm;\n", "\tdouble errornorm = 1.0, preerrornorm;\n", 2),
    ],
}


def guard_macros(text, names):
    for name in names:
        pat = re.compile(r"^(#define\s+%s\s+[^\n]*)$" % re.escape(name), re.M)
        m = pat.findall(text)
        if len(m) != 1:
            raise SystemExit("config hook for %s matched %d times" % (name, len(m)))
        text = pat.sub(lambda mm: "#ifndef %s\n%s\n#endif" % (name, mm.group(1)), text)
    return text


def stage(ref):
    os.makedirs(SRC, exist_ok=True)
    for f in SOURCES + HEADERS:
        with open(os.path.join(ref, f), "r", encoding="latin-1") as fh:
            text = fh.read()
        for old, new, count in PATCHES.get(f, []):
            got = text.count(old)
            if got != count:
                raise SystemExit("patch in %s matched %d times, expected %d: %r" % (f, got, count, old[:60]))
            text = text.replace(old, new)
        if f in GUARDED:
            text = guard_macros(text, GUARDED[f])
        with open(os.path.join(SRC, f), "w", encoding="latin-1") as fh:
            fh.write(text)
    shutil.copy(os.path.join(HERE, "ref_harness.cpp"), os.path.join(SRC, "ref_harness.cpp"))


def compile_variant(name, jobs):
    objdir = os.path.join(OUT, "obj_" + name)
    os.makedirs(objdir, exist_ok=True)
    flags = ["g++", "-O3", "-fopenmp", "-ffp-contract=off", "-fPIC", "-w", "-I", SRC,
             "-Dmain=ref_main"] + VARIANTS[name]
    srcs = [os.path.join(SRC, f) for f in SOURCES] + [os.path.join(SRC, "ref_harness.cpp")]

    def one(s):
        obj = os.path.join(objdir, os.path.basename(s) + ".o")
        subprocess.run(flags + ["-x", "c++", "-c", s, "-o", obj], check=True)
        return obj

    with ThreadPoolExecutor(max_workers=jobs) as ex:
        objs = list(ex.map(one, srcs))
    lib = os.path.join(OUT, "libref_%s.so" % name)
    subprocess.run(["g++", "-shared", "-fopenmp", "-Wl,-Bsymbolic", "-o", lib] + objs + ["-lm"], check=True)
    return lib


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default=os.environ.get("HZ_REFERENCE_DIR", DEFAULT_REF),
                    help="the reference tree (default: $HZ_REFERENCE_DIR, else %s)" % DEFAULT_REF)
    ap.add_argument("--from-stage", action="store_true", help="compile the sources staged under oracle/_ref/src")
    ap.add_argument("--stage-only", action="store_true", help="copy and patch the sources, do not compile")
    ap.add_argument("--auto", action="store_true",
                    help="the tree if it exists, else the staged sources, else nothing (exit 0)")
    ap.add_argument("-j", type=int, default=os.cpu_count() or 4)
    a = ap.parse_args()
    if a.auto:
        if os.path.isdir(a.ref):
            a.from_stage = False
        elif os.path.isdir(SRC):
            a.from_stage = True
        else:
            print("no reference tree and no staged sources: reference build skipped", file=sys.stderr)
            return 0
    if not a.from_stage:
        if not os.path.isdir(a.ref):
            print("reference tree %s not found" % a.ref, file=sys.stderr)
            return 1
        stage(a.ref)
    elif not os.path.isdir(SRC):
        print("no staged sources under %s" % SRC, file=sys.stderr)
        return 1
    if a.stage_only:
        return 0
    for v in VARIANTS:
        print(compile_variant(v, a.j))
    return 0


if __name__ == "__main__":
    sys.exit(main())
