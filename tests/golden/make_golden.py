#!/usr/bin/env python3
"""Generate the golden fixtures in tests/golden/ from the reference itself.

Each case runs in its own process against oracle/_ref/libref_<variant>.so
(the reference's C code, patched and compiled by oracle/build_ref.py), since
the reference keeps its tube arrays in function statics.  Fixtures hold the
input distance grid and the reference's outputs for it: WENO gradient and
curvature grids, tube index list, per-point arrays, a sample of matrix
entries, the dense products A p and A^H p for a seeded p, and the CompBiCG
density for a point-source right-hand side solved to 1e-13.  The dense
case holds the per-point arrays of the three dense assemblers of
HelmholtzKernel.c, a sample of their matrix entries and their products with
a seeded vector.  The Godunov case holds the reference's upwind |grad phi|
(finite_difference3D.c:5-27) for seeded one-sided derivatives.  The digest
case pins the reference's grid stages on the 256^3 torus by SHA-256 digests;
the solve case holds the reference's CompBiCG density for the 64^3 sphere.

Usage:  python oracle/build_ref.py && python tests/golden/make_golden.py
"""
import json
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

CASES = {
    # reference defaults: [-2,2]^3, FACTOR 2, Neumann, exterior; sphere R=1
    # offset from the grid nodes so no projection lands on a cell face.
    "ref_neumann_sphere_n16": dict(variant="neumann", N=16, wave=2.0, shape="sphere", radius=1.0,
                                   center=(0.013, 0.021, 0.007), rhs_kind=2),
    "ref_neumann_sphere_n24": dict(variant="neumann", N=24, wave=5.0, shape="sphere", radius=1.0,
                                   center=(0.013, 0.021, 0.007), rhs_kind=2),
    # the benchmark domain and formulation: [-1,1]^3, FACTOR 3, Dirichlet
    "ref_dirichlet_sphere_n20": dict(variant="dirichlet", N=20, wave=5.0, shape="sphere", radius=0.5,
                                     center=(0.0, 0.0, 0.0), rhs_kind=0),
    # a torus small enough for a dense reference run (R=0.5, r=0.25 keeps
    # the 3h tube inside the domain and away from the core circle at N=32)
    "ref_dirichlet_torus_n32": dict(variant="dirichlet", N=32, wave=4.0, shape="torus", R=0.5, r=0.25,
                                    rhs_kind=0),
}


# Dense assemblers of HelmholtzKernel.c on the reference's own configuration:
# DoubleLayerKernel (tube |d| <= FACTOR h), new_HelmholtzKernelCombo on the
# driver's default annulus [delta0, epsilon0] = [0.1 h, sqrt(h)] (eta -1,
# large3Dexample2.c:37,61-63,298-305), new_HelmholtzKernel on frame.h's sphere.
DENSE_CASES = {
    "ref_neumann_dense_n16": dict(variant="neumann", N=16, wave=2.0, shape="sphere", radius=1.0,
                                  center=(0.013, 0.021, 0.007), eta=-1.0),
}


def distance(case, int_l, int_u):
    from helmholtz_3d_torrone_gb300 import geometry as G
    if case["shape"] == "sphere":
        return G.sphere(case["N"], radius=case["radius"], center=case["center"], int_l=int_l, int_u=int_u)
    return G.torus(case["N"], R=case["R"], r=case["r"], int_l=int_l, int_u=int_u)


def run_case(name):
    import oracle as O
    case = CASES[name]
    ref = O.Reference(case["variant"])
    N, k = case["N"], case["wave"]
    d = distance(case, ref.int_l, ref.int_u)
    # silence the reference's printf chatter
    devnull = os.open(os.devnull, os.O_WRONLY)
    os.dup2(devnull, 1)
    ref.setup(N, k, d)
    gx, gy, gz, mc, gc = ref.grids()
    idx = ref.tube()
    n = len(idx)
    tp = ref.tube_points(n)
    rng = np.random.default_rng(1234)
    pi = rng.integers(0, n, 512).astype(np.int32)
    pj = rng.integers(0, n, 512).astype(np.int32)
    pi[:16] = pj[:16]
    ent = ref.entries(n, pi, pj)
    are, aim = ref.dense(n)
    A = are + 1j * aim
    p = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    Ap = A @ p
    AHp = A.conj().T @ p
    orc = O.Oracle()
    par = ref.params(N, k)
    tpo = dict(xs=tp["xs"], nrm=tp["nrm"], w=tp["w"], reg=tp["reg"])
    b = orc.rhs(par, tpo, np.zeros(3), case["rhs_kind"])
    x = ref.compbicg(are, aim, b)
    fi = rng.standard_normal((64, 7))
    wv = np.array([ref.weno(f, 0.1, 5) for f in fi] + [ref.weno(f[:5], 0.1, 3) for f in fi])
    meta = dict(name=name, N=N, wave=k, int_l=ref.int_l, int_u=ref.int_u, factor=ref.factor,
                tau_factor=ref.tau_factor, dirichlet=ref.dirichlet, interior=ref.interior,
                rhs_kind=case["rhs_kind"], n=n)
    np.savez_compressed(os.path.join(HERE, name + ".npz"), d=d, gx=gx, gy=gy, gz=gz, mc=mc, gc=gc, idx=idx,
                        xs=tp["xs"], nrm=tp["nrm"], delta=tp["delta"], jac=tp["jac"], reg=tp["reg"], w=tp["w"],
                        pi=pi, pj=pj, entries=ent, p=p, Ap=Ap, AHp=AHp, b=b, x=x, weno_in=fi, weno_out=wv,
                        meta=json.dumps(meta))
    return name, n


def run_dense_case(name):
    import oracle as O
    case = DENSE_CASES[name]
    ref = O.Reference(case["variant"])
    N, k = case["N"], case["wave"]
    d = distance(case, ref.int_l, ref.int_u)
    devnull = os.open(os.devnull, os.O_WRONLY)
    os.dup2(devnull, 1)
    ref.setup(N, k, d)
    fl = ref.dense_flags()
    par = ref.params(N, k)
    H = par.H
    orc = O.Oracle()
    grids = list(ref.grids())
    rng = np.random.default_rng(4321)
    out = dict(d=d)

    def sample(K, n, tag):
        pi = rng.integers(0, n, 1024)
        pj = rng.integers(0, n, 1024)
        pi[:32] = pj[:32]
        v = rng.standard_normal(n) + 1j * rng.standard_normal(n)
        out[tag + "_pi"], out[tag + "_pj"] = pi, pj
        out[tag + "_entries"] = K[pi, pj]
        out[tag + "_v"] = v
        out[tag + "_Kv"] = K @ v

    def opts(delta0, eps, onesided, wavenum=k, eta=case["eta"]):
        return O.DenseOpts(delta0, eps, wavenum, eta, fl["poly"], fl["sine"], onesided, fl["combo_interior"],
                           fl["radius"], *fl["center"])

    eps = ref.ref_eps()
    od = opts(0.0, eps, fl["trad_onesided"])
    n_dl = orc.L.or_dense_points(O.DENSE_DOUBLE_LAYER, O.C.byref(par), O.C.byref(od), O._d(d),
                                 *[O._d(np.ascontiguousarray(g)) for g in grids], 0, None)
    pts, K = ref.double_layer(n_dl, eps)
    out["dl_pts"] = pts
    sample(K, n_dl, "dl")
    delta0, eps0 = 0.1 * H, np.sqrt(H)
    oc = opts(delta0, eps0, fl["combo_onesided"])
    n_c = orc.L.or_dense_points(O.DENSE_COMBO, O.C.byref(par), O.C.byref(oc), O._d(d),
                                *[O._d(np.ascontiguousarray(g)) for g in grids], 0, None)
    pts, KP, KS, regcount = ref.combo(n_c, delta0, eps0, k, case["eta"])
    out["combo_pts"] = pts
    sample(KS if fl["sine"] else KP, n_c, "combo")
    n_s = orc.L.or_dense_points(O.DENSE_SPHERE, O.C.byref(par), O.C.byref(oc), None, None, None, None, None, None,
                                0, None)
    pts, KP, KS = ref.sphere_kernel(n_s, delta0, eps0)
    out["sphere_pts"] = pts
    sample(KS if fl["sine"] else KP, n_s, "sphere")
    meta = dict(name=name, N=N, wave=k, int_l=ref.int_l, int_u=ref.int_u, factor=ref.factor,
                tau_factor=ref.tau_factor, dirichlet=ref.dirichlet, interior=ref.interior, epsilon=eps,
                delta0=delta0, epsilon0=eps0, eta=case["eta"], regcount=int(regcount), n_dl=int(n_dl),
                n_combo=int(n_c), n_sphere=int(n_s), flags={k2: (v if not isinstance(v, tuple) else list(v))
                                                           for k2, v in fl.items()})
    meta["flags"]["radius"] = float(fl["radius"])
    meta["flags"]["center"] = [float(c) for c in fl["center"]]
    np.savez_compressed(os.path.join(HERE, name + ".npz"), meta=json.dumps(meta), **out)
    return name, n_dl


# The at-scale configurations, too large to store: the reference's grid
# stages on the 256^3 torus (R=0.6, r=0.25, [-1,1]^3, tube 3h) pinned by
# SHA-256 digests of its exact outputs (grids, tube index list, x*, normals,
# Jacobian, regularisation factor) and a strided sample of delta and w (they
# hold cos(), which differs between libm and CUDA in the last bit).
DIGEST_CASES = {
    "ref_dirichlet_torus_n256_digest": dict(variant="dirichlet", N=256, wave=20.0, shape="torus", R=0.6, r=0.25,
                                            stride=97),
}


def digest(a):
    import hashlib
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def run_digest_case(name):
    import oracle as O
    case = DIGEST_CASES[name]
    ref = O.Reference(case["variant"])
    N, k = case["N"], case["wave"]
    d = distance(case, ref.int_l, ref.int_u)
    devnull = os.open(os.devnull, os.O_WRONLY)
    os.dup2(devnull, 1)
    ref.setup(N, k, d)
    out = {"d": digest(d)}
    for nm, g in zip(("gx", "gy", "gz", "mc", "gc"), ref.grids()):
        out[nm] = digest(g)
    idx = ref.tube()
    n = len(idx)
    out["idx"] = digest(idx.astype(np.int64))
    tp = ref.tube_points(n)
    for nm in ("xs", "nrm", "jac", "reg"):
        out[nm] = digest(tp[nm])
    st = case["stride"]
    meta = dict(name=name, N=N, wave=k, int_l=ref.int_l, int_u=ref.int_u, factor=ref.factor,
                tau_factor=ref.tau_factor, dirichlet=ref.dirichlet, interior=ref.interior, n=n, R=case["R"],
                r=case["r"], stride=st, flagged=int(tp["flagged"]), sha256=out)
    np.savez_compressed(os.path.join(HERE, name + ".npz"), meta=json.dumps(meta), delta=tp["delta"][::st],
                        w=tp["w"][::st])
    return name, n


# Benchmark configuration 1 solved by the reference: sphere R=0.5 at the
# origin on 64^3 over [-1,1]^3, tube 3h, k=5, Dirichlet data of a point
# source at the origin; the reference's dense matrix (omp_get_Ccomp) and its
# CompBiCG, run to 1e-13.  The input grid is regenerated by the test
# (geometry.sphere) and pinned by its digest; the density is stored.
SOLVE_CASES = {
    "ref_dirichlet_sphere_n64_solve": dict(variant="dirichlet", N=64, wave=5.0, shape="sphere", radius=0.5,
                                           center=(0.0, 0.0, 0.0), rhs_kind=0),
}


def run_solve_case(name):
    import oracle as O
    case = SOLVE_CASES[name]
    ref = O.Reference(case["variant"])
    N, k = case["N"], case["wave"]
    d = distance(case, ref.int_l, ref.int_u)
    devnull = os.open(os.devnull, os.O_WRONLY)
    os.dup2(devnull, 1)
    ref.setup(N, k, d)
    idx = ref.tube()
    n = len(idx)
    tp = ref.tube_points(n)
    are, aim = ref.dense(n)
    orc = O.Oracle()
    par = ref.params(N, k)
    b = orc.rhs(par, dict(xs=tp["xs"], nrm=tp["nrm"], w=tp["w"], reg=tp["reg"]), np.zeros(3), case["rhs_kind"])
    x = ref.compbicg(are, aim, b)
    del are, aim
    meta = dict(name=name, N=N, wave=k, int_l=ref.int_l, int_u=ref.int_u, factor=ref.factor,
                tau_factor=ref.tau_factor, dirichlet=ref.dirichlet, interior=ref.interior, n=n,
                radius=case["radius"], center=list(case["center"]), rhs_kind=case["rhs_kind"], acc=1e-13,
                sha256=dict(d=digest(d), idx=digest(idx.astype(np.int64)), b=digest(b)))
    np.savez_compressed(os.path.join(HERE, name + ".npz"), meta=json.dumps(meta), x=x)
    return name, n


# Godunov upwind |grad phi| (finite_difference3D.c:5-27), the Hamiltonian
# of the level-set reinitialisation: seeded one-sided derivatives with
# zeros and both signs mixed in, for signage -1, 0 and +1.
GODUNOV_CASES = {"ref_godunov": dict(variant="neumann", count=1500, seed=5)}


def run_godunov_case(name):
    import oracle as O
    case = GODUNOV_CASES[name]
    ref = O.Reference(case["variant"])
    rng = np.random.default_rng(case["seed"])
    x = rng.standard_normal((case["count"], 6))
    x[rng.random(x.shape) < 0.15] = 0.0
    sig = rng.choice([-1.0, 0.0, 1.0], size=case["count"])
    out = np.array([ref.godunov(s, *row) for s, row in zip(sig, x)])
    np.savez_compressed(os.path.join(HERE, name + ".npz"), signage=sig, derivs=x, out=out)
    return name


def main():
    # One process per case: the reference exits (status 0) on some inputs and
    # keeps per-process statics, so each case gets a fresh, time-limited child.
    names = sys.argv[1:] or (list(CASES) + list(DENSE_CASES) + list(GODUNOV_CASES) + list(DIGEST_CASES) +
                             list(SOLVE_CASES))
    for name in names:
        out = os.path.join(HERE, name + ".npz")
        if os.path.exists(out):
            os.remove(out)
        cmd = [sys.executable, os.path.abspath(__file__), "--one", name]
        r = subprocess.run(cmd, timeout=1800)
        if r.returncode != 0 or not os.path.exists(out):
            raise SystemExit("case %s failed (exit %d, output %s)" % (name, r.returncode,
                                                                   "present" if os.path.exists(out) else "missing"))
        print(name, "ok")


if __name__ == "__main__":
    if len(sys.argv) == 3 and sys.argv[1] == "--one":
        if sys.argv[2] in DENSE_CASES:
            run_dense_case(sys.argv[2])
        elif sys.argv[2] in GODUNOV_CASES:
            run_godunov_case(sys.argv[2])
        elif sys.argv[2] in DIGEST_CASES:
            run_digest_case(sys.argv[2])
        elif sys.argv[2] in SOLVE_CASES:
            run_solve_case(sys.argv[2])
        else:
            run_case(sys.argv[2])
    else:
        main()
