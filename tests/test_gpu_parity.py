"""GPU parity: the CUDA path through the C ABI against the reference's golden
vectors and against the CPU oracle.

Tolerances:
  * grids (WENO gradient, curvatures), tube index list, x*, normals,
    Jacobian and regularisation factors: bit-exact (same FP64 operation
    order, no fused multiply-add);
  * delta_eps and w: 1e-15 relative (CUDA cos vs. the C library's);
  * FP64 matvec: 1e-12 relative (summation order differs);
  * FP64 BiCG density solved to 1e-13: 1e-10 relative (spec bound);
  * GMRES (FP64 or FP32 + FP64 refinement) to 1e-12 / 1e-11: 1e-9 relative;
  * FP32 sweep vs FP64: 2e-5 relative (FP32 arithmetic).
"""
import json

import numpy as np
import pytest

from conftest import golden, rel_err

pytestmark = pytest.mark.gpu

CASES = ["ref_neumann_sphere_n16", "ref_neumann_sphere_n24", "ref_dirichlet_sphere_n20",
         "ref_dirichlet_torus_n32"]


def hz_params_of(hz, g):
    m = json.loads(str(g["meta"]))
    return hz.params(m["N"], m["wave"], int_l=m["int_l"], int_u=m["int_u"], factor=m["factor"],
                     tau_factor=m["tau_factor"], dirichlet=m["dirichlet"], interior=m["interior"]), m


def bits_equal(a, b):
    return np.array_equal(np.ascontiguousarray(a).view(np.uint64), np.ascontiguousarray(b).view(np.uint64))


@pytest.fixture(scope="module")
def built(hz):
    ops = {}
    for case in CASES:
        g = golden(case)
        p, m = hz_params_of(hz, g)
        op = hz.Operator(p)
        op.set_distance(g["d"])
        op.build()
        ops[case] = (op, g, m)
    yield ops
    for op, _, _ in ops.values():
        op.close()


@pytest.mark.parametrize("case", CASES)
def test_grids_bitexact_vs_reference(built, case):
    op, g, m = built[case]
    gx, gy, gz, mc, gc = op.grids()
    for key, a in [("gx", gx), ("gy", gy), ("gz", gz), ("mc", mc), ("gc", gc)]:
        assert bits_equal(a, g[key]), key


@pytest.mark.parametrize("case", CASES)
def test_tube_bitexact_vs_reference(built, case):
    op, g, m = built[case]
    t = op.tube()
    assert op.n == m["n"]
    assert np.array_equal(t["idx"], g["idx"])
    for key in ["xs", "nrm", "jac", "reg"]:
        assert bits_equal(t[key], g[key]), key
    for key in ["delta", "w"]:
        assert rel_err(t[key], g[key]) < 1e-15, key


@pytest.mark.parametrize("case", CASES)
def test_matvec_f64_vs_reference(hz, built, case):
    op, g, m = built[case]
    q = op.matvec(g["p"], precision=hz.PREC_F64)
    qh = op.matvec(g["p"], precision=hz.PREC_F64, adjoint=True)
    assert rel_err(q, g["Ap"]) < 1e-12
    assert rel_err(qh, g["AHp"]) < 1e-12
    q2, qh2 = op.matvec_pair(g["p"], g["p"], precision=hz.PREC_F64)
    assert rel_err(q2, g["Ap"]) < 1e-12
    assert rel_err(qh2, g["AHp"]) < 1e-12


@pytest.mark.parametrize("case", CASES)
def test_matvec_f32_close_to_f64(hz, built, case):
    op, g, m = built[case]
    q = op.matvec(g["p"], precision=hz.PREC_F32)
    qh = op.matvec(g["p"], precision=hz.PREC_F32, adjoint=True)
    assert rel_err(q, g["Ap"]) < 2e-5
    assert rel_err(qh, g["AHp"]) < 2e-5
    q2, qh2 = op.matvec_pair(g["p"], g["p"], precision=hz.PREC_F32)
    assert rel_err(q2, g["Ap"]) < 2e-5
    assert rel_err(qh2, g["AHp"]) < 2e-5


def test_every_sweep_variant_and_autotune(hz, built):
    """Each compiled FP32 sweep variant gives the reference's products to
    FP32 accuracy; the autotuner (and timed products) run outside a graph."""
    op, g, m = built["ref_dirichlet_torus_n32"]
    cfg = 0
    while True:
        try:
            op.set_sweep_config(cfg)
        except hz.HzError:
            break
        q, qh = op.matvec_pair(g["p"], g["p"], precision=hz.PREC_F32)
        assert rel_err(q, g["Ap"]) < 2e-5, cfg
        assert rel_err(qh, g["AHp"]) < 2e-5, cfg
        assert rel_err(op.matvec(g["p"], precision=hz.PREC_F32), g["Ap"]) < 2e-5, cfg
        cfg += 1
    assert cfg >= 4
    best, ms = op.autotune()
    assert 0 <= best < cfg and ms > 0
    op.sweep_timing(1)
    q = op.matvec(g["p"], precision=hz.PREC_F32)
    t, k = op.sweep_timing(-1)
    op.sweep_timing(0)
    assert k >= 1 and t > 0
    assert rel_err(q, g["Ap"]) < 2e-5


@pytest.mark.parametrize("case", CASES)
def test_bicg_f64_vs_reference_compbicg(hz, built, case):
    op, g, m = built[case]
    b = op.rhs_point_source(np.zeros(3), m["rhs_kind"])
    assert rel_err(b, g["b"]) < 1e-14
    x, info = op.solve(g["b"], method=hz.BICG, precision=hz.PREC_F64, tol=1e-13, maxit=2000, stagnation=1)
    assert info["resid"] < 1e-12
    assert rel_err(x, g["x"]) < 1e-10


@pytest.mark.parametrize("case", CASES)
def test_bicgstab_and_refined_agree(hz, built, case):
    op, g, m = built[case]
    x64, i64 = op.solve(g["b"], method=hz.BICGSTAB, precision=hz.PREC_F64, tol=1e-12)
    assert rel_err(x64, g["x"]) < 1e-9
    xr, ir = op.solve(g["b"], method=hz.BICG, precision=hz.PREC_F32_REFINED, tol=1e-11, inner_tol=1e-5)
    assert ir["resid_f64"] < 1e-11
    assert rel_err(xr, g["x"]) < 1e-9
    xs, iS = op.solve(g["b"], method=hz.BICGSTAB, precision=hz.PREC_F32_REFINED, tol=1e-11, inner_tol=1e-5)
    assert rel_err(xs, g["x"]) < 1e-9


@pytest.mark.parametrize("case", CASES)
def test_gmres_vs_reference(hz, built, case):
    """Restarted GMRES (FP64, and as the inner solver of the refinement)
    reaches the reference's CompBiCG density; its recurrence residual is the
    true FP64 residual."""
    op, g, m = built[case]
    b = g["b"]
    x, info = op.solve(b, method=hz.GMRES, precision=hz.PREC_F64, tol=1e-12, restart=20)
    assert info["resid"] < 1e-12
    true = np.linalg.norm(b - op.matvec(x)) / np.linalg.norm(b)
    assert true < 5e-12
    assert rel_err(x, g["x"]) < 1e-9
    xr, ir = op.solve(b, method=hz.GMRES, precision=hz.PREC_F32_REFINED, tol=1e-11, inner_tol=1e-5, restart=20)
    assert ir["resid_f64"] < 1e-11 and ir["outer"] >= 1
    assert rel_err(xr, g["x"]) < 1e-9


def test_stencils_standalone_bitexact(hz):
    g = golden("ref_neumann_sphere_n24")
    m = json.loads(str(g["meta"]))
    H = (m["int_u"] - m["int_l"]) / m["N"]
    gx, gy, gz = hz.assign_gradient(g["d"], m["N"], H)
    mc, gc = hz.assign_curvatures(g["d"], m["N"], H)
    for key, a in [("gx", gx), ("gy", gy), ("gz", gz), ("mc", mc), ("gc", gc)]:
        assert bits_equal(a, g[key]), key


def test_dense_bicg_vs_reference(hz):
    g = golden("ref_neumann_sphere_n16")
    import oracle as O
    o = O.Oracle()
    m = json.loads(str(g["meta"]))
    p = O.Params(m["N"], m["int_l"], m["int_u"], m["wave"], m["factor"], m["tau_factor"], m["dirichlet"],
                 m["interior"])
    tp = {k: g[k] for k in ["xs", "nrm", "reg", "w"]}
    are, aim = o.dense(p, tp)
    x, info = hz.dense_bicg(are + 1j * aim, g["b"], tol=1e-13, maxit=1000)
    assert rel_err(x, g["x"]) < 1e-10


def test_phase_split_mode(hz):
    """hz_set_phase_mode: the FP32 sweep with the phase reduced through a
    split k/(2 pi) stays within the FP32 bound of the FP64 product (A, A^H
    and the fused pair), and a refined solve in that mode equals the FP64
    solve."""
    from helmholtz_3d_torrone_gb300 import geometry as G
    N, k = 32, 20.0
    p = hz.params(N, k, int_l=-1.0, int_u=1.0, factor=3.0, dirichlet=1)
    with hz.Operator(p) as op:
        # the multi right-hand-side tests' torus: on this grid every
        # projected point and its interpolation cell lie inside [-1,1]^3
        op.set_distance(G.torus(N, R=0.5, r=0.25))
        op.build()
        rng = np.random.default_rng(7)
        v = rng.standard_normal(op.n) + 1j * rng.standard_normal(op.n)
        q64, qt64 = op.matvec(v), op.matvec(v, adjoint=True)
        errs = {}
        for mode in (hz.PHASE_DIRECT, hz.PHASE_SPLIT):
            op.set_phase_mode(mode)
            q, qt = op.matvec_pair(v, v, precision=hz.PREC_F32)
            assert rel_err(q, q64) <= 2e-5 and rel_err(qt, qt64) <= 2e-5
            assert rel_err(op.matvec(v, precision=hz.PREC_F32), q64) <= 2e-5
            errs[mode] = rel_err(q, q64)
        op.set_phase_mode(hz.PHASE_SPLIT)
        b = op.rhs_point_source(np.array([0.5, 0.0, 0.0]), hz.RHS_POINT_DIRICHLET)
        x, info = op.solve(b, method=hz.BICG, precision=hz.PREC_F32_REFINED, tol=1e-11)
        x64, _ = op.solve(b, method=hz.BICG, precision=hz.PREC_F64, tol=1e-12)
        assert rel_err(x, x64) < 1e-8
        with pytest.raises(hz.HzError):
            op.set_phase_mode(2)
