"""Multi right-hand-side products and batched solves (one kernel evaluation
per pair for a block of right-hand sides), through the C ABI.

Tolerances: FP64 multi product vs single products 1e-12; FP32 multi vs FP64
2e-5; batched solves vs single solves 1e-7 (both stopped at 1e-9)."""
import numpy as np
import pytest

from conftest import golden, rel_err

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def torus_op(hz):
    from helmholtz_3d_torrone_gb300 import geometry as G
    N, k = 32, 4.0
    p = hz.params(N, k, int_l=-1.0, int_u=1.0, factor=3.0, dirichlet=1)
    op = hz.Operator(p)
    op.set_distance(G.torus(N, R=0.5, r=0.25))
    op.build()
    yield op
    op.close()


@pytest.mark.parametrize("nrhs", [1, 5, 8, 13])
def test_multi_products_match_single(hz, torus_op, nrhs):
    op = torus_op
    rng = np.random.default_rng(nrhs)
    P = rng.standard_normal((nrhs, op.n)) + 1j * rng.standard_normal((nrhs, op.n))
    Q64 = op.matvec_multi(P, precision=hz.PREC_F64)
    Q32 = op.matvec_multi(P, precision=hz.PREC_F32)
    for r in range(nrhs):
        q = op.matvec(P[r], precision=hz.PREC_F64)
        assert rel_err(Q64[r], q) < 1e-12
        assert rel_err(Q32[r], q) < 2e-5


def test_plane_wave_rhs(hz, torus_op):
    from helmholtz_3d_torrone_gb300 import geometry as G
    op = torus_op
    dirs = G.fibonacci_sphere(6)
    t = op.tube()
    k = op.p.wave
    B = op.rhs_plane_waves(dirs)
    expect = np.exp(1j * k * (t["xs"] @ dirs.T)).T
    assert rel_err(B, expect) < 1e-13
    Bn = op.rhs_plane_waves(dirs, kind=hz.RHS_POINT_NEUMANN)
    dn = -(t["nrm"] @ dirs.T).T
    assert rel_err(Bn, 1j * k * dn * expect) < 1e-13


@pytest.mark.parametrize("precision", ["f64", "refined"])
def test_batched_solve_matches_single(hz, torus_op, precision):
    from helmholtz_3d_torrone_gb300 import geometry as G
    op = torus_op
    dirs = G.fibonacci_sphere(10)
    B = op.rhs_plane_waves(dirs)
    prec = hz.PREC_F64 if precision == "f64" else hz.PREC_F32_REFINED
    X, info, res = op.solve_multi(B, method=hz.BICGSTAB, precision=prec, tol=1e-9, inner_tol=1e-5)
    assert np.all(res < 1e-9)
    for r in [0, 4, 9]:
        x, _ = op.solve(B[r], method=hz.BICGSTAB, precision=hz.PREC_F64, tol=1e-9)
        assert rel_err(X[r], x) < 1e-7


@pytest.mark.parametrize("precision", ["f64", "refined"])
def test_multi_columns_leave_when_converged(hz, torus_op, precision):
    """A zero column and columns of different difficulty (plane waves and a
    point source): stopped columns leave the packed sweep, the others still
    equal their single solves, and the zero column stays zero."""
    from helmholtz_3d_torrone_gb300 import geometry as G
    op = torus_op
    B = op.rhs_plane_waves(G.fibonacci_sphere(10))
    B[3] = 0.0
    B[7] = op.rhs_point_source(np.array([0.5, 0.0, 0.0]), hz.RHS_POINT_DIRICHLET)
    prec = hz.PREC_F64 if precision == "f64" else hz.PREC_F32_REFINED
    X, info, res = op.solve_multi(B, method=hz.BICGSTAB, precision=prec, tol=1e-9, inner_tol=1e-5)
    assert np.all(res < 1e-9)
    assert not np.any(X[3])
    passes = 1  # 10 columns fit one pass of the 16-column block (FP32 and FP64)
    assert info["pair_evals"] <= (2 * info["iterations"] + info["outer"]) * op.n * op.n * passes
    for r in [0, 7, 9]:
        x, _ = op.solve(B[r], method=hz.BICGSTAB, precision=hz.PREC_F64, tol=1e-9)
        assert rel_err(X[r], x) < 1e-7
