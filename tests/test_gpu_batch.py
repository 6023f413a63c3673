"""Batches of independent operators (hz_batch_*): uneven ellipsoids with
different grids and wave numbers.

* FP32 batched product (one persistent launch over all operators) equals
  each operator's own FP32 product with the direct phase (the batch sweep's)
  to 1e-10 (same tiles; only the grouping of cross-tile sums differs) for
  every batch sweep shape;
* FP64 batched product equals each operator's FP64 product bit for bit;
* the batched FP32 + FP64-refinement BiCGSTAB solve equals each operator's
  FP64 solve to 1e-8 (both to 1e-11).
"""
import numpy as np
import pytest

from conftest import rel_err

pytestmark = pytest.mark.gpu

# grids fine enough that the 3h tube keeps the WENO stencils off each
# ellipsoid's medial surface (coarser ones project points off the grid, where
# the reference exits as well)
CASES = [(32, (0.7, 0.5, 0.4), 4.0), (40, (0.45, 0.6, 0.3), 5.0), (56, (0.3, 0.35, 0.5), 6.0),
         (20, (0.5, 0.5, 0.5), 3.0)]


@pytest.fixture(scope="module")
def batch(hz):
    from helmholtz_3d_torrone_gb300 import geometry as G
    ops = []
    for N, axes, k in CASES:
        op = hz.Operator(hz.params(N, k, int_l=-1.0, int_u=1.0, factor=3.0, dirichlet=1))
        op.set_distance(G.ellipsoid(N, axes=axes))
        op.build()
        ops.append(op)
    b = hz.Batch(ops)
    yield b, ops
    b.close()
    for op in ops:
        op.close()


def test_batch_products(hz, batch):
    b, ops = batch
    rng = np.random.default_rng(11)
    vs = [rng.standard_normal(op.n) + 1j * rng.standard_normal(op.n) for op in ops]
    q64 = b.matvec(vs, precision=hz.PREC_F64)
    for op, v, q in zip(ops, vs, q64):
        assert np.array_equal(q, op.matvec(v, precision=hz.PREC_F64))
    # the batch sweep reduces the phase directly (HZ_PHASE_DIRECT); compare
    # with each operator's own FP32 product in that mode
    for op in ops:
        op.set_phase_mode(hz.PHASE_DIRECT)
    ref32 = [op.matvec(v, precision=hz.PREC_F32) for op, v in zip(ops, vs)]
    for op in ops:
        op.set_phase_mode(hz.PHASE_SPLIT)
    for shape in range(4):
        b.set_variant(shape)
        q32 = b.matvec(vs, precision=hz.PREC_F32)
        for q, r, q6 in zip(q32, ref32, q64):
            assert rel_err(q, r) <= 1e-10, shape
            assert rel_err(q, q6) <= 2e-5, shape
    best, ms = b.autotune()
    assert 0 <= best < 4 and ms > 0


def test_batch_refined_solve(hz, batch):
    b, ops = batch
    bs = [op.rhs_point_source(np.array([0.05, 0.02, 0.01]), hz.RHS_POINT_DIRICHLET) for op in ops]
    xs, info, res = b.solve(bs, precision=hz.PREC_F32_REFINED, tol=1e-11, inner_tol=1e-5, maxit=400)
    assert np.all(res < 1e-11) and info["outer"] >= 1
    for op, rhs, x in zip(ops, bs, xs):
        x64, i64 = op.solve(rhs, method=hz.BICGSTAB, precision=hz.PREC_F64, tol=1e-12)
        assert rel_err(x, x64) < 1e-8


@pytest.mark.parametrize("precision", ["f64", "refined"])
def test_batch_columns_leave_when_converged(hz, batch, precision):
    """A zero right-hand side never iterates and the others stop at their own
    iteration counts: the launch is re-described over the columns still
    iterating, so the pairs evaluated are fewer than lockstep would take,
    and every system still equals its own FP64 solve."""
    b, ops = batch
    bs = [op.rhs_point_source(np.array([0.05, 0.02, 0.01]), hz.RHS_POINT_DIRICHLET) for op in ops]
    bs[1] = np.zeros_like(bs[1])
    prec = hz.PREC_F64 if precision == "f64" else hz.PREC_F32_REFINED
    xs, info, res = b.solve(bs, precision=prec, tol=1e-11, inner_tol=1e-5, maxit=400)
    assert np.all(res < 1e-11)
    assert not np.any(xs[1])
    sq = sum(op.n * op.n for i, op in enumerate(ops) if i != 1)
    lockstep = 2 * info["iterations"] * sq + info["outer"] * sq
    assert info["pair_evals"] < lockstep
    for i, (op, rhs, x) in enumerate(zip(ops, bs, xs)):
        if i == 1:
            continue
        x64, _ = op.solve(rhs, method=hz.BICGSTAB, precision=hz.PREC_F64, tol=1e-12)
        assert rel_err(x, x64) < 1e-8
