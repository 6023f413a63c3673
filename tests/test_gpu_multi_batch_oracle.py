"""Multi right-hand-side and batched products and solves against the oracle
(the pinned FP64 C restatement of the reference, oracle/ibim_oracle.c), not
against this library's single-vector path.

* every column of a 13-column multi-RHS block (FP64 and FP32 passes) against
  the oracle's product of that column: 1e-12 (FP64), 2e-5 (FP32);
* every operator of an uneven batch (one persistent launch over four
  ellipsoids with different grids and wave numbers) against the oracle's
  product on that operator's own tube: 1e-12 (FP64), 2e-5 (FP32);
* lockstep multi-RHS solves of five plane waves (BiCGSTAB and GMRES, FP32 +
  FP64 refinement to 1e-11, and plain FP64 GMRES to 1e-12) against the
  oracle's BiCG solve of each wave to 1e-13: 1e-8.
"""
import numpy as np
import pytest

from conftest import rel_err

pytestmark = pytest.mark.gpu


def _oracle_params(O, N, k):
    return O.Params(N, -1.0, 1.0, k, 3.0, 2.0, 1, 0)


def test_multi_rhs_columns_vs_oracle(hz, oracle):
    import oracle as O
    from helmholtz_3d_torrone_gb300 import geometry as G
    N, k = 32, 4.0
    d = G.torus(N, R=0.5, r=0.25)
    with hz.Operator(hz.params(N, k, int_l=-1.0, int_u=1.0, factor=3.0, dirichlet=1)) as op:
        op.set_distance(d)
        op.build()
        po = _oracle_params(O, N, k)
        tp = oracle.pipeline(po, d)
        assert np.array_equal(tp["idx"], op.tube()["idx"])
        rng = np.random.default_rng(13)
        P = rng.standard_normal((13, op.n)) + 1j * rng.standard_normal((13, op.n))
        Q64 = op.matvec_multi(P, precision=hz.PREC_F64)
        Q32 = op.matvec_multi(P, precision=hz.PREC_F32)
        for r in range(P.shape[0]):
            qo = oracle.matvec(po, tp, P[r])
            assert rel_err(Q64[r], qo) < 1e-12, r
            assert rel_err(Q32[r], qo) < 2e-5, r
        # lockstep refined solve of plane waves against the oracle's solves
        dirs = G.fibonacci_sphere(5)
        B = op.rhs_plane_waves(dirs)
        xos = [oracle.bicg(po, tp, B[r], acc=1e-13)[0] for r in range(B.shape[0])]
        runs = [dict(method=hz.BICGSTAB, precision=hz.PREC_F32_REFINED, tol=1e-11, inner_tol=1e-5),
                dict(method=hz.GMRES, precision=hz.PREC_F32_REFINED, tol=1e-11, inner_tol=1e-5, restart=40),
                dict(method=hz.GMRES, precision=hz.PREC_F64, tol=1e-12, restart=30)]
        for kw in runs:
            X, info, res = op.solve_multi(B, **kw)
            assert np.all(res < kw["tol"]), (kw, res)
            for r in range(B.shape[0]):
                assert rel_err(X[r], xos[r]) < 1e-8, (kw, r)


def test_batch_products_vs_oracle(hz, oracle):
    import oracle as O
    from helmholtz_3d_torrone_gb300 import geometry as G
    cases = [(32, (0.7, 0.5, 0.4), 4.0), (40, (0.45, 0.6, 0.3), 5.0), (20, (0.5, 0.5, 0.5), 3.0)]
    ops, tps, pos, ds = [], [], [], []
    for N, axes, k in cases:
        d = G.ellipsoid(N, axes=axes)
        op = hz.Operator(hz.params(N, k, int_l=-1.0, int_u=1.0, factor=3.0, dirichlet=1))
        op.set_distance(d)
        op.build()
        ops.append(op)
        po = _oracle_params(O, N, k)
        pos.append(po)
        tps.append(oracle.pipeline(po, d))
    b = hz.Batch(ops)
    try:
        rng = np.random.default_rng(17)
        vs = [rng.standard_normal(op.n) + 1j * rng.standard_normal(op.n) for op in ops]
        q64 = b.matvec(vs, precision=hz.PREC_F64)
        q32 = b.matvec(vs, precision=hz.PREC_F32)
        for po, tp, v, a, c in zip(pos, tps, vs, q64, q32):
            qo = oracle.matvec(po, tp, v)
            assert rel_err(a, qo) < 1e-12
            assert rel_err(c, qo) < 2e-5
    finally:
        b.close()
        for op in ops:
            op.close()
