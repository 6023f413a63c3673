"""Error paths of the C ABI, with the faults injected from the host.

Each case feeds the library an input that the reference would stop on and
checks the status code the C ABI returns instead, then checks that the
operator (and its CUDA context) still works:

* a NaN in the right-hand side: the reference's NaN guard exits
  (large3Dexample2.c:2641); here hz_solve returns HZ_ERR_NONFINITE;
* a corrupted distance grid whose projected point x* = z - d grad d leaves
  the grid: the reference exits in cal_interpgrad (interpolate3D.c:21-36);
  here hz_build returns HZ_ERR_GRID;
* a right-hand side with sum b_i^2 = 0, so that BiCG's first <r, rt> is zero
  (rt0 = conj(b), BICGSTAB.c:104-130): the reference divides by zero; here
  the solve stops with HZ_ERR_BREAKDOWN;
* a data wait of the pair sweeps that runs out (poll limit 0 set by
  hz_set_wait_limit): the CTA lets its copies in flight land and exits, the
  call returns HZ_ERR_DEVICE_WAIT, and with the default limit restored the
  same product is computed correctly.

No case faults, traps or hangs the GPU.
"""
import numpy as np
import pytest

from conftest import rel_err

pytestmark = pytest.mark.gpu

N, K = 20, 5.0


def _sphere(hz):
    from helmholtz_3d_torrone_gb300 import geometry as G
    d = G.sphere(N, radius=0.5, center=(0.011, 0.017, 0.005))
    p = hz.params(N, K, int_l=-1.0, int_u=1.0, factor=3.0, tau_factor=2.0, dirichlet=1)
    return p, d


def test_nan_rhs_gives_nonfinite(hz):
    p, d = _sphere(hz)
    with hz.Operator(p) as op:
        op.set_distance(d)
        n = op.build()
        b = op.rhs_point_source(np.zeros(3), hz.RHS_POINT_DIRICHLET)
        bad = b.copy()
        bad[n // 3] = complex(np.nan, 0.0)
        for method, prec in ((hz.BICG, hz.PREC_F64), (hz.GMRES, hz.PREC_F64), (hz.BICG, hz.PREC_F32_REFINED)):
            with pytest.raises(hz.HzError) as e:
                op.solve(bad, method=method, precision=prec, tol=1e-10)
            assert e.value.code == hz.HZ_ERR_NONFINITE, (method, prec)
        # the operator still solves clean data
        x, info = op.solve(b, method=hz.BICG, precision=hz.PREC_F64, tol=1e-10)
        assert info["converged"] == 1 and info["resid"] < 1e-10


def _corrupted(d):
    """The distance grid with one node outside the tube raised to +40, next to
    a tube node at |d| ~ 2.3h: every WENO5 forward difference of that node
    sees the spike, its gradient becomes ~190 and its projection lands near
    x = 44, far outside [-1, 1]^3."""
    d2 = d.copy()
    d2[8, 18, 9] = 40.0
    return d2


def test_offgrid_projection_gives_grid_error(hz, oracle):
    import oracle as O
    p, d = _sphere(hz)
    d2 = _corrupted(d)
    # the oracle (the reference's cell test, interpolate3D.c:21-36) flags it
    tp = oracle.pipeline(O.make_params(N, K), d2)
    assert tp["bad"] > 0
    with hz.Operator(p) as op:
        op.set_distance(d2)
        with pytest.raises(hz.HzError) as e:
            op.build()
        assert e.value.code == hz.HZ_ERR_GRID
        # a clean grid builds on the same operator afterwards
        op.set_distance(d)
        assert op.build() == len(oracle.pipeline(O.make_params(N, K), d)["idx"])


def test_zero_rho_rhs_gives_breakdown(hz):
    p, d = _sphere(hz)
    with hz.Operator(p) as op:
        op.set_distance(d)
        n = op.build()
        b = np.zeros(n, dtype=complex)
        b[0], b[1] = 1.0, 1j  # sum b_i^2 = 1 - 1 = 0 exactly: <r0, rt0> = 0
        assert np.sum(b * b) == 0
        with pytest.raises(hz.HzError) as e:
            op.solve(b, method=hz.BICG, precision=hz.PREC_F64, tol=1e-10)
        assert e.value.code == hz.HZ_ERR_BREAKDOWN


def test_data_wait_runs_out(hz):
    p, d = _sphere(hz)
    rng = np.random.default_rng(3)
    with hz.Operator(p) as op:
        op.set_distance(d)
        n = op.build()
        v = rng.standard_normal(n) + 1j * rng.standard_normal(n)
        want = {prec: op.matvec(v, precision=prec) for prec in (hz.PREC_F64, hz.PREC_F32)}
        try:
            hz.set_wait_limit(0)  # every data wait gives up before its first poll
            for prec in (hz.PREC_F64, hz.PREC_F32):
                with pytest.raises(hz.HzError) as e:
                    op.matvec(v, precision=prec)
                assert e.value.code == hz.HZ_ERR_DEVICE_WAIT, prec
        finally:
            hz.set_wait_limit(-1)
        # the context is intact and the default limit gives the same products
        for prec in (hz.PREC_F64, hz.PREC_F32):
            assert rel_err(op.matvec(v, precision=prec), want[prec]) < 1e-15
