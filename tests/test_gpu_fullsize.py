"""Size-independent properties at the benchmark's full size: the torus
R = 0.6, r = 0.25 on 256^3 over [-1,1]^3, tube 3h (n = 581,420), k = 20.

* The tube index list is the lexicographic list of nodes with
  |phi| <= 3h, bit for bit (the reference's rule, large3Dexample2.c:548-597;
  at 256^3 h and 3h are exact binary fractions, so numpy's comparison is
  the same comparison).
* The FP32 fused sweep is linear: A(p + 2i q) = A p + 2i A q to FP32
  rounding (2e-6 of the norms).
* The fused sweep's two products are adjoint: <A p, w> = <p, A^H w> to
  FP32 rounding (1e-5 relative).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

N, K = 256, 20.0


@pytest.fixture(scope="module")
def full(hz):
    from helmholtz_3d_torrone_gb300 import geometry as G
    d = G.torus(N, R=0.6, r=0.25, int_l=-1.0, int_u=1.0)
    p = hz.params(N, K, int_l=-1.0, int_u=1.0, factor=3.0, tau_factor=2.0, dirichlet=1)
    op = hz.Operator(p)
    op.set_distance(d)
    op.build()
    yield op, d
    op.close()


def test_tube_index_list_full_size(full):
    op, d = full
    eps = 3.0 * (2.0 / N)
    expect = np.flatnonzero(np.abs(d).ravel() <= eps)
    assert op.n == expect.size == 581420
    assert np.array_equal(op.tube()["idx"], expect)


def test_fp32_sweep_linear_and_adjoint_full_size(hz, full):
    op, d = full
    rng = np.random.default_rng(256)
    p = rng.standard_normal(op.n) + 1j * rng.standard_normal(op.n)
    q = rng.standard_normal(op.n) + 1j * rng.standard_normal(op.n)
    w = rng.standard_normal(op.n) + 1j * rng.standard_normal(op.n)
    Ap, AHw = op.matvec_pair(p, w, precision=hz.PREC_F32)
    Aq = op.matvec(q, precision=hz.PREC_F32)
    Apq = op.matvec(p + 2j * q, precision=hz.PREC_F32)
    scale = np.linalg.norm(Ap) + 2 * np.linalg.norm(Aq)
    assert np.linalg.norm(Apq - (Ap + 2j * Aq)) <= 2e-6 * scale
    lhs, rhs = np.vdot(w, Ap), np.vdot(AHw, p)
    assert abs(lhs - rhs) <= 1e-5 * max(abs(lhs), np.linalg.norm(Ap) * np.linalg.norm(w) * 1e-3)
