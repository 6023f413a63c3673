"""Adjoint gradients of the receiver misfit J = sum |u(x_m) - t_m|^2
(hz_misfit_gradient) against central finite differences of the FP64 solve:
with respect to the boundary data b (through a torch.autograd.Function and
torch.autograd.gradcheck), the wave number k, and the tube-point weights.
Tolerance 1e-5 relative, solves at 1e-13."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

N, K = 24, 4.0


def make_op(hz, wave=K):
    from helmholtz_3d_torrone_gb300 import geometry as G
    p = hz.params(N, wave, int_l=-1.0, int_u=1.0, factor=3.0, dirichlet=1)
    op = hz.Operator(p)
    op.set_distance(G.sphere(N, radius=0.5, center=(0.011, 0.017, 0.005)))
    op.build()
    return op


def problem(op, hz):
    from helmholtz_3d_torrone_gb300 import geometry as G
    rx = G.random_sphere_points(16, 0.9, seed=5)
    r = np.linalg.norm(rx - np.array([0.05, 0.0, 0.0]), axis=1)
    target = np.exp(1j * K * r) / (4 * np.pi * r)  # field of a slightly shifted source
    b = op.rhs_point_source(np.zeros(3), hz.RHS_POINT_DIRICHLET)
    return b, rx, target


def J_of(op, hz, b, rx, target):
    x, _ = op.solve(b, method=hz.BICG, precision=hz.PREC_F64, tol=1e-13)
    u = op.evaluate(rx, x, hz.DOUBLE_LAYER)
    return float(np.sum(np.abs(u - target) ** 2))


def test_gradient_wrt_boundary_data_gradcheck(hz):
    torch = pytest.importorskip("torch")
    op = make_op(hz)
    b, rx, target = problem(op, hz)
    f = hz.misfit_function(op, rx, target, method=hz.BICG, precision=hz.PREC_F64, tol=1e-13)
    # gradcheck on a few coordinates: perturb only a random subset of b
    rng = np.random.default_rng(1)
    idx = rng.choice(op.n, 6, replace=False)
    base_re, base_im = torch.tensor(b.real), torch.tensor(b.imag)

    def sub(vr, vi):
        br, bi = base_re.clone(), base_im.clone()
        br[idx] = vr
        bi[idx] = vi
        return f(br, bi)

    vr = base_re[idx].clone().requires_grad_(True)
    vi = base_im[idx].clone().requires_grad_(True)
    assert torch.autograd.gradcheck(sub, (vr, vi), eps=1e-6, atol=1e-9, rtol=1e-5)
    op.close()


def test_gradient_wrt_wave_number(hz):
    op = make_op(hz)
    b, rx, target = problem(op, hz)
    J, g, dk, gw, info = op.misfit_gradient(b, rx, target, method=hz.BICG, precision=hz.PREC_F64, tol=1e-13)
    assert abs(J - J_of(op, hz, b, rx, target)) < 1e-12 * J
    h = 1e-6
    jp = J_of(make_op(hz, K + h), hz, b, rx, target)
    jm = J_of(make_op(hz, K - h), hz, b, rx, target)
    fd = (jp - jm) / (2 * h)
    assert abs(dk - fd) < 1e-5 * abs(fd)
    op.close()


def test_gradient_wrt_weights(hz):
    """dJ/dw_s by the adjoint, checked along the direction that scales every
    weight by (1 + t): there A(t) = (1 + t) K W + I/2 and E(t) = (1 + t) E,
    so dJ/dt at t = 0 = sum_s w_s dJ/dw_s, compared with a central finite
    difference of dense solves built from the oracle's matrix."""
    op = make_op(hz)
    b, rx, target = problem(op, hz)
    J, g, dk, gw, info = op.misfit_gradient(b, rx, target, method=hz.BICG, precision=hz.PREC_F64, tol=1e-13)
    t = op.tube()
    directional = float(np.sum(t["w"] * gw))
    import oracle as O
    o = O.Oracle()
    po = O.Params(N, -1.0, 1.0, K, 3.0, 2.0, 1, 0)
    tp = {"xs": t["xs"], "nrm": t["nrm"], "reg": t["reg"], "w": t["w"]}
    are, aim = o.dense(po, tp)
    Kw = (are + 1j * aim) - 0.5 * np.eye(op.n)

    def Jt(eps):
        At = (1 + eps) * Kw + 0.5 * np.eye(op.n)
        x = np.linalg.solve(At, b)
        u = (1 + eps) * o.evaluate(po, tp, x, rx, True)
        return float(np.sum(np.abs(u - target) ** 2))

    fd = (Jt(1e-6) - Jt(-1e-6)) / 2e-6
    assert abs(directional - fd) < 1e-5 * abs(fd)
    op.close()
