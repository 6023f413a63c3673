"""Adjoint gradients against central finite differences of the reference's
own FP64 C solve.

J = sum_m |u(x_m) - t_m|^2.  The forward values in the differences come from
the reference build (oracle/_ref, run in child processes by
oracle/ref_worker.py): its grids, tube and per-point set-up
(ASSIGN_GRADIENT, BothCurvs, large3Dexample2.c:548-597,4340-4452), its dense
matrix of omp_get_Ccomp entries (:4463-4564) and CompBiCG
(BICGSTAB.c:5-339) to 1e-13; the receiver field is the double-layer sum
(:1810-1824, oracle restatement) over the reference's tube points.  The
gradients under test come from the GPU (hz_misfit_gradient,
hz_shape_gradient).

* dJ/db: torch.autograd.gradcheck of a Function whose forward is the
  reference solve and whose backward is the GPU adjoint (step 1e-6,
  rtol 1e-5);
* dJ/dk (b held fixed): central difference, step 1e-6, within 1e-5;
* dJ/dphi at grid nodes: central differences, step 1e-6, of reference
  solves of the perturbed grid (b = point-source data at the perturbed
  projections).  J is only piecewise smooth in phi (a pair crossing the
  near-field radius, an upwind or limiter branch flipping), so a node is
  kept where the quotients with steps 1e-6 and 2e-6 agree to 1e-5 of the
  largest quotient.  Where no branch lies near the node the GPU gradient
  equals the quotient to about 1e-8 of the largest one; a branch within a
  step of the node bends both quotients alike, so it passes that screen
  while the adjoint (the derivative on one side) differs by up to a few
  1e-5.  The test asks for 1e-6 on at least 8 nodes and 1e-4 on all.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

H_FD = 1e-6


def _ref_field(O, oracle, tube, x, N, k, rx):
    p = O.Params(N, -1.0, 1.0, k, 3.0, 2.0, 1, 0)
    return oracle.evaluate(p, tube, x, rx, True)


@pytest.fixture(scope="module")
def sphere24(hz):
    from helmholtz_3d_torrone_gb300 import geometry as G
    N, K = 24, 4.0
    d = G.sphere(N, radius=0.5, center=(0.011, 0.017, 0.005))
    rx = G.random_sphere_points(16, 0.9, seed=5)
    r = np.linalg.norm(rx - np.array([0.05, 0.0, 0.0]), axis=1)
    target = np.exp(1j * K * r) / (4 * np.pi * r)
    p = hz.params(N, K, int_l=-1.0, int_u=1.0, factor=3.0, dirichlet=1)
    op = hz.Operator(p)
    op.set_distance(d)
    op.build()
    b = op.rhs_point_source(np.zeros(3), hz.RHS_POINT_DIRICHLET)
    yield dict(op=op, d=d, rx=rx, target=target, b=b, N=N, K=K)
    op.close()


def test_dJ_db_gradcheck_vs_reference_solve(hz, oracle, sphere24):
    torch = pytest.importorskip("torch")
    import oracle as O
    from oracle.ref_worker import RefWorker
    c = sphere24
    op, b, rx, target, N, K = c["op"], c["b"], c["rx"], c["target"], c["N"], c["K"]
    rng = np.random.default_rng(1)
    idx = rng.choice(op.n, 6, replace=False)
    with RefWorker("dirichlet", N, K, c["d"]) as ref:
        assert ref.tube["n"] == op.n
        assert np.array_equal(ref.tube["idx"], op.tube()["idx"])

        def full_b(vr, vi):
            bb = b.copy()
            bb[idx] = vr.detach().numpy() + 1j * vi.detach().numpy()
            return bb

        class RefMisfit(torch.autograd.Function):
            @staticmethod
            def forward(ctx, vr, vi):
                bb = full_b(vr, vi)
                ctx.b = bb
                u = _ref_field(O, oracle, ref.tube, ref.solve(bb), N, K, rx)
                return torch.tensor(float(np.sum(np.abs(u - target) ** 2)), dtype=torch.float64)

            @staticmethod
            def backward(ctx, g_out):
                J, g, dk, gw, info = op.misfit_gradient(ctx.b, rx, target, method=hz.BICG, precision=hz.PREC_F64,
                                                        tol=1e-13)
                return g_out * torch.from_numpy(g.real[idx].copy()), g_out * torch.from_numpy(g.imag[idx].copy())

        vr = torch.tensor(b.real[idx]).requires_grad_(True)
        vi = torch.tensor(b.imag[idx]).requires_grad_(True)
        assert torch.autograd.gradcheck(RefMisfit.apply, (vr, vi), eps=H_FD, atol=1e-9, rtol=1e-5)
        # the GPU's J equals the reference's at the base point
        J, _, _, _, _ = op.misfit_gradient(b, rx, target, method=hz.BICG, precision=hz.PREC_F64, tol=1e-13)
        u = _ref_field(O, oracle, ref.tube, ref.solve(b), N, K, rx)
        Jr = float(np.sum(np.abs(u - target) ** 2))
        assert abs(J - Jr) <= 1e-10 * Jr


def test_dJ_dk_vs_reference_solve(hz, oracle, sphere24):
    import oracle as O
    from oracle.ref_worker import RefWorker
    c = sphere24
    op, b, rx, target, N, K = c["op"], c["b"], c["rx"], c["target"], c["N"], c["K"]
    J, g, dk, gw, info = op.misfit_gradient(b, rx, target, method=hz.BICG, precision=hz.PREC_F64, tol=1e-13)
    Js = []
    for k in (K + H_FD, K - H_FD):
        with RefWorker("dirichlet", N, k, c["d"]) as ref:
            u = _ref_field(O, oracle, ref.tube, ref.solve(b), N, k, rx)
            Js.append(float(np.sum(np.abs(u - target) ** 2)))
    fd = (Js[0] - Js[1]) / (2 * H_FD)
    assert abs(dk - fd) <= 1e-5 * abs(fd), (dk, fd)


def test_dJ_dphi_vs_reference_solve(hz, oracle):
    import oracle as O
    from oracle.ref_worker import solve_many
    from helmholtz_3d_torrone_gb300 import geometry as G
    N, K = 20, 4.0
    src = np.array([0.02, -0.01, 0.03])
    d = G.sphere(N, radius=0.5, center=(0.011, 0.017, 0.005))
    rx = G.random_sphere_points(16, 0.9, seed=5)
    r = np.linalg.norm(rx - src, axis=1)
    t = 1.1 * np.exp(1j * K * r) / (4 * np.pi * r)
    p = hz.params(N, K, int_l=-1.0, int_u=1.0, factor=3.0, dirichlet=1)
    with hz.Operator(p) as op:
        op.set_distance(d)
        op.build()
        J, gphi, info = op.shape_gradient(src, rx, t, method=hz.BICG, precision=hz.PREC_F64, tol=1e-13,
                                          maxit=2000)
    po = O.Params(N, -1.0, 1.0, K, 3.0, 2.0, 1, 0)

    def b_of(tube):
        return oracle.rhs(po, tube, src, 0)

    H = 2.0 / N
    eps = 3.0 * H
    rng = np.random.default_rng(3)
    inner = np.argwhere(np.abs(d) < eps - 0.5 * H)
    outer = np.argwhere((np.abs(d) > eps + 0.5 * H) & (np.abs(d) < eps + 2.0 * H))
    nodes = [tuple(int(v) for v in inner[i]) for i in rng.choice(len(inner), 12, replace=False)]
    nodes += [tuple(int(v) for v in outer[i]) for i in rng.choice(len(outer), 4, replace=False)]
    grids = [d]
    for q in nodes:
        for h in (H_FD, 2 * H_FD):
            for sgn in (1, -1):
                g = d.copy()
                g[q] += sgn * h
                grids.append(g)
    res = solve_many("dirichlet", N, K, grids, b_of)
    Jr = []
    for tube, x in res:
        u = oracle.evaluate(po, tube, x, rx, True)
        Jr.append(float(np.sum(np.abs(u - t) ** 2)))
    assert abs(J - Jr[0]) <= 1e-10 * Jr[0]
    q1, q2 = [], []
    for i in range(len(nodes)):
        jp1, jm1, jp2, jm2 = Jr[1 + 4 * i: 5 + 4 * i]
        q1.append((jp1 - jm1) / (2 * H_FD))
        q2.append((jp2 - jm2) / (4 * H_FD))
    q1, q2 = np.array(q1), np.array(q2)
    scale = np.max(np.abs(q1))
    assert scale > 0
    smooth = np.abs(q1 - q2) <= 1e-5 * scale
    assert np.count_nonzero(smooth) >= 8, (q1, q2)
    gq = np.array([gphi[q] for q in nodes])
    err = np.abs(gq - q1)[smooth] / scale
    assert np.count_nonzero(err <= 1e-6) >= 8, (err, gq[smooth], q1[smooth])
    assert np.max(err) <= 1e-4, (err, gq[smooth], q1[smooth])
