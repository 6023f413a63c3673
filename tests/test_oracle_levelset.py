"""CPU check of the oracle's level-set reinitialisation (the checker used by
the GPU tests): it drives a non-distance ellipsoid level set to the exact
signed distance inside the 3h tube."""
import numpy as np


def test_oracle_reinit_converges(oracle):
    from helmholtz_3d_torrone_gb300 import geometry as G
    N = 32
    H = 2.0 / N
    phi = G.ellipsoid_levelset(N)
    d = G.ellipsoid(N)
    tube = np.abs(d) <= 3 * H
    before = np.max(np.abs(phi - d)[tube])
    r = oracle.reinit(N, H, phi, 40)
    after = np.max(np.abs(r - d)[tube])
    assert after < 2e-3 < before


def test_ellipsoid_distance_is_exact():
    """Closest-point distance vs a dense surface sampling (with the medial
    degenerate case at the centre)."""
    from helmholtz_3d_torrone_gb300 import geometry as G
    N = 16
    a = np.array([0.7, 0.5, 0.4])
    d = G.ellipsoid(N, axes=tuple(a))
    assert abs(d[N // 2, N // 2, N // 2] - 0.4) < 1e-12  # the centre lies 0.4 from the surface
    from scipy.spatial import cKDTree
    u, v = np.meshgrid(np.linspace(0, np.pi, 800), np.linspace(0, 2 * np.pi, 1600))
    P = np.stack([a[0] * np.sin(u) * np.cos(v), a[1] * np.sin(u) * np.sin(v), a[2] * np.cos(u)], -1).reshape(-1, 3)
    H = 2.0 / N
    t = -1.0 + np.arange(N + 1) * H
    idx = np.argwhere(np.ones_like(d, bool))[::5]
    pts = np.stack([t[idx[:, 1]], t[idx[:, 0]], t[idx[:, 2]]], 1)
    bf, _ = cKDTree(P).query(pts)
    inside = (pts ** 2 / a ** 2).sum(1) < 1
    bf = np.where(inside, bf, -bf)
    assert np.max(np.abs(bf - d[idx[:, 0], idx[:, 1], idx[:, 2]])) < 2e-3
