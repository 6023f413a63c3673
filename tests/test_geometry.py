"""CPU checks of the analytic inputs every test and benchmark is built from
(helmholtz_3d_torrone_gb300/geometry.py): grid coordinates, signed
distances, level sets and seeded point sets."""
import numpy as np

from helmholtz_3d_torrone_gb300 import geometry as G


def test_node_coordinates_follow_the_reference_layout():
    # node (i, j, k) sits at (x, y, z) = (l + j H, l + i H, l + k H)
    H, X, Y, Z = G.node_coords(8, -2.0, 2.0)
    assert H == 0.5
    assert X.shape == (1, 9, 1) and Y.shape == (9, 1, 1) and Z.shape == (1, 1, 9)
    assert X[0, 3, 0] == -0.5 and Y[5, 0, 0] == 0.5 and Z[0, 0, 8] == 2.0


def test_sphere_and_torus_distances():
    N = 32
    H, X, Y, Z = G.node_coords(N)
    d = G.sphere(N, radius=0.5, center=(0.1, 0.0, -0.05))
    r = np.sqrt((X - 0.1) ** 2 + Y ** 2 + (Z + 0.05) ** 2)
    assert np.allclose(d, 0.5 - r, atol=0, rtol=0)
    t = G.torus(N, R=0.6, r=0.25)
    # the origin lies on the axis, R - r outside the tube; nothing is deeper than r inside
    assert t[N // 2, N // 2, N // 2] == 0.25 - 0.6
    assert np.max(t) <= 0.25 + 1e-15
    # |grad d| = 1 in the band (central differences, interior nodes only:
    # np.gradient is one-sided on the grid's faces)
    M = 64
    t = G.torus(M, R=0.6, r=0.25)
    g = np.gradient(t, 2.0 / M)
    mag = np.sqrt(g[0] ** 2 + g[1] ** 2 + g[2] ** 2)[2:-2, 2:-2, 2:-2]
    band = (np.abs(t) < 3 * 2.0 / M)[2:-2, 2:-2, 2:-2]
    assert np.max(np.abs(mag[band] - 1.0)) < 0.02


def test_bumpy_sphere_level_set_zero_on_the_surface():
    N = 40
    phi = G.bumpy_sphere_levelset(N, r0=0.5, amp=0.08)
    H, X, Y, Z = G.node_coords(N)
    shape = (N + 1,) * 3
    X, Y, Z = (np.broadcast_to(a, shape) for a in (X, Y, Z))
    rad = np.sqrt(X ** 2 + Y ** 2 + Z ** 2)
    theta = np.arccos(np.clip(np.divide(Z, rad, out=np.zeros(shape), where=rad > 0), -1, 1))
    ph = np.arctan2(Y, X)
    surf = 0.5 * (1 + 0.08 * np.cos(3 * theta) * np.sin(2 * ph))
    assert np.allclose(phi, surf - rad, rtol=0, atol=1e-14)
    assert phi[N // 2, N // 2, N // 2] == 0.5  # positive inside
    # amp = 0 is the round sphere's distance
    assert np.allclose(G.bumpy_sphere_levelset(N, amp=0.0), G.sphere(N, 0.5), rtol=0, atol=1e-15)


def test_point_sets():
    d = G.fibonacci_sphere(64)
    assert d.shape == (64, 3) and np.allclose(np.linalg.norm(d, axis=1), 1.0)
    # nearly uniform: the mean direction is close to zero
    assert np.linalg.norm(d.mean(axis=0)) < 0.05
    p = G.random_sphere_points(100, 0.9, seed=7)
    assert p.shape == (100, 3) and np.allclose(np.linalg.norm(p, axis=1), 0.9)
    assert np.array_equal(p, G.random_sphere_points(100, 0.9, seed=7))
