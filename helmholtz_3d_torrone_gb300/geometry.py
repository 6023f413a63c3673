"""Synthetic signed-distance grids (the input the reference reads from
``distance<N>.txt``, large3Dexample2.c:405-424).

All grids use the reference's node layout: array index [i, j, k] holds the
node (x, y, z) = (int_l + j*H, int_l + i*H, int_l + k*H) (i is y, j is x,
k is z), and d > 0 inside the body (functions.c:590).
"""
import numpy as np


def node_coords(N, int_l=-1.0, int_u=1.0):
    """Return (H, X, Y, Z) broadcastable over the [i, j, k] grid."""
    H = (int_u - int_l) / N
    t = int_l + np.arange(N + 1, dtype=np.float64) * H
    Y = t[:, None, None]
    X = t[None, :, None]
    Z = t[None, None, :]
    return H, X, Y, Z


def sphere(N, radius=0.5, center=(0.0, 0.0, 0.0), int_l=-1.0, int_u=1.0):
    H, X, Y, Z = node_coords(N, int_l, int_u)
    cx, cy, cz = center
    return np.ascontiguousarray(radius - np.sqrt((X - cx) ** 2 + (Y - cy) ** 2 + (Z - cz) ** 2))


def torus(N, R=0.6, r=0.25, int_l=-1.0, int_u=1.0):
    """Torus around the z axis, tube radius r at distance R from the axis."""
    H, X, Y, Z = node_coords(N, int_l, int_u)
    q = np.sqrt(X ** 2 + Y ** 2) - R
    return np.ascontiguousarray(r - np.sqrt(q ** 2 + Z ** 2))


def ellipsoid(N, axes=(0.7, 0.5, 0.4), int_l=-1.0, int_u=1.0, iters=60):
    """Exact signed distance to an axis-aligned ellipsoid (closest point by
    Newton iteration on the Lagrange multiplier, Eberly's method)."""
    H, X, Y, Z = node_coords(N, int_l, int_u)
    shape = np.broadcast_shapes(X.shape, Y.shape, Z.shape)
    p = np.stack([np.broadcast_to(a, shape).ravel() for a in (X, Y, Z)], axis=1)
    a = np.asarray(axes, dtype=np.float64)
    y = np.abs(p)
    inside = np.sum((y / a) ** 2, axis=1) < 1.0
    # Closest point x_i = a_i^2 y_i / (t + a_i^2) where t solves
    # F(t) = sum_i (a_i y_i / (t + a_i^2))^2 - 1 = 0 on t > -min a_i^2.
    # F is convex and decreasing there, so Newton started left of the root
    # (F >= 0 at t0 = max_i (a_i y_i - a_i^2)) climbs to it monotonically.
    amin2 = a.min() ** 2
    floor = -amin2 * (1.0 - 1e-12)
    t = np.max(a[None, :] * y - a[None, :] ** 2, axis=1)
    t = np.maximum(t, floor)
    for _ in range(iters):
        den = t[:, None] + a[None, :] ** 2
        r = a[None, :] * y / den
        F = np.sum(r * r, axis=1) - 1.0
        dF = -2.0 * np.sum(r * r / den, axis=1)
        step = np.divide(F, dF, out=np.zeros_like(F), where=dF != 0)
        t = np.maximum(t - step, floor)
    x = a[None, :] ** 2 * y / (t[:, None] + a[None, :] ** 2)
    # Degenerate case (point on the plane of the shortest axis, inside the
    # evolute): the root sits at t = -min a_i^2 and the closest point leaves
    # that plane; solve for its shortest-axis coordinate from the surface.
    im = int(np.argmin(a))
    deg = t <= floor * (1.0 - 1e-9)
    if np.any(deg):
        others = [i for i in range(3) if i != im]
        xd = np.zeros((int(deg.sum()), 3))
        for i in others:
            gap = a[i] ** 2 - a[im] ** 2
            # an axis as short as the shortest one: the closest point keeps
            # no component along it (only the centre plane is degenerate)
            xd[:, i] = a[i] ** 2 * y[deg, i] / gap if gap > 0 else 0.0
        rest = 1.0 - sum((xd[:, i] / a[i]) ** 2 for i in others)
        xd[:, im] = a[im] * np.sqrt(np.maximum(rest, 0.0))
        x[deg] = xd
    dist = np.sqrt(np.sum((x - y) ** 2, axis=1))
    s = np.where(inside, dist, -dist)
    return np.ascontiguousarray(s.reshape(shape))


def fibonacci_sphere(m, radius=1.0, seed=None):
    """m points quasi-uniform on a sphere (golden-angle spiral)."""
    k = np.arange(m) + 0.5
    z = 1.0 - 2.0 * k / m
    rho = np.sqrt(np.maximum(0.0, 1.0 - z * z))
    ang = np.pi * (3.0 - np.sqrt(5.0)) * k
    pts = np.stack([rho * np.cos(ang), rho * np.sin(ang), z], axis=1)
    return radius * pts


def random_sphere_points(m, radius, seed):
    """m seeded points uniform on the sphere of the given radius."""
    rng = np.random.default_rng(seed)
    v = rng.normal(size=(m, 3))
    v /= np.linalg.norm(v, axis=1, keepdims=True)
    return radius * v


def ellipsoid_levelset(N, axes=(0.7, 0.5, 0.4), scale=0.3, int_l=-1.0, int_u=1.0):
    """A smooth level set of an ellipsoid that is not a distance function
    (positive inside): scale * (1 - sqrt(sum x_i^2 / a_i^2)).  Feed it to the
    reinitialisation to obtain the signed distance."""
    H, X, Y, Z = node_coords(N, int_l, int_u)
    a = np.asarray(axes, dtype=np.float64)
    phi = scale * (1.0 - np.sqrt(X ** 2 / a[0] ** 2 + Y ** 2 / a[1] ** 2 + Z ** 2 / a[2] ** 2))
    return np.ascontiguousarray(np.broadcast_to(phi, (N + 1,) * 3))


def bumpy_sphere_levelset(N, r0=0.5, amp=0.08, int_l=-1.0, int_u=1.0):
    """Level set r(theta, phi) - |x| of the bumpy sphere
    r(theta, phi) = r0 (1 + amp cos(3 theta) sin(2 phi)) (positive inside,
    theta polar from +z, phi azimuth); not a distance function."""
    H, X, Y, Z = node_coords(N, int_l, int_u)
    shape = (N + 1,) * 3
    X, Y, Z = (np.broadcast_to(a, shape) for a in (X, Y, Z))
    rad = np.sqrt(X ** 2 + Y ** 2 + Z ** 2)
    theta = np.arccos(np.clip(np.divide(Z, rad, out=np.zeros(shape), where=rad > 0), -1.0, 1.0))
    ph = np.arctan2(Y, X)
    return np.ascontiguousarray(r0 * (1.0 + amp * np.cos(3 * theta) * np.sin(2 * ph)) - rad)
