"""Synthetic collocation point clouds of the benchmark workloads.

All generators return float64 arrays of shape (n, 3) in their fixed
(original) order.  Random clouds use numpy's PCG64 ``default_rng(seed)``.
"""
import numpy as np


def fibonacci_sphere(n):
    """Unit sphere, Fibonacci lattice: z_i = 1 - 2(i+1/2)/n, theta_i = i*pi*(3-sqrt 5)."""
    i = np.arange(n, dtype=np.float64)
    z = 1.0 - 2.0 * (i + 0.5) / n
    r = np.sqrt(np.maximum(0.0, 1.0 - z * z))
    th = i * (np.pi * (3.0 - np.sqrt(5.0)))
    return np.ascontiguousarray(np.stack([r * np.cos(th), r * np.sin(th), z], axis=1))


def sphere_surface(n, seed):
    """Uniform random points on the unit sphere (normalised Gaussians)."""
    g = np.random.default_rng(seed).standard_normal((n, 3))
    return np.ascontiguousarray(g / np.linalg.norm(g, axis=1, keepdims=True))


def ellipsoid_surface(n, seed, axes=(1.0, 0.5, 0.25)):
    """Uniform (area-weighted) random points on an ellipsoid surface.

    Method: sample the unit sphere uniformly, map x -> A x, and accept with
    probability equal to the local area stretch divided by its maximum
    (rejection sampling; the stretch of the map at unit normal direction u is
    |A| * |A^-1 u|).
    """
    rng = np.random.default_rng(seed)
    a = np.asarray(axes, dtype=np.float64)
    inv = 1.0 / a
    gmax = np.max(inv)
    out = np.empty((0, 3))
    while out.shape[0] < n:
        m = 2 * (n - out.shape[0]) + 64
        g = rng.standard_normal((m, 3))
        u = g / np.linalg.norm(g, axis=1, keepdims=True)
        w = np.linalg.norm(u * inv, axis=1) / gmax
        keep = rng.random(m) < w
        out = np.concatenate([out, u[keep] * a], axis=0)
    return np.ascontiguousarray(out[:n])


def cube_surface(n, seed):
    """Uniform random points on the surface of the unit cube [0,1]^3 (6 equal faces)."""
    rng = np.random.default_rng(seed)
    face = rng.integers(0, 6, n)
    uv = rng.random((n, 2))
    p = np.empty((n, 3))
    ax = face // 2
    side = (face % 2).astype(np.float64)
    for a in range(3):
        sel = ax == a
        others = [b for b in range(3) if b != a]
        p[sel, a] = side[sel]
        p[sel, others[0]] = uv[sel, 0]
        p[sel, others[1]] = uv[sel, 1]
    return np.ascontiguousarray(p)


GEOMETRIES = {
    "sphere": lambda n, seed: sphere_surface(n, seed),
    "ellipsoid": lambda n, seed: ellipsoid_surface(n, seed),
    "cube": lambda n, seed: cube_surface(n, seed),
}
