"""Rays that graze box planes far from the world origin, shared by the oracle's
CPU tests and the GPU tests.

k rays start far from the origin in x (200..3000) with tiny direction x
components (2e-6..3e-5), each towards its own triangle in the plane a few ulps
of the origin away in x: a plane distance (plane - o) / d of the order of the
rounding of o / d itself.  Each triangle ends 0.05..3 past its hit in z, so
the box's exit there lies within that rounding of the entry.  A box test whose
plane distances carry an absolute error of the size of |o / d| ulps (the fused
form fma(plane, 1/d, -o/d)) misses about half of these boxes; one with only
relative errors (the reference's (plane - o) * (1/d)) misses none."""
import numpy as np

import pyoracle as O


def grazing_walls(k=4096, seed=9):
    """(vertices, triangles, rays): ray i hits triangle i, and only it."""
    rng = np.random.default_rng(seed)
    x = rng.uniform(200, 3000, k).astype(np.float32)
    dx = (rng.uniform(2e-6, 3e-5, k) * rng.choice([-1, 1], k)).astype(np.float32)
    xk = (x + np.sign(dx) * rng.integers(1, 40, k) * np.spacing(x)).astype(np.float32)
    y = (2.0 * np.arange(k)).astype(np.float32)
    th = (xk.astype(np.float64) - x) / dx
    z0, z1 = th - rng.uniform(0.5, 5, k), th + rng.uniform(0.05, 3, k)
    V = np.zeros(3 * k, O.VERTEX)
    V["position"][0::3] = np.column_stack([xk, y - 0.5, z0, np.ones(k)])
    V["position"][1::3] = np.column_stack([xk, y + 0.5, z0, np.ones(k)])
    V["position"][2::3] = np.column_stack([xk, y, z1, np.ones(k)])
    T = np.zeros(k, O.TRIANGLE)
    T["v"] = np.arange(3 * k).reshape(k, 3)
    rays = np.zeros(k, O.RAY)
    rays["org"] = np.column_stack([x, y, np.zeros(k)])
    rays["dir"] = np.column_stack([dx, np.zeros(k), np.ones(k)])
    rays["tmin"], rays["tmax"] = 1e-4, 1e9
    return V, T, rays
