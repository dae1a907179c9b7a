"""The FP64 distance helper the GPU tie checks rely on, pinned against the oracle's brute-force
closest points (CPU only)."""
import numpy as np
import pytest

from fp64_geometry import prim_dist64
from zombie_gb300 import problems as P


@pytest.mark.parametrize("dim", [2, 3])
def test_fp64_distance_to_the_closest_primitive_matches_the_oracle(oracle, dim):
    if dim == 2:
        pos, idx = P.star_polygon(512)
    else:
        pos, idx, _ = P.displaced_icosphere(3, seed=5)
    x = np.random.default_rng(0).uniform(-1.3, 1.3, (3000, dim)).astype(np.float32)
    _, _, od, oi = oracle.Boundary(dim, pos, idx, use_bvh=False).closest_point(x)
    d64 = prim_dist64(pos, idx, oi, x)
    assert np.max(np.abs(d64 - od)) <= 2.4e-7 + 1e-6 * od.max()


def test_fp64_triangle_distance_is_the_minimum_over_the_triangle():
    rng = np.random.default_rng(1)
    n = 500
    a, b, c = rng.normal(size=(3, n, 3))
    p = 2.0 * rng.normal(size=(n, 3))
    pos = np.concatenate([a, b, c]).astype(np.float64)
    idx = np.stack([np.arange(n), n + np.arange(n), 2 * n + np.arange(n)], 1)
    d = prim_dist64(pos, idx, np.arange(n), p)
    # dense barycentric sampling never comes closer than the exact distance
    best = np.full(n, np.inf)
    for i in range(41):
        for j in range(41 - i):
            u, v = i / 40, j / 40
            q = a + u * (b - a) + v * (c - a)
            best = np.minimum(best, np.linalg.norm(p - q, axis=1))
    assert np.all(best >= d - 1e-12)
    assert np.all(best - d <= 0.05)
