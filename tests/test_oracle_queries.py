"""Oracle geometric queries: BVH traversals agree with brute force; silhouette flags and
boundary sampling follow their definitions."""
import numpy as np
import pytest

from zombie_gb300 import _abi as A
from zombie_gb300 import problems as P


def _scene(dim):
    if dim == 2:
        pos, idx = P.star_polygon(512)
    else:
        pos, idx, _ = P.displaced_icosphere(3, seed=3)
    return pos, idx


@pytest.mark.parametrize("dim", [2, 3])
def test_closest_point_bvh_matches_brute_force(oracle, dim):
    pos, idx = _scene(dim)
    rng = np.random.default_rng(0)
    x = rng.uniform(-1.4, 1.4, (2000, dim)).astype(np.float32)
    b = oracle.Boundary(dim, pos, idx, use_bvh=True)
    f = oracle.Boundary(dim, pos, idx, use_bvh=False)
    _, _, d1, p1 = b.closest_point(x)
    _, _, d2, p2 = f.closest_point(x)
    assert np.array_equal(d1, d2)
    assert np.mean(p1 == p2) > 0.99   # the rest are exact ties (shared vertices)
    tie = p1 != p2
    assert np.array_equal(d1[tie], d2[tie])


@pytest.mark.parametrize("dim", [2, 3])
def test_intersect_bvh_matches_brute_force(oracle, dim):
    pos, idx = _scene(dim)
    rng = np.random.default_rng(1)
    o = rng.uniform(-0.5, 0.5, (2000, dim)).astype(np.float32)
    d = rng.normal(size=(2000, dim)).astype(np.float32)
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    tmax = rng.uniform(0.1, 3.0, 2000).astype(np.float32)
    nz = np.zeros_like(o)
    on = np.zeros(2000, np.int32)
    b = oracle.Boundary(dim, pos, idx, use_bvh=True)
    f = oracle.Boundary(dim, pos, idx, use_bvh=False)
    h1, _, _, t1, p1 = b.intersect(o, nz, d, tmax, on)
    h2, _, _, t2, p2 = f.intersect(o, nz, d, tmax, on)
    assert np.array_equal(h1, h2)
    assert np.array_equal(t1[h1 == 1], t2[h2 == 1])
    # a ray from the interior crosses a closed boundary an odd number of times
    c = f.count_hits(o, d, np.full(2000, 1e30, np.float32))
    assert np.all(c % 2 == 1)


@pytest.mark.parametrize("dim", [2, 3])
def test_star_radius_bvh_matches_brute_force(oracle, dim):
    pos, idx = _scene(dim)
    rng = np.random.default_rng(2)
    x = rng.uniform(-0.7, 0.7, (1500, dim)).astype(np.float32)
    minr = np.full(1500, 1e-3, np.float32)
    maxr = rng.uniform(0.05, 2.0, 1500).astype(np.float32)
    flip = np.zeros(1500, np.int32)
    for kind, k in [(A.ZGPU_BOUNDARY_NEUMANN, None), (A.ZGPU_BOUNDARY_ROBIN, 2.0)]:
        kk = None if k is None else np.full(idx.shape[0], k, np.float32)
        b = oracle.Boundary(dim, pos, idx, kind=kind, kmin=kk, kmax=kk, silhouette_precision=0.0, use_bvh=True)
        f = oracle.Boundary(dim, pos, idx, kind=kind, kmin=kk, kmax=kk, silhouette_precision=0.0, use_bvh=False)
        r1 = b.star_radius(x, minr, maxr, 1e-3, flip)
        r2 = f.star_radius(x, minr, maxr, 1e-3, flip)
        assert np.array_equal(r1, r2)
        assert np.all(r1 <= np.maximum(maxr, minr)) and np.all(r1 >= minr)


@pytest.mark.parametrize("dim", [2, 3])
def test_robin_node_bounds_keep_the_brute_force_radius(oracle, dim):
    """Robin coefficients that vary per face, with perfectly absorbing (FLT_MAX) and purely
    reflecting (0) faces mixed in: the node-level bounds of the BVH traversal prune work
    but give the radius of the all-primitive loop."""
    if dim == 2:
        pos, idx = P.star_polygon(2048)
    else:
        pos, idx, _ = P.displaced_icosphere(4, seed=5)
    rng = np.random.default_rng(7)
    n = idx.shape[0]
    kmax = rng.uniform(0.5, 6.0, n).astype(np.float32)
    kmin = (kmax * rng.uniform(0.3, 1.0, n)).astype(np.float32)
    absorbing = rng.random(n) < 0.05
    reflecting = rng.random(n) < 0.1
    kmin[absorbing] = kmax[absorbing] = A.FLT_MAX
    kmin[reflecting] = kmax[reflecting] = 0.0
    m = 1500
    x = rng.uniform(-0.6, 0.6, (m, dim)).astype(np.float32)
    minr = np.full(m, 1e-3, np.float32)
    maxr = np.where(rng.random(m) < 0.5, A.FLT_MAX, rng.uniform(0.05, 3.0, m)).astype(np.float32)
    flip = np.zeros(m, np.int32)
    b = oracle.Boundary(dim, pos, idx, kind=A.ZGPU_BOUNDARY_ROBIN, kmin=kmin, kmax=kmax, silhouette_precision=0.0)
    f = oracle.Boundary(dim, pos, idx, kind=A.ZGPU_BOUNDARY_ROBIN, kmin=kmin, kmax=kmax, silhouette_precision=0.0,
                        use_bvh=False)
    oracle.counters()
    r1 = b.star_radius(x, minr, maxr, 1e-3, flip)
    visited = oracle.counters()["star_radius"]["prims"]
    r2 = f.star_radius(x, minr, maxr, 1e-3, flip)
    assert np.array_equal(r1, r2)
    assert visited < 0.25 * m * n


def test_silhouette_flags_convex_and_concave(oracle):
    # a convex square: every vertex is convex -> ignored for single-sided problems
    sq = np.array([[0, 0], [1, 0], [1, 1], [0, 1]], np.float32)
    si = np.array([[0, 1], [1, 2], [2, 3], [3, 0]], np.int32)
    has, ign = oracle.Boundary(2, sq, si, kind=A.ZGPU_BOUNDARY_NEUMANN).flags()
    assert has.all() and ign.all()
    # an L shape has exactly one reflex vertex (index 3 at (1,1)), kept by both neighbours
    L = np.array([[0, 0], [2, 0], [2, 1], [1, 1], [1, 2], [0, 2]], np.float32)
    Li = np.array([[i, (i + 1) % 6] for i in range(6)], np.int32)
    has, ign = oracle.Boundary(2, L, Li, kind=A.ZGPU_BOUNDARY_NEUMANN).flags()
    kept = [(i, j) for i in range(6) for j in range(2) if not ign[i, j]]
    assert sorted(kept) == [(2, 1), (3, 0)]
    # double-sided problems ignore nothing
    _, ign2 = oracle.Boundary(2, L, Li, kind=A.ZGPU_BOUNDARY_NEUMANN, solve_double_sided=True).flags()
    assert not ign2.any()
    # a closed convex polyhedron: all edges convex
    v, f = P.icosphere(1)
    has, ign = oracle.Boundary(3, v.astype(np.float32), f.astype(np.int32), kind=A.ZGPU_BOUNDARY_NEUMANN).flags()
    assert has.all() and ign.all()


def test_l_shape_star_radius(oracle):
    """From a point that sees the reflex corner of an L, the star radius stops at the corner."""
    L = np.array([[0, 0], [2, 0], [2, 1], [1, 1], [1, 2], [0, 2]], np.float32)
    Li = np.array([[i, (i + 1) % 6] for i in range(6)], np.int32)
    b = oracle.Boundary(2, L, Li, kind=A.ZGPU_BOUNDARY_NEUMANN, silhouette_precision=0.0)
    x = np.array([[0.5, 1.5], [1.5, 0.5], [0.5, 0.5]], np.float32)
    r = b.star_radius(x, np.full(3, 1e-3, np.float32), np.full(3, 10.0, np.float32), 1e-3, np.zeros(3, np.int32))
    corner = np.array([1.0, 1.0])
    # (0.5,1.5) and (1.5,0.5) see one face of the corner front-facing and one back-facing
    assert abs(r[0] - np.linalg.norm(x[0] - corner)) < 1e-6
    assert abs(r[1] - np.linalg.norm(x[1] - corner)) < 1e-6
    # from (0.5,0.5) both faces at the corner are back-facing: not a silhouette
    assert r[2] == pytest.approx(10.0)


@pytest.mark.parametrize("use_bvh", [True, False])
def test_boundary_sampling_is_unbiased(oracle, use_bvh):
    """E[G h / pdf] over sampleReflectingBoundary equals the boundary integral in the ball."""
    pos, idx = P.star_polygon(1024)
    b = oracle.Boundary(2, pos, idx, kind=A.ZGPU_BOUNDARY_NEUMANN, use_bvh=use_bvh)
    x = np.array([[0.1, -0.5]], np.float32)
    R = 0.6
    N = 100000
    u = np.random.default_rng(3).random((N, 2)).astype(np.float32)
    found, pt, _, pdf = b.sample(np.repeat(x, N, 0), np.full(N, R, np.float32), u)
    d = np.linalg.norm(pt - x, axis=1)
    G = np.log(R / np.maximum(d, 1e-4)) / (2 * np.pi)
    val = np.where((found == 1) & (d < R), G * pt[:, 1] / np.maximum(pdf, 1e-30), 0.0)
    a = pos[idx[:, 0]].astype(np.float64)
    c = pos[idx[:, 1]].astype(np.float64)
    t = (np.arange(256) + 0.5) / 256
    z = a[:, None, :] + (c - a)[:, None, :] * t[None, :, None]
    dz = np.linalg.norm(z - x, axis=2)
    Gq = np.where(dz < R, np.log(R / np.maximum(dz, 1e-4)) / (2 * np.pi), 0.0)
    quad = ((Gq * z[:, :, 1]).mean(1) * np.linalg.norm(c - a, axis=1)).sum()
    assert abs(val.mean() - quad) <= 4 * val.std() / np.sqrt(N) + 1e-5


def test_offset_point_moves_off_the_surface(oracle):
    import ctypes as C
    p = np.array([0.75, -0.4], np.float32)
    n = np.array([0.6, -0.8], np.float32)
    out = np.zeros(2, np.float32)
    oracle.lib().orc_offset_point(2, p.ctypes.data, n.ctypes.data, out.ctypes.data)
    assert np.dot(out - p, n) > 0
    p3 = np.array([0.01, 0.5, -2.0], np.float32)
    n3 = np.array([0.0, 0.6, 0.8], np.float32)
    out3 = np.zeros(3, np.float32)
    oracle.lib().orc_offset_point(3, p3.ctypes.data, n3.ctypes.data, out3.ctypes.data)
    assert out3[0] == p3[0] and np.dot(out3 - p3, n3) > 0
