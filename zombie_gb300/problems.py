"""Synthetic model problems: boundary meshes, manufactured solutions and evaluation points.

The workloads are defined by their shapes and seeds only (no dataset is involved):
  * star polygon r(t) = r0 (1 + amp sin(k t)) discretised into n CCW line segments;
  * icosphere subdivided L times, vertices displaced radially by 0.15 * sum of 4 seeded
    low-order real spherical harmonics;
  * manufactured solutions u, from which Dirichlet data g = u, Neumann/Robin data
    h = du/dn + kappa u and the source f = -Lap u + sigma u follow in closed form
    (the device evaluates them from the zgpu_analytic descriptor).
"""
import math

import numpy as np

from . import _abi as A
from . import io as _io


# ----------------------------------------------------------------------------- meshes
def star_polygon(n_segments, r0=1.0, amp=0.3, freq=5, phase=0.0, center=(0.0, 0.0)):
    t = 2.0 * np.pi * np.arange(n_segments) / n_segments
    r = r0 * (1.0 + amp * np.sin(freq * t + phase))
    pos = np.stack([center[0] + r * np.cos(t), center[1] + r * np.sin(t)], 1).astype(np.float32)
    idx = np.stack([np.arange(n_segments), (np.arange(n_segments) + 1) % n_segments], 1).astype(np.int32)
    return pos, idx


def polygon_inside_and_radius(points, positions, center=(0.0, 0.0)):
    """Exact inside test for a polygon that is star-shaped about `center` with vertices
    ordered by angle: the ray from the centre through p crosses exactly one segment."""
    p = np.asarray(points, np.float64) - np.asarray(center)
    v = np.asarray(positions, np.float64) - np.asarray(center)
    n = v.shape[0]
    ang_v = np.mod(np.arctan2(v[:, 1], v[:, 0]), 2 * np.pi)
    ang_p = np.mod(np.arctan2(p[:, 1], p[:, 0]), 2 * np.pi)
    k = np.searchsorted(ang_v, ang_p, side="right") - 1
    k = np.mod(k, n)
    a = v[k]
    b = v[(k + 1) % n]
    d = p / np.maximum(np.linalg.norm(p, axis=1, keepdims=True), 1e-30)
    e = b - a
    denom = d[:, 0] * e[:, 1] - d[:, 1] * e[:, 0]
    t = (a[:, 0] * e[:, 1] - a[:, 1] * e[:, 0]) / np.where(np.abs(denom) < 1e-30, 1e-30, denom)
    rad = np.linalg.norm(p, axis=1)
    return rad < t, t


def icosphere(level):
    """Unit icosphere with outward (CCW seen from outside) triangles."""
    phi = (1.0 + 5 ** 0.5) / 2.0
    verts = [(-1, phi, 0), (1, phi, 0), (-1, -phi, 0), (1, -phi, 0), (0, -1, phi), (0, 1, phi),
             (0, -1, -phi), (0, 1, -phi), (phi, 0, -1), (phi, 0, 1), (-phi, 0, -1), (-phi, 0, 1)]
    faces = [(0, 11, 5), (0, 5, 1), (0, 1, 7), (0, 7, 10), (0, 10, 11), (1, 5, 9), (5, 11, 4), (11, 10, 2),
             (10, 7, 6), (7, 1, 8), (3, 9, 4), (3, 4, 2), (3, 2, 6), (3, 6, 8), (3, 8, 9), (4, 9, 5), (2, 4, 11),
             (6, 2, 10), (8, 6, 7), (9, 8, 1)]
    v = np.array(verts, np.float64)
    v /= np.linalg.norm(v, axis=1, keepdims=True)
    f = np.array(faces, np.int64)
    for _ in range(level):
        nv = v.shape[0]
        e = np.concatenate([f[:, [0, 1]], f[:, [1, 2]], f[:, [2, 0]]], 0)
        e.sort(axis=1)
        key = e[:, 0] * (nv + 1) + e[:, 1]
        uniq, inv = np.unique(key, return_inverse=True)
        a = uniq // (nv + 1)
        b = uniq % (nv + 1)
        mid = v[a] + v[b]
        mid /= np.linalg.norm(mid, axis=1, keepdims=True)
        v = np.concatenate([v, mid], 0)
        m = inv.reshape(3, -1).T + nv  # m01, m12, m20 per face
        f0, f1, f2 = f[:, 0], f[:, 1], f[:, 2]
        m01, m12, m20 = m[:, 0], m[:, 1], m[:, 2]
        f = np.concatenate([np.stack([f0, m01, m20], 1), np.stack([f1, m12, m01], 1),
                            np.stack([f2, m20, m12], 1), np.stack([m01, m12, m20], 1)], 0)
    # orient outward
    c = v[f].mean(1)
    n = np.cross(v[f[:, 1]] - v[f[:, 0]], v[f[:, 2]] - v[f[:, 0]])
    flip = (n * c).sum(1) < 0
    f[flip] = f[flip][:, [0, 2, 1]]
    return v, f


def _real_sh(l, m, theta, phi):
    """Unnormalised real spherical harmonic of degree l<=3, order m (theta polar angle)."""
    x = np.sin(theta) * np.cos(phi)
    y = np.sin(theta) * np.sin(phi)
    z = np.cos(theta)
    table = {
        (1, -1): y, (1, 0): z, (1, 1): x,
        (2, -2): x * y, (2, -1): y * z, (2, 0): 3 * z * z - 1, (2, 1): x * z, (2, 2): x * x - y * y,
        (3, -3): y * (3 * x * x - y * y), (3, -2): x * y * z, (3, -1): y * (5 * z * z - 1), (3, 0): z * (5 * z * z - 3),
        (3, 1): x * (5 * z * z - 1), (3, 2): z * (x * x - y * y), (3, 3): x * (x * x - 3 * y * y),
    }
    return table[(l, m)]


class SHDisplacement:
    """r(dir) = 1 + 0.15 * sum_k c_k Y_k(dir) with 4 seeded low-order harmonics, scaled so
    that |sum| <= 1 (keeps the surface star-shaped about the origin)."""

    def __init__(self, seed=0, n_terms=4, scale=0.15):
        rng = np.random.default_rng(seed)
        lm = [(l, m) for l in (1, 2, 3) for m in range(-l, l + 1)]
        pick = rng.choice(len(lm), n_terms, replace=False)
        self.terms = [lm[i] for i in pick]
        c = rng.uniform(-1.0, 1.0, n_terms)
        self.coeffs = c / np.abs(c).sum()
        self.scale = scale

    def radius(self, dirs):
        d = np.asarray(dirs, np.float64)
        d = d / np.linalg.norm(d, axis=1, keepdims=True)
        theta = np.arccos(np.clip(d[:, 2], -1, 1))
        phi = np.arctan2(d[:, 1], d[:, 0])
        s = np.zeros(d.shape[0])
        for (l, m), c in zip(self.terms, self.coeffs):
            s += c * _real_sh(l, m, theta, phi)
        return 1.0 + self.scale * np.clip(s, -1.0, 1.0)


def displaced_icosphere(level, seed=0):
    v, f = icosphere(level)
    sh = SHDisplacement(seed)
    r = sh.radius(v)
    return (v * r[:, None]).astype(np.float32), f.astype(np.int32), sh


def bounding_box(positions, make_square=True, scale=1.0):
    """computeBoundingBox (utils/fcpw_geometric_queries.h:292-317)."""
    p = np.asarray(positions, np.float32)
    cm = p.mean(0)
    q = (p - cm) * scale + cm
    lo, hi = q.min(0), q.max(0)
    if make_square:
        c = 0.5 * (lo + hi)
        h = 0.5 * (hi - lo).max()
        lo, hi = c - h, c + h
    return lo.astype(np.float32), hi.astype(np.float32)


def partition_boundary_mesh(on_reflecting, positions, indices):
    """partitionBoundaryMesh (utils/fcpw_geometric_queries.h:460-510): split by primitive midpoint."""
    return _io.partition_boundary_mesh(on_reflecting, positions, indices)


# ------------------------------------------------------------------ manufactured solutions
def analytic(terms=(), q=(0.0, 0.0, 0.0), l=(0.0, 0.0, 0.0), d=0.0):
    """terms: iterable of (c, a[3], b[3], phi) for c exp(a.x) cos(b.x + phi)."""
    s = A.Analytic()
    terms = list(terms)
    assert len(terms) <= A.ZGPU_MAX_TERMS
    s.n_terms = len(terms)
    for k, (c, a, b, ph) in enumerate(terms):
        s.c[k] = c
        for i in range(3):
            s.a[k][i] = a[i] if i < len(a) else 0.0
            s.b[k][i] = b[i] if i < len(b) else 0.0
        s.phi[k] = ph
    for i in range(3):
        s.q[i] = q[i]
        s.l[i] = l[i]
    s.d = d
    return s


def eval_analytic(s, x):
    """u, grad u, Laplacian of a zgpu_analytic in FP64 (numpy), for RMSE and checks."""
    x = np.asarray(x, np.float64)
    dim = x.shape[1]
    u = np.full(x.shape[0], float(s.d))
    g = np.zeros_like(x)
    lap = np.zeros(x.shape[0])
    for i in range(dim):
        u += s.q[i] * x[:, i] ** 2 + s.l[i] * x[:, i]
        g[:, i] += 2 * s.q[i] * x[:, i] + s.l[i]
        lap += 2 * s.q[i]
    for k in range(s.n_terms):
        a = np.array([s.a[k][i] for i in range(dim)])
        b = np.array([s.b[k][i] for i in range(dim)])
        E = np.exp(x @ a)
        ang = x @ b + s.phi[k]
        Cc, S = np.cos(ang), np.sin(ang)
        u += s.c[k] * E * Cc
        g += s.c[k] * E[:, None] * (a[None, :] * Cc[:, None] - b[None, :] * S[:, None])
        lap += s.c[k] * E * ((a @ a - b @ b) * Cc - 2 * (a @ b) * S)
    return u, g, lap


def solution_expcos(quad=0.0):
    """u = e^x cos y + quad (x^2 + y^2)."""
    return analytic([(1.0, (1.0, 0.0, 0.0), (0.0, 1.0, 0.0), 0.0)], q=(quad, quad, 0.0))


def solution_sin_sinh_cos(offset=0.5):
    """u = sin(x) sinh(sqrt2 y) cos(z) + offset (harmonic), as 4 exp-cos terms."""
    r2 = math.sqrt(2.0)
    terms = []
    for s1 in (1.0, -1.0):
        for s2 in (1.0, -1.0):
            terms.append((0.25 * s1, (0.0, s1 * r2, 0.0), (1.0, 0.0, s2), -math.pi / 2))
    return analytic(terms, d=offset)


def solution_exp_cos_z2():
    """u = exp(0.5 x) cos(y) + z^2."""
    return analytic([(1.0, (0.5, 0.0, 0.0), (0.0, 1.0, 0.0), 0.0)], q=(0.0, 0.0, 1.0))


def make_pde(solution, sigma=0.0, dirichlet=True, robin=False, robin_coeff=0.0, source=True,
             constant_source=None):
    p = A.Pde()
    p.absorption_coeff = sigma
    p.solution = solution
    if constant_source is not None:
        p.is_source_constant = 1
        p.source_kind = A.ZGPU_FIELD_CONSTANT
        p.source_value = constant_source
    elif source:
        p.is_source_constant = 0
        p.source_kind = A.ZGPU_FIELD_ANALYTIC
    else:
        p.is_source_constant = 1
        p.source_kind = A.ZGPU_FIELD_ZERO
    p.dirichlet_kind = A.ZGPU_FIELD_ANALYTIC if dirichlet else A.ZGPU_FIELD_ZERO
    p.robin_kind = A.ZGPU_FIELD_ANALYTIC if robin else A.ZGPU_FIELD_ZERO
    p.are_robin_conditions_pure_neumann = 1 if robin_coeff == 0.0 else 0
    p.are_robin_coeffs_nonnegative = 1 if robin_coeff >= 0.0 else 0
    if robin_coeff != 0.0:
        p.robin_coeff_kind = A.ZGPU_FIELD_CONSTANT
        p.robin_coeff_value = robin_coeff
        p.robin_coeff_value_aligned = robin_coeff
    p.memory = A.ZGPU_MEM_HOST
    return p


def with_grid_fields(pr, fields=("dirichlet",), shape=None, interpolate=True, robin_coeff=None):
    """Replaces analytic PDE fields of pr by dense grids sampled at the cell centres of the
    domain box (DenseGrid<float, 1, DIM>): "dirichlet" (g = u) and "source" (f = -Lap u +
    sigma u).  robin_coeff: a callable kappa(x) sampled onto a "robin_coeff" grid (the Robin
    data stays analytic, h = du/dn + kappa(x) u, so u remains the exact solution); the
    boundary's per-primitive coefficient bounds become the grid's range.  The grid arrays are
    kept on pr.grids (the descriptor points at them)."""
    D = pr.dim
    shape = tuple(shape or ((1024, 1024) if D == 2 else (96, 96, 96)))
    lo = np.asarray(pr.domain_min[:D], np.float64)
    hi = np.asarray(pr.domain_max[:D], np.float64)
    axes = [lo[i] + (np.arange(shape[i]) + 0.5) * (hi[i] - lo[i]) / shape[i] for i in range(D)]
    centres = np.stack(np.meshgrid(*axes, indexing="ij"), -1).reshape(-1, D)
    u, _, lap = eval_analytic(pr.solution, centres)
    pr.grids = getattr(pr, "grids", [])

    def grid(values):
        v = np.ascontiguousarray(values, np.float32)
        pr.grids.append(v)
        g = A.Grid()
        g.values = v.ctypes.data
        for i in range(D):
            g.shape[i] = shape[i]
            g.grid_min[i] = lo[i]
            g.grid_max[i] = hi[i]
        g.enable_interpolation = int(interpolate)
        return g
    for f in fields:
        if f == "dirichlet":
            pr.pde.dirichlet_kind = A.ZGPU_FIELD_GRID
            pr.pde.dirichlet_grid = grid(u)
        elif f == "source":
            pr.pde.source_kind = A.ZGPU_FIELD_GRID
            pr.pde.is_source_constant = 0
            pr.pde.source_grid = grid(-lap + pr.pde.absorption_coeff * u)
        else:
            raise ValueError(f"unknown grid field {f}")
    if robin_coeff is not None:
        k = np.asarray(robin_coeff(centres), np.float32)
        pr.pde.robin_coeff_kind = A.ZGPU_FIELD_GRID
        pr.pde.robin_coeff_grid = grid(k)
        pr.pde.are_robin_conditions_pure_neumann = 0
        pr.pde.are_robin_coeffs_nonnegative = int(k.min() >= 0.0)
        n = len(pr.reflecting[1])
        pr.robin_coeff_range = (np.full(n, k.min(), np.float32), np.full(n, k.max(), np.float32))
    pr.pde.memory = A.ZGPU_MEM_HOST
    pr.name += "_grid"
    return pr


def default_walk_settings(eps_abs=1e-3, eps_refl=1e-3, silhouette_precision=1e-3, rr=0.0,
                          splitting=A.FLT_MAX, max_len=1024, tikhonov=0, maximal=None, double_sided=False,
                          ignore_abs=False, ignore_refl=False, ignore_src=False):
    s = A.WalkSettingsC()
    s.epsilon_shell_for_absorbing_boundary = eps_abs
    s.epsilon_shell_for_reflecting_boundary = eps_refl
    s.silhouette_precision = silhouette_precision
    s.russian_roulette_threshold = rr
    s.splitting_threshold = splitting
    s.max_walk_length = max_len
    s.steps_before_applying_tikhonov = tikhonov
    s.steps_before_using_maximal_spheres = max_len if maximal is None else maximal
    s.solve_double_sided = int(double_sided)
    s.use_gradient_control_variates = 1
    s.use_gradient_antithetic_variates = 1
    s.use_cosine_sampling_for_derivatives = 0
    s.ignore_absorbing_boundary_contribution = int(ignore_abs)
    s.ignore_reflecting_boundary_contribution = int(ignore_refl)
    s.ignore_source_contribution = int(ignore_src)
    s.print_logs = 0
    return s


def seeds_for(n, base=0x5eed):
    """Per-point pcg32 seeds: SplitMix64 of (base * golden + point index)."""
    with np.errstate(over="ignore"):
        z = np.arange(n, dtype=np.uint64) + np.uint64((base * 0x9E3779B97F4A7C15) & 0xFFFFFFFFFFFFFFFF)
        z = z + np.uint64(0x9E3779B97F4A7C15)
        z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        z = z ^ (z >> np.uint64(31))
    return z


# ------------------------------------------------------------------------ workloads
class Problem:
    """A boundary-value problem ready for either solver."""

    def __init__(self, dim, name):
        self.dim = dim
        self.name = name
        self.absorbing = None       # (positions, indices)
        self.reflecting = None      # (positions, indices)
        self.reflecting_kind = A.ZGPU_BOUNDARY_NEUMANN
        self.robin_coeff = 0.0
        self.robin_coeff_range = None   # per-primitive (min, max) coefficient bounds; None: robin_coeff
        # threshold of the silhouette-ignore rule (getIgnoreCandidateSilhouetteCallback,
        # utils/fcpw_geometric_queries.h:1029-1038): 0 keeps every non-convex vertex/edge.
        # The reference default 1e-3 drops nearly flat concave features of finely
        # tessellated curves and biases Walk on Stars near inflection points.
        self.ignore_silhouette_precision = 0.0
        self.domain_min = None
        self.domain_max = None
        self.pde = None
        self.solution = None
        self.settings = None
        self.points = None          # (P, dim) float32
        self.n_walks = None         # (P,) int32
        self.solver = A.ZGPU_SOLVER_WALK_ON_SPHERES

    def exact(self, x=None):
        u, _, _ = eval_analytic(self.solution, self.points if x is None else x)
        return u


def laplace_wos_2d(n_segments=1024, grid=128, spp=256, eps=1e-3, max_len=1024):
    """2D Laplace, pure Dirichlet, Walk on Spheres on the star polygon (g = e^x cos y)."""
    pr = Problem(2, f"laplace_wos_2d_s{n_segments}_g{grid}_w{spp}")
    pos, idx = star_polygon(n_segments)
    pr.absorbing = (pos, idx)
    pr.domain_min, pr.domain_max = bounding_box(pos)
    pr.solution = solution_expcos(0.0)
    pr.pde = make_pde(pr.solution, sigma=0.0, source=False)
    pr.settings = default_walk_settings(eps_abs=eps, max_len=max_len)
    pr.points = _interior_grid_2d(pos, pr.domain_min, pr.domain_max, grid, eps)
    pr.n_walks = np.full(pr.points.shape[0], spp, np.int32)
    pr.solver = A.ZGPU_SOLVER_WALK_ON_SPHERES
    return pr


def mixed_wost_2d(n_segments=4096, grid=256, spp=512, sigma=0.0, eps=1e-3, max_len=1024):
    """2D mixed Dirichlet (theta in [0,pi)) / Neumann (theta in [pi,2pi)) Walk on Stars,
    u = e^x cos y + 0.25 (x^2 + y^2); sigma = 0 gives the constant source f = -1."""
    pr = Problem(2, f"mixed_wost_2d_s{n_segments}_g{grid}_w{spp}_sigma{sigma:g}")
    pos, idx = star_polygon(n_segments)
    absorbing, reflecting = partition_boundary_mesh(
        lambda m: np.mod(np.arctan2(m[:, 1], m[:, 0]), 2 * np.pi) >= np.pi, pos, idx)
    pr.absorbing, pr.reflecting = absorbing, reflecting
    pr.domain_min, pr.domain_max = bounding_box(pos)
    pr.solution = solution_expcos(0.25)
    if sigma == 0.0:
        pr.pde = make_pde(pr.solution, sigma=0.0, robin=True, constant_source=-1.0)
    else:
        pr.pde = make_pde(pr.solution, sigma=sigma, robin=True)
    pr.settings = default_walk_settings(eps_abs=eps, eps_refl=eps, max_len=max_len)
    pr.points = _interior_grid_2d(pos, pr.domain_min, pr.domain_max, grid, eps)
    pr.n_walks = np.full(pr.points.shape[0], spp, np.int32)
    pr.solver = A.ZGPU_SOLVER_WALK_ON_STARS
    return pr


def mixed_star_scene(seed, n_segments, n_points, spp, eps=1e-3, max_len=1024):
    """One scene of the batched many-solve: a seeded random star polygon (about the origin)
    with Neumann conditions on the half theta in [a, a + pi) for a random split angle a,
    Dirichlet on the rest, u = e^x cos y + 0.25 (x^2 + y^2), f = -1; n_points uniform
    interior points clear of the epsilon shell; spp walks each."""
    rng = np.random.default_rng(seed)
    amp, freq, phase = rng.uniform(0.1, 0.35), int(rng.integers(3, 8)), rng.uniform(0, 2 * np.pi)
    split = rng.uniform(0, 2 * np.pi)
    pr = Problem(2, f"mixed_star_s{seed}_n{n_segments}_p{n_points}_w{spp}")
    pos, idx = star_polygon(n_segments, amp=amp, freq=freq, phase=phase)
    absorbing, reflecting = partition_boundary_mesh(
        lambda m: np.mod(np.arctan2(m[:, 1], m[:, 0]) - split, 2 * np.pi) < np.pi, pos, idx)
    pr.absorbing, pr.reflecting = absorbing, reflecting
    pr.domain_min, pr.domain_max = bounding_box(pos)
    pr.solution = solution_expcos(0.25)
    pr.pde = make_pde(pr.solution, sigma=0.0, robin=True, constant_source=-1.0)
    pr.settings = default_walk_settings(eps_abs=eps, eps_refl=eps, max_len=max_len)
    pts = []
    have = 0
    while have < n_points:
        p = rng.uniform(pr.domain_min[:2], pr.domain_max[:2], (2 * (n_points - have) + 64, 2))
        inside, rad = polygon_inside_and_radius(p, pos)
        keep = inside & (rad - np.linalg.norm(p, axis=1) > 4 * eps)
        pts.append(p[keep]); have += int(keep.sum())
    pr.points = np.concatenate(pts)[:n_points].astype(np.float32)
    pr.n_walks = np.full(n_points, spp, np.int32)
    pr.solver = A.ZGPU_SOLVER_WALK_ON_STARS
    return pr


def batched_scenes(n_scenes=64, seed=0, point_scale=1.0, segments=(256, 16384), points=(10_000, 500_000),
                   spps=(64, 128, 256, 512)):
    """The batched many-solve workload: n_scenes independent 2D mixed problems with segment
    counts log-uniform in `segments`, evaluation point counts log-uniform in `points` (times
    point_scale) and walk counts uniform over `spps`."""
    rng = np.random.default_rng(seed)
    out = []
    for k in range(n_scenes):
        nseg = int(np.exp(rng.uniform(np.log(segments[0]), np.log(segments[1]))))
        npts = max(16, int(point_scale * np.exp(rng.uniform(np.log(points[0]), np.log(points[1])))))
        spp = int(rng.choice(spps))
        out.append(mixed_star_scene(int(rng.integers(1 << 31)), nseg, npts, spp))
    return out


def _interior_grid_2d(pos, lo, hi, grid, eps):
    xs = lo[0] + (np.arange(grid) + 0.5) * (hi[0] - lo[0]) / grid
    ys = lo[1] + (np.arange(grid) + 0.5) * (hi[1] - lo[1]) / grid
    X, Y = np.meshgrid(xs, ys, indexing="xy")
    p = np.stack([X.ravel(), Y.ravel()], 1)
    inside, rad = polygon_inside_and_radius(p, pos)
    # keep points clear of the epsilon shell (distance along the ray bounds the true distance
    # from above, so use a conservative margin of 2 eps on the radial gap)
    gap = rad - np.linalg.norm(p, axis=1)
    keep = inside & (gap > 4 * eps)
    return p[keep].astype(np.float32)


def robin_wost_3d(level=6, n_points=1_000_000, spp=128, kappa=2.0, seed=0, rr=0.5, max_len=1024, eps=1e-3):
    """3D pure-Robin Walk on Stars on a displaced icosphere, u = sin x sinh(sqrt2 y) cos z + 0.5."""
    pr = Problem(3, f"robin_wost_3d_l{level}_p{n_points}_w{spp}")
    pos, idx, sh = displaced_icosphere(level, seed)
    pr.reflecting = (pos, idx)
    pr.reflecting_kind = A.ZGPU_BOUNDARY_ROBIN
    pr.robin_coeff = kappa
    pr.domain_min, pr.domain_max = bounding_box(pos)
    pr.solution = solution_sin_sinh_cos(0.5)
    pr.pde = make_pde(pr.solution, sigma=0.0, dirichlet=False, robin=True, robin_coeff=kappa, source=False)
    pr.settings = default_walk_settings(eps_abs=eps, eps_refl=eps, rr=rr, max_len=max_len)
    pr.points = interior_points_3d(sh, level, n_points, seed + 1)
    pr.n_walks = np.full(pr.points.shape[0], spp, np.int32)
    pr.solver = A.ZGPU_SOLVER_WALK_ON_STARS
    pr.sh = sh
    return pr


def screened_wos_3d(level=8, n_points=4_000_000, spp=64, sigma=4.0, seed=0, eps=1e-3, max_len=1024):
    """3D screened Poisson (sigma = 4), pure Dirichlet, u = exp(0.5x) cos y + z^2."""
    pr = Problem(3, f"screened_wos_3d_l{level}_p{n_points}_w{spp}")
    pos, idx, sh = displaced_icosphere(level, seed)
    pr.absorbing = (pos, idx)
    pr.domain_min, pr.domain_max = bounding_box(pos)
    pr.solution = solution_exp_cos_z2()
    pr.pde = make_pde(pr.solution, sigma=sigma, source=True)
    pr.settings = default_walk_settings(eps_abs=eps, max_len=max_len)
    pr.points = interior_points_3d(sh, level, n_points, seed + 1)
    pr.n_walks = np.full(pr.points.shape[0], spp, np.int32)
    pr.solver = A.ZGPU_SOLVER_WALK_ON_SPHERES
    pr.sh = sh
    return pr


def interior_points_3d(sh, level, n, seed):
    """Uniform points inside the displaced icosphere, kept clear of the boundary by the
    chord sag of the level-`level` tessellation (so they are inside the mesh as well)."""
    rng = np.random.default_rng(seed)
    edge = 1.3 * 1.1 / (2 ** level)       # icosahedron edge 1.05 at unit radius, halved per level
    margin = 0.5 * edge * edge + 2e-3      # sag of a chord of that length, plus the epsilon shell
    out = []
    need = n
    while need > 0:
        m = int(need * 2.2) + 1024
        p = rng.uniform(-1.2, 1.2, (m, 3))
        r = np.linalg.norm(p, axis=1)
        ok = r < sh.radius(p) * (1.0 - 0.0) - margin
        p = p[ok][:need]
        out.append(p)
        need -= p.shape[0]
    return np.concatenate(out, 0).astype(np.float32)
