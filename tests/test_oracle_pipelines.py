"""The oracle's boundary value caching and reverse Walk on Stars end to end on the CPU (a 2D star
polygon and a 3D displaced icosphere, level 4), with the host samplers of zombie_gb300.bvc and
the oracle's own closest-point queries: the estimates (and the splatted gradients) recover
manufactured solutions; the reverse walks' splat weights match an FP64 restatement (one step
per walk, 2D / 3D, harmonic / Yukawa); and two FP32 / estimator
properties of the reference's algorithm that the 3D GPU tests are configured around are pinned:

* the 3D Yukawa ball evaluates I_{3/2}(mu R) as cosh(mu R) - sinh(mu R) / (mu R)
  (core/distributions.h:848-851), which cancels in FP32 near mu R = 1e-3: gradient estimates
  from boundary samples offset 1e-3 into a sigma = 4 domain contain NaN normal derivatives,
  at an offset of 1e-2 none;
* the reverse walks' unnormalised absorbing estimate (the one used with absorption) counts
  walks absorbed in the epsilon shell as reaching the boundary: for g = 1 it reads clearly
  below 1 with a 1e-3 shell and about 1 with a 1e-4 shell (same walks otherwise)."""
import numpy as np
import pytest

from zombie_gb300 import _abi as A
from zombie_gb300 import problems as P
from zombie_gb300.api import SampleType


class _Queries:
    """The distance queries the samplers need, answered by the oracle's brute-force closest points."""
    dim = 3

    def __init__(self, boundary, inside):
        self.b = boundary
        self.inside = inside

    def compute_dist_to_absorbing_boundary(self, x, compute_signed_distance=False):
        d = self.b.closest_point(np.asarray(x, np.float32))[2]
        return np.where(self.inside(x), -d, d).astype(np.float32) if compute_signed_distance else d

    def compute_dist_to_reflecting_boundary(self, x, compute_signed_distance=False):
        return np.full(len(x), np.finfo(np.float32).max, np.float32)


def _scene(oracle, sigma):
    pr = P.screened_wos_3d(level=4, n_points=300, spp=4, sigma=sigma)
    ob = oracle.Boundary(3, *pr.absorbing)

    def inside(x):
        x = np.asarray(x, np.float64)
        return np.linalg.norm(x, axis=1) < pr.sh.radius(x)
    return pr, ob, inside, _Queries(ob, inside)


def _boundary_estimates(oracle, pr, ob, cache, n_walks):
    """computeBoundaryEstimates on the oracle: u and du/dn along the sample normals."""
    n = len(cache)
    pts = dict(pt=cache.pt, normal=cache.normal, type=cache.type, estimation_quantity=np.full(n, 1, np.int32),
               dist_to_absorbing=cache.dist_to_absorbing, dist_to_reflecting=cache.dist_to_reflecting,
               n_walks=np.full(n, n_walks, np.int32), seed=cache.seed, first_sphere_radius=np.zeros(n, np.float32),
               direction_for_derivative=np.ascontiguousarray(cache.normal))
    st = dict(solution_mean=np.zeros(n), solution_m2=np.zeros(n), n_solution_estimates=np.zeros(n, np.int32),
              total_walk_length=np.zeros(n, np.int64), total_splits=np.zeros(n, np.int64),
              gradient_mean=np.zeros((n, 3)), gradient_m2=np.zeros((n, 3)), n_gradient_estimates=np.zeros(n, np.int32),
              total_first_source_contribution=np.zeros(n), total_derivative_contribution=np.zeros(n))
    oracle.solve(A.ZGPU_SOLVER_WALK_ON_STARS, 3, ob, None, pr.domain_min, pr.domain_max, pr.pde, pr.settings, pts, st)
    cache.solution[:] = st["solution_mean"]
    cache.normal_derivative[:] = st["total_derivative_contribution"] / np.maximum(st["n_solution_estimates"], 1)


def _boundary_cache(pr, ob, inside, q, n, offset, seed):
    from zombie_gb300 import bvc
    s = bvc.UniformTriangleBoundarySampler(*pr.absorbing, inside, seed=seed)
    s.initialize(offset, False)
    return s.generate_samples(s.get_sample_count(n, False), int(SampleType.OnAbsorbingBoundary), offset, q, False)


def _domain_cache(pr, inside, q, n, seed):
    from zombie_gb300 import bvc
    lo, hi = np.asarray(pr.domain_min[:3]), np.asarray(pr.domain_max[:3])
    u = np.random.default_rng(seed).uniform(lo, hi, (200000, 3))
    vol = float(np.prod(hi - lo)) * float(np.mean(inside(u)))
    return bvc.UniformDomainSampler(inside, lo, hi, vol, seed=seed + 1).generate_samples(n, q)


def test_oracle_bvc_screened_3d_recovers_the_solution(oracle):
    """sigma = 4, u = exp(0.5x) cos y + z^2: boundary samples offset 1e-2 with walk estimates of
    u and du/dn, domain samples with source values, splatted onto interior points."""
    pr, ob, inside, q = _scene(oracle, 4.0)
    c = _boundary_cache(pr, ob, inside, q, 4096, 1e-2, 11)
    _boundary_estimates(oracle, pr, ob, c, 32)
    d = _domain_cache(pr, inside, q, 16384, 12)
    d.contribution[:] = oracle.eval_pde(3, pr.pde, d.pt)[0]
    m = len(pr.points)
    dist = ob.closest_point(pr.points)[2]
    ev = dict(pt=np.ascontiguousarray(pr.points), type=np.zeros(m, np.int32), dist_to_absorbing=dist.astype(np.float32),
              dist_to_reflecting=np.full(m, np.finfo(np.float32).max, np.float32), mean=np.zeros((m, 5)),
              m2=np.zeros((m, 5)), count=np.zeros((m, 5), np.int32), gradient_mean=np.zeros((m, 5, 3)),
              gradient_m2=np.zeros((m, 5, 3)))
    for cc in (c, d):
        smp = {k: np.ascontiguousarray(getattr(cc, k)) for k in
               ("pt", "normal", "pdf", "type", "estimate_normal_aligned", "solution", "normal_derivative",
                "contribution", "robin_coeff")}
        oracle.bvc_splat(3, 4.0, smp, ev, radius_clamp=1e-3, cutoff_absorbing=0.05)
    far = dist >= 0.05
    est, ex = ev["mean"].sum(1)[far], pr.exact()[far]
    rmse = float(np.sqrt(np.mean((est - ex) ** 2)))
    assert np.all(np.isfinite(c.normal_derivative))
    assert rmse < 0.1 * float(np.std(ex)) + 0.02, rmse
    assert np.corrcoef(est, ex)[0, 1] > 0.98


def test_oracle_yukawa_3d_gradient_cancels_in_fp32_at_small_balls(oracle):
    """Normal derivatives of boundary samples in a sigma = 4 domain: NaN for some samples offset
    1e-3 (first ball mu R ~ 2e-3), none offset 1e-2 (mu R ~ 2e-2)."""
    pr, ob, inside, q = _scene(oracle, 4.0)
    nans = {}
    for offset in (1e-3, 1e-2):
        c = _boundary_cache(pr, ob, inside, q, 2000, offset, 11)
        _boundary_estimates(oracle, pr, ob, c, 64)
        assert np.all(np.isfinite(c.solution))
        nans[offset] = int(np.isnan(c.normal_derivative).sum())
    assert nans[1e-3] > 0 and nans[1e-2] == 0, nans


def _rws(oracle, pr, ob, samples_list, eps_abs):
    m = len(pr.points)
    ev = dict(pt=np.ascontiguousarray(pr.points), normal=np.zeros((m, 3), np.float32), type=np.zeros(m, np.int32),
              totals=np.zeros((m, A.ZGPU_RWS_TOTALS)))
    ws = P.default_walk_settings(eps_abs=eps_abs, max_len=1024)
    for c, offset in samples_list:
        smp = {k: np.ascontiguousarray(getattr(c, k)) for k in
               ("pt", "normal", "type", "estimate_normal_aligned", "pdf", "contribution", "dist_to_absorbing", "seed")}
        oracle.rws_solve(3, ob, None, pr.domain_min, pr.domain_max, pr.pde, ws, smp, ev, offset, stream=0)
    return ev["totals"]


def test_oracle_reverse_walks_3d_recover_the_solution(oracle):
    """sigma = 0 (self-normalised absorbing part) with the source of u = exp(0.5x) cos y + z^2."""
    pr, ob, inside, q = _scene(oracle, 0.0)
    offset = 5e-3
    a = _boundary_cache(pr, ob, inside, q, 32768, offset, 21)
    sd = q.compute_dist_to_absorbing_boundary(a.pt, True)
    a.contribution[:] = oracle.eval_pde(3, pr.pde, a.pt - sd[:, None] * a.normal)[1]
    d = _domain_cache(pr, inside, q, 32768, 22)
    d.contribution[:] = oracle.eval_pde(3, pr.pde, d.pt)[0]
    t = _rws(oracle, pr, ob, [(a, offset), (d, offset)], 1e-3)
    pk = t[:, A.ZGPU_RWS_POISSON_KERNEL]
    assert np.all(pk > 0)
    est = t[:, A.ZGPU_RWS_ABSORBING] / pk + t[:, A.ZGPU_RWS_SOURCE] / len(d)
    far = ob.closest_point(pr.points)[2] > 0.05
    ex = pr.exact()[far]
    rmse = float(np.sqrt(np.mean((est[far] - ex) ** 2)))
    assert rmse < 0.3 * float(np.std(ex)) + 0.03, rmse
    assert np.corrcoef(est[far], ex)[0, 1] > 0.95


def test_oracle_unnormalised_reverse_estimate_ends_walks_in_the_epsilon_shell(oracle):
    """g = 1, sigma = 0, offset 5e-3, read without the Poisson-kernel normalisation: the same
    walks with a 1e-3 absorbing shell read clearly below 1, with a 1e-4 shell about 1."""
    pr, ob, inside, q = _scene(oracle, 0.0)
    offset = 5e-3
    a = _boundary_cache(pr, ob, inside, q, 65536, offset, 21)
    a.contribution[:] = 1.0
    far = ob.closest_point(pr.points)[2] > 0.05
    means = {}
    for eps in (1e-3, 1e-4):
        t = _rws(oracle, pr, ob, [(a, offset)], eps)
        means[eps] = float((t[:, A.ZGPU_RWS_ABSORBING] / len(a))[far].mean())
    assert means[1e-4] - means[1e-3] > 0.04, means
    assert abs(means[1e-4] - 1.0) < 0.06, means


def test_oracle_bvc_laplace_2d_splats_values_and_gradients(oracle):
    """u = e^x cos y on the 1024-segment star polygon: 8192 boundary samples offset 1e-3 with
    256 walks each for u and du/dn; the splat recovers u and grad u at interior grid points."""
    from zombie_gb300 import bvc
    pos, idx = P.star_polygon(1024)
    ob = oracle.Boundary(2, pos, idx)

    def inside(x):
        return P.polygon_inside_and_radius(np.asarray(x, np.float64), pos)[0]

    class Q2(_Queries):
        dim = 2
    q = Q2(ob, inside)
    pde = P.make_pde(P.solution_expcos(0.0), source=False)
    ws = P.default_walk_settings(eps_abs=1e-3, max_len=1024)
    s = bvc.UniformLineSegmentBoundarySampler(pos, idx, inside, seed=11)
    s.initialize(1e-3, False)
    c = s.generate_samples(8192, int(SampleType.OnAbsorbingBoundary), 1e-3, q, False)
    n = len(c)
    pts = dict(pt=c.pt, normal=c.normal, type=c.type, estimation_quantity=np.full(n, 1, np.int32),
               dist_to_absorbing=c.dist_to_absorbing, dist_to_reflecting=c.dist_to_reflecting,
               n_walks=np.full(n, 256, np.int32), seed=c.seed, first_sphere_radius=np.zeros(n, np.float32),
               direction_for_derivative=np.ascontiguousarray(c.normal))
    st = dict(solution_mean=np.zeros(n), solution_m2=np.zeros(n), n_solution_estimates=np.zeros(n, np.int32),
              total_walk_length=np.zeros(n, np.int64), total_splits=np.zeros(n, np.int64),
              gradient_mean=np.zeros((n, 2)), gradient_m2=np.zeros((n, 2)), n_gradient_estimates=np.zeros(n, np.int32),
              total_first_source_contribution=np.zeros(n), total_derivative_contribution=np.zeros(n))
    oracle.solve(A.ZGPU_SOLVER_WALK_ON_STARS, 2, ob, None, np.array([-1.3, -1.3]), np.array([1.3, 1.3]), pde, ws,
                 pts, st)
    c.solution[:] = st["solution_mean"]
    c.normal_derivative[:] = st["total_derivative_contribution"] / np.maximum(st["n_solution_estimates"], 1)
    g = (np.arange(24) + 0.5) / 24 * 2.6 - 1.3
    X, Y = np.meshgrid(g, g, indexing="ij")
    grid = np.stack([X.ravel(), Y.ravel()], 1).astype(np.float32)
    grid = grid[inside(grid)]
    dist = ob.closest_point(grid)[2]
    m = len(grid)
    ev = dict(pt=np.ascontiguousarray(grid), type=np.zeros(m, np.int32), dist_to_absorbing=dist.astype(np.float32),
              dist_to_reflecting=np.full(m, np.finfo(np.float32).max, np.float32), mean=np.zeros((m, 5)),
              m2=np.zeros((m, 5)), count=np.zeros((m, 5), np.int32), gradient_mean=np.zeros((m, 5, 2)),
              gradient_m2=np.zeros((m, 5, 2)))
    smp = {k: np.ascontiguousarray(getattr(c, k)) for k in ("pt", "normal", "pdf", "type", "estimate_normal_aligned",
                                                            "solution", "normal_derivative", "contribution",
                                                            "robin_coeff")}
    oracle.bvc_splat(2, 0.0, smp, ev, radius_clamp=1e-3, cutoff_absorbing=0.05)
    far = dist >= 0.05
    x = grid[far].astype(np.float64)
    u = np.exp(x[:, 0]) * np.cos(x[:, 1])
    gu = np.stack([u, -np.exp(x[:, 0]) * np.sin(x[:, 1])], 1).ravel()
    est = ev["mean"].sum(1)[far]
    ge = ev["gradient_mean"].sum(1)[far].ravel()
    assert np.all(ev["count"][~far] == 0)
    assert np.sqrt(np.mean((est - u) ** 2)) < 0.1 * np.std(u) + 0.02
    assert np.sqrt(np.mean((ge - gu) ** 2)) < 0.25 * np.std(gu) + 0.05
    assert np.corrcoef(ge, gu)[0, 1] > 0.98


@pytest.mark.parametrize("dim,sigma", [(2, 0.0), (2, 2.0), (3, 0.0), (3, 2.0)])
def test_oracle_reverse_splat_matches_an_independent_restatement(oracle, dim, sigma):
    """One step per reverse walk (max walk length 1, maximal spheres from the first step, no
    reflecting boundary): every sample splats only its first ball, centred at the sample with
    radius its distance to the absorbing boundary, so each evaluation point's totals are
    sum_s G_ball(max(clamp, |x - y_s|); R_s) / pdf_s * contribution_s (divided by the normal
    offset for absorbing samples; the Poisson-kernel total adds the weights of unscreened
    absorbing samples) over the balls holding it (splatContribution,
    variance_reduction/reverse_walk_solver.h:236-302).  The ball Green's functions are
    restated in FP64 with scipy's Bessel functions (core/distributions.h:453-1005)."""
    from scipy import special
    rng = np.random.default_rng(70 + dim + int(sigma))
    if dim == 2:
        pos, idx = P.star_polygon(1024)
        inside = lambda x: P.polygon_inside_and_radius(np.asarray(x, np.float64), pos)[0]
        lo, hi = np.array([-1.3, -1.3]), np.array([1.3, 1.3])
    else:
        pos, idx, sh = P.displaced_icosphere(3, 0)
        inside = lambda x: np.linalg.norm(np.asarray(x, np.float64), axis=1) < sh.radius(np.asarray(x, np.float64))
        lo, hi = pos.min(0) - 0.05, pos.max(0) + 0.05
    ob = oracle.Boundary(dim, pos, idx)

    def interior(n):
        x = rng.uniform(lo, hi, (4 * n, dim)).astype(np.float32)
        return x[inside(x)][:n]
    ns, ne, offset, clamp = 64, 600, 0.01, 1e-3
    y = interior(ns)
    R = ob.closest_point(y)[2].astype(np.float32)
    typ = np.where(np.arange(ns) % 2 == 0, 0, 1).astype(np.int32)       # source / absorbing samples
    pdf = rng.uniform(0.5, 2.0, ns).astype(np.float32)
    contrib = rng.uniform(-1.0, 1.0, ns).astype(np.float32)
    smp = dict(pt=y, normal=np.zeros_like(y), type=typ, estimate_normal_aligned=np.zeros(ns, np.int32), pdf=pdf,
               contribution=contrib, dist_to_absorbing=R, seed=np.arange(1, ns + 1, dtype=np.uint64))
    x = interior(ne)
    ev = dict(pt=x, normal=np.zeros_like(x), type=np.zeros(len(x), np.int32), totals=np.zeros((len(x), 6)))
    pde = P.make_pde(P.solution_expcos(0.0), sigma=sigma)
    ws = P.default_walk_settings(eps_abs=1e-4, max_len=1, maximal=0)
    oracle.rws_solve(dim, ob, None, lo, hi, pde, ws, smp, ev, offset, radius_clamp=clamp, stream=0)

    # FP64 restatement
    mu = np.sqrt(sigma)
    d = np.linalg.norm(x.astype(np.float64)[:, None, :] - y.astype(np.float64)[None, :, :], axis=2)   # [ne, ns]
    Rd = R.astype(np.float64)[None, :]
    r = np.maximum(clamp, d)
    if dim == 2 and sigma == 0:
        G = np.log(Rd / r) / (2 * np.pi)
    elif dim == 2:
        G = (special.k0(mu * r) - special.i0(mu * r) * special.k0(mu * Rd) / special.i0(mu * Rd)) / (2 * np.pi)
    elif sigma == 0:
        G = (1.0 / r - 1.0 / Rd) / (4 * np.pi)
    else:
        G = (np.exp(-mu * r) - np.exp(-mu * Rd) * np.sinh(mu * r) / np.sinh(mu * Rd)) / (4 * np.pi * r)
    inball = d < Rd
    w = np.where(inball, G / pdf[None, :], 0.0)
    w = np.where(typ[None, :] == 1, w / offset, w)
    src = (w * np.where(typ == 0, contrib, 0.0)[None, :]).sum(1)
    ab = (w * np.where(typ == 1, contrib, 0.0)[None, :]).sum(1)
    pk = (w * (typ == 1)[None, :]).sum(1) if sigma == 0 else np.zeros(len(x))
    # points within FP32 rounding of a ball's edge may fall either side: leave them out
    clear = np.all(np.abs(d - Rd) > 1e-4 * Rd, axis=1)
    t = ev["totals"]
    assert np.sum(np.any(inball, axis=1) & clear) > 50
    for got, want in ((t[:, 4], src), (t[:, 0], ab), (t[:, 5], pk)):
        assert np.allclose(got[clear], want[clear], rtol=2e-4, atol=2e-5 * np.abs(want).max() + 1e-12)
    assert np.all(t[:, [1, 2, 3]] == 0.0)
