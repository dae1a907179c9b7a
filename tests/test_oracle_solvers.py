"""The oracle's walk estimators against FP64 manufactured solutions (small sizes)."""
import numpy as np
import pytest

from zombie_gb300 import _abi as A
from zombie_gb300 import problems as P


def run_oracle(oracle, pr, n_threads=None, seeds=None):
    D = pr.dim
    ab = oracle.Boundary(D, *pr.absorbing) if pr.absorbing is not None and len(pr.absorbing[1]) else None
    rf = None
    if pr.reflecting is not None and len(pr.reflecting[1]):
        kmin = kmax = None
        if pr.reflecting_kind == A.ZGPU_BOUNDARY_ROBIN:
            if pr.robin_coeff_range is not None:
                kmin, kmax = pr.robin_coeff_range
            else:
                kmin = kmax = np.full(len(pr.reflecting[1]), pr.robin_coeff, np.float32)
        rf = oracle.Boundary(D, *pr.reflecting, kind=pr.reflecting_kind, kmin=kmin, kmax=kmax,
                             silhouette_precision=pr.ignore_silhouette_precision)
    n = pr.points.shape[0]
    if ab is not None:
        d = ab.closest_point(pr.points)[2]
    else:
        m = np.minimum(pr.domain_min - pr.points, pr.points - pr.domain_max)
        d = np.linalg.norm(m, axis=1).astype(np.float32)
    pts = dict(pt=pr.points, dist_to_absorbing=d, n_walks=pr.n_walks,
               seed=P.seeds_for(n) if seeds is None else seeds, first_sphere_radius=np.zeros(n, np.float32))
    st = dict(solution_mean=np.zeros(n), solution_m2=np.zeros(n), n_solution_estimates=np.zeros(n, np.int32),
              total_walk_length=np.zeros(n, np.int64), total_splits=np.zeros(n, np.int64))
    steps = oracle.solve(pr.solver, D, ab, rf, pr.domain_min, pr.domain_max, pr.pde, pr.settings, pts, st, n_threads)
    return st, steps


def run_oracle_with(oracle, pr, st=None, estimation_quantity=None, extra_stats=None, n_threads=None, direction=None):
    """run_oracle with extra point fields and statistics, accumulating into st across calls."""
    D = pr.dim
    ab = oracle.Boundary(D, *pr.absorbing) if pr.absorbing is not None and len(pr.absorbing[1]) else None
    rf = None
    if pr.reflecting is not None and len(pr.reflecting[1]):
        rf = oracle.Boundary(D, *pr.reflecting, kind=pr.reflecting_kind,
                             silhouette_precision=pr.ignore_silhouette_precision)
    n = pr.points.shape[0]
    d = ab.closest_point(pr.points)[2] if ab is not None else None
    pts = dict(pt=pr.points, dist_to_absorbing=d, n_walks=pr.n_walks, seed=P.seeds_for(n),
               first_sphere_radius=np.zeros(n, np.float32))
    if estimation_quantity is not None:
        pts["estimation_quantity"] = estimation_quantity
    if direction is not None:
        pts["direction_for_derivative"] = np.ascontiguousarray(direction, np.float32)
    if st is None:
        st = dict(solution_mean=np.zeros(n), solution_m2=np.zeros(n), n_solution_estimates=np.zeros(n, np.int32),
                  total_walk_length=np.zeros(n, np.int64), total_splits=np.zeros(n, np.int64))
        st.update({k: v.copy() for k, v in (extra_stats or {}).items()})
    oracle.solve(pr.solver, D, ab, rf, pr.domain_min, pr.domain_max, pr.pde, pr.settings, pts, st, n_threads)
    return st


def zscores(st, exact):
    n = st["n_solution_estimates"].astype(np.float64)
    se = np.sqrt(st["solution_m2"] / np.maximum(n - 1, 1) / np.maximum(n, 1))
    return (st["solution_mean"] - exact) / np.maximum(se, 1e-12)


def test_wos_laplace_2d_matches_analytic(oracle):
    pr = P.laplace_wos_2d(n_segments=1024, grid=20, spp=512)
    st, steps = run_oracle(oracle, pr)
    z = zscores(st, pr.exact())
    assert steps > 0
    assert abs(z.mean()) < 4.0 / np.sqrt(len(z)) + 0.1   # epsilon-shell bias is O(1e-3)
    assert np.mean(np.abs(z) > 3.5) < 0.02


def test_wost_mixed_2d_matches_analytic(oracle):
    pr = P.mixed_wost_2d(n_segments=2048, grid=16, spp=512)
    st, _ = run_oracle(oracle, pr)
    z = zscores(st, pr.exact())
    assert abs(z.mean()) < 0.35
    assert np.mean(np.abs(z) > 3.5) < 0.03


def test_wost_screened_2d_matches_analytic(oracle):
    pr = P.mixed_wost_2d(n_segments=2048, grid=12, spp=256, sigma=1.0)
    st, _ = run_oracle(oracle, pr)
    z = zscores(st, pr.exact())
    assert abs(z.mean()) < 0.45
    assert np.mean(np.abs(z) > 3.5) < 0.04


def test_wost_robin_3d_matches_analytic(oracle):
    pr = P.robin_wost_3d(level=3, n_points=120, spp=256, kappa=2.0)
    st, _ = run_oracle(oracle, pr)
    z = zscores(st, pr.exact())
    assert abs(z.mean()) < 0.45
    assert np.mean(np.abs(z) > 3.5) < 0.04


def test_wos_screened_3d_matches_analytic(oracle):
    pr = P.screened_wos_3d(level=3, n_points=150, spp=256, sigma=4.0)
    st, _ = run_oracle(oracle, pr)
    z = zscores(st, pr.exact())
    assert abs(z.mean()) < 0.45
    assert np.mean(np.abs(z) > 3.5) < 0.04


def test_progressive_accumulation(oracle):
    """Two calls of W walks merge (common.h:268-310) into the same moments as one call of 2W."""
    pr = P.laplace_wos_2d(n_segments=256, grid=10, spp=64)
    n = pr.points.shape[0]
    ab = oracle.Boundary(2, *pr.absorbing)
    d = ab.closest_point(pr.points)[2]
    seeds = P.seeds_for(n)

    def fresh():
        return dict(solution_mean=np.zeros(n), solution_m2=np.zeros(n), n_solution_estimates=np.zeros(n, np.int32),
                    total_walk_length=np.zeros(n, np.int64), total_splits=np.zeros(n, np.int64))
    a = fresh()
    for _ in range(2):
        pts = dict(pt=pr.points, dist_to_absorbing=d, n_walks=pr.n_walks, seed=seeds, first_sphere_radius=np.zeros(n, np.float32))
        oracle.solve(pr.solver, 2, ab, None, pr.domain_min, pr.domain_max, pr.pde, pr.settings, pts, a)
    b = fresh()
    pts = dict(pt=pr.points, dist_to_absorbing=d, n_walks=2 * pr.n_walks, seed=seeds, first_sphere_radius=np.zeros(n, np.float32))
    oracle.solve(pr.solver, 2, ab, None, pr.domain_min, pr.domain_max, pr.pde, pr.settings, pts, b)
    # walk w of the second call uses stream w + 64 == walk w + 64 of the single call
    assert np.array_equal(a["n_solution_estimates"], b["n_solution_estimates"])
    assert np.allclose(a["solution_mean"], b["solution_mean"], rtol=0, atol=1e-9)
    assert np.allclose(a["solution_m2"], b["solution_m2"], rtol=1e-9, atol=1e-9)
    assert np.array_equal(a["total_walk_length"], b["total_walk_length"])


def test_russian_roulette_and_splitting_stay_unbiased(oracle):
    pr = P.laplace_wos_2d(n_segments=512, grid=10, spp=512)
    pr.pde = P.make_pde(pr.solution, sigma=2.0, source=True)   # screened: throughput decays
    pr.settings = P.default_walk_settings(rr=0.9, splitting=1.5)
    st, _ = run_oracle(oracle, pr)
    z = zscores(st, pr.exact())
    assert abs(z.mean()) < 0.5
    assert np.mean(np.abs(z) > 3.5) < 0.04


@pytest.mark.parametrize("make", [lambda: P.laplace_wos_2d(n_segments=512, grid=10, spp=256),
                                  lambda: P.mixed_wost_2d(n_segments=512, grid=8, spp=256)])
def test_oracle_gradient_estimates_match_the_analytic_gradient(oracle, make):
    """The oracle's estimateSolutionAndGradient (antithetic pairs, stratified first steps,
    control variates from a first call) against grad u of the manufactured solution."""
    pr = make()
    n, D = pr.points.shape
    eq = np.full(n, A.ZGPU_ESTIMATE_SOLUTION_AND_GRADIENT, np.int32)
    extra = dict(gradient_mean=np.zeros((n, D)), gradient_m2=np.zeros((n, D)),
                 n_gradient_estimates=np.zeros(n, np.int32))
    st = None
    for call in range(2):
        st = run_oracle_with(oracle, pr, st, estimation_quantity=eq, extra_stats=extra)
    _, grad, _ = P.eval_analytic(pr.solution, pr.points)
    g = st["gradient_mean"].reshape(n, D)
    ng = st["n_gradient_estimates"].astype(np.float64)
    assert np.all(ng == 2 * pr.n_walks)
    se = np.sqrt(st["gradient_m2"].reshape(n, D) / np.maximum(ng - 1, 1)[:, None] / ng[:, None])
    z = (g - grad) / np.maximum(se, 1e-12)
    assert np.mean(np.abs(z) <= 4) > 0.98
    assert abs(np.mean(z)) < 0.3


def _axis_directions(n, D, seed):
    """Signed coordinate axes: the gradient moments of that axis are then exactly the
    moments of the directional derivative."""
    rng = np.random.default_rng(seed)
    axis = rng.integers(0, D, n)
    v = np.zeros((n, D), np.float32)
    v[np.arange(n), axis] = rng.choice([-1.0, 1.0], n)
    return v, axis


def _screened_2d():
    pr = P.laplace_wos_2d(n_segments=512, grid=16, spp=256)
    pr.pde = P.make_pde(pr.solution, sigma=2.0, source=True)      # f = 2u: a non-constant source
    return pr


@pytest.mark.parametrize("make", [lambda: P.laplace_wos_2d(n_segments=512, grid=16, spp=256), _screened_2d])
def test_oracle_cosine_sampled_directional_derivatives(oracle, make):
    """useCosineSamplingForDerivatives (walk_on_spheres.h:500-504): first steps drawn about
    each point's directionForDerivative; the directional derivative (getEstimatedDerivative,
    the running sum of (boundary + source gradient) . direction) matches grad u . direction,
    and equals the gradient mean projected on the direction.  The source control variate is
    the mean first source contribution of the earlier walks (getMeanFirstSourceContribution)."""
    pr = make()
    pr.settings.use_cosine_sampling_for_derivatives = 1
    n, D = pr.points.shape
    dirs, axis = _axis_directions(n, D, 3)
    eq = np.full(n, A.ZGPU_ESTIMATE_SOLUTION_AND_GRADIENT, np.int32)
    extra = dict(gradient_mean=np.zeros((n, D)), gradient_m2=np.zeros((n, D)), n_gradient_estimates=np.zeros(n, np.int32),
                 total_first_source_contribution=np.zeros(n), total_derivative_contribution=np.zeros(n))
    st = None
    for call in range(2):
        st = run_oracle_with(oracle, pr, st, estimation_quantity=eq, extra_stats=extra, direction=dirs)
    u, grad, _ = P.eval_analytic(pr.solution, pr.points)
    ng = st["n_gradient_estimates"].astype(np.float64)
    assert np.all(ng == 2 * pr.n_walks)
    assert np.array_equal(st["n_solution_estimates"], st["n_gradient_estimates"])
    g = st["gradient_mean"].reshape(n, D)
    deriv = st["total_derivative_contribution"] / ng
    proj = np.sum(g * dirs, axis=1)
    scale = np.sqrt(np.mean(proj ** 2))
    assert np.max(np.abs(deriv - proj)) <= 1e-4 * scale
    se = np.sqrt(st["gradient_m2"].reshape(n, D)[np.arange(n), axis] / np.maximum(ng - 1, 1) / ng)
    z = (deriv - np.sum(grad * dirs, axis=1)) / np.maximum(se, 1e-12)
    assert np.mean(np.abs(z) <= 3.5) > 0.98
    assert abs(np.mean(z)) < 4 / np.sqrt(n)
    if pr.pde.is_source_constant == 0:
        # the first source contributions are kept: their mean is the source part of u
        fs = st["total_first_source_contribution"] / st["n_solution_estimates"]
        assert np.all(np.isfinite(fs)) and np.any(fs != 0.0)
    else:
        assert np.all(st["total_first_source_contribution"] == 0.0)


def test_oracle_cosine_sampling_concentrates_on_the_direction(oracle):
    """Cosine-weighted first steps about the direction lower the variance of the directional
    derivative against uniform first steps (same walks otherwise)."""
    out = {}
    for cosine in (0, 1):
        pr = P.laplace_wos_2d(n_segments=512, grid=10, spp=256)
        pr.settings.use_cosine_sampling_for_derivatives = cosine
        pr.settings.use_gradient_control_variates = 0
        n, D = pr.points.shape
        dirs = np.tile(np.array([[1.0, 0.0]], np.float32), (n, 1))
        eq = np.full(n, A.ZGPU_ESTIMATE_SOLUTION_AND_GRADIENT, np.int32)
        extra = dict(gradient_mean=np.zeros((n, D)), gradient_m2=np.zeros((n, D)),
                     n_gradient_estimates=np.zeros(n, np.int32))
        st = run_oracle_with(oracle, pr, None, estimation_quantity=eq, extra_stats=extra, direction=dirs)
        out[cosine] = np.median(st["gradient_m2"].reshape(n, D)[:, 0] / np.maximum(st["n_gradient_estimates"] - 1, 1))
    assert out[1] < out[0]


@pytest.mark.parametrize("make,fields", [(lambda: P.laplace_wos_2d(n_segments=512, grid=10, spp=256), ("dirichlet",)),
                                         (_screened_2d, ("dirichlet", "source"))])
def test_oracle_dense_grid_fields_follow_the_analytic_fields(oracle, make, fields):
    """g and f read from 512^2 bilinear grids sampled from the same fields: the walks are the
    same (same streams, same lengths) and the estimates differ by the interpolation error."""
    a = make()
    b = P.with_grid_fields(make(), fields, shape=(512, 512))
    sa, _ = run_oracle(oracle, a)
    sb, _ = run_oracle(oracle, b)
    assert np.array_equal(sa["total_walk_length"], sb["total_walk_length"])
    d = sb["solution_mean"] - sa["solution_mean"]
    assert np.max(np.abs(d)) < 3e-3
    assert abs(d.mean()) < 2e-4


def test_oracle_robin_coefficient_grid_is_unbiased(oracle):
    """A spatially varying Robin coefficient read from a trilinear grid (Robin data h = du/dn
    + kappa(x) u, per-primitive coefficient bounds from the grid's range): estimates stay
    within their standard errors of u."""
    pr = P.with_grid_fields(P.robin_wost_3d(level=3, n_points=60, spp=128), (), shape=(24, 24, 24),
                            robin_coeff=lambda x: 1.5 + 0.5 * np.sin(2.0 * x[:, 0]) * np.cos(x[:, 1]))
    st, _ = run_oracle(oracle, pr)
    z = zscores(st, pr.exact())
    assert abs(z.mean()) < 0.5
    assert np.mean(np.abs(z) > 3.5) < 0.05
