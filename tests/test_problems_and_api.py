"""Synthetic workloads and host-side API logic (no GPU calls)."""
import numpy as np
import pytest

from zombie_gb300 import _abi as A
from zombie_gb300 import api
from zombie_gb300 import problems as P


def test_star_polygon_is_ccw_and_closed():
    pos, idx = P.star_polygon(1024)
    a, b = pos[idx[:, 0]], pos[idx[:, 1]]
    area = 0.5 * np.sum(a[:, 0] * b[:, 1] - a[:, 1] * b[:, 0])
    assert area > 0
    assert np.array_equal(np.sort(idx[:, 0]), np.sort(idx[:, 1]))


@pytest.mark.parametrize("level", [0, 2, 4])
def test_icosphere_is_watertight_and_outward(level):
    v, f = P.icosphere(level)
    assert f.shape[0] == 20 * 4 ** level
    edges = set()
    for t in f:
        for j in range(3):
            edges.add((t[j], t[(j + 1) % 3]))
    assert all((b, a) in edges for a, b in edges)
    n = np.cross(v[f[:, 1]] - v[f[:, 0]], v[f[:, 2]] - v[f[:, 0]])
    assert np.all((n * v[f].mean(1)).sum(1) > 0)


def test_displaced_icosphere_stays_star_shaped():
    v, f, sh = P.displaced_icosphere(4, seed=0)
    r = np.linalg.norm(v, axis=1)
    assert 0.8 <= r.min() and r.max() <= 1.2
    n = np.cross(v[f[:, 1]] - v[f[:, 0]], v[f[:, 2]] - v[f[:, 0]])
    assert np.all((n * v[f].mean(1)).sum(1) > 0)


def test_partition_keeps_orientation():
    pos, idx = P.star_polygon(64)
    (ap, ai), (rp, ri) = P.partition_boundary_mesh(lambda m: m[:, 1] < 0, pos, idx)
    assert ai.shape[0] + ri.shape[0] == 64
    for p, i in ((ap, ai), (rp, ri)):
        a, b = p[i[:, 0]], p[i[:, 1]]
        # each segment keeps its CCW direction: it turns counter-clockwise about the origin
        assert np.all(a[:, 0] * b[:, 1] - a[:, 1] * b[:, 0] > 0)


@pytest.mark.parametrize("sol", [P.solution_expcos(0.25), P.solution_sin_sinh_cos(0.5), P.solution_exp_cos_z2()])
def test_analytic_derivatives_match_finite_differences(sol):
    rng = np.random.default_rng(0)
    x = rng.uniform(-1, 1, (50, 3))
    u, g, lap = P.eval_analytic(sol, x)
    h = 1e-4
    for i in range(3):
        e = np.zeros(3); e[i] = h
        up = P.eval_analytic(sol, x + e)[0]
        um = P.eval_analytic(sol, x - e)[0]
        assert np.allclose((up - um) / (2 * h), g[:, i], atol=1e-6)
    lap_fd = sum((P.eval_analytic(sol, x + np.eye(3)[i] * 1e-3)[0] - 2 * u
                  + P.eval_analytic(sol, x - np.eye(3)[i] * 1e-3)[0]) / 1e-6 for i in range(3))
    assert np.allclose(lap_fd, lap, atol=1e-4)


def test_harmonic_solutions_are_harmonic():
    x = np.random.default_rng(1).uniform(-1, 1, (20, 3))
    for s in (P.solution_expcos(0.0), P.solution_sin_sinh_cos(0.5)):
        assert np.allclose(P.eval_analytic(s, x)[2], 0.0, atol=1e-6)   # float32 coefficients


def test_oracle_pde_fields_follow_the_solution(oracle):
    pr = P.mixed_wost_2d(n_segments=64, grid=8, spp=1, sigma=1.0)
    x = pr.points
    n = np.tile(np.array([[0.6, -0.8]], np.float32), (x.shape[0], 1))
    src, dirv, rob = oracle.eval_pde(2, pr.pde, x, n)
    u, g, lap = P.eval_analytic(pr.solution, x)
    assert np.allclose(dirv, u, rtol=1e-5, atol=1e-5)
    assert np.allclose(src, -lap + 1.0 * u, rtol=1e-4, atol=1e-4)
    assert np.allclose(rob, g[:, :2] @ np.array([0.6, -0.8]), rtol=1e-4, atol=1e-4)


def test_walk_settings_defaults_follow_reference():
    # the 4-argument constructor (point_estimation/common.h:21-40)
    s = api.WalkSettings(1e-3, 1e-3, 1024, False)
    assert s.silhouette_precision == 1e-3 and s.russian_roulette_threshold == 0.0
    assert s.splitting_threshold == A.FLT_MAX
    assert s.steps_before_using_maximal_spheres == 1024 and s.steps_before_applying_tikhonov == 0
    assert s.use_gradient_control_variates and s.use_gradient_antithetic_variates
    assert not s.ignore_source_contribution and not s.print_logs
    c = s.to_c()
    assert c.max_walk_length == 1024 and abs(c.epsilon_shell_for_absorbing_boundary - 1e-3) < 1e-9
    full = api.WalkSettings(1e-3, 2e-3, 1e-3, 0.5, 2.0, 100, 3, 50, True, False, False, True, False, True, False, True)
    assert full.splitting_threshold == 2.0 and full.steps_before_using_maximal_spheres == 50 and full.print_logs


def test_factories_validate_dim_and_channels():
    import zombie_gb300 as Z
    with pytest.raises(ValueError):
        Z.Core.PDE(dim=4)
    with pytest.raises(ValueError):
        Z.Core.PDE(dim=2, channels=4)
    pde = Z.Core.PDE(dim=3)
    assert pde.dim == 3 and not pde.has_non_zero_robin_coeff()
    pde.are_robin_conditions_pure_neumann = False
    pde.robin_coeff = Z.Core.get_constant_robin_coefficient_callback(2.0)
    assert pde.has_non_zero_robin_coeff()
    ic = Z.Utils.get_ignore_candidate_silhouette_callback()
    assert ic(-0.1, 0) and not ic(0.1, 0)
    assert not Z.Utils.get_ignore_candidate_silhouette_callback(True)(-0.1, 0)
    w = Z.Utils.get_branch_traversal_weight_callback()
    assert w(0.0) == pytest.approx(1.0 / (4 * np.pi * 1e-2))


def test_solver_rejects_host_callbacks():
    q = api.GeometricQueries(True, [-1, -1], [1, 1], dim=2)
    with pytest.raises(api.ZgpuError) as e:
        api.WalkOnStars(q, walk_state_callback=lambda s: None, dim=2)
    assert e.value.status == A.ZGPU_ERR_UNSUPPORTED_CALLBACK


def test_pde_descriptor_round_trip():
    pr = P.robin_wost_3d(level=1, n_points=10, spp=4)
    pde = api.PDE.from_c(3, pr.pde)
    c = pde.to_c()
    for f in ("absorption_coeff", "robin_kind", "robin_coeff_kind", "robin_coeff_value", "dirichlet_kind",
              "are_robin_conditions_pure_neumann", "source_kind"):
        assert getattr(c, f) == getattr(pr.pde, f)
    assert c.solution.n_terms == 4
