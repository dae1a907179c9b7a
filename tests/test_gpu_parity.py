"""GPU parity: every query and solver of libzgpu.so against the CPU oracle, through the C ABI."""
import numpy as np
import pytest

from zombie_gb300 import _abi as A
from zombie_gb300 import problems as P

pytestmark = pytest.mark.gpu


def _scene(dim, level=3):
    if dim == 2:
        return P.star_polygon(1024)
    pos, idx, _ = P.displaced_icosphere(level, seed=5)
    return pos, idx


def _handler(zgpu, dim, pos, idx, kind, kappa=None, ignore_prec=0.0):
    from zombie_gb300 import api
    ic = api.IgnoreCandidateSilhouette(False, ignore_prec)
    if kind == A.ZGPU_BOUNDARY_ABSORBING:
        h = api.GpuDirichletBoundaryHandler(dim)
        h.build_acceleration_structure(pos, idx)
    elif kind == A.ZGPU_BOUNDARY_NEUMANN:
        h = api.GpuNeumannBoundaryHandler(dim)
        h.build_acceleration_structure(pos, idx, ic)
    else:
        k = np.full(idx.shape[0], kappa, np.float32)
        h = api.GpuRobinBoundaryHandler(dim)
        h.build_acceleration_structure(pos, idx, ic, k, k)
    return h


@pytest.mark.parametrize("dim", [2, 3])
def test_closest_point_parity(zgpu, oracle, dim):
    pos, idx = _scene(dim)
    x = np.random.default_rng(0).uniform(-1.4, 1.4, (20000, dim)).astype(np.float32)
    g = _handler(zgpu, dim, pos, idx, A.ZGPU_BOUNDARY_ABSORBING)
    o = oracle.Boundary(dim, pos, idx, use_bvh=False)
    gp, gn, gd, gi = g.closest_point(x)
    op, on, od, oi = o.closest_point(x)
    # FP32 distances agree within 1e-6 relative, or 2.4e-7 absolute (2 ulp at unit scale) for
    # points within a few 1e-3 of the surface, where x - closest point cancels
    err = np.abs(gd - od)
    tol = np.maximum(1e-6 * od, 2.4e-7)
    assert np.all(err <= tol)
    same = gi == oi
    assert same.mean() > 0.98
    # where the indices differ it is a tie, for every mismatch: the GPU's primitive is as
    # close to the query as the oracle's (FP64 distances of the FP32 inputs)
    from fp64_geometry import prim_dist64
    bad = np.nonzero(~same)[0]
    if len(bad):
        dg, do = prim_dist64(pos, idx, gi[bad], x[bad]), prim_dist64(pos, idx, oi[bad], x[bad])
        assert np.all(np.abs(dg - do) <= np.maximum(1e-6 * do, 2.4e-7))
    assert np.allclose(gp[same], op[same], atol=1e-6)
    assert np.allclose(gn[same], on[same], atol=1e-6)


@pytest.mark.parametrize("dim", [2, 3])
def test_ray_intersection_parity(zgpu, oracle, dim):
    pos, idx = _scene(dim)
    rng = np.random.default_rng(1)
    n = 20000
    o = rng.uniform(-0.6, 0.6, (n, dim)).astype(np.float32)
    d = rng.normal(size=(n, dim)).astype(np.float32)
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    tm = rng.uniform(0.05, 2.5, n).astype(np.float32)
    z = np.zeros_like(o)
    on = np.zeros(n, np.int32)
    g = _handler(zgpu, dim, pos, idx, A.ZGPU_BOUNDARY_NEUMANN)
    ob = oracle.Boundary(dim, pos, idx, kind=A.ZGPU_BOUNDARY_NEUMANN, use_bvh=False)
    gh, gpt, gn, gt, gi = g.intersect(o, z, d, tm, on)
    oh, opt, on_, ot, oi = ob.intersect(o, z, d, tm, on)
    agree = gh == oh
    assert agree.mean() > 0.9995          # misses only for hits within float noise of tMax
    both = (gh == 1) & (oh == 1)
    assert np.all(np.abs(gt[both] - ot[both]) <= 1e-5 * np.maximum(ot[both], 1.0))
    assert (gi[both] == oi[both]).mean() > 0.999
    cnt = g.count_hits(o, d, np.full(n, 1e30, np.float32))
    assert np.array_equal(cnt, ob.count_hits(o, d, np.full(n, 1e30, np.float32)))


@pytest.mark.parametrize("dim,kind,kappa", [(2, A.ZGPU_BOUNDARY_NEUMANN, None), (2, A.ZGPU_BOUNDARY_ROBIN, 2.0),
                                            (3, A.ZGPU_BOUNDARY_NEUMANN, None), (3, A.ZGPU_BOUNDARY_ROBIN, 2.0)])
def test_star_radius_parity(zgpu, oracle, dim, kind, kappa):
    pos, idx = _scene(dim)
    rng = np.random.default_rng(2)
    n = 8000
    x = rng.uniform(-0.7, 0.7, (n, dim)).astype(np.float32)
    mn = np.full(n, 1e-3, np.float32)
    mx = rng.uniform(0.05, 2.0, n).astype(np.float32)
    fl = np.zeros(n, np.int32)
    g = _handler(zgpu, dim, pos, idx, kind, kappa)
    k = None if kappa is None else np.full(idx.shape[0], kappa, np.float32)
    ob = oracle.Boundary(dim, pos, idx, kind=kind, kmin=k, kmax=k, silhouette_precision=0.0, use_bvh=False)
    gr = g.star_radius(x, mn, mx, 1e-3, fl)
    orr = ob.star_radius(x, mn, mx, 1e-3, fl)
    rel = np.abs(gr - orr) / np.maximum(orr, 1e-30)
    # silhouette distances agree to FP32 rounding; the Robin bound r = (h/c) exp(c^2/(h kappa))
    # amplifies the rounding of its exponent (ill-conditioned in FP32 for small h)
    assert np.median(rel) <= 1e-6
    assert np.quantile(rel, 0.999) <= (1e-5 if kappa is None else 2e-3)
    assert np.mean(rel <= 1e-5) > (0.999 if kappa is None else 0.97)
    assert np.all(gr <= np.maximum(mx, mn) * (1 + 1e-6))


def _mixed_robin(n, seed):
    rng = np.random.default_rng(seed)
    kmax = rng.uniform(0.5, 6.0, n).astype(np.float32)
    kmin = (kmax * rng.uniform(0.3, 1.0, n)).astype(np.float32)
    absorbing, reflecting = rng.random(n) < 0.05, rng.random(n) < 0.1
    kmin[absorbing] = kmax[absorbing] = A.FLT_MAX
    kmin[reflecting] = kmax[reflecting] = 0.0
    return kmin, kmax


@pytest.mark.parametrize("dim", [2, 3])
def test_robin_node_bounds_after_coefficient_update(zgpu, oracle, dim):
    """Per-face Robin coefficients (perfectly absorbing and purely reflecting faces mixed in),
    set by updateCoefficientValues on a boundary built with other values: the refitted node
    ranges give the radii of a boundary built with the new values and of the oracle."""
    from zombie_gb300 import api
    pos, idx = _scene(dim, level=4)
    n = idx.shape[0]
    kmin, kmax = _mixed_robin(n, 11)
    ones = np.ones(n, np.float32)
    updated = api.GpuRobinBoundaryHandler(dim)
    updated.build_acceleration_structure(pos, idx, api.IgnoreCandidateSilhouette(False, 0.0), ones, ones)
    updated.update_coefficient_values(kmin, kmax)
    fresh = api.GpuRobinBoundaryHandler(dim)
    fresh.build_acceleration_structure(pos, idx, api.IgnoreCandidateSilhouette(False, 0.0), kmin, kmax)
    rng = np.random.default_rng(12)
    m = 6000
    x = rng.uniform(-0.6, 0.6, (m, dim)).astype(np.float32)
    mn = np.full(m, 1e-3, np.float32)
    mx = np.where(rng.random(m) < 0.5, A.FLT_MAX, rng.uniform(0.05, 3.0, m)).astype(np.float32)
    fl = np.zeros(m, np.int32)
    ru = updated.star_radius(x, mn, mx, 1e-3, fl)
    rf = fresh.star_radius(x, mn, mx, 1e-3, fl)
    assert np.array_equal(ru, rf)
    ob = oracle.Boundary(dim, pos, idx, kind=A.ZGPU_BOUNDARY_ROBIN, kmin=kmin, kmax=kmax, silhouette_precision=0.0,
                         use_bvh=False)
    orr = ob.star_radius(x, mn, mx, 1e-3, fl)
    rel = np.abs(ru - orr) / np.maximum(orr, 1e-30)
    assert np.median(rel) <= 1e-6
    assert np.quantile(rel, 0.99) <= 2e-3
    assert np.mean(rel <= 1e-5) > 0.95


@pytest.mark.parametrize("dim", [2, 3])
def test_line_of_sight_parity(zgpu, oracle, dim):
    pos, idx = _scene(dim)
    rng = np.random.default_rng(3)
    n = 20000
    a = rng.uniform(-0.8, 0.8, (n, dim)).astype(np.float32)
    b = rng.uniform(-0.8, 0.8, (n, dim)).astype(np.float32)
    z = np.zeros_like(a)
    off = np.zeros(n, np.int32)
    g = _handler(zgpu, dim, pos, idx, A.ZGPU_BOUNDARY_NEUMANN)
    ob = oracle.Boundary(dim, pos, idx, kind=A.ZGPU_BOUNDARY_NEUMANN, use_bvh=False)
    assert (g.occluded(a, b, z, z, off, off) == ob.occluded(a, b, z, z, off, off)).mean() > 0.9995


def test_boundary_sampling_is_unbiased(zgpu):
    pos, idx = P.star_polygon(1024)
    g = _handler(zgpu, 2, pos, idx, A.ZGPU_BOUNDARY_NEUMANN)
    x = np.array([[0.1, -0.5]], np.float32)
    R, N = 0.6, 400000
    u = np.random.default_rng(4).random((N, 2)).astype(np.float32)
    found, pt, _, pdf = g.sample(np.repeat(x, N, 0), np.full(N, R, np.float32), u)
    d = np.linalg.norm(pt - x, axis=1)
    G = np.log(R / np.maximum(d, 1e-4)) / (2 * np.pi)
    val = np.where((found == 1) & (d < R), G * pt[:, 1] / np.maximum(pdf, 1e-30), 0.0)
    a = pos[idx[:, 0]].astype(np.float64)
    c = pos[idx[:, 1]].astype(np.float64)
    t = (np.arange(256) + 0.5) / 256
    zz = a[:, None, :] + (c - a)[:, None, :] * t[None, :, None]
    dz = np.linalg.norm(zz - x, axis=2)
    Gq = np.where(dz < R, np.log(R / np.maximum(dz, 1e-4)) / (2 * np.pi), 0.0)
    quad = ((Gq * zz[:, :, 1]).mean(1) * np.linalg.norm(c - a, axis=1)).sum()
    assert abs(val.mean() - quad) <= 4 * val.std() / np.sqrt(N) + 1e-5


# ------------------------------------------------------------------------- solvers
def _screened_2d(grid=20, spp=512):
    pr = P.laplace_wos_2d(n_segments=1024, grid=grid, spp=spp)
    pr.pde = P.make_pde(pr.solution, sigma=2.0, source=True)      # f = 2u: a non-constant source
    return pr


def _gpu_and_oracle(zgpu, oracle, pr):
    from zombie_gb300.runner import GpuProblem, summarize
    import test_oracle_solvers as T
    gp = GpuProblem(pr)
    arr = gp.host_arrays()
    rep = gp.solve(arr)
    g = summarize(arr, pr.exact())
    st, steps = T.run_oracle(oracle, pr, seeds=gp.seeds)
    return g, st, steps, rep


def _cross_z(g, st):
    n = st["n_solution_estimates"].astype(np.float64)
    se_o = np.sqrt(st["solution_m2"] / np.maximum(n - 1, 1) / np.maximum(n, 1))
    se = np.sqrt(g["se"] ** 2 + se_o ** 2)
    return (g["mean"] - st["solution_mean"]) / np.maximum(se, 1e-12)


def _exact_z(g):
    return g["err"] / np.maximum(g["se"], 1e-12)


CASES = {
    "wos_laplace_2d": lambda: P.laplace_wos_2d(n_segments=1024, grid=40, spp=256),
    "wost_mixed_2d": lambda: P.mixed_wost_2d(n_segments=4096, grid=32, spp=256),
    "wost_screened_2d": lambda: P.mixed_wost_2d(n_segments=2048, grid=24, spp=256, sigma=1.0),
    "wost_robin_3d": lambda: P.robin_wost_3d(level=4, n_points=400, spp=256),
    "wos_screened_3d": lambda: P.screened_wos_3d(level=4, n_points=400, spp=256),
    # PDE data from dense grids sampled at cell centres (bilinear / trilinear / nearest)
    "wos_laplace_2d_grid": lambda: P.with_grid_fields(P.laplace_wos_2d(n_segments=1024, grid=40, spp=256)),
    "wos_screened_2d_grid": lambda: P.with_grid_fields(_screened_2d(grid=32, spp=256), ("dirichlet", "source")),
    "wost_mixed_2d_nearest_grid": lambda: P.with_grid_fields(P.mixed_wost_2d(n_segments=2048, grid=24, spp=256),
                                                             shape=(4096, 4096), interpolate=False),
    "wost_robin_3d_kappa_grid": lambda: P.with_grid_fields(
        P.robin_wost_3d(level=4, n_points=400, spp=256), (), shape=(48, 48, 48),
        robin_coeff=lambda x: 1.5 + 0.5 * np.sin(2.0 * x[:, 0]) * np.cos(x[:, 1])),
    "wos_screened_3d_grid": lambda: P.with_grid_fields(P.screened_wos_3d(level=4, n_points=400, spp=256),
                                                       ("dirichlet", "source"), shape=(96, 96, 96)),
}


@pytest.mark.parametrize("case", sorted(CASES))
def test_solver_matches_oracle_and_exact(zgpu, oracle, case):
    pr = CASES[case]()
    g, st, steps, rep = _gpu_and_oracle(zgpu, oracle, pr)
    assert rep.error_word == 0 and rep.total_steps > 0
    # the same walks (same pcg32 streams): totals agree closely, per-point estimates agree
    assert abs(rep.total_steps - steps) <= 0.02 * steps
    z = _cross_z(g, st)
    assert np.mean(np.abs(z) > 3) <= 0.01
    assert abs(z.mean()) <= 4.0 / np.sqrt(len(z)) + 0.05
    # and both agree with the FP64 manufactured solution
    ez = _exact_z(g)
    assert abs(ez.mean()) <= 0.5
    assert np.mean(np.abs(ez) > 3.5) <= 0.04


@pytest.mark.parametrize("make,fields,shape", [
    (lambda: P.laplace_wos_2d(n_segments=1024, grid=40, spp=128), ("dirichlet",), (1024, 1024)),
    (lambda: _screened_2d(grid=32, spp=128), ("dirichlet", "source"), (1024, 1024)),
    (lambda: P.screened_wos_3d(level=4, n_points=400, spp=128), ("dirichlet", "source"), (128, 128, 128))])
def test_dense_grid_fields_follow_the_analytic_fields(zgpu, make, fields, shape):
    """The device's grid lookups (host grids copied by the solve) replace analytic g and f
    without changing a walk: equal walk lengths, estimates within the interpolation error."""
    from zombie_gb300.runner import GpuProblem
    a, b = make(), P.with_grid_fields(make(), fields, shape=shape)
    ga, gb = GpuProblem(a), GpuProblem(b)
    xa, xb = ga.host_arrays(), gb.host_arrays()
    ra, rb = ga.solve(xa), gb.solve(xb)
    assert ra.total_steps == rb.total_steps and rb.error_word == 0
    assert np.array_equal(xa["total_walk_length"], xb["total_walk_length"])
    d = xb["solution_mean"] - xa["solution_mean"]
    assert np.max(np.abs(d)) < 3e-3
    assert abs(d.mean()) < 2e-4


def test_dense_grid_fields_are_validated(zgpu):
    """Grid fields with an empty shape, an empty box or no values are rejected; the
    allocation-free entry point takes device-resident grids only."""
    from zombie_gb300.runner import GpuProblem
    from zombie_gb300 import ZgpuError
    pr = P.with_grid_fields(P.laplace_wos_2d(n_segments=256, grid=8, spp=4), shape=(16, 16))
    for breakage in ("shape", "box", "values"):
        pr2 = P.with_grid_fields(P.laplace_wos_2d(n_segments=256, grid=8, spp=4), shape=(16, 16))
        if breakage == "shape":
            pr2.pde.dirichlet_grid.shape[1] = 0
        elif breakage == "box":
            pr2.pde.dirichlet_grid.grid_max[0] = pr2.pde.dirichlet_grid.grid_min[0]
        else:
            pr2.pde.dirichlet_grid.values = None
        gp = GpuProblem(pr2)
        with pytest.raises(ZgpuError):
            gp.solve(gp.host_arrays())
    gp = GpuProblem(pr)
    rep = gp.solve(gp.host_arrays())
    assert rep.error_word == 0 and rep.total_steps > 0


def test_wos_walks_reproduce_oracle_walks(zgpu, oracle):
    """With identical pcg32 streams, WoS walks on the GPU follow the oracle's walks: the
    per-point means agree far below the Monte Carlo error."""
    pr = P.laplace_wos_2d(n_segments=1024, grid=24, spp=128)
    g, st, steps, rep = _gpu_and_oracle(zgpu, oracle, pr)
    close = np.abs(g["mean"] - st["solution_mean"]) <= 1e-3 * g["se"] + 1e-6
    assert close.mean() > 0.9


def test_progressive_accumulation_matches_single_call(zgpu):
    from zombie_gb300.runner import GpuProblem
    pr = P.mixed_wost_2d(n_segments=1024, grid=16, spp=64)
    gp = GpuProblem(pr)
    a = gp.host_arrays()
    gp.solve(a)
    fsr1 = a["first_sphere_radius"].copy()
    gp.solve(a)
    assert np.array_equal(fsr1, a["first_sphere_radius"])
    b = gp.host_arrays(n_walks=128)
    gp.solve(b)
    assert np.array_equal(a["n_solution_estimates"], b["n_solution_estimates"])
    assert np.allclose(a["solution_mean"], b["solution_mean"], atol=1e-9)
    assert np.allclose(a["solution_m2"], b["solution_m2"], rtol=1e-8, atol=1e-8)


def test_device_and_host_memory_paths_agree(zgpu):
    from zombie_gb300.runner import GpuProblem
    pr = P.mixed_wost_2d(n_segments=2048, grid=24, spp=64)
    gp = GpuProblem(pr)
    h = gp.host_arrays()
    gp.solve(h)
    d = gp.device_arrays()
    gp.solve(d)
    assert np.array_equal(h["n_solution_estimates"], d["n_solution_estimates"].cpu().numpy())
    assert np.allclose(h["solution_mean"], d["solution_mean"].cpu().numpy(), atol=1e-12)


def test_russian_roulette_and_splitting(zgpu, oracle):
    pr = P.laplace_wos_2d(n_segments=512, grid=16, spp=256)
    pr.pde = P.make_pde(pr.solution, sigma=2.0, source=True)
    pr.settings = P.default_walk_settings(rr=0.9, splitting=1.5)
    g, st, steps, rep = _gpu_and_oracle(zgpu, oracle, pr)
    assert rep.error_word == 0
    assert rep.rr_terminated > 0
    z = _cross_z(g, st)
    assert np.mean(np.abs(z) > 3) <= 0.02
    assert abs(_exact_z(g).mean()) <= 0.5


def test_public_api_with_sample_point_lists(zgpu):
    """The reference's call shape: WalkOnStars(queries).solve(pde, settings, n_walks, pts, stats)."""
    import zombie_gb300 as Z
    pr = P.mixed_wost_2d(n_segments=1024, grid=8, spp=64)
    q = Z.Core.GeometricQueries(True, pr.domain_min, pr.domain_max, dim=2)
    ab = Z.Utils.FcpwDirichletBoundaryHandler(dim=2)
    ab.build_acceleration_structure(*pr.absorbing)
    Z.Utils.populate_geometric_queries_for_dirichlet_boundary(ab, q, dim=2)
    rf = Z.Utils.FcpwNeumannBoundaryHandler(dim=2)
    rf.build_acceleration_structure(*pr.reflecting, Z.Utils.get_ignore_candidate_silhouette_callback(False, 0.0))
    Z.Utils.populate_geometric_queries_for_neumann_boundary(rf, Z.Utils.get_branch_traversal_weight_callback(), q, dim=2)
    pde = Z.api.PDE.from_c(2, pr.pde)
    ws = Z.Solvers.WalkSettings(1e-3, 1e-3, 1e-3, 0.0, A.FLT_MAX, 1024, 0, 1024, False, True, True, False, False,
                                False, False, False)
    d = q.compute_dist_to_absorbing_boundary(pr.points)
    pts = [Z.Solvers.SamplePoint(p, np.zeros(2), Z.Solvers.SampleType.InDomain, Z.Solvers.EstimationQuantity.Solution,
                                 1.0, float(di), float("inf"), seed=i + 1, dim=2) for i, (p, di) in enumerate(zip(pr.points, d))]
    stats = Z.Solvers.create_sample_statistics_list(len(pts), dim=2)
    solver = Z.Solvers.WalkOnStars(q, dim=2)
    calls = []
    solver.solve(pde, ws, [64] * len(pts), pts, stats, False, lambda n, t: calls.append(n))
    assert calls == [len(pts)]
    est = np.array([s.get_estimated_solution() for s in stats])
    assert all(s.get_solution_estimate_count() == 64 for s in stats)
    assert all(p.first_sphere_radius > 0 for p in pts)
    assert np.sqrt(np.mean((est - pr.exact()) ** 2)) < 0.3
    assert q.inside_domain(pr.points).all()


def test_invalid_arguments_return_errors(zgpu):
    import ctypes as C
    from zombie_gb300 import _lib
    from zombie_gb300.api import default_context
    L = _lib.lib()
    ctx = default_context()
    h = C.c_void_p()
    pos = np.zeros((4, 2), np.float32)
    idx = np.array([[0, 5]], np.int32)   # vertex index out of range
    st = L.zgpu_boundary_create(ctx.h, 2, A.ptr(pos), 4, A.ptr(idx), 1, 0, None, None, 0, 1e-3, 4, C.byref(h))
    assert st == A.ZGPU_ERR_INVALID_ARG and b"out of range" in L.zgpu_last_error()
    st = L.zgpu_boundary_create(ctx.h, 4, A.ptr(pos), 4, A.ptr(idx), 1, 0, None, None, 0, 1e-3, 4, C.byref(h))
    assert st == A.ZGPU_ERR_INVALID_ARG
    st = L.zgpu_solve(ctx.h, 7, None, None, None, None, None, None, None)
    assert st == A.ZGPU_ERR_INVALID_ARG
    # a grid field without values is an error, not silently a zero field
    from zombie_gb300.runner import GpuProblem
    gp = GpuProblem(P.laplace_wos_2d(n_segments=64, grid=4, spp=4))
    pde = gp.pde.to_c()
    pde.source_kind = A.ZGPU_FIELD_GRID
    with pytest.raises(_lib.ZgpuError) as e:
        gp.solver.solve_arrays(pde, gp.problem.settings, gp.host_arrays())
    assert e.value.status == A.ZGPU_ERR_INVALID_ARG and "no values" in str(e.value)
    # an unknown field kind too
    pde.source_kind = 9
    with pytest.raises(_lib.ZgpuError) as e:
        gp.solver.solve_arrays(pde, gp.problem.settings, gp.host_arrays())
    assert e.value.status == A.ZGPU_ERR_INVALID_ARG


@pytest.mark.parametrize("make", [lambda: P.laplace_wos_2d(n_segments=1024, grid=32, spp=64),
                                  lambda: P.screened_wos_3d(level=4, n_points=2000, spp=32)])
def test_cooperative_queries_reproduce_per_lane_queries(zgpu, make):
    """Walk on Spheres with closest-point queries answered by the whole warp gives the same
    walks, bit for bit, as one lane per query (the same primitive wins every query)."""
    from zombie_gb300.runner import GpuProblem
    pr = make()
    out = []
    for mode in (1, 2):
        opt = A.SolveOptions()
        opt.query_mode = mode
        gp = GpuProblem(pr, options=opt)
        d = gp.device_arrays()
        rep = gp.solve(d)
        assert rep.error_word == 0
        out.append((rep, {k: d[k].cpu().numpy() for k in ("solution_mean", "solution_m2", "n_solution_estimates",
                                                          "total_walk_length")}))
    (r1, a), (r2, b) = out
    assert r1.total_steps == r2.total_steps
    for k in ("n_solution_estimates", "total_walk_length"):
        assert np.array_equal(a[k], b[k]), k
    # the FP64 per-point sums are accumulated by atomics in walk-completion order, which the
    # query mode changes: the moments agree to the last few bits
    for k in ("solution_mean", "solution_m2"):
        assert np.allclose(a[k], b[k], rtol=1e-12, atol=1e-15), k


def test_batched_solve_equals_individual_solves(zgpu):
    """Independent 2D problems in one launch (scene table + per-point scene id) run the walks
    each problem runs alone: identical counts and walk lengths, moments to the last bits."""
    from zombie_gb300.runner import GpuBatch, GpuProblem
    scenes = P.batched_scenes(n_scenes=5, seed=3, point_scale=0.004, segments=(256, 4096))
    batch = GpuBatch(scenes)
    arr = batch.device_arrays()
    rep = batch.solve(arr)
    assert rep.error_word == 0
    for k, g in enumerate(batch.problems):
        d = g.device_arrays()
        g.solve(d)
        lo, hi = batch.offsets[k], batch.offsets[k + 1]
        for key in ("n_solution_estimates", "total_walk_length"):
            assert np.array_equal(d[key].cpu().numpy(), arr[key][lo:hi].cpu().numpy()), (k, key)
        # the batched and single-scene kernels are separate instantiations: last-bit float
        # differences of a walk total reach m2 amplified by its cancellation
        for key in ("solution_mean", "solution_m2"):
            assert np.allclose(d[key].cpu().numpy(), arr[key][lo:hi].cpu().numpy(), rtol=1e-9, atol=1e-12), (k, key)
    # and the batch solves its problems: within a few standard errors of the exact solutions
    n = arr["n_solution_estimates"].cpu().numpy().astype(np.float64)
    err = arr["solution_mean"].cpu().numpy() - batch.exact()
    se = np.sqrt(arr["solution_m2"].cpu().numpy() / np.maximum(n - 1, 1) / n)
    assert np.mean(np.abs(err) <= 4 * se + 1e-6) > 0.99


def test_batched_3d_solve_equals_individual_solves(zgpu):
    """3D problems of one solver batched (different meshes, absorption and sources): each
    point runs the walks of its problem solved alone."""
    from zombie_gb300.runner import GpuBatch
    scenes = [P.screened_wos_3d(level=3, n_points=150, spp=64, sigma=4.0, seed=1),
              P.screened_wos_3d(level=4, n_points=200, spp=32, sigma=1.0, seed=2),
              P.laplace_wos_2d(n_segments=64, grid=4, spp=4)]
    with pytest.raises(ValueError):
        GpuBatch(scenes)                                  # one dimension per batch
    scenes = scenes[:2] + [P.screened_wos_3d(level=3, n_points=100, spp=16, sigma=0.0, seed=3)]
    batch = GpuBatch(scenes)
    arr = batch.device_arrays()
    rep = batch.solve(arr)
    assert rep.error_word == 0
    for k, g in enumerate(batch.problems):
        d = g.device_arrays()
        g.solve(d)
        lo, hi = batch.offsets[k], batch.offsets[k + 1]
        for key in ("n_solution_estimates", "total_walk_length"):
            assert np.array_equal(d[key].cpu().numpy(), arr[key][lo:hi].cpu().numpy()), (k, key)
        for key in ("solution_mean", "solution_m2"):
            assert np.allclose(d[key].cpu().numpy(), arr[key][lo:hi].cpu().numpy(), rtol=1e-9, atol=1e-12), (k, key)


def test_batched_solve_rejects_scene_ids_outside_the_table(zgpu):
    import ctypes as C
    from zombie_gb300 import _lib
    from zombie_gb300.runner import GpuBatch
    batch = GpuBatch(P.batched_scenes(n_scenes=2, seed=4, point_scale=0.002, segments=(256, 512)))
    arr = batch.device_arrays()
    arr["scene_id"][3] = 7
    with pytest.raises(_lib.ZgpuError) as e:
        batch.solve(arr)
    assert e.value.status == A.ZGPU_ERR_DEVICE_STATE


def test_autotuned_and_graph_replayed_solves_run_the_same_walks(zgpu):
    """The autotuner's launch configuration and a solve replayed from its captured CUDA graph
    run the walks of the default launch (walk randomness depends on walk ids only)."""
    from zombie_gb300.runner import GpuProblem
    gp = GpuProblem(P.mixed_wost_2d(n_segments=1024, grid=32, spp=64))
    ref = gp.device_arrays()
    gp.solve(ref)
    opt, rate = gp.solver.autotune(gp.pde, gp.problem.settings, gp.device_arrays(), sample_points=512, sample_walks=8)
    assert opt.block_size in (32, 64, 128) and rate > 0
    again, _ = gp.solver.autotune(gp.pde, gp.problem.settings, gp.device_arrays())
    assert (again.block_size, again.blocks_per_sm) == (opt.block_size, opt.blocks_per_sm)   # cached per scene
    tuned = gp.device_arrays()
    gp.solve(tuned, options=opt)
    opt.use_graph = 1
    graph = gp.device_arrays()
    for call in range(3):                      # the first call captures, the others replay
        for k in ("solution_mean", "solution_m2", "n_solution_estimates", "total_walk_length", "total_splits",
                  "first_sphere_radius"):
            graph[k].zero_()
        rep = gp.solve(graph, options=opt)
        assert rep.error_word == 0 and rep.total_steps > 0
        for d in (tuned, graph):
            for k in ("n_solution_estimates", "total_walk_length"):
                assert np.array_equal(ref[k].cpu().numpy(), d[k].cpu().numpy()), (call, k)
            for k in ("solution_mean", "solution_m2"):
                assert np.allclose(ref[k].cpu().numpy(), d[k].cpu().numpy(), rtol=1e-12, atol=1e-15), (call, k)


def test_cooperative_robin_star_radii_match_per_lane_walks(zgpu):
    """Walk on Stars on a Robin boundary with star radii answered by the whole warp runs the
    per-lane walks (node upper bounds met in another order can move a radius in rare ties):
    nearly all points keep identical walk lengths and every estimate agrees within its error."""
    from zombie_gb300.runner import GpuProblem
    pr = P.robin_wost_3d(level=4, n_points=1500, spp=64)
    out = []
    for mode in (1, 2):
        opt = A.SolveOptions()
        opt.query_mode = mode
        gp = GpuProblem(pr, options=opt)
        d = gp.device_arrays()
        rep = gp.solve(d)
        assert rep.error_word == 0
        out.append((rep, {k: d[k].cpu().numpy() for k in ("solution_mean", "solution_m2", "n_solution_estimates",
                                                          "total_walk_length")}))
    (r1, a), (r2, b) = out
    assert abs(r1.total_steps - r2.total_steps) <= 0.01 * r1.total_steps
    assert np.mean(a["total_walk_length"] == b["total_walk_length"]) > 0.95
    n = a["n_solution_estimates"].astype(np.float64)
    se = np.sqrt((a["solution_m2"] + b["solution_m2"]) / np.maximum(n - 1, 1) / n)
    assert np.mean(np.abs(a["solution_mean"] - b["solution_mean"]) <= 3 * se + 1e-9) > 0.99


@pytest.mark.parametrize("make", [lambda: P.laplace_wos_2d(n_segments=1024, grid=24, spp=512),
                                  lambda: P.mixed_wost_2d(n_segments=1024, grid=20, spp=512),
                                  lambda: P.screened_wos_3d(level=4, n_points=300, spp=512)])
def test_gradient_estimates_match_the_analytic_gradient(zgpu, make):
    """estimateSolutionAndGradient (control variates, antithetic pairs, stratified first
    steps): per-point gradient estimates within their standard errors of grad u, and the
    solution estimates stay unbiased."""
    from zombie_gb300.runner import GpuProblem
    pr = make()
    gp = GpuProblem(pr)
    d = gp.device_arrays(gradients=True)
    gp.solve(d)          # first call: no control variate yet (no previous estimate)
    gp.solve(d)          # second call: control variates from the first call's estimates
    D = pr.dim
    u, grad, _ = P.eval_analytic(pr.solution, pr.points)
    n = d["n_gradient_estimates"].cpu().numpy().astype(np.float64)
    assert np.all(n == 2 * pr.n_walks)            # antithetic pairs: walks rounded to even
    gm = d["gradient_mean"].cpu().numpy().reshape(-1, D)
    gse = np.sqrt(d["gradient_m2"].cpu().numpy().reshape(-1, D) / np.maximum(n - 1, 1)[:, None] / n[:, None])
    z = (gm - grad) / np.maximum(gse, 1e-12)
    assert np.mean(np.abs(z) <= 4) > 0.99
    assert abs(np.mean(z)) < 0.15
    sn = d["n_solution_estimates"].cpu().numpy().astype(np.float64)
    sz = (d["solution_mean"].cpu().numpy() - u) / np.sqrt(d["solution_m2"].cpu().numpy() / np.maximum(sn - 1, 1) / sn)
    assert np.mean(np.abs(sz) <= 4) > 0.99


def test_gradient_estimates_match_the_oracle(zgpu, oracle):
    """GPU and oracle run the same gradient walks (same streams, strata and mirroring): the
    per-point gradient estimates agree far inside their standard errors."""
    import sys
    import os
    sys.path.insert(0, os.path.dirname(__file__))
    from test_oracle_solvers import run_oracle_with
    from zombie_gb300.runner import GpuProblem
    pr = P.laplace_wos_2d(n_segments=512, grid=12, spp=128)
    n, D = pr.points.shape
    eq = np.full(n, A.ZGPU_ESTIMATE_SOLUTION_AND_GRADIENT, np.int32)
    extra = dict(gradient_mean=np.zeros((n, D)), gradient_m2=np.zeros((n, D)),
                 n_gradient_estimates=np.zeros(n, np.int32))
    st = None
    for _ in range(2):
        st = run_oracle_with(oracle, pr, st, estimation_quantity=eq, extra_stats=extra)
    gp = GpuProblem(pr)
    d = gp.device_arrays(gradients=True)
    gp.solve(d)
    gp.solve(d)
    assert np.array_equal(d["n_gradient_estimates"].cpu().numpy(), st["n_gradient_estimates"])
    gg = d["gradient_mean"].cpu().numpy().reshape(n, D)
    og = st["gradient_mean"].reshape(n, D)
    se = np.sqrt(st["gradient_m2"].reshape(n, D) / np.maximum(st["n_gradient_estimates"] - 1, 1)[:, None]
                 / st["n_gradient_estimates"][:, None])
    assert np.mean(np.abs(gg - og) <= 0.1 * se + 1e-6) > 0.95
    assert np.all(np.abs(gg - og) <= 3 * se + 1e-6)


def _axis_directions(n, D, seed):
    rng = np.random.default_rng(seed)
    axis = rng.integers(0, D, n)
    v = np.zeros((n, D), np.float32)
    v[np.arange(n), axis] = rng.choice([-1.0, 1.0], n)
    return v, axis


@pytest.mark.parametrize("make", [lambda: P.laplace_wos_2d(n_segments=1024, grid=24, spp=512), _screened_2d,
                                  lambda: P.mixed_wost_2d(n_segments=1024, grid=20, spp=512),
                                  lambda: P.screened_wos_3d(level=4, n_points=300, spp=512)])
def test_cosine_sampled_directional_derivatives(zgpu, make):
    """useCosineSamplingForDerivatives: first steps cosine-weighted about each point's
    directionForDerivative; getEstimatedDerivative (running sum of the walks' directional
    derivatives) matches grad u . direction within its standard errors and equals the
    gradient mean projected on the direction."""
    import torch
    from zombie_gb300.runner import GpuProblem
    pr = make()
    pr.settings.use_cosine_sampling_for_derivatives = 1
    gp = GpuProblem(pr)
    d = gp.device_arrays(gradients=True)
    n, D = pr.points.shape
    dirs, axis = _axis_directions(n, D, 11)
    d.arrays["direction_for_derivative"] = torch.from_numpy(dirs).to(d["pt"].device)
    gp.solve(d)
    gp.solve(d)
    ng = d["n_gradient_estimates"].cpu().numpy().astype(np.float64)
    assert np.all(ng == 2 * pr.n_walks)
    deriv = d["total_derivative_contribution"].cpu().numpy() / ng
    g = d["gradient_mean"].cpu().numpy().reshape(n, D)
    proj = np.sum(g * dirs, axis=1)
    assert np.max(np.abs(deriv - proj)) <= 1e-4 * np.sqrt(np.mean(proj ** 2))
    _, grad, _ = P.eval_analytic(pr.solution, pr.points)
    se = np.sqrt(d["gradient_m2"].cpu().numpy().reshape(n, D)[np.arange(n), axis] / np.maximum(ng - 1, 1) / ng)
    z = (deriv - np.sum(grad * dirs, axis=1)) / np.maximum(se, 1e-12)
    assert np.mean(np.abs(z) <= 4) > 0.99
    assert abs(np.mean(z)) < 4 / np.sqrt(n)


def test_cosine_sampled_derivatives_match_the_oracle(zgpu, oracle):
    """GPU and oracle on the same cosine-sampled gradient walks with a non-constant source
    (source control variate from the first call's mean first source contribution) and
    arbitrary unit directions: gradients, directional derivatives and first source sums
    agree far inside their standard errors."""
    import sys
    import os
    import torch
    sys.path.insert(0, os.path.dirname(__file__))
    from test_oracle_solvers import run_oracle_with
    from zombie_gb300.runner import GpuProblem
    pr = _screened_2d(grid=12, spp=128)
    pr.settings.use_cosine_sampling_for_derivatives = 1
    n, D = pr.points.shape
    v = np.random.default_rng(12).normal(size=(n, D))
    dirs = (v / np.linalg.norm(v, axis=1, keepdims=True)).astype(np.float32)
    eq = np.full(n, A.ZGPU_ESTIMATE_SOLUTION_AND_GRADIENT, np.int32)
    extra = dict(gradient_mean=np.zeros((n, D)), gradient_m2=np.zeros((n, D)), n_gradient_estimates=np.zeros(n, np.int32),
                 total_first_source_contribution=np.zeros(n), total_derivative_contribution=np.zeros(n))
    st = None
    for _ in range(2):
        st = run_oracle_with(oracle, pr, st, estimation_quantity=eq, extra_stats=extra, direction=dirs)
    gp = GpuProblem(pr)
    d = gp.device_arrays(gradients=True)
    d.arrays["direction_for_derivative"] = torch.from_numpy(dirs).to(d["pt"].device)
    gp.solve(d)
    gp.solve(d)
    ng = st["n_gradient_estimates"].astype(np.float64)
    assert np.array_equal(d["n_gradient_estimates"].cpu().numpy(), st["n_gradient_estimates"])
    se = np.sqrt(st["gradient_m2"].reshape(n, D) / np.maximum(ng - 1, 1)[:, None] / ng[:, None])
    gg = d["gradient_mean"].cpu().numpy().reshape(n, D)
    og = st["gradient_mean"].reshape(n, D)
    assert np.mean(np.abs(gg - og) <= 0.1 * se + 1e-6) > 0.95
    assert np.all(np.abs(gg - og) <= 3 * se + 1e-6)
    sed = np.sqrt(np.sum(se ** 2, axis=1))
    gd = d["total_derivative_contribution"].cpu().numpy() / ng
    od = st["total_derivative_contribution"] / ng
    assert np.mean(np.abs(gd - od) <= 0.1 * sed + 1e-6) > 0.95
    fs_g = d["total_first_source_contribution"].cpu().numpy()
    fs_o = st["total_first_source_contribution"]
    assert np.any(fs_o != 0.0)
    assert np.allclose(fs_g, fs_o, rtol=1e-3, atol=1e-3 * np.max(np.abs(fs_o)))


@pytest.mark.parametrize("dim,level", [(2, None), (3, 3), (3, 7)])
def test_device_built_bvh_answers_like_the_host_built_one(zgpu, dim, level):
    """The linear BVH built on the GPU (Morton order, 4-wide collapse) gives the host-built
    tree's closest points, ray hits and hit counts, and the same Walk on Spheres walks."""
    from zombie_gb300 import api
    if dim == 2:
        pos, idx = P.star_polygon(4096)
    else:
        pos, idx, _ = P.displaced_icosphere(level, seed=5)
    host = api.GpuDirichletBoundaryHandler(dim)
    host.build_acceleration_structure(pos, idx)
    dev = api.GpuDirichletBoundaryHandler(dim)
    dev.build_acceleration_structure(pos, idx, build_on_device=True)
    assert dev.info()["depth"] <= 20
    assert dev.signed_volume() == pytest.approx(host.signed_volume(), rel=1e-5)
    rng = np.random.default_rng(9)
    x = rng.uniform(-1.3, 1.3, (20000, dim)).astype(np.float32)
    hp, hn, hd, hi = host.closest_point(x)
    dp, dn, dd, di = dev.closest_point(x)
    assert np.array_equal(hd, dd)
    # equal distances everywhere; a different primitive is an exact tie (shared vertex or
    # edge) that the two trees' box tests meet in another order
    same = hi == di
    assert same.mean() > 0.99
    assert np.array_equal(hp[same], dp[same])
    d = rng.normal(size=(20000, dim)).astype(np.float32)
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    tm = np.full(20000, 5.0, np.float32)
    z = np.zeros_like(x)
    on = np.zeros(20000, np.int32)
    h1 = host.intersect(x, z, d, tm, on)
    h2 = dev.intersect(x, z, d, tm, on)
    assert np.array_equal(h1[0], h2[0]) and np.array_equal(h1[3], h2[3])
    assert np.array_equal(host.count_hits(x, d, tm), dev.count_hits(x, d, tm))


@pytest.mark.parametrize("dim,kind,level", [(2, A.ZGPU_BOUNDARY_NEUMANN, None), (3, A.ZGPU_BOUNDARY_NEUMANN, 3),
                                            (3, A.ZGPU_BOUNDARY_NEUMANN, 5), (2, A.ZGPU_BOUNDARY_ROBIN, None),
                                            (3, A.ZGPU_BOUNDARY_ROBIN, 4)])
def test_device_built_reflecting_boundary_answers_like_the_host_built_one(zgpu, oracle, dim, kind, level):
    """Reflecting boundaries built on the GPU (adjacency, silhouette flags, normal cones,
    Robin coefficient ranges and the silhouette-candidate tree all on the device): closest
    points as on the host-built tree; Neumann star radii (closest silhouette points) identical;
    Robin star radii against the oracle's brute force as for host-built trees, and refitted
    by a coefficient update exactly like a fresh device build."""
    from zombie_gb300 import api
    if dim == 2:
        pos, idx = P.star_polygon(4096)
    else:
        pos, idx, _ = P.displaced_icosphere(level, seed=5)
    n = idx.shape[0]
    ic = api.IgnoreCandidateSilhouette(False, 0.0)
    robin = kind == A.ZGPU_BOUNDARY_ROBIN
    kmin, kmax = _mixed_robin(n, 21) if robin else (None, None)
    cls = api.GpuRobinBoundaryHandler if robin else api.GpuNeumannBoundaryHandler
    host, dev = cls(dim), cls(dim)
    args = (pos, idx, ic, kmin, kmax) if robin else (pos, idx, ic)
    host.build_acceleration_structure(*args)
    dev.build_acceleration_structure(*args, build_on_device=True)
    assert dev.info()["depth"] <= 20
    assert dev.signed_volume() == pytest.approx(host.signed_volume(), rel=1e-5)
    rng = np.random.default_rng(31)
    m = 8000
    x = rng.uniform(-0.7, 0.7, (m, dim)).astype(np.float32)
    assert np.array_equal(host.closest_point(x)[2], dev.closest_point(x)[2])
    mn = np.full(m, 1e-3, np.float32)
    mx = np.where(rng.random(m) < 0.3, A.FLT_MAX, rng.uniform(0.05, 2.0, m)).astype(np.float32)
    for flip in (0, 1):
        fl = np.full(m, flip, np.int32)
        rh = host.star_radius(x, mn, mx, 1e-3, fl)
        rd = dev.star_radius(x, mn, mx, 1e-3, fl)
        if not robin:
            assert np.array_equal(rh, rd)
            continue
        ob = oracle.Boundary(dim, pos, idx, kind=kind, kmin=kmin, kmax=kmax, silhouette_precision=0.0, use_bvh=False)
        orr = ob.star_radius(x, mn, mx, 1e-3, fl)
        for r in (rh, rd):
            rel = np.abs(r - orr) / np.maximum(orr, 1e-30)
            assert np.median(rel) <= 1e-6
            assert np.quantile(rel, 0.99) <= 2e-3
            assert np.mean(rel <= 1e-5) > 0.95
    if robin:
        k2min, k2max = _mixed_robin(n, 22)
        dev.update_coefficient_values(k2min, k2max)
        fresh = cls(dim)
        fresh.build_acceleration_structure(pos, idx, ic, k2min, k2max, build_on_device=True)
        fl = np.zeros(m, np.int32)
        assert np.array_equal(dev.star_radius(x, mn, mx, 1e-3, fl), fresh.star_radius(x, mn, mx, 1e-3, fl))


@pytest.mark.parametrize("make", [lambda: P.mixed_wost_2d(n_segments=4096, grid=32, spp=128),
                                  lambda: P.robin_wost_3d(level=4, n_points=400, spp=128)])
def test_solves_on_device_built_boundaries(zgpu, make):
    """Walk on Stars over boundaries built entirely on the GPU: Neumann walks are the walks of
    the host-built boundaries (identical queries); Robin estimates agree within their errors."""
    from zombie_gb300.runner import GpuProblem, summarize
    pr = make()
    a, b = GpuProblem(pr), GpuProblem(pr, build_on_device=True)
    xa, xb = a.host_arrays(), b.host_arrays()
    ra, rb = a.solve(xa), b.solve(xb)
    assert ra.error_word == 0 and rb.error_word == 0
    if pr.reflecting_kind == A.ZGPU_BOUNDARY_NEUMANN:
        assert ra.total_steps == rb.total_steps
        assert np.array_equal(xa["total_walk_length"], xb["total_walk_length"])
    ga, gb = summarize(xa, pr.exact()), summarize(xb, pr.exact())
    z = (ga["mean"] - gb["mean"]) / np.maximum(np.sqrt(ga["se"] ** 2 + gb["se"] ** 2), 1e-12)
    assert np.mean(np.abs(z) > 3.5) < 0.02
    ez = gb["err"] / np.maximum(gb["se"], 1e-12)
    assert abs(ez.mean()) < 0.5


def test_step_budget_drops_walks_and_reports_it(zgpu):
    """zgpu_solve_options.step_budget caps the loop iterations of a walk state: a budget
    below the walks' lengths returns ZGPU_ERR_TIMEOUT_BUDGET, a generous one changes nothing."""
    from zombie_gb300 import _lib
    from zombie_gb300.runner import GpuProblem
    pr = P.laplace_wos_2d(n_segments=512, grid=16, spp=32)
    gp = GpuProblem(pr)
    ref = gp.device_arrays()
    gp.solve(ref)
    opt = A.SolveOptions()
    opt.step_budget = 2
    with pytest.raises(_lib.ZgpuError) as e:
        gp.solve(gp.device_arrays(), options=opt)
    assert e.value.status == A.ZGPU_ERR_TIMEOUT_BUDGET
    opt.step_budget = 100000
    d = gp.device_arrays()
    gp.solve(d, options=opt)
    for k in ("n_solution_estimates", "total_walk_length"):
        assert np.array_equal(ref[k].cpu().numpy(), d[k].cpu().numpy())
