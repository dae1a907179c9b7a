"""The sorted-wavefront schedule of the walk loop against the persistent walk kernel.

Both schedules run the same walks: each walk keeps its pcg32 stream and its arithmetic, and
the wavefront only moves the closest-point query from the end of a step to the start of the
next.  On the same inputs they must therefore agree walk for walk: the same estimate counts,
walk lengths and step / escape / length-limit / Russian-roulette counters, and per-point
means equal up to the order of the FP64 sums (walks finish in another order).  The oracle
parity of the wavefront itself is covered by the solver tests, whose 2D Walk on Stars cases
run on it under the automatic schedule; Walk on Spheres on the wavefront is held to the
persistent kernel here, whose oracle parity the solver tests cover.
"""
import numpy as np
import pytest

from zombie_gb300 import _abi as A
from zombie_gb300 import problems as P

pytestmark = pytest.mark.gpu


def _wos_source_rr():
    pr = P.laplace_wos_2d(n_segments=512, grid=16, spp=256)
    pr.pde = P.make_pde(pr.solution, sigma=2.0, source=True)      # f = 2u: sampled source points
    pr.settings = P.default_walk_settings(rr=0.9)
    return pr


def _double_sided():
    pr = P.mixed_wost_2d(n_segments=1024, grid=24, spp=64)
    pr.settings = P.default_walk_settings(double_sided=True)
    return pr


CASES = {
    "mixed_2d": lambda: P.mixed_wost_2d(n_segments=2048, grid=32, spp=128),
    "screened_2d": lambda: P.mixed_wost_2d(n_segments=2048, grid=24, spp=128, sigma=1.0),
    "mixed_2d_grid_fields": lambda: P.with_grid_fields(P.mixed_wost_2d(n_segments=1024, grid=24, spp=64),
                                                       ("dirichlet", "source")),
    "double_sided_2d": _double_sided,
    "robin_rr_3d": lambda: P.robin_wost_3d(level=4, n_points=400, spp=128),
    "wos_laplace_2d": lambda: P.laplace_wos_2d(n_segments=1024, grid=32, spp=128),
    "wos_source_rr_2d": _wos_source_rr,
    "wos_screened_3d": lambda: P.screened_wos_3d(level=4, n_points=400, spp=128),
    # more walks (9.9M) than the pool holds (2^23): slots are refilled over many rounds
    "mixed_2d_pool_rounds": lambda: P.mixed_wost_2d(n_segments=1024, grid=136, spp=1024),
}


def _solve(gp, schedule, **opts):
    opt = A.SolveOptions()
    opt.schedule = schedule
    opt.query_mode = A.ZGPU_QUERY_MODE_LANE
    for k, v in opts.items():
        setattr(opt, k, v)
    arrays = gp.device_arrays()
    rep = gp.solve(arrays, options=opt)
    return {k: arrays[k].cpu().numpy() for k in ("solution_mean", "solution_m2", "n_solution_estimates",
                                                  "total_walk_length", "first_sphere_radius")}, rep


@pytest.mark.parametrize("case", sorted(CASES))
def test_wavefront_runs_the_persistent_kernels_walks(zgpu, case):
    from zombie_gb300.runner import GpuProblem
    gp = GpuProblem(CASES[case]())
    a, ra = _solve(gp, A.ZGPU_SCHEDULE_PERSISTENT)
    b, rb = _solve(gp, A.ZGPU_SCHEDULE_WAVEFRONT)
    assert ra.error_word == 0 and rb.error_word == 0
    assert ra.total_walks == rb.total_walks > 0
    assert (ra.total_steps, ra.escaped_walks, ra.exceeded_walks, ra.rr_terminated) == \
           (rb.total_steps, rb.escaped_walks, rb.exceeded_walks, rb.rr_terminated)
    assert np.array_equal(a["n_solution_estimates"], b["n_solution_estimates"])
    assert np.array_equal(a["total_walk_length"], b["total_walk_length"])
    assert np.array_equal(a["first_sphere_radius"], b["first_sphere_radius"])
    assert np.allclose(a["solution_mean"], b["solution_mean"], rtol=1e-9, atol=1e-12)
    assert np.allclose(a["solution_m2"], b["solution_m2"], rtol=1e-8, atol=1e-10)


def test_batched_wavefront_runs_the_persistent_kernels_walks(zgpu):
    """A batched many-solve on the wavefront (records sorted by scene, then by cell in the
    scene's box) runs the walks of the persistent batched kernel."""
    from zombie_gb300.runner import GpuBatch
    batch = GpuBatch(P.batched_scenes(n_scenes=5, seed=3, point_scale=0.004, segments=(256, 4096)))
    out = {}
    for sched in (A.ZGPU_SCHEDULE_PERSISTENT, A.ZGPU_SCHEDULE_WAVEFRONT):
        opt = A.SolveOptions()
        opt.schedule = sched
        arrays = batch.device_arrays()
        rep = batch.solve(arrays, options=opt)
        assert rep.error_word == 0 and rep.total_steps > 0
        out[sched] = (rep, {k: arrays[k].cpu().numpy() for k in ("solution_mean", "n_solution_estimates",
                                                                  "total_walk_length")})
    (ra, a), (rb, b) = out[A.ZGPU_SCHEDULE_PERSISTENT], out[A.ZGPU_SCHEDULE_WAVEFRONT]
    assert (ra.total_steps, ra.escaped_walks, ra.exceeded_walks) == (rb.total_steps, rb.escaped_walks, rb.exceeded_walks)
    assert np.array_equal(a["n_solution_estimates"], b["n_solution_estimates"])
    assert np.array_equal(a["total_walk_length"], b["total_walk_length"])
    assert np.allclose(a["solution_mean"], b["solution_mean"], rtol=1e-9, atol=1e-12)


def test_automatic_schedule_picks_the_wavefront_in_2d(zgpu):
    """Auto (0) runs 2D Walk on Stars on the wavefront: its statistics are the wavefront's."""
    from zombie_gb300.runner import GpuProblem
    gp = GpuProblem(P.mixed_wost_2d(n_segments=1024, grid=16, spp=64))
    a, ra = _solve(gp, A.ZGPU_SCHEDULE_AUTO)
    b, rb = _solve(gp, A.ZGPU_SCHEDULE_WAVEFRONT)
    assert ra.total_steps == rb.total_steps
    assert np.array_equal(a["total_walk_length"], b["total_walk_length"])


def test_wavefront_replayed_from_its_graph_runs_the_same_walks(zgpu):
    """use_graph on the wavefront: chunks of iterations replayed from a captured graph (the
    capture reused by the second solve) run the walks of the launched iterations."""
    from zombie_gb300.runner import GpuProblem
    gp = GpuProblem(P.mixed_wost_2d(n_segments=1024, grid=40, spp=256))
    ref, rr = _solve(gp, A.ZGPU_SCHEDULE_WAVEFRONT)
    for _ in range(2):
        got, rg = _solve(gp, A.ZGPU_SCHEDULE_WAVEFRONT, use_graph=1)
        assert rg.total_steps == rr.total_steps and rg.kernel_launches == rr.kernel_launches
        assert np.array_equal(ref["total_walk_length"], got["total_walk_length"])
        assert np.allclose(ref["solution_mean"], got["solution_mean"], rtol=1e-9, atol=1e-12)


def test_wavefront_step_budget_drops_the_same_walks(zgpu):
    from zombie_gb300._lib import ZgpuError
    from zombie_gb300.runner import GpuProblem
    gp = GpuProblem(P.mixed_wost_2d(n_segments=1024, grid=16, spp=64))
    out = {}
    for sched in (A.ZGPU_SCHEDULE_PERSISTENT, A.ZGPU_SCHEDULE_WAVEFRONT):
        opt = A.SolveOptions()
        opt.schedule = sched
        opt.step_budget = 6
        arrays = gp.device_arrays()
        with pytest.raises(ZgpuError) as e:
            gp.solve(arrays, options=opt)
        assert e.value.status == A.ZGPU_ERR_TIMEOUT_BUDGET
        out[sched] = arrays["n_solution_estimates"].cpu().numpy()
    assert np.array_equal(out[A.ZGPU_SCHEDULE_PERSISTENT], out[A.ZGPU_SCHEDULE_WAVEFRONT])
    assert out[A.ZGPU_SCHEDULE_WAVEFRONT].sum() < 64 * len(out[A.ZGPU_SCHEDULE_WAVEFRONT])


def test_wavefront_refuses_what_it_cannot_serve(zgpu):
    from zombie_gb300._lib import ZgpuError
    from zombie_gb300.runner import GpuProblem

    def refused(gp, **opts):
        opt = A.SolveOptions()
        opt.schedule = A.ZGPU_SCHEDULE_WAVEFRONT
        for k, v in opts.items():
            setattr(opt, k, v)
        with pytest.raises(ZgpuError) as e:
            gp.solve(gp.device_arrays(), options=opt)
        return e.value.status

    gp = GpuProblem(P.mixed_wost_2d(n_segments=512, grid=8, spp=8))
    assert refused(gp, query_mode=A.ZGPU_QUERY_MODE_WARP) == A.ZGPU_ERR_UNSUPPORTED
    assert refused(gp, schedule=3) == A.ZGPU_ERR_INVALID_ARG
    # gradient walks keep to the persistent kernel
    opt = A.SolveOptions()
    opt.schedule = A.ZGPU_SCHEDULE_WAVEFRONT
    with pytest.raises(ZgpuError) as e:
        gp.solve(gp.device_arrays(gradients=True), options=opt)
    assert e.value.status == A.ZGPU_ERR_UNSUPPORTED
    # walk splitting needs split scratch the wavefront does not keep
    pr = P.mixed_wost_2d(n_segments=512, grid=8, spp=8)
    pr.settings = P.default_walk_settings(splitting=1.5)
    assert refused(GpuProblem(pr)) == A.ZGPU_ERR_UNSUPPORTED
