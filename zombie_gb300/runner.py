"""Runs the synthetic model problems (zombie_gb300.problems) through the public API.

`GpuProblem` builds the boundary handlers and sample arrays once; `solve()` runs one call of
WalkOnSpheres/WalkOnStars::solve over all points (host arrays: the end-to-end path;
device tensors: inputs already resident in HBM).
"""
import numpy as np

from . import _abi as A
from . import problems as P
from .api import (GeometricQueries, GpuDirichletBoundaryHandler, GpuNeumannBoundaryHandler, GpuRobinBoundaryHandler,
                  IgnoreCandidateSilhouette, PDE, SampleArrays, WalkOnSpheres, WalkOnStars, default_context)


class GpuProblem:
    def __init__(self, problem, context=None, seed_base=0x5eed, options=None, build_on_device=False):
        self.problem = problem
        self.ctx = context or default_context()
        D = problem.dim
        self.queries = GeometricQueries(True, problem.domain_min, problem.domain_max, dim=D)
        ic = IgnoreCandidateSilhouette(bool(problem.settings.solve_double_sided), problem.ignore_silhouette_precision)
        if problem.absorbing is not None and len(problem.absorbing[1]) > 0:
            h = GpuDirichletBoundaryHandler(D, self.ctx)
            h.build_acceleration_structure(*problem.absorbing, build_on_device=build_on_device)
            self.queries.absorbing = h
        if problem.reflecting is not None and len(problem.reflecting[1]) > 0:
            if problem.reflecting_kind == A.ZGPU_BOUNDARY_ROBIN:
                h = GpuRobinBoundaryHandler(D, self.ctx)
                n = len(problem.reflecting[1])
                if problem.robin_coeff_range is not None:
                    kmin, kmax = problem.robin_coeff_range
                else:
                    kmin = kmax = np.full(n, problem.robin_coeff, np.float32)
                h.build_acceleration_structure(*problem.reflecting, ic, kmin, kmax, build_on_device=build_on_device)
            else:
                h = GpuNeumannBoundaryHandler(D, self.ctx)
                h.build_acceleration_structure(*problem.reflecting, ic, build_on_device=build_on_device)
            self.queries.reflecting = h
        self.pde = PDE.from_c(D, problem.pde)
        self.solver = (WalkOnSpheres if problem.solver == A.ZGPU_SOLVER_WALK_ON_SPHERES else WalkOnStars)(
            self.queries, dim=D, context=self.ctx, options=options)
        self.points = problem.points
        self.dist = self.queries.compute_dist_to_absorbing_boundary(self.points)
        self.seeds = P.seeds_for(self.points.shape[0], seed_base)

    def host_arrays(self, n_walks=None, gradients=False):
        nw = self.problem.n_walks if n_walks is None else np.broadcast_to(np.asarray(n_walks, np.int32),
                                                                          (self.points.shape[0],))
        return SampleArrays.host(self.points, self.dist, nw, self.seeds, gradients=gradients)

    def device_arrays(self, n_walks=None, gradients=False):
        import torch
        h = self.host_arrays(n_walks, gradients)
        dev = {}
        for k, v in h.arrays.items():
            t = torch.from_numpy(np.ascontiguousarray(v).view(np.int64) if v.dtype == np.uint64 else np.ascontiguousarray(v))
            dev[k] = t.to("cuda:%d" % self.ctx.device)
        return SampleArrays(**dev)

    def solve(self, arrays, options=None, cache=None, cache_min_distance=0.05):
        return self.solver.solve_arrays(self.pde, self.problem.settings, arrays, options, cache=cache,
                                        cache_min_distance=cache_min_distance)

    def exact(self):
        return self.problem.exact()


def summarize(arrays, exact):
    """RMSE vs the analytic solution and per-point standard errors, in FP64."""
    def host(x):
        return x.cpu().numpy() if hasattr(x, "cpu") else np.asarray(x)
    mean = host(arrays["solution_mean"]).astype(np.float64)
    m2 = host(arrays["solution_m2"]).astype(np.float64)
    n = host(arrays["n_solution_estimates"]).astype(np.float64)
    var = m2 / np.maximum(n - 1, 1)
    se = np.sqrt(var / np.maximum(n, 1))
    err = mean - exact
    return dict(rmse=float(np.sqrt(np.mean(err ** 2))), mean=mean, se=se, n=n, err=err,
                mean_walk_length=float(host(arrays["total_walk_length"]).sum() / max(1.0, n.sum())))


class GpuBatch:
    """Independent problems solved in one launch (zgpu_solve_batched): each point carries the
    row of its problem in the scene table.  Per-point seeds are those of the single-problem
    solves, so a batched solve runs the same walks as solving each problem alone."""

    def __init__(self, problems, context=None, seed_base=0x5eed, options=None):
        from . import _abi as A
        self.ctx = context or default_context()
        self.problems = [GpuProblem(p, context=self.ctx, seed_base=seed_base) for p in problems]
        self.solver_id = problems[0].solver
        if any(p.solver != self.solver_id for p in problems) or any(p.dim != problems[0].dim for p in problems):
            raise ValueError("a batch holds problems of one dimension and one solver")
        self.options = options
        n = len(self.problems)
        self.q = (A.GeometricQueriesC * n)(*[g.queries.to_c() for g in self.problems])
        self.pde = (A.Pde * n)(*[g.pde.to_c() for g in self.problems])
        self.ws = (A.WalkSettingsC * n)(*[g.problem.settings for g in self.problems])
        self.offsets = np.cumsum([0] + [g.points.shape[0] for g in self.problems])

    @property
    def n_points(self):
        return int(self.offsets[-1])

    def device_arrays(self):
        import torch
        parts = [g.device_arrays() for g in self.problems]
        dev = {}
        for k in parts[0].arrays:
            dev[k] = torch.cat([p.arrays[k] for p in parts])
        sid = np.concatenate([np.full(g.points.shape[0], i, np.int32) for i, g in enumerate(self.problems)])
        dev["scene_id"] = torch.from_numpy(sid).to(dev["pt"].device)
        return SampleArrays(**dev)

    def host_arrays(self):
        parts = [g.host_arrays() for g in self.problems]
        arr = {k: np.concatenate([p.arrays[k] for p in parts]) for k in parts[0].arrays}
        arr["scene_id"] = np.concatenate([np.full(g.points.shape[0], i, np.int32) for i, g in enumerate(self.problems)])
        return SampleArrays(**arr)

    def solve(self, arrays, options=None):
        import ctypes as C
        from . import _abi as A
        from ._lib import check, lib
        from .api import SolveReport
        sp, st = arrays.to_c()
        opt = options or self.options
        rep = A.SolveReport()
        check(lib().zgpu_solve_batched(self.ctx.h, self.solver_id, len(self.problems), self.q, self.pde, self.ws,
                                       C.byref(sp), C.byref(st), C.byref(opt) if opt is not None else None,
                                       C.byref(rep)))
        launches = C.c_int64()
        check(lib().zgpu_last_solve_launches(self.ctx.h, C.byref(launches)))
        return SolveReport(rep, launches.value)

    def exact(self):
        return np.concatenate([g.problem.exact() for g in self.problems])
