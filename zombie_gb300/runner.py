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
    def __init__(self, problem, context=None, seed_base=0x5eed, options=None):
        self.problem = problem
        self.ctx = context or default_context()
        D = problem.dim
        self.queries = GeometricQueries(True, problem.domain_min, problem.domain_max, dim=D)
        ic = IgnoreCandidateSilhouette(bool(problem.settings.solve_double_sided), problem.ignore_silhouette_precision)
        if problem.absorbing is not None and len(problem.absorbing[1]) > 0:
            h = GpuDirichletBoundaryHandler(D, self.ctx)
            h.build_acceleration_structure(*problem.absorbing)
            self.queries.absorbing = h
        if problem.reflecting is not None and len(problem.reflecting[1]) > 0:
            if problem.reflecting_kind == A.ZGPU_BOUNDARY_ROBIN:
                h = GpuRobinBoundaryHandler(D, self.ctx)
                n = len(problem.reflecting[1])
                k = np.full(n, problem.robin_coeff, np.float32)
                h.build_acceleration_structure(*problem.reflecting, ic, k, k)
            else:
                h = GpuNeumannBoundaryHandler(D, self.ctx)
                h.build_acceleration_structure(*problem.reflecting, ic)
            self.queries.reflecting = h
        self.pde = PDE.from_c(D, problem.pde)
        self.solver = (WalkOnSpheres if problem.solver == A.ZGPU_SOLVER_WALK_ON_SPHERES else WalkOnStars)(
            self.queries, dim=D, context=self.ctx, options=options)
        self.points = problem.points
        self.dist = self.queries.compute_dist_to_absorbing_boundary(self.points)
        self.seeds = P.seeds_for(self.points.shape[0], seed_base)

    def host_arrays(self, n_walks=None):
        nw = self.problem.n_walks if n_walks is None else np.broadcast_to(np.asarray(n_walks, np.int32),
                                                                          (self.points.shape[0],))
        return SampleArrays.host(self.points, self.dist, nw, self.seeds)

    def device_arrays(self, n_walks=None):
        import torch
        h = self.host_arrays(n_walks)
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
