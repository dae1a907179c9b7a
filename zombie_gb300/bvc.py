"""Boundary Value Caching (variance_reduction/boundary_value_caching.h, boundary_samplers.h,
domain_samplers.h) over the GPU walk engine.

A boundary value caching solve (Miller et al., "Boundary Value Caching for Walk on Spheres",
2023) estimates the solution and its normal derivative at a cache of boundary samples with
Walk on Stars, then splats every cached value onto every evaluation point through the
free-space Green's function.  Here the walks run in the walk kernels (zgpu_solve: normal
derivatives through the gradient estimator with directionForDerivative = the sample's
normal), the PDE data of the samples come from the device field evaluation
(zgpu_pde_evaluate), and the all-pairs splat is a CUDA kernel (zgpu_bvc_splat).  Sample
generation (CDF tables over the boundary, stratified candidates in the domain) is host-side
bookkeeping, as in the reference.

Caches and evaluation points are structures of arrays (`SampleCache`, `EvaluationPoints`);
`EvaluationPoint` is the reference's per-point view.
"""
import ctypes as C

import numpy as np

from . import _abi as A
from ._lib import check, lib
from .api import (EstimationQuantity, SampleArrays, SampleType, WalkOnStars, default_context, pde_evaluate)


# --------------------------------------------------------------------------- helpers
def _stratified(n, dim, rng):
    """n jittered stratified samples in [0,1)^dim, strata in random order per dimension
    (generateStratifiedSamples, core/sampling.h)."""
    if n <= 0:
        return np.zeros((0, dim), np.float32)
    u = np.empty((n, dim), np.float64)
    for j in range(dim):
        u[:, j] = (rng.permutation(n) + rng.random(n)) / n
    return np.minimum(u, 1.0 - 1e-7).astype(np.float32)


def _inside(fn, x):
    """insideSolveRegion over an (N, D) array: a vectorised callable, or one taking a point."""
    try:
        m = np.asarray(fn(x), bool)
        if m.shape == (x.shape[0],):
            return m
    except Exception:
        pass
    return np.array([bool(fn(p)) for p in x], bool)


def _seeds(rng, n):
    return rng.integers(0, np.iinfo(np.int64).max, n, dtype=np.int64).astype(np.uint64)


class SampleCache:
    """A cache of SamplePoints (common.h:151-195) as arrays, with the members boundary value
    caching fills: robin_coeff, solution, normal_derivative, contribution."""

    def __init__(self, dim, pt, normal, type, pdf, dist_to_absorbing, dist_to_reflecting, aligned=False, seeds=None):
        n = pt.shape[0]
        self.dim = dim
        self.pt = np.ascontiguousarray(pt, np.float32).reshape(n, dim)
        self.normal = np.ascontiguousarray(normal, np.float32).reshape(n, dim)
        self.type = np.ascontiguousarray(np.broadcast_to(np.asarray(type, np.int32), (n,)))
        self.pdf = np.ascontiguousarray(np.broadcast_to(np.asarray(pdf, np.float32), (n,)))
        self.dist_to_absorbing = np.ascontiguousarray(dist_to_absorbing, np.float32)
        self.dist_to_reflecting = np.ascontiguousarray(dist_to_reflecting, np.float32)
        self.estimate_normal_aligned = np.ascontiguousarray(np.broadcast_to(np.asarray(aligned, np.int32), (n,)))
        self.estimation_quantity = np.full(n, int(EstimationQuantity.Solution), np.int32)
        self.direction_for_derivative = np.zeros((n, dim), np.float32)
        self.direction_for_derivative[:, 0] = 1.0
        self.seed = seeds if seeds is not None else _seeds(np.random.default_rng(), n)
        self.first_sphere_radius = np.zeros(n, np.float32)
        self.robin_coeff = np.zeros(n, np.float32)
        self.solution = np.zeros(n, np.float32)
        self.normal_derivative = np.zeros(n, np.float32)
        self.contribution = np.zeros(n, np.float32)

    def __len__(self):
        return self.pt.shape[0]

    @staticmethod
    def empty(dim):
        z = np.zeros((0, dim), np.float32)
        return SampleCache(dim, z, z, np.zeros(0, np.int32), np.zeros(0, np.float32), np.zeros(0, np.float32),
                           np.zeros(0, np.float32), seeds=np.zeros(0, np.uint64))

    def to_c(self):
        s = A.BvcSamplesC()
        s.n = len(self)
        for name in ("pt", "normal", "pdf", "type", "estimate_normal_aligned", "solution", "normal_derivative",
                     "contribution", "robin_coeff"):
            setattr(s, name, A.ptr(getattr(self, name)))
        return s


class EvaluationPoints:
    """EvaluationPoint (boundary_value_caching.h:19-56) for many points: five statistics each
    (absorbing, absorbing normal-aligned, reflecting, reflecting normal-aligned, source) with
    FP64 solution and gradient moments."""

    def __init__(self, pt, normal=None, type=None, dist_to_absorbing=None, dist_to_reflecting=None, dim=None):
        pt = np.asarray(pt, np.float32)
        self.dim = dim or pt.shape[-1]
        n = pt.reshape(-1, self.dim).shape[0]
        self.pt = np.ascontiguousarray(pt.reshape(n, self.dim))
        self.normal = np.zeros((n, self.dim), np.float32) if normal is None else \
            np.ascontiguousarray(normal, np.float32).reshape(n, self.dim)
        self.type = np.full(n, int(SampleType.InDomain), np.int32) if type is None else \
            np.ascontiguousarray(np.broadcast_to(np.asarray(type, np.int32), (n,)))
        self.dist_to_absorbing = np.full(n, np.float32(3.4e38), np.float32) if dist_to_absorbing is None else \
            np.ascontiguousarray(dist_to_absorbing, np.float32)
        self.dist_to_reflecting = np.full(n, np.float32(3.4e38), np.float32) if dist_to_reflecting is None else \
            np.ascontiguousarray(dist_to_reflecting, np.float32)
        self.reset()

    def __len__(self):
        return self.pt.shape[0]

    def reset(self, mask=None):
        n, G, D = len(self), A.ZGPU_BVC_GROUPS, self.dim
        if mask is None:
            self.mean = np.zeros((n, G))
            self.m2 = np.zeros((n, G))
            self.count = np.zeros((n, G), np.int32)
            self.gradient_mean = np.zeros((n, G, D))
            self.gradient_m2 = np.zeros((n, G, D))
        else:
            for a in (self.mean, self.m2, self.count, self.gradient_mean, self.gradient_m2):
                a[mask] = 0

    def get_estimated_solution(self):
        """EvaluationPoint::getEstimatedSolution: the sum of the five statistics' means."""
        return self.mean.sum(axis=1)

    def get_estimated_gradient(self):
        return self.gradient_mean.sum(axis=1)

    def to_c(self):
        e = A.BvcEvalPointsC()
        e.n = len(self)
        for name in ("pt", "type", "dist_to_absorbing", "dist_to_reflecting", "mean", "m2", "count", "gradient_mean",
                     "gradient_m2"):
            setattr(e, name, A.ptr(getattr(self, name)))
        return e


class EvaluationPoint:
    """One evaluation point (boundary_value_caching.h:19-56), a view of EvaluationPoints."""

    def __init__(self, pt, normal, type, dist_to_absorbing_boundary, dist_to_reflecting_boundary):
        self._pts = EvaluationPoints(np.asarray(pt, np.float32)[None], np.asarray(normal, np.float32)[None], [int(type)],
                                     [dist_to_absorbing_boundary], [dist_to_reflecting_boundary])
        self.pt, self.normal, self.type = self._pts.pt[0], self._pts.normal[0], SampleType(int(type))
        self.dist_to_absorbing_boundary = float(dist_to_absorbing_boundary)
        self.dist_to_reflecting_boundary = float(dist_to_reflecting_boundary)

    def get_estimated_solution(self):
        return float(self._pts.get_estimated_solution()[0])

    def get_estimated_gradient(self):
        return list(self._pts.get_estimated_gradient()[0])

    def reset(self):
        self._pts.reset()


def evaluation_points_from_list(points):
    """Gathers a list of EvaluationPoint into one EvaluationPoints (and back with scatter)."""
    dim = points[0].pt.shape[0]
    return EvaluationPoints(np.array([p.pt for p in points]), np.array([p.normal for p in points]),
                            [int(p.type) for p in points], [p.dist_to_absorbing_boundary for p in points],
                            [p.dist_to_reflecting_boundary for p in points], dim=dim)


def scatter_to_list(ev, points):
    for i, p in enumerate(points):
        for name in ("mean", "m2", "count", "gradient_mean", "gradient_m2"):
            getattr(p._pts, name)[0] = getattr(ev, name)[i]


# --------------------------------------------------------------------------- samplers
class _MeshBoundarySampler:
    """Uniform sampling of a segment (2D) / triangle (3D) mesh by area x primitive weight, on
    the mesh displaced along its vertex normals (UniformLineSegmentBoundarySampler /
    UniformTriangleBoundarySampler, boundary_samplers.h:36-186)."""

    def __init__(self, positions, indices, inside_solve_region, primitive_weights=None,
                 primitive_weights_normal_aligned=None, compute_weighted_normals=False, seed=None, dim=None):
        self.positions = np.asarray(positions, np.float64)
        self.dim = dim or self.positions.shape[1]
        self.indices = np.asarray(indices, np.int64).reshape(-1, self.dim)
        n = self.indices.shape[0]
        self.weights = np.ones(n) if primitive_weights is None else np.asarray(primitive_weights, np.float64)
        self.weights_aligned = self.weights.copy() if primitive_weights_normal_aligned is None else \
            np.asarray(primitive_weights_normal_aligned, np.float64)
        if self.weights.shape != (n,) or self.weights_aligned.shape != (n,):
            raise ValueError("weights must be the same size as the number of primitives")
        if not (np.all(np.isfinite(self.weights)) and np.all(self.weights >= 0) and
                np.all(np.isfinite(self.weights_aligned)) and np.all(self.weights_aligned >= 0)):
            raise ValueError("weights must be non-negative and finite")
        self.inside = inside_solve_region
        self.rng = np.random.default_rng(seed)
        self.face_normals_unit = self._face_normals(True)
        fn = self._face_normals(not compute_weighted_normals)
        vn = np.zeros_like(self.positions)
        for k in range(self.dim):
            np.add.at(vn, self.indices[:, k], fn)
        self.vertex_normals = vn / np.maximum(np.linalg.norm(vn, axis=1, keepdims=True), 1e-30)
        self.mass = 0.0
        self.mass_aligned = 0.0
        self.cdf = self.cdf_aligned = None

    def _face_normals(self, normalize):
        p = self.positions[self.indices]
        if self.dim == 2:
            d = p[:, 1] - p[:, 0]
            n = np.stack([d[:, 1], -d[:, 0]], axis=1)
        else:
            n = np.cross(p[:, 1] - p[:, 0], p[:, 2] - p[:, 0])
        if normalize:
            n = n / np.maximum(np.linalg.norm(n, axis=1, keepdims=True), 1e-30)
        return n

    def _offset_faces(self, offset):
        return self.positions[self.indices] + offset * self.vertex_normals[self.indices]

    def _areas(self, p):
        if self.dim == 2:
            return np.linalg.norm(p[:, 1] - p[:, 0], axis=1)
        return 0.5 * np.linalg.norm(np.cross(p[:, 1] - p[:, 0], p[:, 2] - p[:, 0]), axis=1)

    def _table(self, offset, weights):
        # buildCDFTable: faces whose displaced midpoint lies in the solve region, by area x weight
        mid = self.positions[self.indices].mean(axis=1) + offset * self.face_normals_unit
        keep = _inside(self.inside, mid.astype(np.float32))
        w = np.where(keep, self._areas(self._offset_faces(offset)) * weights, 0.0)
        total = float(w.sum())
        return (np.cumsum(w) / total if total > 0 else None), total

    def initialize(self, normal_offset_for_boundary, solve_double_sided):
        self.cdf, self.mass = self._table(-normal_offset_for_boundary, self.weights)
        if solve_double_sided:
            self.cdf_aligned, self.mass_aligned = self._table(normal_offset_for_boundary, self.weights_aligned)

    def get_sample_count(self, n_total_samples, boundary_normal_aligned_samples=False):
        total = self.mass + self.mass_aligned
        if total <= 0:
            return 0
        m = self.mass_aligned if boundary_normal_aligned_samples else self.mass
        return int(np.ceil(n_total_samples * m / total))

    def generate_samples(self, n_samples, sample_type, normal_offset_for_boundary, queries,
                         generate_boundary_normal_aligned_samples=False):
        aligned = bool(generate_boundary_normal_aligned_samples)
        cdf, mass = (self.cdf_aligned, self.mass_aligned) if aligned else (self.cdf, self.mass)
        offset = normal_offset_for_boundary if aligned else -normal_offset_for_boundary
        weights = self.weights_aligned if aligned else self.weights
        if cdf is None or mass <= 0 or n_samples <= 0:
            return SampleCache.empty(self.dim)
        u = _stratified(n_samples, 1, self.rng)[:, 0]
        face = np.minimum(np.searchsorted(cdf, u, side="right"), len(cdf) - 1)
        p = self._offset_faces(offset)[face]
        if self.dim == 2:
            t = self.rng.random(n_samples)[:, None]
            pt = p[:, 0] + t * (p[:, 1] - p[:, 0])
            d = p[:, 1] - p[:, 0]
            nrm = np.stack([d[:, 1], -d[:, 0]], axis=1)
        else:
            r1, r2 = self.rng.random(n_samples), self.rng.random(n_samples)
            s = np.sqrt(r1)
            b0, b1 = 1.0 - s, r2 * s
            pt = b0[:, None] * p[:, 0] + b1[:, None] * p[:, 1] + (1.0 - b0 - b1)[:, None] * p[:, 2]
            nrm = np.cross(p[:, 1] - p[:, 0], p[:, 2] - p[:, 0])
        nrm = nrm / np.maximum(np.linalg.norm(nrm, axis=1, keepdims=True), 1e-30)
        pdf = weights[face] / mass
        pt = pt.astype(np.float32)
        dA = queries.compute_dist_to_absorbing_boundary(pt)
        dR = queries.compute_dist_to_reflecting_boundary(pt)
        return SampleCache(self.dim, pt, nrm, int(sample_type), pdf, dA, dR, aligned=int(aligned),
                           seeds=_seeds(self.rng, n_samples))


class UniformLineSegmentBoundarySampler(_MeshBoundarySampler):
    def __init__(self, positions, indices, inside_solve_region, primitive_weights=None,
                 primitive_weights_normal_aligned=None, compute_weighted_normals=False, seed=None):
        super().__init__(positions, indices, inside_solve_region, primitive_weights, primitive_weights_normal_aligned,
                         compute_weighted_normals, seed, dim=2)


class UniformTriangleBoundarySampler(_MeshBoundarySampler):
    def __init__(self, positions, indices, inside_solve_region, primitive_weights=None,
                 primitive_weights_normal_aligned=None, compute_weighted_normals=False, seed=None):
        super().__init__(positions, indices, inside_solve_region, primitive_weights, primitive_weights_normal_aligned,
                         compute_weighted_normals, seed, dim=3)


class UniformDomainSampler:
    """UniformDomainSampler (domain_samplers.h:17-110): stratified candidates over the solve
    region's box, oversampled by box volume / region volume, kept inside the region, each with
    pdf 1 / region volume."""

    def __init__(self, inside_solve_region, solve_region_min, solve_region_max, solve_region_volume, seed=None):
        self.inside = inside_solve_region
        self.lo = np.asarray(solve_region_min, np.float64)
        self.hi = np.asarray(solve_region_max, np.float64)
        self.volume = float(solve_region_volume)
        self.dim = self.lo.shape[0]
        self.rng = np.random.default_rng(seed)

    def generate_samples(self, n_samples, queries):
        ext = self.hi - self.lo
        pdf = 1.0 / self.volume if self.volume > 0 else 0.0
        n = n_samples
        if self.volume > 0:
            n = int(min(n_samples * float(np.prod(ext)) * pdf, 1e8))
        u = _stratified(n, self.dim, self.rng)
        pt = (self.lo + ext * u).astype(np.float32)
        pt = pt[_inside(self.inside, pt)]
        dA = queries.compute_dist_to_absorbing_boundary(pt)
        dR = queries.compute_dist_to_reflecting_boundary(pt)
        return SampleCache(self.dim, pt, np.zeros_like(pt), int(SampleType.InDomain), pdf, dA, dR,
                           seeds=_seeds(self.rng, pt.shape[0]))


def _sampler_args(args):
    # (inside), (weights, inside) or (weights, weights_normal_aligned, inside), as the
    # reference's create_uniform_*_boundary_sampler overloads (python/zombie_bindings.h)
    if len(args) == 1:
        return args[0], None, None
    if len(args) == 2:
        return args[1], args[0], None
    if len(args) == 3:
        return args[2], args[0], args[1]
    raise TypeError("expected inside_solve_region, optionally preceded by one or two weight arrays")


def create_uniform_line_segment_boundary_sampler(positions, indices, *args, compute_weighted_normals=False, seed=None):
    inside, w, wa = _sampler_args(args)
    return UniformLineSegmentBoundarySampler(positions, indices, inside, w, wa,
                                             compute_weighted_normals=compute_weighted_normals, seed=seed)


def create_uniform_triangle_boundary_sampler(positions, indices, *args, compute_weighted_normals=False, seed=None):
    inside, w, wa = _sampler_args(args)
    return UniformTriangleBoundarySampler(positions, indices, inside, w, wa,
                                          compute_weighted_normals=compute_weighted_normals, seed=seed)


def create_uniform_domain_sampler(inside_solve_region, solve_region_min, solve_region_max, solve_region_volume,
                                  seed=None):
    return UniformDomainSampler(inside_solve_region, solve_region_min, solve_region_max, solve_region_volume, seed)


# ------------------------------------------------------------------- boundary value caching
class BoundaryValueCaching:
    """BoundaryValueCaching<T,DIM> (boundary_value_caching.h:59-178)."""

    def __init__(self, queries, walk_on_stars):
        self.queries = queries
        self.walk_on_stars = walk_on_stars
        self.dim = queries.dim
        self.ctx = walk_on_stars.ctx

    def _set_estimation_data(self, pde, ws, n_sol, n_grad, robin_cutoff, use_fd, cache):
        # setEstimationData (boundary_value_caching.h:565-621)
        n = len(cache)
        n_walks = np.zeros(n, np.int32)
        ds = bool(ws.solve_double_sided)
        flip = np.where(ds & (cache.estimate_normal_aligned != 0), -1.0, 1.0).astype(np.float32)[:, None]
        absorbing = cache.type == int(SampleType.OnAbsorbingBoundary)
        reflecting = cache.type == int(SampleType.OnReflectingBoundary)
        if np.any(~(absorbing | reflecting)):
            raise ValueError("boundary value caching estimates boundary samples only")
        if use_fd:
            cache.type[absorbing] = int(SampleType.InDomain)
            cache.estimation_quantity[absorbing] = int(EstimationQuantity.Solution)
        else:
            cache.direction_for_derivative[absorbing] = (cache.normal * flip)[absorbing]
            cache.estimation_quantity[absorbing] = int(EstimationQuantity.SolutionAndGradient)
        n_walks[absorbing] = n_grad
        if np.any(reflecting):
            if not pde.are_robin_conditions_pure_neumann:
                aligned = (ds & (cache.estimate_normal_aligned != 0)).astype(np.int32)
                kap = pde_evaluate(pde, cache.pt[reflecting], cache.normal[reflecting], aligned[reflecting],
                                   dim=self.dim, context=self.ctx)[3]
                cache.robin_coeff[reflecting] = kap
            grad = reflecting & (np.abs(cache.robin_coeff) > robin_cutoff)
            cache.direction_for_derivative[grad] = (cache.normal * flip)[grad]
            cache.estimation_quantity[grad] = int(EstimationQuantity.SolutionAndGradient)
            n_walks[grad] = n_grad
            sol = reflecting & ~grad
            cache.estimation_quantity[sol] = int(EstimationQuantity.Solution)
            n_walks[sol] = n_sol
        return n_walks

    def compute_boundary_estimates(self, pde, walk_settings, n_walks_for_solution_estimates,
                                   n_walks_for_gradient_estimates, robin_coeff_cutoff_for_normal_derivative, cache,
                                   use_finite_differences=False, run_single_threaded=False, report_progress=None):
        """computeBoundaryEstimates (boundary_value_caching.h:319-343)."""
        n = len(cache)
        if n == 0:
            return None
        n_walks = self._set_estimation_data(pde, walk_settings, n_walks_for_solution_estimates,
                                            n_walks_for_gradient_estimates, robin_coeff_cutoff_for_normal_derivative,
                                            use_finite_differences, cache)
        D = self.dim
        arr = SampleArrays(
            pt=cache.pt, normal=cache.normal, type=cache.type, estimation_quantity=cache.estimation_quantity,
            dist_to_absorbing=cache.dist_to_absorbing, dist_to_reflecting=cache.dist_to_reflecting,
            n_walks=n_walks, seed=cache.seed, first_sphere_radius=cache.first_sphere_radius,
            estimate_normal_aligned=cache.estimate_normal_aligned,
            direction_for_derivative=np.ascontiguousarray(cache.direction_for_derivative),
            solution_mean=np.zeros(n), solution_m2=np.zeros(n), n_solution_estimates=np.zeros(n, np.int32),
            total_walk_length=np.zeros(n, np.int64), total_splits=np.zeros(n, np.int64),
            gradient_mean=np.zeros((n, D)), gradient_m2=np.zeros((n, D)), n_gradient_estimates=np.zeros(n, np.int32),
            total_first_source_contribution=np.zeros(n), total_derivative_contribution=np.zeros(n))
        rep = self.walk_on_stars.solve_arrays(pde, walk_settings, arr)
        self._set_estimated_boundary_data(pde, walk_settings, robin_coeff_cutoff_for_normal_derivative,
                                          use_finite_differences, cache, arr)
        if report_progress is not None:
            report_progress(n, 0)
        return rep

    def _set_estimated_boundary_data(self, pde, ws, robin_cutoff, use_fd, cache, arr):
        # setEstimatedBoundaryData (boundary_value_caching.h:623-650)
        cnt = np.maximum(arr["n_solution_estimates"], 1).astype(np.float64)
        cache.solution[:] = arr["solution_mean"]
        derivative = (arr["total_derivative_contribution"] / cnt).astype(np.float32)
        ds = bool(ws.solve_double_sided)
        reflecting = cache.type == int(SampleType.OnReflectingBoundary)
        if np.any(reflecting) and not ws.ignore_reflecting_boundary_contribution:
            aligned = (ds & (cache.estimate_normal_aligned != 0)).astype(np.int32)
            h = pde_evaluate(pde, cache.pt[reflecting], cache.normal[reflecting], aligned[reflecting], dim=self.dim,
                             context=self.ctx)[2]
            if pde.are_robin_conditions_pure_neumann:
                cache.normal_derivative[reflecting] = h
            else:
                cache.contribution[reflecting] = h
                grad = reflecting & (np.abs(cache.robin_coeff) > robin_cutoff)
                cache.normal_derivative[grad] = derivative[grad]
        other = ~reflecting
        if not np.any(other):
            return
        if use_fd:
            # biased finite-difference normal derivatives from the projection onto the boundary
            x = cache.pt[other]
            sd = self.queries.compute_dist_to_absorbing_boundary(x, compute_signed_distance=True).astype(np.float32)
            proj = x - sd[:, None] * cache.normal[other]
            aligned = (ds & (sd > 0)).astype(np.int32)
            g = np.zeros(x.shape[0], np.float32)
            if not ws.ignore_absorbing_boundary_contribution:
                g = pde_evaluate(pde, proj, None, aligned, dim=self.dim, context=self.ctx)[1]
            cache.normal_derivative[other] = (g - cache.solution[other]) / np.abs(sd)
            cache.type[other] = int(SampleType.OnAbsorbingBoundary)
        else:
            cache.normal_derivative[other] = derivative[other]

    def set_source_values(self, pde, cache, run_single_threaded=False):
        """setSourceValues (boundary_value_caching.h:345-370)."""
        if len(cache) == 0:
            return
        cache.contribution[:] = pde_evaluate(pde, cache.pt, dim=self.dim, context=self.ctx)[0]
        cache.estimation_quantity[:] = int(EstimationQuantity.Skip)

    def splat(self, pde, cache, radius_clamp, kernel_regularization, robin_coeff_cutoff_for_normal_derivative,
              cutoff_dist_to_absorbing_boundary, cutoff_dist_to_reflecting_boundary, evaluation_points,
              report_progress=None):
        """splat (boundary_value_caching.h:380-459) of a whole cache onto all evaluation points,
        on the GPU (zgpu_bvc_splat)."""
        single = isinstance(evaluation_points, EvaluationPoint)
        listed = isinstance(evaluation_points, (list, tuple))
        ev = evaluation_points._pts if single else (evaluation_points_from_list(evaluation_points) if listed
                                                    else evaluation_points)
        if listed:
            for i, p in enumerate(evaluation_points):
                for name in ("mean", "m2", "count", "gradient_mean", "gradient_m2"):
                    getattr(ev, name)[i] = getattr(p._pts, name)[0]
        if len(cache) > 0 and len(ev) > 0:
            p = pde.to_c()
            s, e = cache.to_c(), ev.to_c()
            check(lib().zgpu_bvc_splat(self.ctx.h, self.dim, C.byref(p), C.byref(s), float(radius_clamp),
                                       float(kernel_regularization), float(robin_coeff_cutoff_for_normal_derivative),
                                       float(cutoff_dist_to_absorbing_boundary),
                                       float(cutoff_dist_to_reflecting_boundary), C.byref(e), A.ZGPU_MEM_HOST))
        if listed:
            scatter_to_list(ev, evaluation_points)
        if report_progress is not None:
            report_progress(len(cache), 0)

    def estimate_solution_near_boundary(self, pde, walk_settings, use_distance_to_absorbing_boundary,
                                        cutoff_dist_to_boundary, n_walks, evaluation_points, run_single_threaded=False):
        """estimateSolutionNearBoundary (boundary_value_caching.h:461-563): points closer to the
        boundary than the cutoff get a plain Walk on Stars estimate instead of splats."""
        ev = evaluation_points
        d = ev.dist_to_absorbing if use_distance_to_absorbing_boundary else ev.dist_to_reflecting
        near = np.nonzero(d < cutoff_dist_to_boundary)[0]
        if near.size == 0:
            return
        m = near.size
        arr = SampleArrays(
            pt=np.ascontiguousarray(ev.pt[near]), normal=np.ascontiguousarray(ev.normal[near]),
            type=np.ascontiguousarray(ev.type[near]), dist_to_absorbing=np.ascontiguousarray(ev.dist_to_absorbing[near]),
            dist_to_reflecting=np.ascontiguousarray(ev.dist_to_reflecting[near]),
            n_walks=np.full(m, int(n_walks), np.int32), seed=_seeds(np.random.default_rng(), m),
            first_sphere_radius=np.zeros(m, np.float32),
            solution_mean=np.zeros(m), solution_m2=np.zeros(m), n_solution_estimates=np.zeros(m, np.int32),
            total_walk_length=np.zeros(m, np.int64), total_splits=np.zeros(m, np.int64))
        self.walk_on_stars.solve_arrays(pde, walk_settings, arr)
        ev.reset(near)
        t = ev.type[near]
        group = np.where(t == int(SampleType.OnAbsorbingBoundary), A.ZGPU_BVC_ABSORBING,
                         np.where(t == int(SampleType.OnReflectingBoundary), A.ZGPU_BVC_REFLECTING, A.ZGPU_BVC_SOURCE))
        ev.mean[near, group] = arr["solution_mean"]
        ev.count[near, group] = 1


class BoundaryValueCachingSolver:
    """BoundaryValueCachingSolver<T,DIM> (boundary_value_caching.h:180-247, :813-945)."""

    def __init__(self, queries, absorbing_boundary_sampler, reflecting_boundary_sampler, domain_sampler, context=None,
                 options=None):
        self.queries = queries
        self.dim = queries.dim
        self.absorbing_sampler = absorbing_boundary_sampler
        self.reflecting_sampler = reflecting_boundary_sampler
        self.domain_sampler = domain_sampler
        self.walk_on_stars = WalkOnStars(queries, dim=self.dim, context=context or default_context(), options=options)
        self.bvc = BoundaryValueCaching(queries, self.walk_on_stars)
        e = SampleCache.empty(self.dim)
        self.absorbing_cache, self.absorbing_cache_aligned = e, SampleCache.empty(self.dim)
        self.reflecting_cache, self.reflecting_cache_aligned = SampleCache.empty(self.dim), SampleCache.empty(self.dim)
        self.domain_cache = SampleCache.empty(self.dim)

    def generate_samples(self, absorbing_boundary_cache_size, reflecting_boundary_cache_size, domain_cache_size,
                         normal_offset_for_absorbing_boundary, normal_offset_for_reflecting_boundary,
                         solve_double_sided):
        def gen(sampler, size, stype, offset, aligned):
            if sampler is None:
                return SampleCache.empty(self.dim)
            return sampler.generate_samples(sampler.get_sample_count(size, aligned), stype, offset, self.queries, aligned)
        A_, R_ = int(SampleType.OnAbsorbingBoundary), int(SampleType.OnReflectingBoundary)
        self.absorbing_cache = gen(self.absorbing_sampler, absorbing_boundary_cache_size, A_,
                                   normal_offset_for_absorbing_boundary, False)
        self.absorbing_cache_aligned = gen(self.absorbing_sampler, absorbing_boundary_cache_size, A_,
                                           normal_offset_for_absorbing_boundary, True) if solve_double_sided \
            else SampleCache.empty(self.dim)
        self.reflecting_cache = gen(self.reflecting_sampler, reflecting_boundary_cache_size, R_,
                                    normal_offset_for_reflecting_boundary, False)
        self.reflecting_cache_aligned = gen(self.reflecting_sampler, reflecting_boundary_cache_size, R_,
                                            normal_offset_for_reflecting_boundary, True) if solve_double_sided \
            else SampleCache.empty(self.dim)
        self.domain_cache = self.domain_sampler.generate_samples(domain_cache_size, self.queries) \
            if self.domain_sampler is not None else SampleCache.empty(self.dim)

    def _boundary_caches(self):
        return [self.absorbing_cache, self.absorbing_cache_aligned, self.reflecting_cache,
                self.reflecting_cache_aligned]

    def compute_sample_estimates(self, pde, walk_settings, n_walks_for_solution_estimates,
                                 n_walks_for_gradient_estimates, robin_coeff_cutoff_for_normal_derivative,
                                 use_finite_differences=False, run_single_threaded=False, report_progress=None):
        reports = []
        for c in self._boundary_caches():
            reports.append(self.bvc.compute_boundary_estimates(pde, walk_settings, n_walks_for_solution_estimates,
                                                               n_walks_for_gradient_estimates,
                                                               robin_coeff_cutoff_for_normal_derivative, c,
                                                               use_finite_differences, run_single_threaded,
                                                               report_progress))
        self.bvc.set_source_values(pde, self.domain_cache, run_single_threaded)
        return reports

    def splat(self, pde, radius_clamp, kernel_regularization, robin_coeff_cutoff_for_normal_derivative,
              cutoff_dist_to_absorbing_boundary, cutoff_dist_to_reflecting_boundary, evaluation_points,
              report_progress=None):
        for c in self._boundary_caches() + [self.domain_cache]:
            self.bvc.splat(pde, c, radius_clamp, kernel_regularization, robin_coeff_cutoff_for_normal_derivative,
                           cutoff_dist_to_absorbing_boundary, cutoff_dist_to_reflecting_boundary, evaluation_points,
                           report_progress)

    def estimate_solution_near_boundary(self, pde, walk_settings, cutoff_dist_to_absorbing_boundary,
                                        cutoff_dist_to_reflecting_boundary, n_walks_for_solution_estimates,
                                        evaluation_points, run_single_threaded=False):
        self.bvc.estimate_solution_near_boundary(pde, walk_settings, True, cutoff_dist_to_absorbing_boundary,
                                                 n_walks_for_solution_estimates, evaluation_points)
        self.bvc.estimate_solution_near_boundary(pde, walk_settings, False, cutoff_dist_to_reflecting_boundary,
                                                 n_walks_for_solution_estimates, evaluation_points)

    def get_absorbing_boundary_cache(self, return_boundary_normal_aligned=False):
        return self.absorbing_cache_aligned if return_boundary_normal_aligned else self.absorbing_cache

    def get_reflecting_boundary_cache(self, return_boundary_normal_aligned=False):
        return self.reflecting_cache_aligned if return_boundary_normal_aligned else self.reflecting_cache

    def get_domain_cache(self):
        return self.domain_cache
