"""Reverse Walk on Stars (point_estimation/reverse_walk_on_stars.h, variance_reduction/
reverse_walk_solver.h) over the GPU engine.

Walks start at sample points (absorbing-boundary samples offset into the domain, reflecting
boundary samples, domain samples) and, at every step, splat the sample's contribution onto
every evaluation point inside the walk's star-shaped ball.  The walks and their splats run in
one CUDA kernel (zgpu_rws_solve: a BVH over the evaluation points for the per-step radius
searches, FP64 atomic sums); sample generation reuses the boundary value caching samplers and
the samples' contributions come from the device field evaluation (zgpu_pde_evaluate).
"""
import ctypes as C

import numpy as np

from . import _abi as A
from ._lib import check, lib
from .api import SampleType, SolveReport, default_context, pde_evaluate
from .bvc import SampleCache


class EvaluationPoints:
    """rws::EvaluationPoint (reverse_walk_solver.h:19-45) for many points: running sums of the
    absorbing, absorbing normal-aligned, reflecting, reflecting normal-aligned and source
    contributions and of the Poisson-kernel weights (self-normalisation)."""

    def __init__(self, pt, normal=None, type=None, dist_to_absorbing=None, dist_to_reflecting=None, dim=None):
        pt = np.asarray(pt, np.float32)
        self.dim = dim or pt.shape[-1]
        n = pt.reshape(-1, self.dim).shape[0]
        self.pt = np.ascontiguousarray(pt.reshape(n, self.dim))
        self.normal = np.zeros((n, self.dim), np.float32) if normal is None else \
            np.ascontiguousarray(normal, np.float32).reshape(n, self.dim)
        self.type = np.full(n, int(SampleType.InDomain), np.int32) if type is None else \
            np.ascontiguousarray(np.broadcast_to(np.asarray(type, np.int32), (n,)))
        self.dist_to_absorbing = None if dist_to_absorbing is None else np.asarray(dist_to_absorbing, np.float32)
        self.dist_to_reflecting = None if dist_to_reflecting is None else np.asarray(dist_to_reflecting, np.float32)
        self.reset()

    def __len__(self):
        return self.pt.shape[0]

    def reset(self):
        self.totals = np.zeros((len(self), A.ZGPU_RWS_TOTALS))

    def get_estimated_solution(self, n_absorbing, n_absorbing_aligned, n_reflecting, n_reflecting_aligned, n_source):
        """EvaluationPoint::getEstimatedSolution (reverse_walk_solver.h:129-166) for every point."""
        t = self.totals
        sol = np.zeros(len(self))
        if n_absorbing > 0:
            pk = t[:, A.ZGPU_RWS_POISSON_KERNEL]
            sol += np.where(pk > 0, t[:, A.ZGPU_RWS_ABSORBING] / np.where(pk > 0, pk, 1.0),
                            t[:, A.ZGPU_RWS_ABSORBING] / n_absorbing)
        if n_absorbing_aligned > 0:
            sol += t[:, A.ZGPU_RWS_ABSORBING_ALIGNED] / n_absorbing_aligned
        if n_reflecting > 0:
            sol += t[:, A.ZGPU_RWS_REFLECTING] / n_reflecting
        if n_reflecting_aligned > 0:
            sol += t[:, A.ZGPU_RWS_REFLECTING_ALIGNED] / n_reflecting_aligned
        if n_source > 0:
            sol += t[:, A.ZGPU_RWS_SOURCE] / n_source
        on_abs = self.type == int(SampleType.OnAbsorbingBoundary)
        sol[on_abs] = t[on_abs, A.ZGPU_RWS_ABSORBING]
        return sol

    def to_c(self):
        e = A.RwsEvalPointsC()
        e.n = len(self)
        for name in ("pt", "normal", "type", "totals"):
            setattr(e, name, A.ptr(getattr(self, name)))
        return e


class EvaluationPoint:
    """One rws::EvaluationPoint (reverse_walk_solver.h:19-45, :120-178): its running sums
    (total_absorbing_boundary_contribution, ..., total_poisson_kernel_contribution) and
    get_estimated_solution(n_absorbing, n_absorbing_aligned, n_reflecting, n_reflecting_aligned,
    n_source).  Lists of these go through ReverseWalkOnStarsSolver.solve like EvaluationPoints."""

    _TOTALS = {"total_absorbing_boundary_contribution": A.ZGPU_RWS_ABSORBING,
               "total_absorbing_boundary_normal_aligned_contribution": A.ZGPU_RWS_ABSORBING_ALIGNED,
               "total_reflecting_boundary_contribution": A.ZGPU_RWS_REFLECTING,
               "total_reflecting_boundary_normal_aligned_contribution": A.ZGPU_RWS_REFLECTING_ALIGNED,
               "total_source_contribution": A.ZGPU_RWS_SOURCE,
               "total_poisson_kernel_contribution": A.ZGPU_RWS_POISSON_KERNEL}

    def __init__(self, pt, normal, type, dist_to_absorbing_boundary, dist_to_reflecting_boundary):
        self._pts = EvaluationPoints(np.asarray(pt, np.float32)[None], np.asarray(normal, np.float32)[None],
                                     [int(type)], [dist_to_absorbing_boundary], [dist_to_reflecting_boundary])
        self.pt, self.normal, self.type = self._pts.pt[0], self._pts.normal[0], SampleType(int(type))
        self.dist_to_absorbing_boundary = float(dist_to_absorbing_boundary)
        self.dist_to_reflecting_boundary = float(dist_to_reflecting_boundary)

    def __getattr__(self, name):
        if name in EvaluationPoint._TOTALS:
            return float(self._pts.totals[0, EvaluationPoint._TOTALS[name]])
        raise AttributeError(name)

    def get_estimated_solution(self, n_absorbing, n_absorbing_aligned, n_reflecting, n_reflecting_aligned, n_source):
        return float(self._pts.get_estimated_solution(n_absorbing, n_absorbing_aligned, n_reflecting,
                                                      n_reflecting_aligned, n_source)[0])

    def reset(self):
        self._pts.reset()


def _gather(points):
    ev = EvaluationPoints(np.array([p.pt for p in points]), np.array([p.normal for p in points]),
                          [int(p.type) for p in points], [p.dist_to_absorbing_boundary for p in points],
                          [p.dist_to_reflecting_boundary for p in points], dim=points[0].pt.shape[0])
    ev.totals[:] = np.concatenate([p._pts.totals for p in points])
    return ev


class ReverseWalkOnStarsSolver:
    """ReverseWalkOnStarsSolver<T,DIM> (reverse_walk_solver.h:47-118, :168-372)."""

    def __init__(self, queries, absorbing_boundary_sampler, reflecting_boundary_sampler, domain_sampler, context=None):
        self.queries = queries
        self.dim = queries.dim
        self.absorbing_sampler = absorbing_boundary_sampler
        self.reflecting_sampler = reflecting_boundary_sampler
        self.domain_sampler = domain_sampler
        self.ctx = context or default_context()
        e = SampleCache.empty
        self.absorbing, self.absorbing_aligned = e(self.dim), e(self.dim)
        self.reflecting, self.reflecting_aligned = e(self.dim), e(self.dim)
        self.domain = e(self.dim)
        self.calls = 0
        self.last_reports = []

    def generate_samples(self, absorbing_boundary_sample_count, reflecting_boundary_sample_count, domain_sample_count,
                         normal_offset_for_absorbing_boundary, solve_double_sided):
        """generateSamples (reverse_walk_solver.h:188-213): absorbing samples offset into the
        domain, reflecting samples on the boundary."""
        def gen(sampler, count, stype, offset, aligned):
            if sampler is None or count <= 0:
                return SampleCache.empty(self.dim)
            return sampler.generate_samples(sampler.get_sample_count(count, aligned), stype, offset, self.queries, aligned)
        AB, RB = int(SampleType.OnAbsorbingBoundary), int(SampleType.OnReflectingBoundary)
        self.absorbing = gen(self.absorbing_sampler, absorbing_boundary_sample_count, AB,
                             normal_offset_for_absorbing_boundary, False)
        self.absorbing_aligned = gen(self.absorbing_sampler, absorbing_boundary_sample_count, AB,
                                     normal_offset_for_absorbing_boundary, True) if solve_double_sided \
            else SampleCache.empty(self.dim)
        self.reflecting = gen(self.reflecting_sampler, reflecting_boundary_sample_count, RB, 0.0, False)
        self.reflecting_aligned = gen(self.reflecting_sampler, reflecting_boundary_sample_count, RB, 0.0, True) \
            if solve_double_sided else SampleCache.empty(self.dim)
        self.domain = self.domain_sampler.generate_samples(domain_sample_count, self.queries) \
            if self.domain_sampler is not None and domain_sample_count > 0 else SampleCache.empty(self.dim)

    def _contributions(self, pde, ws, cache):
        """ReverseWalkOnStars::solve's contribution of each sample (reverse_walk_on_stars.h:95-120);
        returns the mask of samples that walk."""
        n = len(cache)
        walk = np.zeros(n, bool)
        if n == 0:
            return walk
        ds = bool(ws.solve_double_sided)
        t = cache.type
        src = (t == int(SampleType.InDomain)) & (not ws.ignore_source_contribution)
        if np.any(src):
            cache.contribution[src] = pde_evaluate(pde, cache.pt[src], dim=self.dim, context=self.ctx)[0]
        ab = (t == int(SampleType.OnAbsorbingBoundary)) & (not ws.ignore_absorbing_boundary_contribution)
        if np.any(ab):
            x = cache.pt[ab]
            sd = self.queries.compute_dist_to_absorbing_boundary(x, compute_signed_distance=True).astype(np.float32)
            proj = x - sd[:, None] * cache.normal[ab]
            cache.contribution[ab] = pde_evaluate(pde, proj, None, (ds & (sd > 0)).astype(np.int32), dim=self.dim,
                                                  context=self.ctx)[1]
        rf = (t == int(SampleType.OnReflectingBoundary)) & (not ws.ignore_reflecting_boundary_contribution)
        if np.any(rf):
            al = (ds & (cache.estimate_normal_aligned != 0)).astype(np.int32)
            cache.contribution[rf] = pde_evaluate(pde, cache.pt[rf], cache.normal[rf], al[rf], dim=self.dim,
                                                  context=self.ctx)[2]
        return src | ab | rf

    def solve(self, pde, walk_settings, normal_offset_for_absorbing_boundary, radius_clamp, kernel_regularization,
              evaluation_points, updated_eval_pt_locations=True, run_single_threaded=False, report_progress=None):
        """solve (reverse_walk_solver.h:304-338): one reverse walk per sample, progressive over
        calls (call k draws pcg32 stream k of every sample).  evaluation_points: EvaluationPoints
        or a list of EvaluationPoint."""
        listed = isinstance(evaluation_points, (list, tuple))
        if listed and len(evaluation_points) == 0:
            self.calls += 1
            return
        ev = _gather(evaluation_points) if listed else evaluation_points
        p = pde.to_c()
        ws = walk_settings.to_c() if hasattr(walk_settings, "to_c") else walk_settings
        q = self.queries.to_c()
        self.last_reports = []
        for cache in (self.absorbing, self.absorbing_aligned, self.reflecting, self.reflecting_aligned, self.domain):
            mask = self._contributions(pde, walk_settings, cache)
            if not np.any(mask) or len(ev) == 0:
                continue
            idx = np.nonzero(mask)[0]
            arrays = {k: np.ascontiguousarray(getattr(cache, k)[idx]) for k in
                      ("pt", "normal", "type", "estimate_normal_aligned", "pdf", "contribution", "dist_to_absorbing",
                       "seed")}
            s = A.RwsSamplesC()
            s.n = idx.size
            for k, v in arrays.items():
                setattr(s, k, A.ptr(v))
            e = ev.to_c()
            rep = A.SolveReport()
            check(lib().zgpu_rws_solve(self.ctx.h, C.byref(q), C.byref(p), C.byref(ws), C.byref(s),
                                       float(normal_offset_for_absorbing_boundary), float(radius_clamp),
                                       float(kernel_regularization), int(self.calls), C.byref(e), A.ZGPU_MEM_HOST,
                                       C.byref(rep)))
            self.last_reports.append(SolveReport(rep))
            if report_progress is not None:
                report_progress(int(idx.size), 0)
        self.calls += 1
        # evaluation points on the absorbing boundary take the boundary value
        on_abs = ev.type == int(SampleType.OnAbsorbingBoundary)
        if np.any(on_abs):
            g = np.zeros(int(on_abs.sum()), np.float32)
            if not walk_settings.ignore_absorbing_boundary_contribution:
                g = pde_evaluate(pde, ev.pt[on_abs], dim=self.dim, context=self.ctx)[1]
            ev.totals[on_abs, A.ZGPU_RWS_ABSORBING] = g
        if listed:
            for i, p in enumerate(evaluation_points):
                p._pts.totals[0] = ev.totals[i]

    def get_absorbing_boundary_sample_pts(self, return_boundary_normal_aligned=False):
        return self.absorbing_aligned if return_boundary_normal_aligned else self.absorbing

    def get_reflecting_boundary_sample_pts(self, return_boundary_normal_aligned=False):
        return self.reflecting_aligned if return_boundary_normal_aligned else self.reflecting

    def get_domain_sample_pts(self):
        return self.domain

    def get_absorbing_boundary_sample_count(self, return_boundary_normal_aligned=False):
        return len(self.get_absorbing_boundary_sample_pts(return_boundary_normal_aligned))

    def get_reflecting_boundary_sample_count(self, return_boundary_normal_aligned=False):
        return len(self.get_reflecting_boundary_sample_pts(return_boundary_normal_aligned))

    def get_domain_sample_count(self):
        return len(self.domain)

    def get_estimated_solution(self, evaluation_points):
        """The evaluation points' solution with this solver's sample counts times the number of
        solve calls whose walks the points accumulated."""
        k = max(self.calls, 1)
        if isinstance(evaluation_points, (list, tuple)):
            n = (k * self.get_absorbing_boundary_sample_count(), k * self.get_absorbing_boundary_sample_count(True),
                 k * self.get_reflecting_boundary_sample_count(), k * self.get_reflecting_boundary_sample_count(True),
                 k * self.get_domain_sample_count())
            return [p.get_estimated_solution(*n) for p in evaluation_points]
        return evaluation_points.get_estimated_solution(
            k * self.get_absorbing_boundary_sample_count(), k * self.get_absorbing_boundary_sample_count(True),
            k * self.get_reflecting_boundary_sample_count(), k * self.get_reflecting_boundary_sample_count(True),
            k * self.get_domain_sample_count())
