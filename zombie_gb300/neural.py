"""Neural-cache solving around the plain walk: online training on the solver's own walk
estimates, a held-out error gate, early walk termination through the cache, and the plain
walk as fallback and judge of the cache's bias.  No counterpart in the reference.

The compute (walks, training, inference) runs in libzgpu.so; this module is the policy:

1. training estimates: walks at `train_spp` from random interior points (plain walks in the
   first round; cached walks in later rounds, whose estimates are less noisy);
2. `cache.train`: Adam on the mean squared error against those estimates;
3. gate: on held-out points the plain walk judges the cached walk: the RMS difference of
   their estimates corrected for both estimates' noise, sqrt(max(0, mean d^2 - mean(se_p^2 +
   se_c^2))), is the error the cache adds to a solve; it must stay below `error_bound`,
   otherwise solves fall back to the plain walk.  (The pointwise error of the cache is the
   wrong measure: its high-frequency part averages out over the first step's sphere.)
4. calibration (before the gate, on other held-out points): the cache's global offset is
   measured against plain walks and removed from its output bias;
5. solve: zgpu_solve_cached when the gate passed, zgpu_solve otherwise.
"""
import time

import numpy as np

from . import problems as P
from .api import NeuralCache, SampleArrays


class NeuralCacheSolver:
    def __init__(self, solver, pde, walk_settings, cache, min_distance=0.05, error_bound=1e-2):
        self.solver = solver                # WalkOnSpheres / WalkOnStars over the problem's queries
        self.pde = pde
        self.settings = walk_settings
        self.cache = cache
        self.min_distance = float(min_distance)
        self.error_bound = float(error_bound)
        self.enabled = False
        self.gate_report = None
        self.history = []

    @property
    def queries(self):
        return self.solver.queries

    def sample_interior(self, n, rng, margin=1e-3):
        """n uniform points of the domain box that lie inside the domain, at least `margin`
        from the absorbing boundary, with their distances."""
        q = self.queries
        lo = np.asarray(q.domain_min, np.float64)[:q.dim]
        hi = np.asarray(q.domain_max, np.float64)[:q.dim]
        pts, dist = [], []
        have = 0
        while have < n:
            x = rng.uniform(lo, hi, (max(2 * (n - have), 1024), q.dim)).astype(np.float32)
            x = x[q.inside_domain(x)]
            d = q.compute_dist_to_absorbing_boundary(x)
            keep = d > margin
            pts.append(x[keep]); dist.append(d[keep])
            have += int(keep.sum())
        return np.concatenate(pts)[:n], np.concatenate(dist)[:n]

    def _arrays(self, x, dist, spp, seed_base):
        n = x.shape[0]
        seeds = P.seeds_for(n, base=seed_base)
        return SampleArrays.host(x, dist, np.full(n, spp, np.int32), seeds)

    def estimate(self, x, dist, spp, seed_base, use_cache):
        arr = self._arrays(x, dist, spp, seed_base)
        rep = self.solver.solve_arrays(self.pde, self.settings, arr, cache=self.cache if use_cache else None,
                                       cache_min_distance=self.min_distance)
        n = arr["n_solution_estimates"].astype(np.float64)
        mean = arr["solution_mean"]
        var = arr["solution_m2"] / np.maximum(n - 1, 1)
        return mean, np.sqrt(var / np.maximum(n, 1)), rep

    def train(self, x, dist, spp, steps, batch_size=1 << 16, rounds=1, seed_base=1 << 40, cached=False):
        """`rounds` of (estimate on x at spp, then `steps` Adam steps).  With cached=True the
        estimates come from cached walks (self-training: shorter walks, less noisy targets
        whose bias the next fit shrinks, as the walk's throughput damps the cache's error)."""
        for r in range(rounds):
            t0 = time.perf_counter()
            y, se, rep = self.estimate(x, dist, spp, seed_base + r * (1 << 32), use_cache=cached)
            t1 = time.perf_counter()
            loss = self.cache.train(x, y.astype(np.float32), steps, batch_size)
            t2 = time.perf_counter()
            self.history.append(dict(round=r, estimate_s=t1 - t0, train_s=t2 - t1, loss=loss,
                                     target_se=float(np.sqrt(np.mean(se ** 2))), steps=rep.total_steps))
        return self.history[-1]

    def gate(self, x, dist, spp, seed_base=1 << 50):
        """Held-out check: plain and cached estimates at x decide whether the cache may end
        walks (the error it adds to a solve, corrected for the estimates' noise, against
        error_bound); also reports the cache's own pointwise error and the mean difference."""
        yp, sp, _ = self.estimate(x, dist, spp, seed_base, use_cache=False)
        yc, sc, _ = self.estimate(x, dist, spp, seed_base + 1, use_cache=True)
        d = yc - yp
        noise = float(np.mean(sp ** 2 + sc ** 2))
        err = float(np.sqrt(max(0.0, float(np.mean(d ** 2)) - noise)))
        c = self.cache.evaluate(x).astype(np.float64)
        pointwise = float(np.sqrt(max(0.0, float(np.mean((c - yp) ** 2)) - float(np.mean(sp ** 2)))))
        mean_se = float(np.sqrt(noise / len(d)))
        self.enabled = err <= self.error_bound
        self.gate_report = dict(solve_error=err, mean_difference=float(np.mean(d)), mean_difference_se=mean_se,
                                cache_pointwise_error=pointwise, bound=self.error_bound, enabled=self.enabled)
        return self.gate_report

    def calibrate(self, x, dist, spp, seed_base=1 << 54):
        """Removes the cache's global offset, which dominates the error it adds to a solve: the
        plain walk measures the mean difference d of cached and plain estimates at x; the same
        cached walks (same seeds, so the same termination points) rerun with the output bias
        raised by 1 measure the mean throughput tau at termination; the output bias then
        drops by d / tau.  Returns (d, tau)."""
        yp, _, _ = self.estimate(x, dist, spp, seed_base, use_cache=False)
        yc, _, _ = self.estimate(x, dist, spp, seed_base + 1, use_cache=True)
        p = self.cache.get_parameters()
        b3 = self.cache.split(p)["b3"]
        b3 += 1.0
        self.cache.set_parameters(p)
        yc1, _, _ = self.estimate(x, dist, spp, seed_base + 1, use_cache=True)
        tau = float(np.mean(yc1 - yc))
        d = float(np.mean(yc - yp))
        b3 -= 1.0 + (d / tau if tau > 1e-6 else 0.0)
        self.cache.set_parameters(p)
        return d, tau

    def solve_arrays(self, arrays):
        return self.solver.solve_arrays(self.pde, self.settings, arrays, cache=self.cache if self.enabled else None,
                                        cache_min_distance=self.min_distance)

    def judge_bias(self, x, dist, spp, seed_base=1 << 52):
        """Plain against cached estimates at the same points: the mean difference and its
        standard error (z = mean / se; |z| large means the cache biases the solve)."""
        yp, sp, _ = self.estimate(x, dist, spp, seed_base, use_cache=False)
        yc, sc, _ = self.estimate(x, dist, spp, seed_base + 1, use_cache=True)
        d = yc - yp
        se = float(np.sqrt(np.mean(sp ** 2 + sc ** 2) / len(d)))
        return dict(mean_difference=float(np.mean(d)), se=se, z=float(np.mean(d) / max(se, 1e-300)),
                    rms_difference=float(np.sqrt(np.mean(d ** 2))))


def make_cache(queries, dim, **kw):
    """A NeuralCache over the queries' domain box."""
    return NeuralCache(dim, np.asarray(queries.domain_min)[:dim], np.asarray(queries.domain_max)[:dim], **kw)
