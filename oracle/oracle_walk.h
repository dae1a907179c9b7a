// oracle_walk.h -- TEST INFRASTRUCTURE, NOT PRODUCT CODE (see oracle_core.h).
//
// CPU restatement of WalkOnSpheres (point_estimation/walk_on_spheres.h) and WalkOnStars
// (point_estimation/walk_on_stars.h) over the oracle's geometric queries
// (core/geometric_queries.h semantics) and the device-evaluable PDE descriptor.
// Deviation kept identical on the GPU: walk w of point i draws from
// pcg32(seed_i, stream = w + n_prev_i) instead of one sequential generator per point
// (common.h:182), so walks are independent of scheduling.
#pragma once

#include "oracle_geometry.h"

namespace orc {

// ---------------------------------------------------------------------------------------
// PDE fields (replaces the std::function members of core/pde.h:19-45)
template <int D>
struct AnalyticEval {
    float u, lap; Vec<D> grad;
};
template <int D>
inline AnalyticEval<D> evalAnalytic(const zgpu_analytic& a, const Vec<D>& x) {
    AnalyticEval<D> r; r.u = a.d; r.lap = 0.0f;
    for (int i = 0; i < D; i++) {
        r.u += a.q[i] * x[i] * x[i] + a.l[i] * x[i];
        r.grad[i] = 2.0f * a.q[i] * x[i] + a.l[i];
        r.lap += 2.0f * a.q[i];
    }
    for (int k = 0; k < a.n_terms && k < ZGPU_MAX_TERMS; k++) {
        float ax = 0.0f, bx = a.phi[k], aa = 0.0f, bb = 0.0f, ab = 0.0f;
        for (int i = 0; i < D; i++) {
            ax += a.a[k][i] * x[i]; bx += a.b[k][i] * x[i];
            aa += a.a[k][i] * a.a[k][i]; bb += a.b[k][i] * a.b[k][i]; ab += a.a[k][i] * a.b[k][i];
        }
        float E = std::exp(ax), C = std::cos(bx), S = std::sin(bx);
        r.u += a.c[k] * E * C;
        for (int i = 0; i < D; i++) r.grad[i] += a.c[k] * E * (a.a[k][i] * C - a.b[k][i] * S);
        r.lap += a.c[k] * E * ((aa - bb) * C - 2.0f * ab * S);
    }
    return r;
}

// DenseGrid<float, 1, DIM>::operator() (utils/dense_grid.h:264-355): cell-centred samples over
// [grid_min, grid_max], row-major with the last axis fastest; nearest cell, or multilinear
// between the cell centres with indices clamped to the grid and fractions to [0, 1].  The
// normal-aligned grid (getDenseGridCallback2/4) answers aligned lookups when given.
template <int D>
inline float gridValue(const zgpu_grid& g, const Vec<D>& x, bool aligned) {
    const float* v = (aligned && g.values_aligned) ? g.values_aligned : g.values;
    int i0[D], i1[D];
    float f[D];
    for (int i = 0; i < D; i++) {
        int n = g.shape[i];
        float t = (x[i] - g.grid_min[i]) / (g.grid_max[i] - g.grid_min[i]);
        if (g.enable_interpolation) {
            float u = n == 1 ? 0.0f : t * (float)n - 0.5f;
            i0[i] = std::clamp((int)std::floor(u), 0, n - 1);
            i1[i] = std::clamp(i0[i] + 1, 0, n - 1);
            f[i] = std::clamp(u - (float)i0[i], 0.0f, 1.0f);
        } else {
            i0[i] = i1[i] = std::clamp((int)std::floor(t * (float)n), 0, n - 1);
            f[i] = 0.0f;
        }
    }
    if (!g.enable_interpolation) {
        int64_t k = 0;
        for (int i = 0; i < D; i++) k = k * g.shape[i] + i0[i];
        return v[k];
    }
    float r = 0.0f;
    for (int corner = 0; corner < (1 << D); corner++) {
        int64_t k = 0;
        float w = 1.0f;
        for (int i = 0; i < D; i++) {
            bool hi = (corner >> i) & 1;
            k = k * g.shape[i] + (hi ? i1[i] : i0[i]);
            w *= hi ? f[i] : 1.0f - f[i];
        }
        r += w * v[k];
    }
    return r;
}

template <int D>
struct Pde {
    const zgpu_pde* p;
    float robinCoeff(const Vec<D>& x, const Vec<D>&, bool aligned) const {
        if (p->robin_coeff_kind == ZGPU_FIELD_ZERO) return 0.0f;
        if (p->robin_coeff_kind == ZGPU_FIELD_GRID) return gridValue<D>(p->robin_coeff_grid, x, aligned);
        return aligned ? p->robin_coeff_value_aligned : p->robin_coeff_value;
    }
    float source(const Vec<D>& x) const {
        if (p->source_kind == ZGPU_FIELD_CONSTANT) return p->source_value;
        if (p->source_kind == ZGPU_FIELD_ANALYTIC) {
            AnalyticEval<D> e = evalAnalytic<D>(p->solution, x);
            return -e.lap + p->absorption_coeff * e.u;
        }
        if (p->source_kind == ZGPU_FIELD_GRID) return gridValue<D>(p->source_grid, x, false);
        return 0.0f;
    }
    float dirichlet(const Vec<D>& x, bool aligned) const {
        if (p->dirichlet_kind == ZGPU_FIELD_CONSTANT) return aligned ? p->dirichlet_value_aligned : p->dirichlet_value;
        if (p->dirichlet_kind == ZGPU_FIELD_ANALYTIC) return evalAnalytic<D>(p->solution, x).u;
        if (p->dirichlet_kind == ZGPU_FIELD_GRID) return gridValue<D>(p->dirichlet_grid, x, aligned);
        return 0.0f;
    }
    // Robin data h = du/dn + kappa u with n the outward normal (Walkin' Robin, Miller et al. 2024)
    float robin(const Vec<D>& x, const Vec<D>& n, bool aligned) const {
        if (p->robin_kind == ZGPU_FIELD_CONSTANT) return aligned ? p->robin_value_aligned : p->robin_value;
        if (p->robin_kind == ZGPU_FIELD_ANALYTIC) {
            AnalyticEval<D> e = evalAnalytic<D>(p->solution, x);
            float s = aligned ? -1.0f : 1.0f;
            return s * dot(e.grad, n) + robinCoeff(x, n, aligned) * e.u;
        }
        if (p->robin_kind == ZGPU_FIELD_GRID) return gridValue<D>(p->robin_grid, x, aligned);
        return 0.0f;
    }
    // pde.h:62-78
    bool hasNonZeroRobinCoeff(const Vec<D>& x) const {
        if (p->are_robin_conditions_pure_neumann) return false;
        Vec<D> n; n[0] = 1.0f;
        return std::fabs(robinCoeff(x, n, true)) > 0.0f || std::fabs(robinCoeff(x, n, false)) > 0.0f;
    }
};

// ---------------------------------------------------------------------------------------
// GeometricQueries<DIM> populated from the two boundaries (core/geometric_queries.h:58-124,
// defaults :210-390, FCPW lambdas utils/fcpw_geometric_queries.h:1062-1291)
template <int D>
struct Queries {
    const Boundary<D>* absorbing = nullptr;
    const Boundary<D>* reflecting = nullptr;
    Vec<D> domainMin, domainMax;
    bool hasNonEmptyReflectingBoundary() const { return reflecting && reflecting->nPrims() > 0; }
    bool hasNonEmptyAbsorbingBoundary() const { return absorbing && absorbing->nPrims() > 0; }

    float computeDistToAbsorbingBoundary(const Vec<D>& x) const {
        if (hasNonEmptyAbsorbingBoundary()) {
            Vec<D> pt, n; float d; int pi;
            absorbing->closestPoint(x, pt, n, d, pi);
            return d;
        }
        // geometric_queries.h:212-217
        Vec<D> u = domainMin - x, v = x - domainMax, m;
        for (int i = 0; i < D; i++) m[i] = std::min(u[i], v[i]);
        return norm(m);
    }
    bool projectToAbsorbingBoundary(Vec<D>& x, Vec<D>& normal, float& distance, bool computeSigned) const {
        if (!hasNonEmptyAbsorbingBoundary()) { distance = 0.0f; return false; }
        Vec<D> pt, n; float d; int pi;
        if (!absorbing->closestPoint(x, pt, n, d, pi)) { normal = Vec<D>(); distance = kMaxFloat; return false; }
        float sd = d;
        if (computeSigned) sd = dot(x - pt, n) >= 0.0f ? d : -d;
        x = pt; normal = n; distance = sd;
        return true;
    }
    bool intersectReflectingBoundary(const Vec<D>& origin, const Vec<D>& normal, const Vec<D>& dir, float tMax,
                                     bool onReflectingBoundary, Vec<D>& pt, Vec<D>& n, float& dist) const {
        if (!hasNonEmptyReflectingBoundary()) return false;
        Vec<D> o = onReflectingBoundary ? offsetPointAlongDirection<D>(origin, -normal) : origin;
        float t; int pi;
        if (!reflecting->intersect(o, dir, tMax, pt, n, t, pi)) return false;
        dist = t;
        return true;
    }
    bool intersectsWithReflectingBoundary(const Vec<D>& xi, const Vec<D>& xj, const Vec<D>& ni, const Vec<D>& nj,
                                          bool offseti, bool offsetj) const {
        if (!hasNonEmptyReflectingBoundary()) return false;
        Vec<D> p1 = offseti ? offsetPointAlongDirection<D>(xi, -ni) : xi;
        Vec<D> p2 = offsetj ? offsetPointAlongDirection<D>(xj, -nj) : xj;
        return reflecting->occluded(p1, p2);
    }
    bool sampleReflectingBoundary(const Vec<D>& x, float radius, const float* u, Vec<D>& pt, Vec<D>& n, float& pdf) const {
        if (!hasNonEmptyReflectingBoundary()) return false;
        return reflecting->sample(x, radius, u, pt, n, pdf);
    }
    float computeStarRadiusForReflectingBoundary(const Vec<D>& x, float minR, float maxR, float precision, bool flip) const {
        if (!hasNonEmptyReflectingBoundary()) return maxR;
        return reflecting->starRadius(x, minR, maxR, precision, flip);
    }
    bool outsideBoundingDomain(const Vec<D>& x) const {
        for (int i = 0; i < D; i++) if (x[i] < domainMin[i] || x[i] > domainMax[i]) return true;
        return false;
    }
};

enum class Code { ReachedAbsorbingBoundary, TerminatedWithRussianRoulette, ExceededMaxWalkLength, EscapedDomain };

// WalkState (common.h:93-130)
template <int D>
struct WalkState {
    float totalReflectingBoundaryContribution = 0.0f, totalSourceContribution = 0.0f;
    Vec<D> currentPt, currentNormal, prevDirection;
    float prevDistance = 0.0f, throughput = 1.0f;
    int walkLength = 0;
    bool onReflectingBoundary = false;
    WalkState() {}
    WalkState(const Vec<D>& p, const Vec<D>& n, const Vec<D>& d, float pd, float tp, int wl, bool onR)
        : currentPt(p), currentNormal(n), prevDirection(d), prevDistance(pd), throughput(tp), walkLength(wl),
          onReflectingBoundary(onR) {}
};

// per-point result of one solve (merged into the caller's statistics)
struct PointStats {
    double mean = 0.0, m2 = 0.0;
    int n = 0;
    int64_t walkLength = 0, splits = 0;
    uint64_t steps = 0;
    void add(double x) { n += 1; double d = x - mean; mean += d / n; double d2 = x - mean; m2 += d * d2; }
};

struct GradStats {
    double mean[3] = {0, 0, 0}, m2[3] = {0, 0, 0};
    int n = 0;
    double firstSource = 0.0, derivative = 0.0;   // addFirstSource/DerivativeContribution sums
    void add(const double* x, int D) {
        n += 1;
        for (int i = 0; i < D; i++) { double d = x[i] - mean[i]; mean[i] += d / n; m2[i] += d * (x[i] - mean[i]); }
    }
};

template <int D>
struct Solver {
    const Queries<D>& q;
    Pde<D> pde;
    const zgpu_walk_settings& ws;

    std::unique_ptr<GreensFnBall<D>> makeGreens(bool yukawa) const {
        if (yukawa) return std::unique_ptr<GreensFnBall<D>>(new YukawaGreensFnBall<D>(pde.p->absorption_coeff));
        return std::unique_ptr<GreensFnBall<D>>(new HarmonicGreensFnBall<D>());
    }

    // walk_on_spheres.h:193-226 / walk_on_stars.h:309-343
    bool applyWeightWindow(Pcg32& rng, WalkState<D>& s, std::queue<WalkState<D>>& queue) const {
        if (s.throughput > ws.splitting_threshold) {
            float left = s.throughput - ws.splitting_threshold;
            s.throughput = ws.splitting_threshold;
            WalkState<D> split(s.currentPt, s.currentNormal, s.prevDirection, s.prevDistance, s.throughput, 0,
                               s.onReflectingBoundary);
            while (left > ws.splitting_threshold) { left -= ws.splitting_threshold; queue.push(split); }
            if (rng.nextFloat() < left / ws.splitting_threshold) queue.push(split);
        } else if (s.throughput < ws.russian_roulette_threshold) {
            float survival = s.throughput / ws.russian_roulette_threshold;
            if (survival < rng.nextFloat()) { s.throughput = 0.0f; return true; }
            s.throughput = ws.russian_roulette_threshold;
        }
        return false;
    }

    // ------------------------------- Walk on Spheres ---------------------------------
    // walk_on_spheres.h:229-291
    Code wosWalk(float dist, std::unique_ptr<GreensFnBall<D>>& g, Pcg32& rng, WalkState<D>& s,
                 std::queue<WalkState<D>>& queue, uint64_t& steps) const {
        while (dist > ws.epsilon_shell_for_absorbing_boundary) {
            steps++;
            g->updateBall(s.currentPt, dist);
            if (!ws.ignore_source_contribution) {  // :171-190
                float src;
                if (pde.p->is_source_constant) {
                    src = g->norm() * pde.source(s.currentPt);
                } else {
                    float r, pdf;
                    Vec<D> y = g->sampleVolume(rng, r, pdf);
                    src = g->norm() * pde.source(y);
                }
                s.totalSourceContribution += s.throughput * src;
            }
            Vec<D> dir = sampleUnitSphereUniform<D>(rng);
            s.currentPt = s.currentPt + dist * dir;
            s.throughput *= g->directionSampledPoissonKernel(s.currentPt);
            if (q.outsideBoundingDomain(s.currentPt)) return Code::EscapedDomain;
            if (applyWeightWindow(rng, s, queue)) return Code::TerminatedWithRussianRoulette;
            s.walkLength++;
            if (s.walkLength >= ws.max_walk_length) return Code::ExceededMaxWalkLength;
            if (pde.p->absorption_coeff > 0.0f && ws.steps_before_applying_tikhonov == s.walkLength) g = makeGreens(true);
            dist = q.computeDistToAbsorbingBoundary(s.currentPt);
        }
        return Code::ReachedAbsorbingBoundary;
    }

    // walk_on_spheres.h:294-318
    float wosTerminal(Code code, WalkState<D>& s) const {
        if ((code == Code::ReachedAbsorbingBoundary || code == Code::ExceededMaxWalkLength) &&
            !ws.ignore_absorbing_boundary_contribution) {
            float sd;
            q.projectToAbsorbingBoundary(s.currentPt, s.currentNormal, sd, ws.solve_double_sided);
            bool aligned = ws.solve_double_sided && sd > 0.0f;
            return pde.dirichlet(s.currentPt, aligned);
        }
        return 0.0f;
    }

    // walk_on_spheres.h:321-414 (rng per walk; see file header)
    void wosEstimate(const Vec<D>& pt, int type, float distAbs, int nWalks, uint64_t seed, bool hasPrev,
                     bool normalAligned, float& firstSphereRadius, PointStats& st) const {
        if (type == ZGPU_SAMPLE_ON_ABSORBING_BOUNDARY) {
            if (!hasPrev) {
                float c = 0.0f;
                if (!ws.ignore_absorbing_boundary_contribution)
                    c = pde.dirichlet(pt, ws.solve_double_sided && normalAligned);
                st.add(c);
                firstSphereRadius = 0.0f;
            }
            return;
        } else if (distAbs <= ws.epsilon_shell_for_absorbing_boundary) {
            nWalks = 1;
        }
        if (!hasPrev) firstSphereRadius = distAbs;
        std::queue<WalkState<D>> queue;
        for (int w = 0; w < nWalks; w++) {
            Pcg32 rng(seed, (uint64_t)w + streamBase);
            WalkState<D> s(pt, Vec<D>(), Vec<D>(), 0.0f, 1.0f, 0, false);
            queue.push(s);
            int splits = -1;
            float total = 0.0f;
            bool success = false;
            while (!queue.empty()) {
                s = queue.front(); queue.pop();
                splits++;
                bool yukawa = pde.p->absorption_coeff > 0.0f && ws.steps_before_applying_tikhonov == 0;
                std::unique_ptr<GreensFnBall<D>> g = makeGreens(yukawa);
                float dist = splits == 0 ? distAbs : q.computeDistToAbsorbingBoundary(s.currentPt);
                Code code = wosWalk(dist, g, rng, s, queue, st.steps);
                if (code != Code::EscapedDomain) {
                    float term = wosTerminal(code, s);
                    total += s.throughput * term + s.totalSourceContribution;
                    st.walkLength += s.walkLength;
                    success = true;
                }
            }
            if (success) { st.add((double)total); st.splits += splits; }
        }
    }

    // ------------------------------- Walk on Stars -----------------------------------
    // walk_on_stars.h:190-250
    void reflectingContribution(const GreensFnBall<D>& g, float starRadius, bool flip, Pcg32& rng, WalkState<D>& s) const {
        if (q.hasNonEmptyReflectingBoundary() && !ws.ignore_reflecting_boundary_contribution) {
            float u[D];
            for (int i = 0; i < D; i++) u[i] = rng.nextFloat();
            Vec<D> bpt, bn; float pdf;
            if (q.sampleReflectingBoundary(s.currentPt, starRadius, u, bpt, bn, pdf)) {
                Vec<D> toSample = bpt - s.currentPt;
                float distToSample = norm(toSample);
                float alpha = s.onReflectingBoundary ? 2.0f : 1.0f;
                bool aligned = false;
                if (ws.solve_double_sided) {
                    toSample = toSample / distToSample;
                    if (flip) {
                        aligned = true;
                    } else if (dot(toSample, bn) < -ws.silhouette_precision) {
                        bool flipSample = true;
                        if (alpha > 1.0f) flipSample = dot(toSample, s.currentNormal) < -ws.silhouette_precision;
                        if (flipSample) aligned = true;
                    }
                }
                Vec<D> bnA = bn * (aligned ? -1.0f : 1.0f);
                if (pdf > 0.0f && distToSample < starRadius &&
                    !q.intersectsWithReflectingBoundary(s.currentPt, bpt, s.currentNormal, bnA, s.onReflectingBoundary, true)) {
                    float r = std::max(g.rClamp, distToSample);
                    float G = g.evaluate(r);
                    float h = pde.robin(bpt, bn, ws.solve_double_sided && aligned);
                    s.totalReflectingBoundaryContribution += s.throughput * alpha * G * h / pdf;
                }
            }
        }
    }
    // walk_on_stars.h:253-275
    void starSourceContribution(GreensFnBall<D>& g, const Vec<D>& dir, float hitDist, Pcg32& rng, WalkState<D>& s) const {
        if (!ws.ignore_source_contribution) {
            float r, pdf;
            Vec<D> y = g.sampleVolume(dir, rng, r, pdf);
            if (r <= hitDist) s.totalSourceContribution += s.throughput * g.norm() * pde.source(y);
        }
    }
    // walk_on_stars.h:278-307
    float stepThroughput(const GreensFnBall<D>& g, const WalkState<D>& s) const {
        if (s.onReflectingBoundary && s.prevDistance > std::numeric_limits<float>::epsilon()) {
            float kappa = 0.0f;
            Vec<D> n = s.currentNormal;
            if (!pde.p->are_robin_conditions_pure_neumann) {
                bool flip = false;
                if (ws.solve_double_sided) { flip = dot(s.prevDirection, s.currentNormal) < 0.0f; n = n * (flip ? -1.0f : 1.0f); }
                kappa = pde.robinCoeff(s.currentPt, s.currentNormal, ws.solve_double_sided && flip);
            }
            float refl = g.reflectance(s.prevDistance, s.prevDirection, n, kappa);
            float maxRefl = pde.p->are_robin_coeffs_nonnegative ? 1.0f : 2.0f;
            return std::min(std::max(refl, 0.0f), maxRefl);
        }
        return g.directionSampledPoissonKernel(s.currentPt);
    }
    float shrunkStarRadius(const Vec<D>& x, float distAbs, bool flip) const {
        float R = q.computeStarRadiusForReflectingBoundary(x, ws.epsilon_shell_for_reflecting_boundary, distAbs,
                                                          ws.silhouette_precision, flip);
        if (q.hasNonEmptyReflectingBoundary() && ws.epsilon_shell_for_reflecting_boundary <= distAbs)
            R = std::max(0.99f * R, ws.epsilon_shell_for_reflecting_boundary);
        return R;
    }
    // walk_on_stars.h:346-490
    Code wostWalk(float distAbs, float firstSphereRadius, bool flip, std::unique_ptr<GreensFnBall<D>>& g, Pcg32& rng,
                  WalkState<D>& s, std::queue<WalkState<D>>& queue, uint64_t& steps) const {
        bool firstStep = true;
        while (distAbs > ws.epsilon_shell_for_absorbing_boundary) {
            steps++;
            float starRadius;
            if (firstStep && firstSphereRadius > 0.0f) {
                starRadius = firstSphereRadius;
            } else {
                flip = false;
                if (ws.solve_double_sided && s.onReflectingBoundary) {
                    if (s.prevDistance > 0.0f && dot(s.prevDirection, s.currentNormal) < 0.0f) {
                        s.currentNormal = -s.currentNormal; flip = true;
                    }
                }
                if (ws.steps_before_using_maximal_spheres <= s.walkLength) starRadius = distAbs;
                else if (s.onReflectingBoundary && pde.hasNonZeroRobinCoeff(s.currentPt)) starRadius = ws.epsilon_shell_for_reflecting_boundary;
                else starRadius = shrunkStarRadius(s.currentPt, distAbs, flip);
            }
            g->updateBall(s.currentPt, starRadius);
            Vec<D> dir = sampleUnitSphereUniform<D>(rng);
            if (s.onReflectingBoundary && dot(s.currentNormal, dir) > 0.0f) dir = -dir;
            Vec<D> hitPt, hitN; float hitDist = kMaxFloat;
            bool hit = q.intersectReflectingBoundary(s.currentPt, s.currentNormal, dir, starRadius, s.onReflectingBoundary,
                                                     hitPt, hitN, hitDist);
            if (!hit) {
                Vec<D> p0 = s.onReflectingBoundary ? offsetPointAlongDirection<D>(s.currentPt, -s.currentNormal) : s.currentPt;
                hitPt = p0 + starRadius * dir;
                hitDist = starRadius;
                hitN = Vec<D>();
            }
            reflectingContribution(*g, starRadius, flip, rng, s);
            starSourceContribution(*g, dir, hitDist, rng, s);
            s.prevDistance = hitDist;
            s.prevDirection = dir;
            s.currentPt = hitPt;
            s.currentNormal = hitN;
            s.onReflectingBoundary = hit;
            s.throughput *= stepThroughput(*g, s);
            if (!s.onReflectingBoundary && q.outsideBoundingDomain(s.currentPt)) return Code::EscapedDomain;
            if (applyWeightWindow(rng, s, queue)) return Code::TerminatedWithRussianRoulette;
            s.walkLength++;
            if (s.walkLength >= ws.max_walk_length) return Code::ExceededMaxWalkLength;
            if (pde.p->absorption_coeff > 0.0f && ws.steps_before_applying_tikhonov == s.walkLength) g = makeGreens(true);
            distAbs = q.computeDistToAbsorbingBoundary(s.currentPt);
            firstStep = false;
        }
        return Code::ReachedAbsorbingBoundary;
    }
    // walk_on_stars.h:493-516
    float wostTerminal(Code code, WalkState<D>& s) const {
        if (code == Code::ReachedAbsorbingBoundary && !ws.ignore_absorbing_boundary_contribution) {
            float sd;
            q.projectToAbsorbingBoundary(s.currentPt, s.currentNormal, sd, ws.solve_double_sided);
            bool aligned = ws.solve_double_sided && sd > 0.0f;
            return pde.dirichlet(s.currentPt, aligned);
        }
        return 0.0f;
    }
    // walk_on_stars.h:519-662
    void wostEstimate(const Vec<D>& pt, const Vec<D>& normal, int type, float distAbs, int nWalks, uint64_t seed,
                      bool hasPrev, bool normalAligned, float& firstSphereRadius, PointStats& st) const {
        if (type == ZGPU_SAMPLE_ON_ABSORBING_BOUNDARY) {
            if (!hasPrev) {
                float c = 0.0f;
                if (!ws.ignore_absorbing_boundary_contribution)
                    c = pde.dirichlet(pt, ws.solve_double_sided && normalAligned);
                st.add(c);
                firstSphereRadius = 0.0f;
            }
            return;
        } else if (distAbs <= ws.epsilon_shell_for_absorbing_boundary) {
            nWalks = 1;
        }
        Vec<D> currentNormal = normal, prevDirection = normal;
        float prevDistance = kMaxFloat;
        bool flip = false;
        if (ws.solve_double_sided && type == ZGPU_SAMPLE_ON_REFLECTING_BOUNDARY && normalAligned) {
            currentNormal = -currentNormal; prevDirection = -prevDirection; flip = true;
        }
        if (!hasPrev) {
            if (distAbs <= ws.epsilon_shell_for_absorbing_boundary || ws.steps_before_using_maximal_spheres == 0)
                firstSphereRadius = distAbs;
            else if (type == ZGPU_SAMPLE_ON_REFLECTING_BOUNDARY && pde.hasNonZeroRobinCoeff(pt))
                firstSphereRadius = ws.epsilon_shell_for_reflecting_boundary;
            else
                firstSphereRadius = shrunkStarRadius(pt, distAbs, flip);
        }
        std::queue<WalkState<D>> queue;
        for (int w = 0; w < nWalks; w++) {
            Pcg32 rng(seed, (uint64_t)w + streamBase);
            WalkState<D> s(pt, currentNormal, prevDirection, prevDistance, 1.0f, 0, type == ZGPU_SAMPLE_ON_REFLECTING_BOUNDARY);
            queue.push(s);
            int splits = -1;
            float total = 0.0f;
            bool success = false;
            while (!queue.empty()) {
                s = queue.front(); queue.pop();
                splits++;
                bool yukawa = pde.p->absorption_coeff > 0.0f && ws.steps_before_applying_tikhonov == 0;
                std::unique_ptr<GreensFnBall<D>> g = makeGreens(yukawa);
                float dist = distAbs, fsr = firstSphereRadius;
                if (splits > 0) { dist = q.computeDistToAbsorbingBoundary(s.currentPt); fsr = 0.0f; }
                Code code = wostWalk(dist, fsr, flip, g, rng, s, queue, st.steps);
                if (code != Code::EscapedDomain) {
                    float term = wostTerminal(code, s);
                    total += s.throughput * term + s.totalReflectingBoundaryContribution + s.totalSourceContribution;
                    st.walkLength += s.walkLength;
                    success = true;
                }
            }
            if (success) { st.add((double)total); st.splits += splits; }
        }
    }

    // ------------------------------- solution and gradient ----------------------------
    // Latin-hypercube stratum of sample k among m for dimension j of point `key` (the device's
    // permutation: k -> (a k + b) mod m, a coprime to m, a and b hashed from (key, j))
    static uint32_t lhsStratum(uint64_t key, int j, uint32_t k, uint32_t m) {
        if (m <= 1) return 0;
        uint64_t h = key ^ (0x9E3779B97F4A7C15ull * (uint64_t)(j + 1));
        h = (h ^ (h >> 30)) * 0xBF58476D1CE4E5B9ull;
        h = (h ^ (h >> 27)) * 0x94D049BB133111EBull;
        h ^= h >> 31;
        uint32_t a = 1u + (uint32_t)(h % (uint64_t)(m - 1));
        for (int guard = 0; guard < 64; guard++) {
            uint32_t x = a, y = m;
            while (y) { uint32_t t = x % y; x = y; y = t; }
            if (x == 1u) break;
            a = a + 1u < m ? a + 1u : 1u;
        }
        const uint32_t b = (uint32_t)((h >> 32) % m);
        return (uint32_t)(((uint64_t)a * k + b) % m);
    }
    static Vec<D> sphereFromUniform(const float* u) {
        Vec<D> v;
        if (D == 2) { v[0] = std::cos(2.0f * kPi * u[0]); v[1] = std::sin(2.0f * kPi * u[0]); }
        else {
            float z = 1.0f - 2.0f * u[0], r = std::sqrt(std::max(0.0f, 1.0f - z * z));
            v[0] = r * std::cos(2.0f * kPi * u[1]); v[1] = r * std::sin(2.0f * kPi * u[1]); v[D - 1] = z;
        }
        return v;
    }

    // cosine-weighted hemisphere direction about the last axis (core/sampling.h:124-129,
    // :186-216: 2D uniform abscissa; 3D Shirley-Chiu concentric disk lifted to the hemisphere)
    static Vec<D> hemisphereCosine(const float* u) {
        Vec<D> v;
        if (D == 2) {
            float x = 2.0f * u[0] - 1.0f;
            v[0] = x; v[1] = std::sqrt(std::max(0.0f, 1.0f - x * x));
        } else {
            float a = 2.0f * u[0] - 1.0f, b = 2.0f * u[1] - 1.0f, r = 0.0f, phi = 0.0f;
            if (a != 0.0f || b != 0.0f) {
                if (std::fabs(a) > std::fabs(b)) { r = a; phi = 0.25f * kPi * (b / a); }
                else { r = b; phi = 0.5f * kPi - 0.25f * kPi * (a / b); }
            }
            v[0] = r * std::cos(phi); v[1] = r * std::sin(phi); v[D - 1] = std::sqrt(std::max(0.0f, 1.0f - r * r));
        }
        return v;
    }
    static float hemisphereCosinePdf(float c) { return D == 2 ? 0.5f * c : c / kPi; }
    // direction d given in the frame whose last axis is n (core/sampling.h:151-157, :236-246;
    // 3D: the orthonormal basis of Duff et al., JCGT 2017)
    static Vec<D> toFrame(const Vec<D>& n, const Vec<D>& d) {
        Vec<D> r;
        if (D == 2) {
            r[0] = d[0] * n[1] + d[1] * n[0];
            r[1] = -d[0] * n[0] + d[1] * n[1];
        } else {
            float sg = std::copysign(1.0f, n[D - 1]);
            float a = -1.0f / (sg + n[D - 1]);
            float b = n[0] * n[1] * a;
            float t1[3] = {1.0f + sg * n[0] * n[0] * a, sg * b, -sg * n[0]};
            float t2[3] = {b, sg + n[1] * n[1] * a, -n[1]};
            for (int i = 0; i < D; i++) r[i] = d[0] * t1[i] + d[1] * t2[i] + d[D - 1] * n[i];
        }
        return r;
    }

    // estimateSolutionAndGradient (walk_on_spheres.h:417-593, walk_on_stars.h:665-848) with the
    // parallel restatement the device uses: antithetic walks 2k, 2k+1 share pcg32 stream k and
    // mirror the first step; the first-step samples form a Latin hypercube assigned by a
    // per-point permutation; the control variates are the previous call's estimate (cvB) and
    // mean first source contribution (cvS); dirD is directionForDerivative.
    void gradEstimate(int solver, const Vec<D>& pt, float distB, int nWalks, uint64_t seed, int nPrev, float cvB,
                      float cvS, const Vec<D>& dirD, PointStats& st, GradStats& gs) const {
        const bool anti = ws.use_gradient_antithetic_variates != 0;
        const int count = nWalks <= 0 ? 0 : (anti ? 2 * std::max(1, nWalks / 2) : nWalks);
        const float R0 = 0.99f * distB;
        if (count == 0 || !(R0 > 0.0f)) return;
        const uint32_t m = (uint32_t)(2 * (anti ? count / 2 : count));
        const uint64_t key = seed ^ (uint64_t)nPrev;
        std::queue<WalkState<D>> queue;
        for (int w = 0; w < count; w++) {
            const uint32_t pair = anti ? (uint32_t)(w >> 1) : (uint32_t)w;
            const bool mirror = anti && (w & 1);
            Pcg32 rng(seed, (uint64_t)pair + (uint64_t)nPrev);
            bool yukawa = pde.p->absorption_coeff > 0.0f && ws.steps_before_applying_tikhonov == 0;
            std::unique_ptr<GreensFnBall<D>> g = makeGreens(yukawa);
            g->updateBall(pt, R0);
            float us[3] = {0, 0, 0}, ub[3] = {0, 0, 0};
            for (int j = 0; j < D - 1; j++) {
                us[j] = std::min(((float)lhsStratum(key, j, 2 * pair, m) + rng.nextFloat()) / (float)m, 0.99999994f);
                ub[j] = std::min(((float)lhsStratum(key, j, 2 * pair + 1, m) + rng.nextFloat()) / (float)m, 0.99999994f);
            }
            WalkState<D> s(pt, Vec<D>(), Vec<D>(), 0.0f, 1.0f, 0, false);
            float firstSrc = 0.0f;
            Vec<D> sDir;
            if (!ws.ignore_source_contribution) {
                float nrmG = g->norm();
                if (pde.p->is_source_constant) {
                    firstSrc = nrmG * pde.source(pt);
                } else {
                    Vec<D> dirS = sphereFromUniform(us);
                    float r, pdf;
                    g->sampleVolume(dirS, rng, r, pdf);
                    pdf = g->evaluate(r) / nrmG;
                    Vec<D> ys = mirror ? pt - r * dirS : pt + r * dirS;
                    firstSrc = nrmG * pde.source(ys);
                    sDir = (1.0f / (pdf * nrmG)) * g->gradient(r, ys);
                }
                s.totalSourceContribution += s.throughput * firstSrc;
            }
            Vec<D> dirB;
            float bPdf;
            if (ws.use_cosine_sampling_for_derivatives) {
                Vec<D> loc = hemisphereCosine(ub);
                if (rng.nextFloat() < 0.5f) loc[D - 1] = -loc[D - 1];
                bPdf = 0.5f * hemisphereCosinePdf(std::fabs(loc[D - 1]));
                dirB = toFrame(dirD, loc);
            } else {
                dirB = sphereFromUniform(ub);
                bPdf = D == 2 ? 1.0f / (2.0f * kPi) : 1.0f / (4.0f * kPi);
            }
            if (mirror) dirB = -dirB;
            Vec<D> yb = pt + R0 * dirB;
            s.throughput *= g->poissonKernelCentre() / bPdf;
            Vec<D> bDir = (1.0f / (bPdf * s.throughput)) * g->poissonKernelGradient(yb);
            s.currentPt = yb;
            if (solver == ZGPU_SOLVER_WALK_ON_STARS) { s.prevDistance = R0; s.prevDirection = dirB; }
            queue.push(s);
            int splits = -1;
            float total = 0.0f;
            bool success = false;
            while (!queue.empty()) {
                s = queue.front(); queue.pop();
                splits++;
                std::unique_ptr<GreensFnBall<D>> gw = makeGreens(yukawa);
                float dist = q.computeDistToAbsorbingBoundary(s.currentPt);
                Code code;
                if (solver == ZGPU_SOLVER_WALK_ON_SPHERES) code = wosWalk(dist, gw, rng, s, queue, st.steps);
                else code = wostWalk(dist, 0.0f, false, gw, rng, s, queue, st.steps);
                if (code != Code::EscapedDomain) {
                    float term = solver == ZGPU_SOLVER_WALK_ON_SPHERES ? wosTerminal(code, s) : wostTerminal(code, s);
                    total += s.throughput * term + s.totalReflectingBoundaryContribution + s.totalSourceContribution;
                    st.walkLength += s.walkLength;
                    success = true;
                }
            }
            if (success) {
                st.add((double)total);
                st.splits += splits;
                double gv[3] = {0, 0, 0};
                const float bc = total - firstSrc;
                float deriv = 0.0f;
                for (int i = 0; i < D; i++) {
                    float gb = (bc - cvB) * bDir[i], gsrc = (firstSrc - cvS) * sDir[i];
                    deriv += gb * dirD[i] + gsrc * dirD[i];
                    gv[i] = (double)(gb + gsrc);
                }
                gs.add(gv, D);
                gs.firstSource += firstSrc;
                gs.derivative += deriv;
            }
        }
    }

    uint64_t streamBase = 0;   // stream offset: solution-estimate count before this call
};

}  // namespace orc
