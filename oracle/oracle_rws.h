// oracle_rws.h -- TEST INFRASTRUCTURE, NOT PRODUCT CODE (see oracle_core.h).
//
// CPU restatement of ReverseWalkOnStars::solve for one sample (point_estimation/
// reverse_walk_on_stars.h:90-165, walk :265-393) with the splat of ReverseWalkOnStarsSolver
// (variance_reduction/reverse_walk_solver.h:236-302): every step searches its star-shaped
// ball for evaluation points by brute force (the reference uses a nanoflann k-d tree; any
// exact radius search gives the same set).  The walk draws from pcg32(seed, stream), its
// split states wait in a FIFO queue, as on the device.
#pragma once

#include "oracle_walk.h"

namespace orc {

template <int D>
struct RwsEval {
    int64_t n;
    const float* pt;
    const float* normal;
    const int32_t* type;
};

template <int D>
void reverseWalkSample(const Solver<D>& sv, const Vec<D>& pt, const Vec<D>& normal, int type, bool aligned, float pdf,
                       float contribution, float distAbs, uint64_t seed, uint64_t stream, const RwsEval<D>& ev,
                       float normalOffset, float radiusClamp, float reg, bool selfNormalize, double* totals,
                       uint64_t& steps) {
    const zgpu_walk_settings& ws = sv.ws;
    const auto& q = sv.q;
    const bool ds = ws.solve_double_sided != 0;
    int group;
    if (type == ZGPU_SAMPLE_ON_ABSORBING_BOUNDARY) group = aligned ? ZGPU_RWS_ABSORBING_ALIGNED : ZGPU_RWS_ABSORBING;
    else if (type == ZGPU_SAMPLE_ON_REFLECTING_BOUNDARY) group = aligned ? ZGPU_RWS_REFLECTING_ALIGNED : ZGPU_RWS_REFLECTING;
    else group = ZGPU_RWS_SOURCE;
    Pcg32 rng(seed, stream);
    const bool onRefl0 = type == ZGPU_SAMPLE_ON_REFLECTING_BOUNDARY;
    Vec<D> prevDir = (ds && onRefl0 && aligned) ? -1.0f * normal : normal;
    std::queue<WalkState<D>> queue;
    queue.push(WalkState<D>(pt, normal, prevDir, kMaxFloat, 1.0f, 0, onRefl0));
    bool first = true;
    int states = 0;
    while (!queue.empty() && states++ < 64) {
        WalkState<D> s = queue.front();
        queue.pop();
        bool yukawa = sv.pde.p->absorption_coeff > 0.0f && ws.steps_before_applying_tikhonov == 0;
        std::unique_ptr<GreensFnBall<D>> g = sv.makeGreens(yukawa);
        float dist = first ? distAbs : q.computeDistToAbsorbingBoundary(s.currentPt);
        first = false;
        while (dist > ws.epsilon_shell_for_absorbing_boundary) {
            steps++;
            bool flip = false;
            if (ds && s.onReflectingBoundary && s.prevDistance > 0.0f && dot(s.prevDirection, s.currentNormal) < 0.0f) {
                s.currentNormal = -1.0f * s.currentNormal;
                flip = true;
            }
            float R;
            if (ws.steps_before_using_maximal_spheres <= s.walkLength) {
                R = dist;
            } else if (s.onReflectingBoundary && sv.pde.hasNonZeroRobinCoeff(s.currentPt)) {
                R = ws.epsilon_shell_for_reflecting_boundary;
            } else {
                R = q.computeStarRadiusForReflectingBoundary(s.currentPt, ws.epsilon_shell_for_reflecting_boundary, dist,
                                                             ws.silhouette_precision, flip);
                if (ws.epsilon_shell_for_reflecting_boundary <= dist)
                    R = std::max(0.99f * R, ws.epsilon_shell_for_reflecting_boundary);
            }
            g->updateBall(s.currentPt, R);
            // splatContribution
            const float alpha = s.onReflectingBoundary ? 2.0f : 1.0f;
            for (int64_t e = 0; e < ev.n; e++) {
                const Vec<D> xe = load<D>(ev.pt + e * D);
                const float d2 = norm2(xe - s.currentPt);
                if (!(d2 < R * R)) continue;
                const int te = ev.type ? ev.type[e] : ZGPU_SAMPLE_IN_DOMAIN;
                if (te == ZGPU_SAMPLE_ON_ABSORBING_BOUNDARY) continue;
                const Vec<D> ne = ev.normal ? load<D>(ev.normal + e * D) : Vec<D>();
                if (q.intersectsWithReflectingBoundary(s.currentPt, xe, s.currentNormal, ne, s.onReflectingBoundary,
                                                       te == ZGPU_SAMPLE_ON_REFLECTING_BOUNDARY))
                    continue;
                float r = std::max(radiusClamp, std::sqrt(d2));
                float G = g->evaluate(r);
                if (reg > 0.0f) G *= regGreens(D, r / reg);
                float w = alpha * s.throughput * G / pdf;
                if (group <= ZGPU_RWS_ABSORBING_ALIGNED) w /= normalOffset;
                totals[e * ZGPU_RWS_TOTALS + group] += (double)(w * contribution);
                if (selfNormalize && group == ZGPU_RWS_ABSORBING) totals[e * ZGPU_RWS_TOTALS + ZGPU_RWS_POISSON_KERNEL] += w;
            }
            Vec<D> dir = sampleUnitSphereUniform<D>(rng);
            if (s.onReflectingBoundary && dot(s.currentNormal, dir) > 0.0f) dir = -1.0f * dir;
            Vec<D> hitPt, hitN;
            float hitDist = kMaxFloat;
            bool hit = q.intersectReflectingBoundary(s.currentPt, s.currentNormal, dir, R, s.onReflectingBoundary, hitPt,
                                                     hitN, hitDist);
            if (!hit) {
                Vec<D> p0 = s.onReflectingBoundary ? offsetPointAlongDirection<D>(s.currentPt, -1.0f * s.currentNormal)
                                                   : s.currentPt;
                hitPt = p0 + R * dir;
                hitDist = R;
                hitN = Vec<D>();
            }
            s.prevDistance = hitDist;
            s.prevDirection = dir;
            s.currentPt = hitPt;
            s.currentNormal = hitN;
            s.onReflectingBoundary = hit;
            s.throughput *= sv.stepThroughput(*g, s);
            if (!s.onReflectingBoundary && q.outsideBoundingDomain(s.currentPt)) break;
            if (sv.applyWeightWindow(rng, s, queue)) break;
            s.walkLength++;
            if (s.walkLength >= ws.max_walk_length) break;
            if (sv.pde.p->absorption_coeff > 0.0f && ws.steps_before_applying_tikhonov == s.walkLength) g = sv.makeGreens(true);
            dist = q.computeDistToAbsorbingBoundary(s.currentPt);
        }
    }
}

}  // namespace orc
