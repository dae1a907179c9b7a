// zgpu_kernels.cuh -- the walk engine kernels (instantiated per dimension by
// zgpu_kernels2.cu / zgpu_kernels3.cu; host dispatch in zgpu_dispatch.cu).
//
//  prepare  : per point, the bookkeeping of estimateSolution before its walk loop
//             (walk_on_spheres.h:321-356, walk_on_stars.h:519-598): boundary points,
//             epsilon-shell points, the first sphere / star radius, walk counts
//  scan     : exclusive prefix sum of walk counts -> global walk ids
//  walk     : persistent wavefront kernel.  Every lane owns one walk; a lane whose walk
//             finishes refills itself from a global walk counter (one atomic per warp for
//             all refilling lanes).  One iteration = one step of walk()
//             (walk_on_spheres.h:229-291, walk_on_stars.h:346-490) fused with the
//             geometric queries of that step.  Walk estimates are FP32; per-point sums
//             are FP64 atomics.
//  finalize : merge of this call's per-point moments into the caller's statistics
//             (SampleStatistics::merge, common.h:268-310), in FP64.
#pragma once
#include "zgpu_internal.h"

namespace zg {
namespace detail {

constexpr unsigned kFull = 0xffffffffu;

// the scene of point i (batched solves read the point's row of the scene table; a row
// outside the table is reported and the point is skipped)
ZG_D const SceneDesc& sceneOfPoint(const SolveParams& P, int64_t i, bool& bad) {
    bad = false;
    if (!P.sceneId) return P.sc;
    const int sid = P.sceneId[i];
    if (sid < 0 || sid >= P.nScenes) { bad = true; return P.sc; }
    return P.scenes[sid];
}

ZG_D bool outsideBox(const SceneDesc& S, const float* x, int D) {
    for (int i = 0; i < D; i++)
        if (x[i] < S.domainMin[i] || x[i] > S.domainMax[i]) return true;
    return false;
}

template <int D>
ZG_D float bboxDistance(const SceneDesc& S, V<D> x) {
    // default computeDistToAbsorbingBoundary (core/geometric_queries.h:212-217)
    V<D> m;
#pragma unroll
    for (int i = 0; i < D; i++) m[i] = fminf(S.domainMin[i] - x[i], x[i] - S.domainMax[i]);
    return len(m);
}

// a pending split walk state, 3 float4 in global scratch (only touched when walks split)
template <int D>
ZG_D void storeSplit(float4* slot, V<D> pt, V<D> nrm, V<D> prevDir, float prevDist, float thr, bool onRefl) {
    float v[12] = {0};
#pragma unroll
    for (int i = 0; i < D; i++) { v[i] = pt[i]; v[3 + i] = nrm[i]; v[6 + i] = prevDir[i]; }
    v[9] = prevDist; v[10] = thr; v[11] = onRefl ? 1.0f : 0.0f;
    slot[0] = make_float4(v[0], v[1], v[2], v[3]);
    slot[1] = make_float4(v[4], v[5], v[6], v[7]);
    slot[2] = make_float4(v[8], v[9], v[10], v[11]);
}

template <int D, int SOLVER, bool SCREENED, bool BATCHED, bool COOP>
struct Walker {
    // warp-cooperative queries are compiled into their own kernels: closest points for Walk
    // on Spheres, Robin star radii for Walk on Stars
    static constexpr bool kCoopClosest = COOP && SOLVER == ZGPU_SOLVER_WALK_ON_SPHERES;
    static constexpr bool kCoopStar = COOP && SOLVER == ZGPU_SOLVER_WALK_ON_STARS;
    const SolveParams& P;
    const SceneDesc* sc;   // batched solves: the walk's row of the scene table
    // the walk's problem; single-scene kernels read the kernel parameter itself, so its fields
    // stay parameter-space loads
    ZG_D const SceneDesc& SC() const {
        if constexpr (BATCHED) return *sc;
        else return P.sc;
    }
    DevicePde<D> pde;
    // walk identity
    int point;
    Pcg32 rng;
    // walk state (WalkState, common.h:93-130)
    V<D> pt, nrm, prevDir;
    float prevDist, thr;
    int wlen;
    bool onRefl, flip, pointFlip;
    float totRefl, totSrc;
    // estimateSolutionAndGradient: this walk's first-step source contribution, control
    // variate and gradient directions
    bool gradMode;
    float firstSrc, cvB, cvS;
    V<D> bGradDir, sGradDir;
    // per-walk accumulation across split states
    float walkTotal;
    bool success;
    int splits;
    long long lenSum;
    // loop state
    float distAbs, fsr;
    bool firstStep, cpValid;
    long long iters;        // loop iterations of this walk state (step budget)
    bool queryPending;      // cooperative mode: the closest-point query of this state is due
    bool radiusPending;     // cooperative mode: the Robin star radius of this step is due
    bool radiusReady;       // ... and answered (pendingR) -- the step resumes from there
    float pendingR;
    int pendingCode;        // cooperative mode: terminate(code) once the query is answered (-1: none)
    V<D> cpPt, cpN;
    Greens<D, SCREENED> g;
    float4* splitSlots;   // this thread's kSplitStack slots of 3 float4
    int nStack;
    // counters
    unsigned long long steps, escaped, exceeded, rr;
    uint32_t err;
    TravStack S;
    int cpSeed;             // this walk's last closest primitive (-1: none), the next query's first bound

    ZG_D Walker(const SolveParams& p, TravStack s) : P(p), S(s) {
        sc = &P.sc;
        pde.p = &SC().pde;
        steps = escaped = exceeded = rr = 0;
        err = 0;
        g.sqrtLambda = sqrtf(fmaxf(SC().pde.absorption_coeff, 0.0f));
    }

    ZG_D void closestQuery() {
        if (kCoopClosest && SC().hasAbs) { queryPending = true; cpValid = false; return; }
        if (SC().hasAbs) {
            ClosestHit<D> h = closestPoint<D, SOLVER == ZGPU_SOLVER_WALK_ON_STARS>(SC().absorbing, pt, S, err, cpSeed);
            cpSeed = h.slot;
            distAbs = h.d;
            cpPt = h.pt;
            if (h.slot >= 0) cpN = primNormal<D>(loadPrim<D>(SC().absorbing, h.slot));
            cpValid = true;
        } else {
            distAbs = bboxDistance<D>(SC(), pt);
            cpValid = false;
        }
    }

    ZG_D void resetGreens() {
        // a new GreensFnBall for every dequeued state (walk_on_spheres.h:376-383, walk_on_stars.h:618-625)
        g.yukawa = SC().pde.absorption_coeff > 0.0f && SC().ws.steps_before_applying_tikhonov == 0;
    }

    ZG_D void start(long long id, int pointIndex) {
        point = pointIndex;
        if (BATCHED) {
            sc = P.scenes + __ldg(P.sceneId + point);
            pde.p = &sc->pde;
            g.sqrtLambda = sqrtf(fmaxf(sc->pde.absorption_coeff, 0.0f));
        }
        long long w = id - __ldg(P.walkStart + point);
        rng.seed(__ldg(P.seed + point), (uint64_t)w + (uint64_t)__ldg(P.nPrev + point));
        pt = vload<D>(P.pt + (size_t)point * D);
        int type = P.type ? __ldg(P.type + point) : ZGPU_SAMPLE_IN_DOMAIN;
        int flags = __ldg(P.pointFlags + point);
        if (SOLVER == ZGPU_SOLVER_WALK_ON_STARS) {
            V<D> n = P.normal ? vload<D>(P.normal + (size_t)point * D) : vzero<D>();
            pointFlip = (flags & kPointFlip) != 0;
            if (pointFlip) n = -n;
            nrm = n; prevDir = n;
            prevDist = kFltMax;
            onRefl = type == ZGPU_SAMPLE_ON_REFLECTING_BOUNDARY;
        } else {
            nrm = vzero<D>(); prevDir = vzero<D>(); prevDist = 0.0f; onRefl = false; pointFlip = false;
        }
        flip = pointFlip;
        thr = 1.0f; wlen = 0; totRefl = 0.0f; totSrc = 0.0f;
        walkTotal = 0.0f; success = false; splits = 0; lenSum = 0; nStack = 0;
        distAbs = __ldg(P.distAbs + point);
        fsr = P.fsr[point];
        firstStep = true;
        cpValid = false;
        gradMode = false;
        queryPending = false;
        radiusPending = false;
        radiusReady = false;
        pendingCode = -1;
        iters = 0;
        cpSeed = -1;
        resetGreens();
        if (flags & kPointGradient) startGradient(w);
    }

    // First step of estimateSolutionAndGradient (walk_on_spheres.h:417-515,
    // walk_on_stars.h:665-790): a ball of radius 0.99 x the distance to the boundary; a
    // source point sampled along a stratified direction, a boundary point on a stratified
    // direction, and the gradient directions of both.  With antithetic variates walks 2k and
    // 2k+1 share pcg32 stream k: the odd walk draws the same first step and mirrors it
    // through the centre, then both continue on identical random numbers.  Stratification is
    // a Latin hypercube over the point's 2M first-step samples of this call (M = walks, or
    // pairs), the strata assigned by a per-point permutation.
    __device__ __noinline__ void startGradient(long long w) {
        const zgpu_walk_settings& ws = SC().ws;
        const bool anti = ws.use_gradient_antithetic_variates != 0;
        const long long pair = anti ? (w >> 1) : w;
        const bool mirror = anti && (w & 1);
        const int nPrev = __ldg(P.nPrev + point);
        if (anti) rng.seed(__ldg(P.seed + point), (uint64_t)pair + (uint64_t)nPrev);
        const long long walks = __ldg(P.walkStart + point + 1) - __ldg(P.walkStart + point);
        const uint32_t m = (uint32_t)(2 * (anti ? walks / 2 : walks));
        const uint64_t key = __ldg(P.seed + point) ^ (uint64_t)nPrev;
        gradMode = true;
        // control variates (walk_on_spheres.h:444-450): the previous estimate and the mean
        // first source contribution of the earlier walks
        const bool cv = ws.use_gradient_control_variates && nPrev > 0;
        cvB = cv ? (float)P.statMean[point] : 0.0f;
        cvS = (cv && P.statFirstSrc) ? (float)(P.statFirstSrc[point] / (double)nPrev) : 0.0f;
        const V<D> x0 = pt;
        const float R0 = fsr;
        g.update(x0, R0);
        float us[D], ub[D];
#pragma unroll
        for (int j = 0; j < D - 1; j++) {
            us[j] = fminf(((float)lhsStratum(key, j, (uint32_t)(2 * pair), m) + rng.uniform()) / (float)m, 0.99999994f);
            ub[j] = fminf(((float)lhsStratum(key, j, (uint32_t)(2 * pair + 1), m) + rng.uniform()) / (float)m, 0.99999994f);
        }
        firstSrc = 0.0f;
        sGradDir = vzero<D>();
        if (!ws.ignore_source_contribution) {
            const float nrmG = g.norm();
            if (SC().pde.is_source_constant) {
                firstSrc = nrmG * pde.source(x0);
            } else {
                const V<D> dirS = sphereFromUniform<D>(us);
                const float r = g.sampleRadius(rng);
                const float pdf = g.evaluate(r) / nrmG;
                const V<D> ys = mirror ? x0 - r * dirS : x0 + r * dirS;
                firstSrc = nrmG * pde.source(ys);
                sGradDir = (1.0f / (pdf * nrmG)) * g.gradient(r, ys);
            }
            totSrc += thr * firstSrc;
        }
        V<D> dirB;
        float bPdf;
        if (ws.use_cosine_sampling_for_derivatives) {
            // cosine-weighted about directionForDerivative, either hemisphere with probability
            // 1/2 (walk_on_spheres.h:500-504)
            V<D> loc = hemisphereCosine<D>(ub);
            if (rng.uniform() < 0.5f) loc[D - 1] = -loc[D - 1];
            bPdf = 0.5f * hemisphereCosinePdf<D>(fabsf(loc[D - 1]));
            dirB = toFrame(derivativeDirection(), loc);
        } else {
            dirB = sphereFromUniform<D>(ub);
            bPdf = D == 2 ? 1.0f / (2.0f * kPi) : 1.0f / (4.0f * kPi);
        }
        if (mirror) dirB = -dirB;
        const V<D> yb = x0 + R0 * dirB;
        thr *= g.poissonKernelCentre() / bPdf;
        bGradDir = (1.0f / (bPdf * thr)) * g.poissonKernelGradient(yb);
        pt = yb;
        if (SOLVER == ZGPU_SOLVER_WALK_ON_STARS) {
            prevDist = R0;
            prevDir = dirB;
            nrm = vzero<D>();
            onRefl = false;
        }
        firstStep = false;
        fsr = 0.0f;
        resetGreens();
        closestQuery();
    }

    // answer of a cooperative closest-point query
    ZG_D void setClosest(float d, int slot) {
        distAbs = d;
        cpPt = pt;
        if (slot >= 0) {
            Prim<D> t = loadPrim<D>(SC().absorbing, slot);
            V<D> q;
            closestOnPrim(t, pt, q);
            cpPt = q;
            cpN = primNormal<D>(t);
        }
        cpValid = true;
        queryPending = false;
    }

    __device__ __noinline__ void pushSplit() {
        // no split slots (a solve that runs without split scratch): report instead of storing
        if (P.splitStack && nStack < kSplitStack) storeSplit<D>(splitSlots + 3 * nStack++, pt, nrm, prevDir, prevDist, thr, onRefl);
        else err |= kErrSplitOverflow;
    }

    __device__ __noinline__ void beginSplit() {
        --nStack;
        float4 a = splitSlots[3 * nStack], b = splitSlots[3 * nStack + 1], c = splitSlots[3 * nStack + 2];
        float v[12] = {a.x, a.y, a.z, a.w, b.x, b.y, b.z, b.w, c.x, c.y, c.z, c.w};
#pragma unroll
        for (int i = 0; i < D; i++) { pt[i] = v[i]; nrm[i] = v[3 + i]; prevDir[i] = v[6 + i]; }
        prevDist = v[9]; thr = v[10]; onRefl = v[11] != 0.0f;
        wlen = 0; totRefl = 0.0f; totSrc = 0.0f;
        flip = pointFlip;
        fsr = 0.0f;
        firstStep = true;
        iters = 0;
        cpSeed = -1;
        resetGreens();
        closestQuery();
        splits++;
    }

    // weight window (walk_on_spheres.h:193-226, walk_on_stars.h:309-343); true -> terminated
    ZG_D bool weightWindow() {
        const float sT = SC().ws.splitting_threshold, rT = SC().ws.russian_roulette_threshold;
        if (thr > sT) {
            if (!(thr <= kFltMax)) {
                // a throughput that overflowed to inf (reflectance bounds up to 2 with negative
                // Robin coefficients) cannot be split into finite states: report it, keep sT
                err |= kErrSplitOverflow;
                thr = sT;
                return false;
            }
            float left = thr - sT;
            thr = sT;
            for (int guard = 0; left > sT && guard < 1 << 20; guard++) {
                left -= sT;
                pushSplit();
            }
            if (rng.uniform() < left / sT) pushSplit();
        } else if (thr < rT) {
            float survival = thr / rT;
            if (survival < rng.uniform()) { thr = 0.0f; return true; }
            thr = rT;
        }
        return false;
    }

    // returns false when the lane's walk is complete
    __device__ __noinline__ bool terminate(int code) {
        if (code == kEscaped) {
            escaped++;
        } else {
            if (code == kExceeded) exceeded++;
            if (code == kRussianRoulette) rr++;
            float term = 0.0f;
            bool payTerminal = code == kReached || (SOLVER == ZGPU_SOLVER_WALK_ON_SPHERES && code == kExceeded);
            if (payTerminal && !SC().ws.ignore_absorbing_boundary_contribution) {
                // projectToAbsorbingBoundary then pde.dirichlet (walk_on_spheres.h:294-318, walk_on_stars.h:493-516)
                if (SC().hasAbs) {
                    if (!cpValid && !kCoopClosest) closestQuery();
                    bool aligned = false;
                    if (SC().ws.solve_double_sided) aligned = dot(pt - cpPt, cpN) > 0.0f;
                    term = pde.dirichlet(cpPt, aligned);
                } else {
                    term = pde.dirichlet(pt, false);
                }
            }
            walkTotal += thr * term + totRefl + totSrc;
            lenSum += wlen;
            success = true;
        }
        if (nStack > 0) { beginSplit(); return true; }
        if (success) {
            if (gradMode) addGradient();
            atomicAdd(P.accSum + point, (double)walkTotal);
            atomicAdd(P.accSq + point, (double)walkTotal * (double)walkTotal);
            atomicAdd(P.accN + point, 1);
            atomicAdd(reinterpret_cast<unsigned long long*>(P.accLen + point), (unsigned long long)lenSum);
            if (splits) atomicAdd(reinterpret_cast<unsigned long long*>(P.accSplits + point), (unsigned long long)splits);
        }
        return false;
    }

    // Ends the walk through the neural cache: records the position, the throughput and the
    // contributions gathered so far; the cache pass adds throughput * cache(x) and merges the
    // walk into its point.  False (keep walking) when the record buffer is full.
    __device__ __noinline__ bool cacheTerminate() {
        unsigned long long slot = atomicAdd(P.counters + kCtrCache, 1ull);
        if ((long long)slot >= P.cacheCap) { err |= kErrCacheOverflow; return false; }
        float4* r = P.cacheRec + 2 * slot;
        r[0] = make_float4(pt[0], pt[1], D == 3 ? pt[D - 1] : 0.0f, thr);
        r[1] = make_float4(walkTotal + totRefl + totSrc, __int_as_float(point), __int_as_float((int)(lenSum + wlen)), 0.0f);
        return true;
    }

    // gradient estimate of a completed walk (walk_on_spheres.h:567-580): the boundary part of
    // its total (minus the control variate) along the boundary gradient direction plus the
    // first source contribution along the source gradient direction
    __device__ __noinline__ void addGradient() {
        const float bc = walkTotal - firstSrc;
        const V<D> dd = derivativeDirection();
        float deriv = 0.0f;
#pragma unroll
        for (int i = 0; i < D; i++) {
            const float gb = (bc - cvB) * bGradDir[i], gs = (firstSrc - cvS) * sGradDir[i];
            deriv += gb * dd[i] + gs * dd[i];
            const double gi = (double)(gb + gs);
            atomicAdd(P.accGrad + (size_t)point * D + i, gi);
            atomicAdd(P.accGradSq + (size_t)point * D + i, gi * gi);
        }
        atomicAdd(P.accGradN + point, 1);
        if (P.accFirstSrc) atomicAdd(P.accFirstSrc + point, (double)firstSrc);
        if (P.accDeriv) atomicAdd(P.accDeriv + point, (double)deriv);
    }

    // SamplePoint::directionForDerivative (common.h:185), the first axis by default
    ZG_D V<D> derivativeDirection() const {
        V<D> d = vzero<D>();
        if (P.dirDeriv) d = vload<D>(P.dirDeriv + (size_t)point * D);
        else d[0] = 1.0f;
        return d;
    }

    // --------------------------------------------------------------- Walk on Spheres step
    ZG_D bool stepWoS() {
        const zgpu_walk_settings& ws = SC().ws;
        if (!(distAbs > ws.epsilon_shell_for_absorbing_boundary)) {
            // the terminal value needs the projection: in cooperative mode the warp answers first
            if (kCoopClosest && SC().hasAbs && !cpValid) { pendingCode = kReached; closestQuery(); return true; }
            return terminate(kReached);
        }
        if (P.cacheMinDist > 0.0f && wlen > 0 && distAbs >= P.cacheMinDist && cacheTerminate()) return false;
        steps++;
        g.update(pt, distAbs);
        if (!ws.ignore_source_contribution) {
            float src;
            if (SC().pde.is_source_constant) {
                src = g.norm() * pde.source(pt);
            } else {
                V<D> d = sampleSphere<D>(rng);
                float r = g.sampleRadius(rng);
                src = g.norm() * pde.source(pt + r * d);
            }
            totSrc += thr * src;
        }
        V<D> dir = sampleSphere<D>(rng);
        pt = pt + distAbs * dir;
        cpValid = false;
        thr *= g.directionSampledPoissonKernel(pt);
        if (outsideBox(SC(), pt.v, D)) return terminate(kEscaped);
        if (weightWindow()) return terminate(kRussianRoulette);
        wlen++;
        if (wlen >= ws.max_walk_length) {
            // WoS pays the terminal value of the projected point: query first when cooperative
            if (kCoopClosest && SC().hasAbs) { pendingCode = kExceeded; closestQuery(); return true; }
            return terminate(kExceeded);
        }
        if (SC().pde.absorption_coeff > 0.0f && ws.steps_before_applying_tikhonov == wlen) g.yukawa = true;
        closestQuery();
        return true;
    }

    // --------------------------------------------------------------- Walk on Stars step
    // answer of a cooperative Robin star-radius query (the shrink of walk_on_stars.h:393-397)
    ZG_D void setStarRadius(float r) {
        const float eps = SC().ws.epsilon_shell_for_reflecting_boundary;
        pendingR = eps <= distAbs ? fmaxf(kRadiusShrink * r, eps) : r;
        radiusPending = false;
        radiusReady = true;
    }

    ZG_D bool stepWoSt() {
        const zgpu_walk_settings& ws = SC().ws;
        float R;
        if (kCoopStar && radiusReady) {
            // resumed after the warp answered this step's Robin star radius
            radiusReady = false;
            R = pendingR;
        } else {
            if (!(distAbs > ws.epsilon_shell_for_absorbing_boundary)) return terminate(kReached);
            if (P.cacheMinDist > 0.0f && wlen > 0 && !onRefl && distAbs >= P.cacheMinDist) {
                bool far = !SC().hasRefl || closestPoint<D>(SC().reflecting, pt, S, err).d >= P.cacheMinDist;
                if (far && cacheTerminate()) return false;
            }
            if (firstStep && fsr > 0.0f) {
                R = fsr;
            } else {
                flip = false;
                if (ws.solve_double_sided && onRefl && prevDist > 0.0f && dot(prevDir, nrm) < 0.0f) {
                    nrm = -nrm;
                    flip = true;
                }
                if (ws.steps_before_using_maximal_spheres <= wlen) {
                    R = distAbs;
                } else if (onRefl && pde.hasNonZeroRobinCoeff(pt)) {
                    R = ws.epsilon_shell_for_reflecting_boundary;
                } else if (kCoopStar && SC().hasRefl) {
                    radiusPending = true;      // the warp answers, then the step resumes here
                    return true;
                } else {
                    R = SC().hasRefl ? starRadius<D>(SC().reflecting, pt, ws.epsilon_shell_for_reflecting_boundary,
                                                     distAbs, ws.silhouette_precision, flip, S, err)
                                     : distAbs;
                    if (SC().hasRefl && ws.epsilon_shell_for_reflecting_boundary <= distAbs)
                        R = fmaxf(kRadiusShrink * R, ws.epsilon_shell_for_reflecting_boundary);
                }
            }
        }
        steps++;
        g.update(pt, R);
        V<D> dir = sampleSphere<D>(rng);
        if (onRefl && dot(nrm, dir) > 0.0f) dir = -dir;
        V<D> origin = onRefl ? offsetPoint<D>(pt, -nrm) : pt;
        V<D> hitPt, hitN;
        float hitDist;
        bool hit = false;
        if (SC().hasRefl) {
            RayHit<D> h = intersectRay<D>(SC().reflecting, origin, dir, R, false, S, err);
            if (h.slot >= 0) {
                hit = true;
                hitDist = h.t;
                hitPt = origin + h.t * dir;
                hitN = primNormal<D>(loadPrim<D>(SC().reflecting, h.slot));
            }
        }
        if (!hit) {
            hitPt = origin + R * dir;
            hitDist = R;
            hitN = vzero<D>();
        }
        // reflecting boundary contribution (walk_on_stars.h:190-250)
        if (SC().hasRefl && !ws.ignore_reflecting_boundary_contribution) {
            float u[D];
#pragma unroll
            for (int i = 0; i < D; i++) u[i] = rng.uniform();
            V<D> bpt, bn;
            float pdf;
            if (sampleBoundary<D>(SC().reflecting, pt, R, u, bpt, bn, pdf)) {
                V<D> toS = bpt - pt;
                float dS = len(toS);
                float alpha = onRefl ? 2.0f : 1.0f;
                bool aligned = false;
                if (ws.solve_double_sided) {
                    toS = (1.0f / dS) * toS;
                    if (flip) {
                        aligned = true;
                    } else if (dot(toS, bn) < -ws.silhouette_precision) {
                        bool fs = true;
                        if (alpha > 1.0f) fs = dot(toS, nrm) < -ws.silhouette_precision;
                        if (fs) aligned = true;
                    }
                }
                V<D> bnA = aligned ? -bn : bn;
                if (pdf > 0.0f && dS < R) {
                    V<D> p1 = onRefl ? offsetPoint<D>(pt, -nrm) : pt;
                    V<D> p2 = offsetPoint<D>(bpt, -bnA);
                    V<D> seg = p2 - p1;
                    float sl = len(seg);
                    bool occluded = false;
                    if (sl > 0.0f) {
                        RayHit<D> oh = intersectRay<D>(SC().reflecting, p1, (1.0f / sl) * seg, sl, true, S, err);
                        occluded = oh.slot >= 0;
                    }
                    if (!occluded) {
                        float r = fmaxf(kRClamp, dS);
                        float G = g.evaluate(r);
                        float h = pde.robin(bpt, bn, ws.solve_double_sided && aligned);
                        totRefl += thr * alpha * G * h / pdf;
                    }
                }
            }
        }
        // source contribution (walk_on_stars.h:253-275)
        if (!ws.ignore_source_contribution) {
            float r = g.sampleRadius(rng);
            if (r <= hitDist) totSrc += thr * g.norm() * pde.source(pt + r * dir);
        }
        prevDist = hitDist;
        prevDir = dir;
        pt = hitPt;
        nrm = hitN;
        onRefl = hit;
        cpValid = false;
        // walk step throughput (walk_on_stars.h:278-307)
        float stepThr;
        if (onRefl && prevDist > kFltEps) {
            float kappa = 0.0f;
            V<D> n = nrm;
            if (!SC().pde.are_robin_conditions_pure_neumann) {
                bool f2 = false;
                if (ws.solve_double_sided) { f2 = dot(prevDir, nrm) < 0.0f; if (f2) n = -n; }
                kappa = pde.robinCoeff(pt, ws.solve_double_sided && f2);
            }
            float refl = g.reflectance(prevDist, prevDir, n, kappa);
            float maxRefl = SC().pde.are_robin_coeffs_nonnegative ? 1.0f : 2.0f;
            stepThr = fminf(fmaxf(refl, 0.0f), maxRefl);
        } else {
            stepThr = g.directionSampledPoissonKernel(pt);
        }
        thr *= stepThr;
        if (!onRefl && outsideBox(SC(), pt.v, D)) return terminate(kEscaped);
        if (weightWindow()) return terminate(kRussianRoulette);
        wlen++;
        if (wlen >= ws.max_walk_length) return terminate(kExceeded);
        if (SC().pde.absorption_coeff > 0.0f && ws.steps_before_applying_tikhonov == wlen) g.yukawa = true;
        closestQuery();
        firstStep = false;
        return true;
    }

    ZG_D bool step() {
        if (P.stepBudget > 0 && ++iters > P.stepBudget) {
            // the iteration budget of this state ran out: drop the walk and report it
            err |= kErrBudget;
            success = false;
            nStack = 0;
            queryPending = radiusPending = false;
            return false;
        }
        if (SOLVER == ZGPU_SOLVER_WALK_ON_SPHERES) {
            if (kCoopClosest && pendingCode >= 0) { const int code = pendingCode; pendingCode = -1; return terminate(code); }
            return stepWoS();
        }
        return stepWoSt();
    }

    // ------------------------------------------------- sorted-wavefront Walk on Stars step
    // The wavefront schedule (zgpu_wave.cuh) keeps each walk's state in a record in device
    // memory between kernels and runs one step as two kernels over records sorted by
    // position: waveRadius (the closest-point query that ends the previous step, the
    // absorbing-boundary test and this step's star radius) and waveAdvance (the rest of the
    // step).  Together they run stepWoSt's statements in its order; only the closest-point
    // query moves from the end of one step to the start of the next, with no random number
    // drawn in between.  Solves on this schedule have no neural cache, no gradient walks, no
    // split scratch and no warp-wide queries, so those branches of stepWoSt are absent here;
    // stepWoSt itself stays as it is, its code generation being sensitive to its shape.
    static constexpr int kWaveVec = D == 2 ? 5 : 6;   // float4 per record

    // record words: pt, nrm, prevDir (D each), prevDist, thr, distAbs, fsr (this step's
    // radius once waveRadius has run), totRefl, totSrc, pcg32 state and increment (two words
    // each), point (-1: a free slot), wlen, closest-point seed, flags
    ZG_D void waveLoad(const float4* rec) {
        float w[4 * kWaveVec];
#pragma unroll
        for (int v = 0; v < kWaveVec; v++) {
            const float4 q = rec[v];
            w[4 * v] = q.x; w[4 * v + 1] = q.y; w[4 * v + 2] = q.z; w[4 * v + 3] = q.w;
        }
#pragma unroll
        for (int i = 0; i < D; i++) { pt[i] = w[i]; nrm[i] = w[D + i]; prevDir[i] = w[2 * D + i]; }
        constexpr int o = 3 * D;
        prevDist = w[o]; thr = w[o + 1]; distAbs = w[o + 2]; fsr = w[o + 3]; totRefl = w[o + 4]; totSrc = w[o + 5];
        rng.state = (uint64_t)__float_as_uint(w[o + 6]) | ((uint64_t)__float_as_uint(w[o + 7]) << 32);
        rng.inc = (uint64_t)__float_as_uint(w[o + 8]) | ((uint64_t)__float_as_uint(w[o + 9]) << 32);
        point = __float_as_int(w[o + 10]);
        if constexpr (BATCHED) {   // the walk's row of the scene table, as start() sets it
            sc = P.scenes + __ldg(P.sceneId + point);
            pde.p = &sc->pde;
            g.sqrtLambda = sqrtf(fmaxf(sc->pde.absorption_coeff, 0.0f));
        }
        wlen = __float_as_int(w[o + 11]);
        cpSeed = __float_as_int(w[o + 12]);
        const int f = __float_as_int(w[o + 13]);
        onRefl = (f & 1) != 0; flip = (f & 2) != 0; pointFlip = (f & 4) != 0; firstStep = (f & 8) != 0;
        g.yukawa = (f & 16) != 0;
        // what start() leaves in the fields a record does not hold
        walkTotal = 0.0f; success = false; splits = 0; lenSum = 0; nStack = 0; gradMode = false; cpValid = false;
        queryPending = radiusPending = radiusReady = false; pendingCode = -1;
        iters = wlen;   // every step() call before this one advanced wlen
    }
    ZG_D void waveStore(float4* rec) const {
        float w[4 * kWaveVec];
#pragma unroll
        for (int i = 0; i < D; i++) { w[i] = pt[i]; w[D + i] = nrm[i]; w[2 * D + i] = prevDir[i]; }
        constexpr int o = 3 * D;
        w[o] = prevDist; w[o + 1] = thr; w[o + 2] = distAbs; w[o + 3] = fsr; w[o + 4] = totRefl; w[o + 5] = totSrc;
        w[o + 6] = __uint_as_float((uint32_t)rng.state); w[o + 7] = __uint_as_float((uint32_t)(rng.state >> 32));
        w[o + 8] = __uint_as_float((uint32_t)rng.inc); w[o + 9] = __uint_as_float((uint32_t)(rng.inc >> 32));
        w[o + 10] = __int_as_float(point);
        w[o + 11] = __int_as_float(wlen);
        w[o + 12] = __int_as_float(cpSeed);
        w[o + 13] = __int_as_float((onRefl ? 1 : 0) | (flip ? 2 : 0) | (pointFlip ? 4 : 0) | (firstStep ? 8 : 0) |
                                   (g.yukawa ? 16 : 0));
#pragma unroll
        for (int k = o + 14; k < 4 * kWaveVec; k++) w[k] = 0.0f;
#pragma unroll
        for (int v = 0; v < kWaveVec; v++) rec[v] = make_float4(w[4 * v], w[4 * v + 1], w[4 * v + 2], w[4 * v + 3]);
    }
    static constexpr int kWavePointWord = 3 * D + 10;

    // terminate(), closestQuery() and weightWindow() for the wavefront members, inline: a
    // wavefront walk has no split states, gradients or cache records, and without their
    // out-of-line paths the walker's address is never taken, so its fields can live in
    // registers (the traversals get a stack descriptor and an error word that are locals of
    // the step member, not the walker's own).  Same statements, same random numbers and the
    // same atomics as the originals for such a walk; a split reports kErrSplitOverflow as
    // pushSplit does without split scratch.  Measured on the default workload: +1.7% over
    // the walker in local memory (966M against 950M walk-steps/s).
    ZG_D bool waveTerminate(TravStack& s, uint32_t& e, int code) {
        if (code == kEscaped) {
            escaped++;
            return false;
        }
        if (code == kExceeded) exceeded++;
        if (code == kRussianRoulette) rr++;
        float term = 0.0f;
        const bool payTerminal = code == kReached || (SOLVER == ZGPU_SOLVER_WALK_ON_SPHERES && code == kExceeded);
        if (payTerminal && !SC().ws.ignore_absorbing_boundary_contribution) {
            if (SC().hasAbs) {
                if (!cpValid) waveClosestQuery(s, e);
                bool aligned = false;
                if (SC().ws.solve_double_sided) aligned = dot(pt - cpPt, cpN) > 0.0f;
                term = pde.dirichlet(cpPt, aligned);
            } else {
                term = pde.dirichlet(pt, false);
            }
        }
        const float total = 0.0f + (thr * term + totRefl + totSrc);
        atomicAdd(P.accSum + point, (double)total);
        atomicAdd(P.accSq + point, (double)total * (double)total);
        atomicAdd(P.accN + point, 1);
        atomicAdd(reinterpret_cast<unsigned long long*>(P.accLen + point), (unsigned long long)(long long)wlen);
        return false;
    }
    // closestQuery() on the caller's stack descriptor and error word
    ZG_D void waveClosestQuery(TravStack& s, uint32_t& e) {
        if (SC().hasAbs) {
            ClosestHit<D> h = closestPoint<D, SOLVER == ZGPU_SOLVER_WALK_ON_STARS>(SC().absorbing, pt, s, e, cpSeed);
            cpSeed = h.slot;
            distAbs = h.d;
            cpPt = h.pt;
            if (h.slot >= 0) cpN = primNormal<D>(loadPrim<D>(SC().absorbing, h.slot));
            cpValid = true;
        } else {
            distAbs = bboxDistance<D>(SC(), pt);
            cpValid = false;
        }
    }
    ZG_D bool waveWeightWindow() {
        const float sT = SC().ws.splitting_threshold, rT = SC().ws.russian_roulette_threshold;
        if (thr > sT) {
            if (!(thr <= kFltMax)) { err |= kErrSplitOverflow; thr = sT; return false; }
            float left = thr - sT;
            thr = sT;
            for (int guard = 0; left > sT && guard < 1 << 20; guard++) {
                left -= sT;
                err |= kErrSplitOverflow;
            }
            if (rng.uniform() < left / sT) err |= kErrSplitOverflow;
        } else if (thr < rT) {
            float survival = thr / rT;
            if (survival < rng.uniform()) { thr = 0.0f; return true; }
            thr = rT;
        }
        return false;
    }

    // first kernel of a step; false when the walk ended (terminated or out of budget)
    ZG_D bool waveRadius() {
        TravStack s = S;
        uint32_t e = 0;
        const bool alive = waveRadiusImpl(s, e);
        err |= e;
        return alive;
    }
    ZG_D bool waveRadiusImpl(TravStack& s, uint32_t& e) {
        if (P.stepBudget > 0 && ++iters > P.stepBudget) { err |= kErrBudget; return false; }
        const zgpu_walk_settings& ws = SC().ws;
        if (!firstStep) waveClosestQuery(s, e);
        if (!(distAbs > ws.epsilon_shell_for_absorbing_boundary)) return waveTerminate(s, e, kReached);
        if (firstStep && fsr > 0.0f) return true;   // the first sphere radius is this step's
        float R;
        flip = false;
        if (ws.solve_double_sided && onRefl && prevDist > 0.0f && dot(prevDir, nrm) < 0.0f) {
            nrm = -nrm;
            flip = true;
        }
        if (ws.steps_before_using_maximal_spheres <= wlen) {
            R = distAbs;
        } else if (onRefl && pde.hasNonZeroRobinCoeff(pt)) {
            R = ws.epsilon_shell_for_reflecting_boundary;
        } else {
            R = SC().hasRefl ? starRadius<D>(SC().reflecting, pt, ws.epsilon_shell_for_reflecting_boundary,
                                             distAbs, ws.silhouette_precision, flip, s, e)
                             : distAbs;
            if (SC().hasRefl && ws.epsilon_shell_for_reflecting_boundary <= distAbs)
                R = fmaxf(kRadiusShrink * R, ws.epsilon_shell_for_reflecting_boundary);
        }
        fsr = R;
        return true;
    }

    // second kernel of a step, from the radius fsr that waveRadius left; false when the walk ended
    ZG_D bool waveAdvance() {
        TravStack s = S;
        uint32_t e = 0;
        const bool alive = waveAdvanceImpl(s, e);
        err |= e;
        return alive;
    }
    ZG_D bool waveAdvanceImpl(TravStack& s, uint32_t& e) {
        const zgpu_walk_settings& ws = SC().ws;
        const float R = fsr;
        steps++;
        g.update(pt, R);
        V<D> dir = sampleSphere<D>(rng);
        if (onRefl && dot(nrm, dir) > 0.0f) dir = -dir;
        V<D> origin = onRefl ? offsetPoint<D>(pt, -nrm) : pt;
        V<D> hitPt, hitN;
        float hitDist;
        bool hit = false;
        if (SC().hasRefl) {
            RayHit<D> h = intersectRay<D>(SC().reflecting, origin, dir, R, false, s, e);
            if (h.slot >= 0) {
                hit = true;
                hitDist = h.t;
                hitPt = origin + h.t * dir;
                hitN = primNormal<D>(loadPrim<D>(SC().reflecting, h.slot));
            }
        }
        if (!hit) {
            hitPt = origin + R * dir;
            hitDist = R;
            hitN = vzero<D>();
        }
        if (SC().hasRefl && !ws.ignore_reflecting_boundary_contribution) {
            float u[D];
#pragma unroll
            for (int i = 0; i < D; i++) u[i] = rng.uniform();
            V<D> bpt, bn;
            float pdf;
            if (sampleBoundary<D>(SC().reflecting, pt, R, u, bpt, bn, pdf)) {
                V<D> toS = bpt - pt;
                float dS = len(toS);
                float alpha = onRefl ? 2.0f : 1.0f;
                bool aligned = false;
                if (ws.solve_double_sided) {
                    toS = (1.0f / dS) * toS;
                    if (flip) {
                        aligned = true;
                    } else if (dot(toS, bn) < -ws.silhouette_precision) {
                        bool fs = true;
                        if (alpha > 1.0f) fs = dot(toS, nrm) < -ws.silhouette_precision;
                        if (fs) aligned = true;
                    }
                }
                V<D> bnA = aligned ? -bn : bn;
                if (pdf > 0.0f && dS < R) {
                    V<D> p1 = onRefl ? offsetPoint<D>(pt, -nrm) : pt;
                    V<D> p2 = offsetPoint<D>(bpt, -bnA);
                    V<D> seg = p2 - p1;
                    float sl = len(seg);
                    bool occluded = false;
                    if (sl > 0.0f) {
                        RayHit<D> oh = intersectRay<D>(SC().reflecting, p1, (1.0f / sl) * seg, sl, true, s, e);
                        occluded = oh.slot >= 0;
                    }
                    if (!occluded) {
                        float r = fmaxf(kRClamp, dS);
                        float G = g.evaluate(r);
                        float h = pde.robin(bpt, bn, ws.solve_double_sided && aligned);
                        totRefl += thr * alpha * G * h / pdf;
                    }
                }
            }
        }
        if (!ws.ignore_source_contribution) {
            float r = g.sampleRadius(rng);
            if (r <= hitDist) totSrc += thr * g.norm() * pde.source(pt + r * dir);
        }
        prevDist = hitDist;
        prevDir = dir;
        pt = hitPt;
        nrm = hitN;
        onRefl = hit;
        cpValid = false;
        float stepThr;
        if (onRefl && prevDist > kFltEps) {
            float kappa = 0.0f;
            V<D> n = nrm;
            if (!SC().pde.are_robin_conditions_pure_neumann) {
                bool f2 = false;
                if (ws.solve_double_sided) { f2 = dot(prevDir, nrm) < 0.0f; if (f2) n = -n; }
                kappa = pde.robinCoeff(pt, ws.solve_double_sided && f2);
            }
            float refl = g.reflectance(prevDist, prevDir, n, kappa);
            float maxRefl = SC().pde.are_robin_coeffs_nonnegative ? 1.0f : 2.0f;
            stepThr = fminf(fmaxf(refl, 0.0f), maxRefl);
        } else {
            stepThr = g.directionSampledPoissonKernel(pt);
        }
        thr *= stepThr;
        if (!onRefl && outsideBox(SC(), pt.v, D)) return waveTerminate(s, e, kEscaped);
        if (waveWeightWindow()) return waveTerminate(s, e, kRussianRoulette);
        wlen++;
        if (wlen >= ws.max_walk_length) return waveTerminate(s, e, kExceeded);
        if (SC().pde.absorption_coeff > 0.0f && ws.steps_before_applying_tikhonov == wlen) g.yukawa = true;
        firstStep = false;   // the closest-point query that ends the step runs in the next waveRadius
        return true;
    }

    // a Walk on Spheres step on the wavefront schedule: stepWoS's statements in its order, the
    // closest-point query that ends the previous step first; false when the walk ended
    ZG_D bool waveStepWoS() {
        TravStack s = S;
        uint32_t e = 0;
        const bool alive = waveStepWoSImpl(s, e);
        err |= e;
        return alive;
    }
    ZG_D bool waveStepWoSImpl(TravStack& s, uint32_t& e) {
        if (P.stepBudget > 0 && ++iters > P.stepBudget) { err |= kErrBudget; return false; }
        const zgpu_walk_settings& ws = SC().ws;
        if (!firstStep) waveClosestQuery(s, e);
        if (!(distAbs > ws.epsilon_shell_for_absorbing_boundary)) return waveTerminate(s, e, kReached);
        steps++;
        g.update(pt, distAbs);
        if (!ws.ignore_source_contribution) {
            float src;
            if (SC().pde.is_source_constant) {
                src = g.norm() * pde.source(pt);
            } else {
                V<D> d = sampleSphere<D>(rng);
                float r = g.sampleRadius(rng);
                src = g.norm() * pde.source(pt + r * d);
            }
            totSrc += thr * src;
        }
        V<D> dir = sampleSphere<D>(rng);
        pt = pt + distAbs * dir;
        cpValid = false;
        thr *= g.directionSampledPoissonKernel(pt);
        if (outsideBox(SC(), pt.v, D)) return waveTerminate(s, e, kEscaped);
        if (waveWeightWindow()) return waveTerminate(s, e, kRussianRoulette);
        wlen++;
        if (wlen >= ws.max_walk_length) return waveTerminate(s, e, kExceeded);
        if (SC().pde.absorption_coeff > 0.0f && ws.steps_before_applying_tikhonov == wlen) g.yukawa = true;
        firstStep = false;
        return true;
    }
};

constexpr int kWalkThreads = 128;
// Minimum resident blocks per SM the walk kernel is compiled for: 8 caps it at 64 registers
// (8 blocks x 4 warps per SM).  Measured on the GB300 against no cap (84 registers, 6 blocks):
// 2D Walk on Stars +18%, 3D Robin Walk on Stars +61%, 3D Walk on Spheres +10%; 7 and 10
// blocks were slower than 8.
#ifndef ZG_WALK_MIN_BLOCKS
#define ZG_WALK_MIN_BLOCKS 8
#endif

// Warp-cooperative search: the largest i in [0, nPoints) with walkStart[i] <= id (all 32
// lanes take part; 32-ary narrowing with one coalesced probe per lane per round).
ZG_D int warpFindPoint(const SolveParams& P, long long id, int lane) {
    int64_t lo = 0, hi = P.nPoints;   // invariant: walkStart[lo] <= id < walkStart[hi]
    while (hi - lo > 32) {
        int64_t stride = (hi - lo + 31) / 32;
        int64_t probe = lo + (int64_t)lane * stride;
        bool le = probe < hi && __ldg(P.walkStart + probe) <= id;
        unsigned b = __ballot_sync(kFull, le);
        int k = 31 - __clz(b);            // lane 0 always holds lo itself
        lo = lo + (int64_t)k * stride;
        hi = lo + stride < hi ? lo + stride : hi;
    }
    int64_t probe = lo + lane;
    bool le = probe < hi && __ldg(P.walkStart + probe) <= id;
    unsigned b = __ballot_sync(kFull, le);
    return (int)(lo + 31 - __clz(b));
}

template <int D, int SOLVER, bool SCREENED, bool BATCHED, bool COOP>
__global__ void __launch_bounds__(kWalkThreads, ZG_WALK_MIN_BLOCKS) walkKernel(const __grid_constant__ SolveParams P) {
    // The one-lane traversal stack lives in local memory (the L1-cached top entries are the
    // hot ones): shared memory holds only the warps' cooperative work areas, which leaves
    // the rest of the SM's 256 KB to L1 for the scene.  Measured on the GB300 against the
    // shared-memory stack: 2D Walk on Stars +4%, 2D Walk on Spheres +9%, 3D Robin +60%.
    extern __shared__ int dynStack[];
    int stackNode[kMaxStack];
    float stackKey[kMaxStack];
    TravStack S{stackNode, stackKey, 1, P.stackEntries};
    CoopWork* coopWork = reinterpret_cast<CoopWork*>(dynStack) + (threadIdx.x >> 5);
    using WalkerT = Walker<D, SOLVER, SCREENED, BATCHED, COOP>;
    WalkerT W(P, S);
    W.splitSlots = P.splitStack ? P.splitStack + ((size_t)blockIdx.x * blockDim.x + threadIdx.x) * 3 * kSplitStack : nullptr;
    const int lane = threadIdx.x & 31;
    const long long total = (long long)__ldg(P.walkStart + P.nPoints);
    bool active = false, exhausted = false;
    for (;;) {
        bool need = !active && !exhausted;
        unsigned m = __ballot_sync(kFull, need);
        if (m) {
            int leader = __ffs(m) - 1;
            unsigned long long base = 0;
            if (lane == leader) base = atomicAdd(P.counters + kCtrNext, (unsigned long long)__popc(m));
            base = __shfl_sync(kFull, base, leader);
            if ((long long)base < total) {
                int p0 = warpFindPoint(P, (long long)base, lane);
                if (need) {
                    long long id = (long long)base + __popc(m & ((1u << lane) - 1u));
                    if (id >= total) {
                        exhausted = true;
                    } else {
                        int p = p0;
                        while (__ldg(P.walkStart + p + 1) <= id) p++;   // walks of a point are contiguous
                        W.start(id, p);
                        active = true;
                    }
                }
            } else if (need) {
                exhausted = true;
            }
        }
        if (!__any_sync(kFull, active)) break;
        if (active) active = W.step();
        if constexpr (WalkerT::kCoopStar) {
            // Robin star radii of this round, one at a time with the whole warp
            unsigned qm = __ballot_sync(kFull, active && W.radiusPending);
            while (qm) {
                const int src = __ffs(qm) - 1;
                qm &= qm - 1;
                V<D> x;
#pragma unroll
                for (int i = 0; i < D; i++) x[i] = __shfl_sync(kFull, W.pt[i], src);
                const float maxR = __shfl_sync(kFull, W.distAbs, src);
                const bool flip = __shfl_sync(kFull, (int)W.flip, src) != 0;
                const float r = coopRobinStarRadius<D>(P.sc.reflecting, x, P.sc.ws.epsilon_shell_for_reflecting_boundary,
                                                       maxR, P.sc.ws.silhouette_precision, flip, *coopWork, lane, W.err);
                if (lane == src) W.setStarRadius(r);
            }
        }
        if constexpr (WalkerT::kCoopClosest) {
            // closest-point queries of this round, one at a time with the whole warp
            unsigned qm = __ballot_sync(kFull, active && W.queryPending);
            while (qm) {
                const int src = __ffs(qm) - 1;
                qm &= qm - 1;
                V<D> x;
#pragma unroll
                for (int i = 0; i < D; i++) x[i] = __shfl_sync(kFull, W.pt[i], src);
                float d;
                int slot;
                coopClosest<D>(P.sc.absorbing, x, *coopWork, lane, d, slot, W.err);
                if (lane == src) W.setClosest(d, slot);
            }
        }
    }
    // warp-reduce the counters, one atomic per warp
    unsigned long long v[4] = {W.steps, W.escaped, W.exceeded, W.rr};
#pragma unroll
    for (int k = 0; k < 4; k++)
        for (int o = 16; o > 0; o >>= 1) v[k] += __shfl_xor_sync(kFull, v[k], o);
    uint32_t e = W.err;
    for (int o = 16; o > 0; o >>= 1) e |= __shfl_xor_sync(kFull, e, o);
    if (lane == 0) {
        atomicAdd(P.counters + kCtrSteps, v[0]);
        if (v[1]) atomicAdd(P.counters + kCtrEscaped, v[1]);
        if (v[2]) atomicAdd(P.counters + kCtrExceeded, v[2]);
        if (v[3]) atomicAdd(P.counters + kCtrRR, v[3]);
        if (e) atomicOr(P.errorWord, e);
    }
}

// ------------------------------------------------------------------------- prepare
constexpr int kQueryThreads = 128;

template <int D>
__global__ void __launch_bounds__(kQueryThreads) prepareKernel(const __grid_constant__ SolveParams P) {
    extern __shared__ int dynStack[];
    TravStack S{dynStack + threadIdx.x, reinterpret_cast<float*>(dynStack + P.stackEntries * blockDim.x) + threadIdx.x,
                (int)blockDim.x, P.stackEntries};
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= P.nPoints) return;
    bool badScene;
    const SceneDesc& sc = sceneOfPoint(P, i, badScene);
    DevicePde<D> pde; pde.p = &sc.pde;
    const zgpu_walk_settings& ws = sc.ws;
    int eq = P.eq ? P.eq[i] : ZGPU_ESTIMATE_SOLUTION;
    int type = P.type ? P.type[i] : ZGPU_SAMPLE_IN_DOMAIN;
    int nPrev = P.statN[i];
    P.nPrev[i] = nPrev;
    P.accSum[i] = 0.0; P.accSq[i] = 0.0; P.accN[i] = 0; P.accLen[i] = 0; P.accSplits[i] = 0;
    if (P.accGrad) {
        for (int k = 0; k < D; k++) { P.accGrad[i * D + k] = 0.0; P.accGradSq[i * D + k] = 0.0; }
        P.accGradN[i] = 0;
        if (P.accFirstSrc) P.accFirstSrc[i] = 0.0;
        if (P.accDeriv) P.accDeriv[i] = 0.0;
    }
    bool hasPrev = nPrev > 0 && P.fsrPersistent;
    int flags = 0;
    long long count = 0;
    float dAbs = P.distAbs[i];
    bool aligned = P.aligned ? P.aligned[i] != 0 : false;
    if (P.solver == ZGPU_SOLVER_WALK_ON_STARS && ws.solve_double_sided && type == ZGPU_SAMPLE_ON_REFLECTING_BOUNDARY && aligned)
        flags |= kPointFlip;
    if (badScene) atomicOr(P.errorWord, kErrBadInput);
    if (eq == ZGPU_ESTIMATE_SOLUTION_AND_GRADIENT && !badScene && P.accGrad) {
        // estimateSolutionAndGradient (walk_on_spheres.h:422-430, walk_on_stars.h:670-684),
        // whatever the point's type (boundary value caching estimates normal derivatives at
        // boundary samples offset into the domain): first ball 0.99 x the distance to the
        // boundary; antithetic pairs halve the draws
        float dB = dAbs;
        if (P.solver == ZGPU_SOLVER_WALK_ON_STARS && sc.hasRefl) {
            float dR;
            if (P.distRefl) {
                dR = P.distRefl[i];
            } else {
                uint32_t err = 0;
                dR = closestPoint<D>(sc.reflecting, vload<D>(P.pt + (size_t)i * D), S, err).d;
                if (err) atomicOr(P.errorWord, err);
            }
            dB = fminf(dB, dR);
        }
        const int nw = max(P.nWalks[i], 0);
        count = nw == 0 ? 0 : (ws.use_gradient_antithetic_variates ? 2 * max(1, nw / 2) : nw);
        P.fsr[i] = kRadiusShrink * dB;
        if (count > 0 && P.fsr[i] > 0.0f) flags |= kPointGradient;
        P.pointFlags[i] = flags;
        P.walkStart[i] = count;
        return;
    }
    if (eq == ZGPU_ESTIMATE_SKIP || badScene) {
        count = 0;
    } else if (type == ZGPU_SAMPLE_ON_ABSORBING_BOUNDARY) {
        if (nPrev == 0) { flags |= kPointBoundaryValue; P.fsr[i] = 0.0f; }
        count = 0;
    } else {
        count = dAbs <= ws.epsilon_shell_for_absorbing_boundary ? 1 : max(P.nWalks[i], 0);
        if (!hasPrev) {
            float r;
            if (P.solver == ZGPU_SOLVER_WALK_ON_SPHERES) {
                r = dAbs;
            } else if (dAbs <= ws.epsilon_shell_for_absorbing_boundary || ws.steps_before_using_maximal_spheres == 0) {
                r = dAbs;
            } else if (type == ZGPU_SAMPLE_ON_REFLECTING_BOUNDARY && pde.hasNonZeroRobinCoeff(vload<D>(P.pt + (size_t)i * D))) {
                r = ws.epsilon_shell_for_reflecting_boundary;
            } else {
                uint32_t err = 0;
                V<D> x = vload<D>(P.pt + (size_t)i * D);
                r = sc.hasRefl ? starRadius<D>(sc.reflecting, x, ws.epsilon_shell_for_reflecting_boundary, dAbs,
                                              ws.silhouette_precision, (flags & kPointFlip) != 0, S, err)
                              : dAbs;
                if (sc.hasRefl && ws.epsilon_shell_for_reflecting_boundary <= dAbs)
                    r = fmaxf(kRadiusShrink * r, ws.epsilon_shell_for_reflecting_boundary);
                if (err) atomicOr(P.errorWord, err);
            }
            P.fsr[i] = r;
        }
    }
    P.pointFlags[i] = flags;
    P.walkStart[i] = count;
}

// ------------------------------------------------------------------------- finalize
template <int D>
__global__ void finalizeKernel(const __grid_constant__ SolveParams P) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= P.nPoints) return;
    bool badScene;
    const SceneDesc& sc = sceneOfPoint(P, i, badScene);
    DevicePde<D> pde; pde.p = &sc.pde;
    int flags = P.pointFlags[i];
    int n2 = P.accN[i];
    double mean2 = 0.0, m22 = 0.0;
    if (flags & kPointBoundaryValue) {
        float v = 0.0f;
        if (!sc.ws.ignore_absorbing_boundary_contribution) {
            bool aligned = sc.ws.solve_double_sided && P.aligned && P.aligned[i] != 0;
            v = pde.dirichlet(vload<D>(P.pt + (size_t)i * D), aligned);
        }
        n2 = 1; mean2 = v; m22 = 0.0;
    } else if (n2 > 0) {
        double s = P.accSum[i], q = P.accSq[i];
        mean2 = s / n2;
        m22 = fmax(0.0, q - s * mean2);
    }
    if (n2 > 0) {
        int n1 = P.nPrev[i];
        int nt = n1 + n2;
        if (n1 == 0) {
            P.statMean[i] = mean2;
            P.statM2[i] = m22;
        } else {
            double m1 = P.statMean[i];
            double delta = mean2 - m1;
            P.statMean[i] = m1 + delta * ((double)n2 / nt);
            P.statM2[i] = P.statM2[i] + m22 + delta * delta * ((double)n1 * (double)n2 / nt);
        }
        P.statN[i] = nt;
    }
    P.statLen[i] += P.accLen[i];
    P.statSplits[i] += P.accSplits[i];
    if (P.accGrad && P.statGradMean && P.statGradN) {
        const int g2 = P.accGradN[i];
        if (g2 > 0) {
            const int g1 = P.statGradN[i];
            const int gt = g1 + g2;
            for (int k = 0; k < D; k++) {
                const double s = P.accGrad[i * D + k], q = P.accGradSq[i * D + k];
                const double m2mean = s / g2, m2m2 = fmax(0.0, q - s * m2mean);
                if (g1 == 0) {
                    P.statGradMean[i * D + k] = m2mean;
                    if (P.statGradM2) P.statGradM2[i * D + k] = m2m2;
                } else {
                    const double m1 = P.statGradMean[i * D + k], delta = m2mean - m1;
                    P.statGradMean[i * D + k] = m1 + delta * ((double)g2 / gt);
                    if (P.statGradM2)
                        P.statGradM2[i * D + k] += m2m2 + delta * delta * ((double)g1 * (double)g2 / gt);
                }
            }
            P.statGradN[i] = gt;
        }
        if (P.accFirstSrc && P.statFirstSrc) P.statFirstSrc[i] += P.accFirstSrc[i];
        if (P.accDeriv && P.statDeriv) P.statDeriv[i] += P.accDeriv[i];
    }
}

// ------------------------------------------------------------------------- query kernels
template <int D>
__global__ void __launch_bounds__(kQueryThreads) closestKernel(BoundaryView b, int64_t n, const float* x, int computeSigned, float* pt, float* nrm,
                              float* dist, int* prim, unsigned int* errw) {
    extern __shared__ int dynStack[];
    TravStack S{dynStack + threadIdx.x, reinterpret_cast<float*>(dynStack + b.stackEntries * blockDim.x) + threadIdx.x,
                (int)blockDim.x, b.stackEntries};
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    uint32_t err = 0;
    V<D> q = vload<D>(x + (size_t)i * D);
    ClosestHit<D> h = closestPoint<D>(b, q, S, err);
    V<D> nn = vzero<D>();
    int idx = -1;
    float d = h.d;
    if (h.slot >= 0) {
        nn = primNormal<D>(loadPrim<D>(b, h.slot));
        idx = b.primIndex[h.slot];
        if (computeSigned && dot(q - h.pt, nn) < 0.0f) d = -d;
    }
    if (pt) vstore<D>(h.pt, pt + (size_t)i * D);
    if (nrm) vstore<D>(nn, nrm + (size_t)i * D);
    if (dist) dist[i] = d;
    if (prim) prim[i] = idx;
    if (err) atomicOr(errw, err);
}

template <int D>
__global__ void __launch_bounds__(kQueryThreads) intersectKernel(BoundaryView b, int64_t n, const float* o, const float* nrmIn, const float* dir,
                                const float* tmax, const int* onb, int* hit, float* pt, float* nrm, float* dist,
                                int* prim, unsigned int* errw) {
    extern __shared__ int dynStack[];
    TravStack S{dynStack + threadIdx.x, reinterpret_cast<float*>(dynStack + b.stackEntries * blockDim.x) + threadIdx.x,
                (int)blockDim.x, b.stackEntries};
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    uint32_t err = 0;
    V<D> origin = vload<D>(o + (size_t)i * D);
    if (onb && onb[i]) origin = offsetPoint<D>(origin, -vload<D>(nrmIn + (size_t)i * D));
    V<D> d = vload<D>(dir + (size_t)i * D);
    RayHit<D> h = intersectRay<D>(b, origin, d, tmax[i], false, S, err);
    bool ok = h.slot >= 0;
    hit[i] = ok;
    V<D> p = ok ? origin + h.t * d : vzero<D>();
    V<D> nn = ok ? primNormal<D>(loadPrim<D>(b, h.slot)) : vzero<D>();
    if (pt) vstore<D>(p, pt + (size_t)i * D);
    if (nrm) vstore<D>(nn, nrm + (size_t)i * D);
    if (dist) dist[i] = ok ? h.t : kFltMax;
    if (prim) prim[i] = ok ? b.primIndex[h.slot] : -1;
    if (err) atomicOr(errw, err);
}

template <int D>
__global__ void __launch_bounds__(kQueryThreads) countHitsKernel(BoundaryView b, int64_t n, const float* o, const float* dir, const float* tmax,
                                int* out, unsigned int* errw) {
    extern __shared__ int dynStack[];
    TravStack S{dynStack + threadIdx.x, reinterpret_cast<float*>(dynStack + b.stackEntries * blockDim.x) + threadIdx.x,
                (int)blockDim.x, b.stackEntries};
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    uint32_t err = 0;
    out[i] = countHits<D>(b, vload<D>(o + (size_t)i * D), vload<D>(dir + (size_t)i * D), tmax[i], S, err);
    if (err) atomicOr(errw, err);
}

template <int D>
__global__ void __launch_bounds__(kQueryThreads) starRadiusKernel(BoundaryView b, int64_t n, const float* x, const float* minR, const float* maxR,
                                 float prec, const int* flip, float* out, unsigned int* errw) {
    extern __shared__ int dynStack[];
    TravStack S{dynStack + threadIdx.x, reinterpret_cast<float*>(dynStack + b.stackEntries * blockDim.x) + threadIdx.x,
                (int)blockDim.x, b.stackEntries};
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    uint32_t err = 0;
    out[i] = starRadius<D>(b, vload<D>(x + (size_t)i * D), minR[i], maxR[i], prec, flip && flip[i], S, err);
    if (err) atomicOr(errw, err);
}

// Warp-cooperative versions of the closest-point and Robin star-radius queries (the walk
// kernel's coopClosest / coopRobinStarRadius): one warp answers one query at a time.
template <int D>
__global__ void __launch_bounds__(kQueryThreads) coopClosestKernel(BoundaryView b, int64_t n, const float* x,
                                                                   int computeSigned, float* pt, float* nrm,
                                                                   float* dist, int* prim, unsigned int* errw) {
    __shared__ CoopWork work[kQueryThreads / 32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int64_t stride = (int64_t)gridDim.x * (kQueryThreads / 32);
    uint32_t err = 0;
    for (int64_t i = (int64_t)blockIdx.x * (kQueryThreads / 32) + warp; i < n; i += stride) {
        const V<D> q = vload<D>(x + (size_t)i * D);
        float d;
        int slot;
        coopClosest<D>(b, q, work[warp], lane, d, slot, err);
        if (lane != 0) continue;
        V<D> cp = q, nn = vzero<D>();
        int idx = -1;
        if (slot >= 0) {
            const Prim<D> t = loadPrim<D>(b, slot);
            closestOnPrim(t, q, cp);
            nn = primNormal<D>(t);
            idx = b.primIndex[slot];
            if (computeSigned && dot(q - cp, nn) < 0.0f) d = -d;
        }
        if (pt) vstore<D>(cp, pt + (size_t)i * D);
        if (nrm) vstore<D>(nn, nrm + (size_t)i * D);
        if (dist) dist[i] = d;
        if (prim) prim[i] = idx;
    }
    if (err && (threadIdx.x & 31) == 0) atomicOr(errw, err);
}

template <int D>
__global__ void __launch_bounds__(kQueryThreads) coopStarRadiusKernel(BoundaryView b, int64_t n, const float* x,
                                                                      const float* minR, const float* maxR, float prec,
                                                                      const int* flip, float* out, unsigned int* errw) {
    __shared__ CoopWork work[kQueryThreads / 32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int64_t stride = (int64_t)gridDim.x * (kQueryThreads / 32);
    uint32_t err = 0;
    for (int64_t i = (int64_t)blockIdx.x * (kQueryThreads / 32) + warp; i < n; i += stride) {
        const float r = coopRobinStarRadius<D>(b, vload<D>(x + (size_t)i * D), minR[i], maxR[i], prec,
                                               flip && flip[i], work[warp], lane, err);
        if (lane == 0) out[i] = r;
    }
    if (err && lane == 0) atomicOr(errw, err);
}

template <int D>
__global__ void __launch_bounds__(kQueryThreads) occludedKernel(BoundaryView b, int64_t n, const float* xi, const float* xj, const float* ni,
                               const float* nj, const int* oi, const int* oj, int* out, unsigned int* errw) {
    extern __shared__ int dynStack[];
    TravStack S{dynStack + threadIdx.x, reinterpret_cast<float*>(dynStack + b.stackEntries * blockDim.x) + threadIdx.x,
                (int)blockDim.x, b.stackEntries};
    int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    uint32_t err = 0;
    V<D> p1 = vload<D>(xi + (size_t)k * D), p2 = vload<D>(xj + (size_t)k * D);
    if (oi && oi[k]) p1 = offsetPoint<D>(p1, -vload<D>(ni + (size_t)k * D));
    if (oj && oj[k]) p2 = offsetPoint<D>(p2, -vload<D>(nj + (size_t)k * D));
    V<D> s = p2 - p1;
    float l = len(s);
    int occ = 0;
    if (l > 0.0f) occ = intersectRay<D>(b, p1, (1.0f / l) * s, l, true, S, err).slot >= 0;
    out[k] = occ;
    if (err) atomicOr(errw, err);
}

template <int D>
__global__ void sampleKernel(BoundaryView b, int64_t n, const float* x, const float* r, const float* u, int* found,
                             float* pt, float* nrm, float* pdf) {
    int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    V<D> p, nn;
    float pp = 0.0f;
    float uu[D];
    for (int i = 0; i < D; i++) uu[i] = u[(size_t)k * D + i];
    bool ok = sampleBoundary<D>(b, vload<D>(x + (size_t)k * D), r[k], uu, p, nn, pp);
    if (!ok) { p = vzero<D>(); nn = vzero<D>(); pp = 0.0f; }
    found[k] = ok;
    vstore<D>(p, pt + (size_t)k * D);
    vstore<D>(nn, nrm + (size_t)k * D);
    pdf[k] = pp;
}

inline unsigned gridFor(int64_t n, int t) { return (unsigned)((n + t - 1) / t); }

}  // namespace detail


inline size_t smemBytes(int stackEntries, int threads) { return (size_t)stackEntries * threads * 8; }
// walk kernel: one CoopWork per warp in cooperative mode (its traversal stacks are local)
inline size_t walkSmemBytes(const SolveParams& p, int threads) {
    return (p.coop || p.coopStar) ? sizeof(CoopWork) * (size_t)(threads / 32) : 0;
}

// walk kernel launchers, explicitly instantiated per (dimension, solver) in zgpu_walk_<D>d_<solver>.cu
template <int D, int SOLVER>
struct WalkLaunch {
    // the walk kernel for a solve: screened or not, batched (a scene table) or one scene,
    // warp-cooperative queries or one lane per query; nullptr for a combination not built
    static const void* kernel(bool screened, bool batched, bool coop) {
        if (batched) {
            if (coop) return nullptr;
            return screened ? (const void*)detail::walkKernel<D, SOLVER, true, true, false>
                            : (const void*)detail::walkKernel<D, SOLVER, false, true, false>;
        }
        if (coop) return screened ? (const void*)detail::walkKernel<D, SOLVER, true, false, true>
                                  : (const void*)detail::walkKernel<D, SOLVER, false, false, true>;
        return screened ? (const void*)detail::walkKernel<D, SOLVER, true, false, false>
                        : (const void*)detail::walkKernel<D, SOLVER, false, false, false>;
    }
    static const void* kernelFor(const SolveParams& p) {
        const bool batched = p.sceneId != nullptr;
        const bool screened = batched ? p.batchScreened != 0 : p.sc.pde.absorption_coeff > 0.0f;
        return kernel(screened, batched, p.coop || p.coopStar);
    }
    static cudaError_t walk(const SolveParams& p, int blocks, int threads, cudaStream_t s) {
        const void* f = kernelFor(p);
        if (!f) return cudaErrorNotSupported;
        const size_t smem = walkSmemBytes(p, threads);
        cudaError_t e = cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
        void* args[] = {const_cast<SolveParams*>(&p)};
        return cudaLaunchKernel(f, dim3(blocks), dim3(threads), args, smem, s);
    }
    static int maxBlocksPerSM(const SolveParams& p, int threads, size_t smem) {
        int n = 0;
        const void* f = kernelFor(p);
        if (!f) return 1;
        cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, f, threads, smem) != cudaSuccess) return 1;
        return n > 0 ? n : 1;
    }
};

// per-dimension launchers of the bookkeeping and query kernels, instantiated in zgpu_kernels{2,3}.cu
template <typename K>
inline void allowStack(K kernel) {
    cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smemBytes(kMaxStack, detail::kQueryThreads));
}

template <int D>
struct Launch {
    static cudaError_t prepare(const SolveParams& p, cudaStream_t s) {
        if (p.nPoints == 0) return cudaSuccess;
        allowStack(detail::prepareKernel<D>);
        detail::prepareKernel<D><<<detail::gridFor(p.nPoints, detail::kQueryThreads), detail::kQueryThreads, smemBytes(p.stackEntries, detail::kQueryThreads), s>>>(p);
        return cudaGetLastError();
    }
    static cudaError_t finalize(const SolveParams& p, cudaStream_t s) {
        if (p.nPoints == 0) return cudaSuccess;
        detail::finalizeKernel<D><<<detail::gridFor(p.nPoints, 256), 256, 0, s>>>(p);
        return cudaGetLastError();
    }
    static cudaError_t closest(const BoundaryView& b, int64_t n, const float* x, int computeSigned, float* pt, float* nrm,
                               float* dist, int* prim, unsigned int* err, cudaStream_t s) {
        if (n == 0) return cudaSuccess;
        allowStack(detail::closestKernel<D>);
        detail::closestKernel<D><<<detail::gridFor(n, detail::kQueryThreads), detail::kQueryThreads, smemBytes(b.stackEntries, detail::kQueryThreads), s>>>(b, n, x, computeSigned, pt, nrm, dist, prim, err);
        return cudaGetLastError();
    }
    static cudaError_t intersect(const BoundaryView& b, int64_t n, const float* o, const float* nrmIn, const float* dir,
                                 const float* tmax, const int* onb, int* hit, float* pt, float* nrm, float* dist, int* prim,
                                 unsigned int* err, cudaStream_t s) {
        if (n == 0) return cudaSuccess;
        allowStack(detail::intersectKernel<D>);
        detail::intersectKernel<D><<<detail::gridFor(n, detail::kQueryThreads), detail::kQueryThreads, smemBytes(b.stackEntries, detail::kQueryThreads), s>>>(b, n, o, nrmIn, dir, tmax, onb, hit, pt, nrm, dist, prim, err);
        return cudaGetLastError();
    }
    static cudaError_t countHits(const BoundaryView& b, int64_t n, const float* o, const float* dir, const float* tmax,
                                 int* out, unsigned int* err, cudaStream_t s) {
        if (n == 0) return cudaSuccess;
        allowStack(detail::countHitsKernel<D>);
        detail::countHitsKernel<D><<<detail::gridFor(n, detail::kQueryThreads), detail::kQueryThreads, smemBytes(b.stackEntries, detail::kQueryThreads), s>>>(b, n, o, dir, tmax, out, err);
        return cudaGetLastError();
    }
    static cudaError_t starRadius(const BoundaryView& b, int64_t n, const float* x, const float* minR, const float* maxR,
                                  float prec, const int* flip, float* out, unsigned int* err, cudaStream_t s) {
        if (n == 0) return cudaSuccess;
        allowStack(detail::starRadiusKernel<D>);
        detail::starRadiusKernel<D><<<detail::gridFor(n, detail::kQueryThreads), detail::kQueryThreads, smemBytes(b.stackEntries, detail::kQueryThreads), s>>>(b, n, x, minR, maxR, prec, flip, out, err);
        return cudaGetLastError();
    }
    static cudaError_t closestCoop(const BoundaryView& b, int64_t n, const float* x, int computeSigned, float* pt,
                                   float* nrm, float* dist, int* prim, unsigned int* err, cudaStream_t s) {
        if (n == 0) return cudaSuccess;
        detail::coopClosestKernel<D><<<detail::gridFor(n, detail::kQueryThreads / 32), detail::kQueryThreads, 0, s>>>(
            b, n, x, computeSigned, pt, nrm, dist, prim, err);
        return cudaGetLastError();
    }
    static cudaError_t starRadiusCoop(const BoundaryView& b, int64_t n, const float* x, const float* minR,
                                      const float* maxR, float prec, const int* flip, float* out, unsigned int* err,
                                      cudaStream_t s) {
        if (n == 0) return cudaSuccess;
        detail::coopStarRadiusKernel<D><<<detail::gridFor(n, detail::kQueryThreads / 32), detail::kQueryThreads, 0, s>>>(
            b, n, x, minR, maxR, prec, flip, out, err);
        return cudaGetLastError();
    }
    static cudaError_t occluded(const BoundaryView& b, int64_t n, const float* xi, const float* xj, const float* ni,
                                const float* nj, const int* oi, const int* oj, int* out, unsigned int* err, cudaStream_t s) {
        if (n == 0) return cudaSuccess;
        allowStack(detail::occludedKernel<D>);
        detail::occludedKernel<D><<<detail::gridFor(n, detail::kQueryThreads), detail::kQueryThreads, smemBytes(b.stackEntries, detail::kQueryThreads), s>>>(b, n, xi, xj, ni, nj, oi, oj, out, err);
        return cudaGetLastError();
    }
    static cudaError_t sample(const BoundaryView& b, int64_t n, const float* x, const float* r, const float* u, int* found,
                              float* pt, float* nrm, float* pdf, cudaStream_t s) {
        if (n == 0) return cudaSuccess;
        detail::sampleKernel<D><<<detail::gridFor(n, detail::kQueryThreads), detail::kQueryThreads, smemBytes(b.stackEntries, detail::kQueryThreads), s>>>(b, n, x, r, u, found, pt, nrm, pdf);
        return cudaGetLastError();
    }
};

}  // namespace zg
