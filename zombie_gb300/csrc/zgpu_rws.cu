// zgpu_rws.cu -- reverse Walk on Stars (point_estimation/reverse_walk_on_stars.h) with the
// splat of variance_reduction/reverse_walk_solver.h.
//
// Each lane walks the samples of a grid-stride sequence, one walk step per loop iteration.
// After the star radius of a step is known, the warp splats every pending lane's ball in turn
// with all 32 lanes (a ball holds up to thousands of evaluation points, a lane's own walk
// would leave the other 31 idle): a 4-wide BVH over the evaluation points, built on the
// device for the call, is traversed warp-uniformly, and a point inside the ball, not on the
// absorbing boundary and visible from the walk position (line of sight against the
// reflecting boundary) receives alpha * throughput * G(r) / pdf times the sample's
// contribution by FP64 atomic add into its running sums.  Split states of the weight window
// wait in a per-lane FIFO, processed in the reference's queue order, all on the sample's one
// pcg32 stream.
#include <cfloat>

#include "zgpu_internal.h"

namespace zg {
namespace {

constexpr int kRwsThreads = 128;
constexpr int kRwsQueue = 8;
constexpr int kPointStack = 64;

// outsideBoundingDomain (core/geometric_queries.h:373-379)
template <int D>
ZG_D bool outsideDomainBox(const SceneDesc& sc, const V<D>& x) {
#pragma unroll
    for (int i = 0; i < D; i++)
        if (x[i] < sc.domainMin[i] || x[i] > sc.domainMax[i]) return true;
    return false;
}

template <int D>
struct RevState {
    V<D> pt, nrm, prevDir;
    float prevDist, thr;
    int wlen;
    bool onRefl;
};

// splatContribution (reverse_walk_solver.h:236-302) of one ball with the whole warp: every
// lane traverses the evaluation points' tree the same way (warp-uniform), child boxes that lie
// inside the ball hand over their whole contiguous range of sorted points, and the points of
// each range are shared out 32 at a time.  Per point: not on the absorbing boundary, line of
// sight from the ball's centre (when the reflecting boundary reaches into the ball), then
// alpha * throughput * G / pdf * contribution by FP64 atomic add.
struct Ball {
    float R, thr, pdf, contrib;
    float visible2;        // squared distance within which no reflecting point lies (no test needed)
    int group;
    bool onRefl, toPoisson, needTest, yukawa;
};

template <int D, bool SCREENED>
ZG_D void coopSplat(const RwsParams& P, const V<D>& x, const V<D>& nrm, const Ball& b, float sqrtLambda, int lane,
                    TravStack& S, uint32_t& err) {
    Greens<D, SCREENED> g;
    g.sqrtLambda = sqrtLambda;
    g.yukawa = b.yukawa;
    g.update(x, b.R);
    BoundaryView t;
    t.nodes = P.evalNodes;
    const float R2 = b.R * b.R;
    const float alpha = b.onRefl ? 2.0f : 1.0f;
    int stack[kPointStack];
    int sp = 0;
    int node = 0;
    for (int guard = 0; guard < (1 << 26); guard++) {
        WideNode<D> w;
        loadNode<D>(t, node, w);
#pragma unroll 1
        for (int k = 0; k < 4; k++) {
            const int c = w.child[k];
            if (c == kEmptyChild || !(boxDist2<D>(w, k, x) < R2)) continue;
            const bool inside = boxMaxDist2<D>(w, k, x) < R2;
            if (!inside && !isLeaf(c)) {
                if (sp < kPointStack) stack[sp++] = c;
                else err |= kErrStackOverflow;
                continue;
            }
            const int2 rg = __ldg(P.evalRanges + (size_t)node * 4 + k);
            for (int base = rg.x; base < rg.x + rg.y; base += 32) {
                const int j = base + lane;
                if (j >= rg.x + rg.y) continue;
                const int e = __ldg(P.evalOrder + j);
                const V<D> xe = vload<D>(P.evalPt + (size_t)e * D);
                const float d2 = len2(xe - x);
                if (!(d2 < R2)) continue;
                const int te = P.evalType ? P.evalType[e] : ZGPU_SAMPLE_IN_DOMAIN;
                if (te == ZGPU_SAMPLE_ON_ABSORBING_BOUNDARY) continue;      // not splatted
                if (b.needTest && !(d2 < b.visible2)) {
                    // intersectsWithReflectingBoundary: the segment between the points, each
                    // offset off the reflecting boundary when it lies on it (a segment shorter
                    // than the distance to the reflecting boundary cannot cross it)
                    const V<D> p1 = b.onRefl ? offsetPoint<D>(x, -nrm) : x;
                    V<D> p2 = xe;
                    if (te == ZGPU_SAMPLE_ON_REFLECTING_BOUNDARY && P.evalNormal)
                        p2 = offsetPoint<D>(xe, -vload<D>(P.evalNormal + (size_t)e * D));
                    const V<D> seg = p2 - p1;
                    const float sl = len(seg);
                    if (sl > 0.0f && intersectRay<D>(P.sc.reflecting, p1, (1.0f / sl) * seg, sl, true, S, err).slot >= 0)
                        continue;
                }
                const float r = fmaxf(P.radiusClamp, sqrtf(d2));
                float G = g.evaluate(r);
                if (P.regularization > 0.0f) G *= kernelRegularizationG<D>(r / P.regularization);
                float weight = alpha * b.thr * G / b.pdf;
                if (b.group <= ZGPU_RWS_ABSORBING_ALIGNED) weight /= P.normalOffset;
                atomicAdd(P.totals + (size_t)e * ZGPU_RWS_TOTALS + b.group, (double)(weight * b.contrib));
                if (b.toPoisson) atomicAdd(P.totals + (size_t)e * ZGPU_RWS_TOTALS + ZGPU_RWS_POISSON_KERNEL, (double)weight);
            }
        }
        if (sp == 0) break;
        node = stack[--sp];
    }
}

// applyWeightWindow (reverse_walk_on_stars.h:230-263): split states join the FIFO
template <int D>
ZG_D bool weightWindow(const zgpu_walk_settings& ws, Pcg32& rng, RevState<D>& s, RevState<D>* q, int qh, int& qn,
                       uint32_t& err) {
    if (s.thr > ws.splitting_threshold) {
        float left = s.thr - ws.splitting_threshold;
        s.thr = ws.splitting_threshold;
        RevState<D> split = s;
        split.wlen = 0;
        while (left > ws.splitting_threshold) {
            left -= ws.splitting_threshold;
            if (qn < kRwsQueue) q[(qh + qn++) % kRwsQueue] = split;
            else err |= kErrSplitOverflow;
        }
        if (rng.uniform() < left / ws.splitting_threshold) {
            if (qn < kRwsQueue) q[(qh + qn++) % kRwsQueue] = split;
            else err |= kErrSplitOverflow;
        }
    } else if (s.thr < ws.russian_roulette_threshold) {
        const float survival = s.thr / ws.russian_roulette_threshold;
        if (survival < rng.uniform()) { s.thr = 0.0f; return true; }
        s.thr = ws.russian_roulette_threshold;
    }
    return false;
}

template <int D, bool SCREENED>
__global__ void __launch_bounds__(kRwsThreads) reverseWalkKernel(const __grid_constant__ RwsParams P) {
    extern __shared__ int dynStack[];
    TravStack S{dynStack + threadIdx.x, reinterpret_cast<float*>(dynStack + P.stackEntries * blockDim.x) + threadIdx.x,
                (int)blockDim.x, P.stackEntries};
    const zgpu_walk_settings& ws = P.sc.ws;
    DevicePde<D> pde;
    pde.p = &P.sc.pde;
    const bool ds = ws.solve_double_sided != 0;
    const float sqrtLambda = sqrtf(fmaxf(P.sc.pde.absorption_coeff, 0.0f));
    const bool yukawa0 = P.sc.pde.absorption_coeff > 0.0f && ws.steps_before_applying_tikhonov == 0;
    const int lane = threadIdx.x & 31;
    uint32_t err = 0;
    unsigned long long steps = 0, walks = 0;
    // this lane's sample (grid-stride) and walk state; the walks advance one step per
    // iteration so that the warp can splat every lane's ball together
    int64_t nextSample = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    bool hasSample = false, haveState = false;
    int states = 0, group = 0;
    bool aligned = false, toPoisson = false;
    float pdf = 1.0f, contrib = 0.0f, dist = FLT_MAX;
    Pcg32 rng;
    rng.state = 0; rng.inc = 1;
    RevState<D> s;
    s.pt = s.nrm = s.prevDir = vzero<D>();
    s.prevDist = 0.0f; s.thr = 0.0f; s.wlen = 0; s.onRefl = false;
    RevState<D> q[kRwsQueue];
    int qh = 0, qn = 0;
    Greens<D, SCREENED> g;
    g.sqrtLambda = sqrtLambda;
    g.yukawa = yukawa0;
    for (long long iter = 0; iter < (1ll << 40); iter++) {
        // the lane's next walk state: a split state of its sample, or a new sample
        if (!haveState && hasSample && qn > 0) {
            if (states < 64) {
                s = q[qh];
                qh = (qh + 1) % kRwsQueue;
                qn--;
                states++;
                g.yukawa = yukawa0;
                dist = P.sc.hasAbs ? closestPoint<D>(P.sc.absorbing, s.pt, S, err).d : FLT_MAX;
                haveState = true;
            } else {
                err |= kErrBudget;              // bounds the splits of one sample
                qn = 0;
            }
        }
        if (!haveState && nextSample < P.nSamples) {
            const int64_t i = nextSample;
            nextSample += stride;
            const int type = P.type[i];
            aligned = P.aligned ? P.aligned[i] != 0 : false;
            pdf = P.pdf[i];
            contrib = P.contribution[i];
            if (type == ZGPU_SAMPLE_ON_ABSORBING_BOUNDARY) group = aligned ? ZGPU_RWS_ABSORBING_ALIGNED : ZGPU_RWS_ABSORBING;
            else if (type == ZGPU_SAMPLE_ON_REFLECTING_BOUNDARY) group = aligned ? ZGPU_RWS_REFLECTING_ALIGNED : ZGPU_RWS_REFLECTING;
            else group = ZGPU_RWS_SOURCE;
            toPoisson = P.selfNormalize && group == ZGPU_RWS_ABSORBING;
            rng.seed(P.seed[i], P.stream);
            walks++;
            // the walk's initial state (reverse_walk_on_stars.h:121-138)
            s.pt = vload<D>(P.pt + (size_t)i * D);
            s.nrm = vload<D>(P.normal + (size_t)i * D);
            s.onRefl = type == ZGPU_SAMPLE_ON_REFLECTING_BOUNDARY;
            s.prevDir = (ds && s.onRefl && aligned) ? -s.nrm : s.nrm;
            s.prevDist = FLT_MAX;
            s.thr = 1.0f;
            s.wlen = 0;
            qh = qn = 0;
            states = 1;
            g.yukawa = yukawa0;
            dist = P.distAbs[i];
            hasSample = haveState = true;
        }
        if (!__any_sync(0xffffffffu, haveState)) break;
        // step, first part (reverse_walk_on_stars.h:265-309): termination, star radius
        bool pending = false;
        Ball b;
        b.R = 0.0f; b.thr = s.thr; b.pdf = pdf; b.contrib = contrib; b.group = group;
        b.onRefl = s.onRefl; b.toPoisson = toPoisson; b.needTest = false; b.yukawa = g.yukawa;
        b.visible2 = 0.0f;
        if (haveState) {
            if (!(dist > ws.epsilon_shell_for_absorbing_boundary)) {
                haveState = false;                                              // reached the boundary
            } else {
                steps++;
                bool flip = false;
                if (ds && s.onRefl && s.prevDist > 0.0f && dot(s.prevDir, s.nrm) < 0.0f) {
                    s.nrm = -s.nrm;
                    flip = true;
                }
                float R;
                if (ws.steps_before_using_maximal_spheres <= s.wlen) {
                    R = dist;
                } else if (s.onRefl && pde.hasNonZeroRobinCoeff(s.pt)) {
                    R = ws.epsilon_shell_for_reflecting_boundary;
                } else {
                    R = P.sc.hasRefl ? starRadius<D>(P.sc.reflecting, s.pt, ws.epsilon_shell_for_reflecting_boundary,
                                                     dist, ws.silhouette_precision, flip, S, err)
                                     : dist;
                    if (ws.epsilon_shell_for_reflecting_boundary <= dist)
                        R = fmaxf(kRadiusShrink * R, ws.epsilon_shell_for_reflecting_boundary);
                }
                g.update(s.pt, R);
                b.R = R;
                b.onRefl = s.onRefl;
                b.yukawa = g.yukawa;
                // line of sight needs testing only when the reflecting boundary reaches into the
                // ball (segments inside a ball no reflecting point enters cannot cross it), and
                // then only for points farther than the closest reflecting point (0.1% margin)
                if (P.sc.hasRefl) {
                    const float dRefl = s.onRefl ? 0.0f : closestPoint<D>(P.sc.reflecting, s.pt, S, err).d;
                    b.needTest = s.onRefl || dRefl < R;
                    b.visible2 = b.needTest ? (0.999f * dRefl) * (0.999f * dRefl) : 0.0f;
                }
                pending = true;
            }
        }
        // the warp splats each pending lane's ball together
        unsigned pm = __ballot_sync(0xffffffffu, pending);
        while (pm) {
            const int src = __ffs(pm) - 1;
            pm &= pm - 1;
            V<D> x, n;
#pragma unroll
            for (int i = 0; i < D; i++) {
                x[i] = __shfl_sync(0xffffffffu, s.pt[i], src);
                n[i] = __shfl_sync(0xffffffffu, s.nrm[i], src);
            }
            Ball bb;
            bb.R = __shfl_sync(0xffffffffu, b.R, src);
            bb.thr = __shfl_sync(0xffffffffu, b.thr, src);
            bb.pdf = __shfl_sync(0xffffffffu, b.pdf, src);
            bb.contrib = __shfl_sync(0xffffffffu, b.contrib, src);
            bb.visible2 = __shfl_sync(0xffffffffu, b.visible2, src);
            bb.group = __shfl_sync(0xffffffffu, b.group, src);
            const int flags = __shfl_sync(0xffffffffu, (int)b.onRefl | ((int)b.toPoisson << 1) | ((int)b.needTest << 2) |
                                                           ((int)b.yukawa << 3), src);
            bb.onRefl = flags & 1; bb.toPoisson = (flags >> 1) & 1; bb.needTest = (flags >> 2) & 1; bb.yukawa = (flags >> 3) & 1;
            coopSplat<D, SCREENED>(P, x, n, bb, sqrtLambda, lane, S, err);
        }
        if (!pending) continue;
        // step, second part (reverse_walk_on_stars.h:314-390): direction, intersection,
        // throughput, weight window
        V<D> dir = sampleSphere<D>(rng);
        if (s.onRefl && dot(s.nrm, dir) > 0.0f) dir = -dir;
        const V<D> origin = s.onRefl ? offsetPoint<D>(s.pt, -s.nrm) : s.pt;
        V<D> hitPt = origin + b.R * dir, hitN = vzero<D>();
        float hitDist = b.R;
        bool hit = false;
        if (P.sc.hasRefl) {
            RayHit<D> h = intersectRay<D>(P.sc.reflecting, origin, dir, b.R, false, S, err);
            if (h.slot >= 0) {
                hit = true;
                hitDist = h.t;
                hitPt = origin + h.t * dir;
                hitN = primNormal<D>(loadPrim<D>(P.sc.reflecting, h.slot));
            }
        }
        s.prevDist = hitDist;
        s.prevDir = dir;
        s.pt = hitPt;
        s.nrm = hitN;
        s.onRefl = hit;
        // computeWalkStepThroughput (reverse_walk_on_stars.h:199-228)
        float stepThr;
        if (s.onRefl && s.prevDist > kFltEps) {
            float kappa = 0.0f;
            V<D> nn = s.nrm;
            if (!P.sc.pde.are_robin_conditions_pure_neumann) {
                bool f2 = false;
                if (ds) { f2 = dot(s.prevDir, s.nrm) < 0.0f; if (f2) nn = -nn; }
                kappa = pde.robinCoeff(s.pt, ds && f2);
            }
            const float refl = g.reflectance(s.prevDist, s.prevDir, nn, kappa);
            stepThr = fminf(fmaxf(refl, 0.0f), P.sc.pde.are_robin_coeffs_nonnegative ? 1.0f : 2.0f);
        } else {
            stepThr = g.directionSampledPoissonKernel(s.pt);
        }
        s.thr *= stepThr;
        if ((!s.onRefl && outsideDomainBox<D>(P.sc, s.pt)) || weightWindow<D>(ws, rng, s, q, qh, qn, err)) {
            haveState = false;                                                  // escaped / roulette
            continue;
        }
        s.wlen++;
        if (s.wlen >= ws.max_walk_length) { haveState = false; continue; }
        if (P.sc.pde.absorption_coeff > 0.0f && ws.steps_before_applying_tikhonov == s.wlen) g.yukawa = true;
        dist = P.sc.hasAbs ? closestPoint<D>(P.sc.absorbing, s.pt, S, err).d : FLT_MAX;
    }
    // warp-reduce the counters, one atomic per warp
    for (int o = 16; o > 0; o >>= 1) {
        steps += __shfl_xor_sync(0xffffffffu, steps, o);
        walks += __shfl_xor_sync(0xffffffffu, walks, o);
        err |= __shfl_xor_sync(0xffffffffu, err, o);
    }
    if (lane == 0) {
        if (steps) atomicAdd(P.counters + 0, steps);
        if (walks) atomicAdd(P.counters + 1, walks);
        if (err) atomicOr(P.errorWord, err);
    }
}

}  // namespace

cudaError_t launchReverseWalks(int D, bool screened, const RwsParams& p, int blocks, cudaStream_t s) {
    if (p.nSamples == 0) return cudaSuccess;
    const size_t smem = (size_t)p.stackEntries * kRwsThreads * 8;
    const void* f = D == 2 ? (screened ? (const void*)reverseWalkKernel<2, true> : (const void*)reverseWalkKernel<2, false>)
                           : (screened ? (const void*)reverseWalkKernel<3, true> : (const void*)reverseWalkKernel<3, false>);
    cudaError_t e = cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    void* args[] = {const_cast<RwsParams*>(&p)};
    return cudaLaunchKernel(f, dim3(blocks), dim3(kRwsThreads), args, smem, s);
}

}  // namespace zg
