// oracle.cpp -- TEST INFRASTRUCTURE, NOT PRODUCT CODE (see oracle_core.h).
//
// C entry points of the CPU oracle for ctypes (tests/, smoke(), bench.py CPU baseline).
// Mirrors the product C ABI shapes (include/zgpu.h) so tests can call both the same way.
#include <chrono>
#include <cstdio>
#include "oracle_walk.h"
#include "oracle_cache.h"
#include "oracle_bvc.h"
#include "oracle_rws.h"

using namespace orc;

namespace {

struct Handle {
    int dim = 2;
    void* b = nullptr;
};

std::atomic<uint64_t> gCounters[15];

// moves this thread's traversal counters into the global totals
void flushCounters() {
    Counters& c = counters();
    for (int k = 0; k < 5; k++) {
        gCounters[k] += c.calls[k]; gCounters[5 + k] += c.nodes[k]; gCounters[10 + k] += c.prims[k];
        c.calls[k] = c.nodes[k] = c.prims[k] = 0;
    }
}

template <int D>
Boundary<D>* makeBoundary(const float* pos, int nV, const int* idx, int nP, int kind, const float* kmin,
                          const float* kmax, int doubleSided, float silPrec, int useBvh) {
    Boundary<D>* b = new Boundary<D>();
    b->kind = kind;
    b->pos.resize(nV);
    for (int i = 0; i < nV; i++) b->pos[i] = load<D>(pos + (size_t)i * D);
    b->idx.resize(nP);
    for (int i = 0; i < nP; i++) for (int k = 0; k < D; k++) b->idx[i][k] = idx[(size_t)i * D + k];
    b->kmin.assign(nP, 0.0f);
    b->kmax.assign(nP, 0.0f);
    if (kind == ZGPU_BOUNDARY_ROBIN && kmin && kmax) {
        for (int i = 0; i < nP; i++) { b->kmin[i] = kmin[i]; b->kmax[i] = kmax[i]; }
    }
    if (kind == ZGPU_BOUNDARY_ABSORBING) {
        for (int i = 0; i < nP; i++) { b->kmin[i] = kMaxFloat; b->kmax[i] = kMaxFloat; }
    }
    b->buildAdjacency(doubleSided != 0, silPrec);
    b->useBvh = useBvh != 0;
    b->buildBvh();
    b->buildCones();
    b->buildFeatureTree();
    return b;
}

template <int D>
void solveImpl(int solver, const zgpu_geometric_queries* gq, const zgpu_pde* pde, const zgpu_walk_settings* ws,
               const zgpu_sample_points* pts, zgpu_sample_statistics* st, int nThreads, uint64_t* stepsOut) {
    Queries<D> q;
    q.absorbing = gq->absorbing ? (const Boundary<D>*)((Handle*)gq->absorbing)->b : nullptr;
    q.reflecting = gq->reflecting ? (const Boundary<D>*)((Handle*)gq->reflecting)->b : nullptr;
    for (int i = 0; i < D; i++) { q.domainMin[i] = gq->domain_min[i]; q.domainMax[i] = gq->domain_max[i]; }
    int64_t n = pts->n;
    std::atomic<int64_t> next{0};
    std::atomic<uint64_t> steps{0};
    auto work = [&]() {
        uint64_t localSteps = 0;
        while (true) {
            int64_t begin = next.fetch_add(16);
            if (begin >= n) break;
            int64_t end = std::min(n, begin + 16);
            for (int64_t i = begin; i < end; i++) {
                int eq = pts->estimation_quantity ? pts->estimation_quantity[i] : ZGPU_ESTIMATE_SOLUTION;
                if (eq == ZGPU_ESTIMATE_SKIP) continue;
                Solver<D> s{q, Pde<D>{pde}, *ws};
                int nPrev = st->n_solution_estimates[i];
                s.streamBase = (uint64_t)nPrev;
                Vec<D> p = load<D>(pts->pt + i * D);
                Vec<D> nrm = pts->normal ? load<D>(pts->normal + i * D) : Vec<D>();
                int type = pts->type ? pts->type[i] : ZGPU_SAMPLE_IN_DOMAIN;
                bool aligned = pts->estimate_normal_aligned ? pts->estimate_normal_aligned[i] != 0 : false;
                float fsr = pts->first_sphere_radius ? pts->first_sphere_radius[i] : 0.0f;
                PointStats ps;
                GradStats gs;
                const bool gradient = eq == ZGPU_ESTIMATE_SOLUTION_AND_GRADIENT &&
                                      st->gradient_mean && st->n_gradient_estimates;
                if (gradient) {
                    float dB = pts->dist_to_absorbing[i];
                    if (solver == ZGPU_SOLVER_WALK_ON_STARS && q.hasNonEmptyReflectingBoundary()) {
                        float dR;
                        if (pts->dist_to_reflecting) dR = pts->dist_to_reflecting[i];
                        else { Vec<D> cp, cn; int pi; q.reflecting->closestPoint(p, cp, cn, dR, pi); }
                        dB = std::min(dB, dR);
                    }
                    const bool cv = ws->use_gradient_control_variates && nPrev > 0;
                    const float cvB = cv ? (float)st->solution_mean[i] : 0.0f;
                    const float cvS = (cv && st->total_first_source_contribution)
                                          ? (float)(st->total_first_source_contribution[i] / (double)nPrev) : 0.0f;
                    Vec<D> dirD;
                    if (pts->direction_for_derivative) dirD = load<D>(pts->direction_for_derivative + i * D);
                    else dirD[0] = 1.0f;
                    s.gradEstimate(solver, p, dB, pts->n_walks[i], pts->seed[i], nPrev, cvB, cvS, dirD, ps, gs);
                    fsr = 0.99f * dB;
                } else if (solver == ZGPU_SOLVER_WALK_ON_SPHERES)
                    s.wosEstimate(p, type, pts->dist_to_absorbing[i], pts->n_walks[i], pts->seed[i], nPrev > 0, aligned, fsr, ps);
                else
                    s.wostEstimate(p, nrm, type, pts->dist_to_absorbing[i], pts->n_walks[i], pts->seed[i], nPrev > 0, aligned, fsr, ps);
                if (gradient && gs.n > 0) {
                    int g1 = st->n_gradient_estimates[i], g2 = gs.n, gt = g1 + g2;
                    for (int k = 0; k < D; k++) {
                        double* gm = st->gradient_mean + (size_t)i * D + k;
                        double* g2m = st->gradient_m2 ? st->gradient_m2 + (size_t)i * D + k : nullptr;
                        if (g1 == 0) { *gm = gs.mean[k]; if (g2m) *g2m = gs.m2[k]; }
                        else {
                            double delta = gs.mean[k] - *gm;
                            *gm += delta * ((double)g2 / gt);
                            if (g2m) *g2m += gs.m2[k] + delta * delta * ((double)g1 * g2 / gt);
                        }
                    }
                    st->n_gradient_estimates[i] = gt;
                }
                if (gradient) {
                    if (st->total_first_source_contribution) st->total_first_source_contribution[i] += gs.firstSource;
                    if (st->total_derivative_contribution) st->total_derivative_contribution[i] += gs.derivative;
                }
                if (pts->first_sphere_radius) pts->first_sphere_radius[i] = fsr;
                localSteps += ps.steps;
                // SampleStatistics::merge (common.h:268-310) in FP64
                if (ps.n > 0) {
                    int n1 = nPrev, n2 = ps.n, nt = n1 + n2;
                    if (n1 == 0) { st->solution_mean[i] = ps.mean; st->solution_m2[i] = ps.m2; }
                    else {
                        double delta = ps.mean - st->solution_mean[i];
                        st->solution_mean[i] += delta * ((double)n2 / nt);
                        st->solution_m2[i] += ps.m2 + delta * delta * ((double)n1 * n2 / nt);
                    }
                    st->n_solution_estimates[i] = nt;
                }
                st->total_walk_length[i] += ps.walkLength;
                st->total_splits[i] += ps.splits;
            }
        }
        steps += localSteps;
        flushCounters();
    };
    if (nThreads <= 1) {
        work();
    } else {
        std::vector<std::thread> th;
        for (int t = 0; t < nThreads; t++) th.emplace_back(work);
        for (auto& t : th) t.join();
    }
    if (stepsOut) *stepsOut = steps.load();
}

}  // namespace


// traversal counters accumulated by orc_solve and the batched queries: calls[5], nodes[5],
// prims[5]; reset after read
extern "C" void orc_counters(uint64_t* out) {
    for (int k = 0; k < 15; k++) out[k] = gCounters[k].exchange(0);
}

extern "C" int orc_hardware_threads() { return (int)std::thread::hardware_concurrency(); }

extern "C" void* orc_boundary_create(int dim, const float* pos, int nV, const int* idx, int nP, int kind, const float* kmin,
                          const float* kmax, int doubleSided, float silPrec, int useBvh) {
    Handle* h = new Handle();
    h->dim = dim;
    if (dim == 2) h->b = makeBoundary<2>(pos, nV, idx, nP, kind, kmin, kmax, doubleSided, silPrec, useBvh);
    else h->b = makeBoundary<3>(pos, nV, idx, nP, kind, kmin, kmax, doubleSided, silPrec, useBvh);
    return h;
}

extern "C" void orc_boundary_destroy(void* hp) {
    Handle* h = (Handle*)hp;
    if (!h) return;
    if (h->dim == 2) delete (Boundary<2>*)h->b; else delete (Boundary<3>*)h->b;
    delete h;
}

// silhouette flags as built (for tests): hasAdj and ignore bits per primitive feature
extern "C" void orc_boundary_flags(void* hp, int* hasAdj, int* ignore) {
    Handle* h = (Handle*)hp;
    if (h->dim == 2) {
        auto* b = (Boundary<2>*)h->b;
        for (int i = 0; i < b->nPrims(); i++) for (int j = 0; j < 2; j++) { hasAdj[i * 2 + j] = b->hasAdj[i][j]; ignore[i * 2 + j] = b->ignore[i][j]; }
    } else {
        auto* b = (Boundary<3>*)h->b;
        for (int i = 0; i < b->nPrims(); i++) for (int j = 0; j < 3; j++) { hasAdj[i * 3 + j] = b->hasAdj[i][j]; ignore[i * 3 + j] = b->ignore[i][j]; }
    }
}

extern "C" double orc_signed_volume(void* hp) {
    Handle* h = (Handle*)hp;
    return h->dim == 2 ? ((Boundary<2>*)h->b)->signedVolume() : ((Boundary<3>*)h->b)->signedVolume();
}

#define ORC_DISPATCH(h, body2, body3) \
    if ((h)->dim == 2) { auto* b = (Boundary<2>*)(h)->b; constexpr int D = 2; (void)b; (void)D; body2; } \
    else { auto* b = (Boundary<3>*)(h)->b; constexpr int D = 3; (void)b; (void)D; body3; } \
    flushCounters();

template <int D>
static void closestImpl(const Boundary<D>* b, int64_t n, const float* x, float* pt, float* nrm, float* d, int* prim) {
    for (int64_t i = 0; i < n; i++) {
        Vec<D> p, nn; float dd; int pi = -1;
        bool ok = b->closestPoint(load<D>(x + i * D), p, nn, dd, pi);
        if (!ok) { p = Vec<D>(); nn = Vec<D>(); dd = kMaxFloat; }
        if (pt) store<D>(p, pt + i * D);
        if (nrm) store<D>(nn, nrm + i * D);
        if (d) d[i] = dd;
        if (prim) prim[i] = pi;
    }
}
extern "C" int orc_closest_point(void* hp, int64_t n, const float* x, float* pt, float* nrm, float* d, int* prim) {
    Handle* h = (Handle*)hp;
    ORC_DISPATCH(h, closestImpl<2>(b, n, x, pt, nrm, d, prim), closestImpl<3>(b, n, x, pt, nrm, d, prim));
    return 0;
}

template <int D>
static void intersectImpl(const Boundary<D>* b, int64_t n, const float* o, const float* nrmIn, const float* dir,
                          const float* tmax, const int* onb, int* hit, float* pt, float* nrm, float* dist, int* prim) {
    for (int64_t i = 0; i < n; i++) {
        Vec<D> origin = load<D>(o + i * D);
        if (onb && onb[i]) origin = offsetPointAlongDirection<D>(origin, -load<D>(nrmIn + i * D));
        Vec<D> p, nn; float t = kMaxFloat; int pi = -1;
        bool ok = b->intersect(origin, load<D>(dir + i * D), tmax[i], p, nn, t, pi);
        hit[i] = ok;
        if (!ok) { p = Vec<D>(); nn = Vec<D>(); t = kMaxFloat; pi = -1; }
        if (pt) store<D>(p, pt + i * D);
        if (nrm) store<D>(nn, nrm + i * D);
        if (dist) dist[i] = t;
        if (prim) prim[i] = pi;
    }
}
extern "C" int orc_intersect(void* hp, int64_t n, const float* o, const float* nrmIn, const float* dir, const float* tmax,
                  const int* onb, int* hit, float* pt, float* nrm, float* dist, int* prim) {
    Handle* h = (Handle*)hp;
    ORC_DISPATCH(h, intersectImpl<2>(b, n, o, nrmIn, dir, tmax, onb, hit, pt, nrm, dist, prim),
                    intersectImpl<3>(b, n, o, nrmIn, dir, tmax, onb, hit, pt, nrm, dist, prim));
    return 0;
}

extern "C" int orc_count_hits(void* hp, int64_t n, const float* o, const float* dir, const float* tmax, int* out) {
    Handle* h = (Handle*)hp;
    ORC_DISPATCH(h,
        for (int64_t i = 0; i < n; i++) out[i] = b->countHits(load<D>(o + i * D), load<D>(dir + i * D), tmax[i]),
        for (int64_t i = 0; i < n; i++) out[i] = b->countHits(load<D>(o + i * D), load<D>(dir + i * D), tmax[i]));
    return 0;
}

extern "C" int orc_star_radius(void* hp, int64_t n, const float* x, const float* minR, const float* maxR, float prec,
                    const int* flip, float* out) {
    Handle* h = (Handle*)hp;
    ORC_DISPATCH(h,
        for (int64_t i = 0; i < n; i++) out[i] = b->starRadius(load<D>(x + i * D), minR[i], maxR[i], prec, flip && flip[i]),
        for (int64_t i = 0; i < n; i++) out[i] = b->starRadius(load<D>(x + i * D), minR[i], maxR[i], prec, flip && flip[i]));
    return 0;
}

template <int D>
static void occludedImpl(const Boundary<D>* b, int64_t n, const float* xi, const float* xj, const float* ni,
                         const float* nj, const int* oi, const int* oj, int* out) {
    for (int64_t k = 0; k < n; k++) {
        Vec<D> p1 = load<D>(xi + k * D), p2 = load<D>(xj + k * D);
        if (oi && oi[k]) p1 = offsetPointAlongDirection<D>(p1, -load<D>(ni + k * D));
        if (oj && oj[k]) p2 = offsetPointAlongDirection<D>(p2, -load<D>(nj + k * D));
        out[k] = b->occluded(p1, p2);
    }
}
extern "C" int orc_occluded(void* hp, int64_t n, const float* xi, const float* xj, const float* ni, const float* nj,
                 const int* oi, const int* oj, int* out) {
    Handle* h = (Handle*)hp;
    ORC_DISPATCH(h, occludedImpl<2>(b, n, xi, xj, ni, nj, oi, oj, out), occludedImpl<3>(b, n, xi, xj, ni, nj, oi, oj, out));
    return 0;
}

template <int D>
static void sampleImpl(const Boundary<D>* b, int64_t n, const float* x, const float* r, const float* u, int* found,
                       float* pt, float* nrm, float* pdf) {
    for (int64_t k = 0; k < n; k++) {
        Vec<D> p, nn; float pp = 0.0f;
        bool ok = b->sample(load<D>(x + k * D), r[k], u + k * D, p, nn, pp);
        found[k] = ok;
        if (!ok) { p = Vec<D>(); nn = Vec<D>(); pp = 0.0f; }
        store<D>(p, pt + k * D); store<D>(nn, nrm + k * D); pdf[k] = pp;
    }
}
extern "C" int orc_sample(void* hp, int64_t n, const float* x, const float* r, const float* u, int* found, float* pt, float* nrm,
               float* pdf) {
    Handle* h = (Handle*)hp;
    ORC_DISPATCH(h, sampleImpl<2>(b, n, x, r, u, found, pt, nrm, pdf), sampleImpl<3>(b, n, x, r, u, found, pt, nrm, pdf));
    return 0;
}

// Green's function helpers for identity tests (distributions.h)
extern "C" float orc_greens_norm(int dim, int yukawa, float lambda, float R) {
    if (dim == 2) {
        std::unique_ptr<GreensFnBall<2>> g(yukawa ? (GreensFnBall<2>*)new YukawaGreensFnBall<2>(lambda) : new HarmonicGreensFnBall<2>());
        g->updateBall(Vec<2>(), R); return g->norm();
    }
    std::unique_ptr<GreensFnBall<3>> g(yukawa ? (GreensFnBall<3>*)new YukawaGreensFnBall<3>(lambda) : new HarmonicGreensFnBall<3>());
    g->updateBall(Vec<3>(), R); return g->norm();
}
extern "C" float orc_greens_evaluate(int dim, int yukawa, float lambda, float R, float r) {
    if (dim == 2) {
        std::unique_ptr<GreensFnBall<2>> g(yukawa ? (GreensFnBall<2>*)new YukawaGreensFnBall<2>(lambda) : new HarmonicGreensFnBall<2>());
        g->updateBall(Vec<2>(), R); return g->evaluate(r);
    }
    std::unique_ptr<GreensFnBall<3>> g(yukawa ? (GreensFnBall<3>*)new YukawaGreensFnBall<3>(lambda) : new HarmonicGreensFnBall<3>());
    g->updateBall(Vec<3>(), R); return g->evaluate(r);
}
// draws n radii from GreensFnBall::sampleVolume(dir, ...) with pcg32(seed, 0)
extern "C" void orc_greens_sample_radii(int dim, int yukawa, float lambda, float R, uint64_t seed, int n, float* out) {
    Pcg32 rng(seed, 0);
    float r, pdf;
    if (dim == 2) {
        std::unique_ptr<GreensFnBall<2>> g(yukawa ? (GreensFnBall<2>*)new YukawaGreensFnBall<2>(lambda) : new HarmonicGreensFnBall<2>());
        g->updateBall(Vec<2>(), R);
        Vec<2> d; d[0] = 1.0f;
        for (int i = 0; i < n; i++) { g->sampleVolume(d, rng, r, pdf); out[i] = r; }
    } else {
        std::unique_ptr<GreensFnBall<3>> g(yukawa ? (GreensFnBall<3>*)new YukawaGreensFnBall<3>(lambda) : new HarmonicGreensFnBall<3>());
        g->updateBall(Vec<3>(), R);
        Vec<3> d; d[0] = 1.0f;
        for (int i = 0; i < n; i++) { g->sampleVolume(d, rng, r, pdf); out[i] = r; }
    }
}
extern "C" double orc_bessel(int which, double x) {
    switch (which) { case 0: return bessel::i0(x); case 1: return bessel::i1(x); case 2: return bessel::k0(x); default: return bessel::k1(x); }
}
extern "C" void orc_pcg32(uint64_t seed, uint64_t stream, int n, uint32_t* outU, float* outF) {
    Pcg32 a(seed, stream), b(seed, stream);
    for (int i = 0; i < n; i++) { if (outU) outU[i] = a.nextUInt(); if (outF) outF[i] = b.nextFloat(); }
}
extern "C" void orc_offset_point(int dim, const float* p, const float* n, float* out) {
    if (dim == 2) store<2>(offsetPointAlongDirection<2>(load<2>(p), load<2>(n)), out);
    else store<3>(offsetPointAlongDirection<3>(load<3>(p), load<3>(n)), out);
}
// the PDE's fields at n points: source, Dirichlet, Robin data and Robin coefficient (any
// output may be NULL), the boundary-normal-aligned values when `aligned`
extern "C" void orc_eval_pde(int dim, const zgpu_pde* pde, int64_t n, const float* x, const float* nrm, int aligned,
                             float* src, float* dir, float* rob, float* kappa) {
    const bool al = aligned != 0;
    for (int64_t i = 0; i < n; i++) {
        if (dim == 2) {
            Pde<2> p{pde}; Vec<2> xx = load<2>(x + i * 2), nn = nrm ? load<2>(nrm + i * 2) : Vec<2>();
            if (src) src[i] = p.source(xx);
            if (dir) dir[i] = p.dirichlet(xx, al);
            if (rob) rob[i] = p.robin(xx, nn, al);
            if (kappa) kappa[i] = p.robinCoeff(xx, nn, al);
        } else {
            Pde<3> p{pde}; Vec<3> xx = load<3>(x + i * 3), nn = nrm ? load<3>(nrm + i * 3) : Vec<3>();
            if (src) src[i] = p.source(xx);
            if (dir) dir[i] = p.dirichlet(xx, al);
            if (rob) rob[i] = p.robin(xx, nn, al);
            if (kappa) kappa[i] = p.robinCoeff(xx, nn, al);
        }
    }
}

// WalkOnSpheres/WalkOnStars::solve over all points with nThreads std::threads (TBB stand-in)
extern "C" int orc_solve(int solver, const zgpu_geometric_queries* q, const zgpu_pde* pde, const zgpu_walk_settings* ws,
              const zgpu_sample_points* pts, zgpu_sample_statistics* st, int nThreads, uint64_t* steps) {
    if (q->dim == 2) solveImpl<2>(solver, q, pde, ws, pts, st, nThreads, steps);
    else solveImpl<3>(solver, q, pde, ws, pts, st, nThreads, steps);
    return 0;
}


// ---------------------------------------------------------------- neural cache oracle
// Parameters arrive as float arrays (the GPU's FP16 table and BF16 weights widened to FP32);
// res = per-level resolutions, lo / inv = domain normalisation.
static CacheModel makeCacheModel(int dim, int levels, int log2T, const float* res, const float* lo, const float* inv,
                                 const float* table, const float* W1, const float* b1, const float* W2,
                                 const float* b2, const float* w3, float b3) {
    CacheModel m;
    m.dim = dim; m.levels = levels; m.log2T = log2T;
    m.res.assign(res, res + levels);
    for (int i = 0; i < dim; i++) { m.lo[i] = lo[i]; m.inv[i] = inv[i]; }
    const size_t T = (size_t)1 << log2T, I = (size_t)2 * levels, H = kCacheHidden;
    m.table.assign(table, table + (size_t)levels * T * 2);
    m.W1.assign(W1, W1 + H * I); m.b1.assign(b1, b1 + H);
    m.W2.assign(W2, W2 + H * H); m.b2.assign(b2, b2 + H);
    m.w3.assign(w3, w3 + H); m.b3 = b3;
    return m;
}

extern "C" void orc_cache_forward(int dim, int levels, int log2T, const float* res, const float* lo, const float* inv,
                                  const float* table, const float* W1, const float* b1, const float* W2,
                                  const float* b2, const float* w3, float b3, int64_t n, const float* x,
                                  double* y, double* enc) {
    CacheModel m = makeCacheModel(dim, levels, log2T, res, lo, inv, table, W1, b1, W2, b2, w3, b3);
    CacheActivations a;
    for (int64_t i = 0; i < n; i++) {
        y[i] = cacheForward(m, x + i * dim, a);
        if (enc) for (int k = 0; k < 2 * levels; k++) enc[i * 2 * levels + k] = a.e[k];
    }
}

// corner indices of every level for each point: out[n][levels][2^dim]
extern "C" void orc_cache_corners(int dim, int levels, int log2T, const float* res, const float* lo, const float* inv,
                                  int64_t n, const float* x, uint32_t* idx, double* w) {
    CacheModel m;
    m.dim = dim; m.levels = levels; m.log2T = log2T;
    m.res.assign(res, res + levels);
    for (int i = 0; i < dim; i++) { m.lo[i] = lo[i]; m.inv[i] = inv[i]; }
    CacheCorner cs[8];
    const int C = 1 << dim;
    for (int64_t i = 0; i < n; i++)
        for (int l = 0; l < levels; l++) {
            cacheCorners(m, l, x + i * dim, cs);
            for (int k = 0; k < C; k++) {
                idx[(i * levels + l) * C + k] = cs[k].index;
                if (w) w[(i * levels + l) * C + k] = cs[k].weight;
            }
        }
}

// mean squared error and its gradient; outputs laid out like the parameters (double)
extern "C" double orc_cache_grads(int dim, int levels, int log2T, const float* res, const float* lo, const float* inv,
                                  const float* table, const float* W1, const float* b1, const float* W2,
                                  const float* b2, const float* w3, float b3, int n, const float* x,
                                  const float* target, double* gTable, double* gW1, double* gb1, double* gW2,
                                  double* gb2, double* gw3, double* gb3) {
    CacheModel m = makeCacheModel(dim, levels, log2T, res, lo, inv, table, W1, b1, W2, b2, w3, b3);
    CacheGrads g;
    double loss = cacheLossAndGrads(m, n, x, target, g);
    std::copy(g.table.begin(), g.table.end(), gTable);
    std::copy(g.W1.begin(), g.W1.end(), gW1);
    std::copy(g.b1.begin(), g.b1.end(), gb1);
    std::copy(g.W2.begin(), g.W2.end(), gW2);
    std::copy(g.b2.begin(), g.b2.end(), gb2);
    std::copy(g.w3.begin(), g.w3.end(), gw3);
    *gb3 = g.b3;
    return loss;
}

// BoundaryValueCaching::splat over all evaluation points (boundary_value_caching.h:427-459 with
// :380-425 per point): the cache's statistics merged into the points' (common.h:268-310)
extern "C" int orc_bvc_splat(int dim, float absorption, const zgpu_bvc_samples* s, float radiusClamp, float reg,
                             float robinCutoff, float cutoffA, float cutoffR, zgpu_bvc_eval_points* ev, int nThreads) {
    std::atomic<int64_t> next{0};
    auto work = [&]() {
        for (;;) {
            const int64_t i = next.fetch_add(1);
            if (i >= ev->n) break;
            const float dA = ev->dist_to_absorbing[i];
            const float dR = ev->dist_to_reflecting ? ev->dist_to_reflecting[i] : std::numeric_limits<float>::max();
            if (dA < cutoffA || dR < cutoffR) continue;
            const int type = ev->type ? ev->type[i] : ZGPU_SAMPLE_IN_DOMAIN;
            SplatStat st[ZGPU_BVC_GROUPS];
            if (dim == 2) bvcSplatPoint<2>(*s, absorption, radiusClamp, reg, robinCutoff, load<2>(ev->pt + i * 2), type, st);
            else bvcSplatPoint<3>(*s, absorption, radiusClamp, reg, robinCutoff, load<3>(ev->pt + i * 3), type, st);
            for (int g = 0; g < ZGPU_BVC_GROUPS; g++) {
                if (st[g].n == 0) continue;
                const size_t k = (size_t)i * ZGPU_BVC_GROUPS + g;
                const int n1 = ev->count[k], n2 = st[g].n, nt = n1 + n2;
                const double d = st[g].mean - ev->mean[k];
                if (n1 == 0) { ev->mean[k] = st[g].mean; ev->m2[k] = st[g].m2; }
                else {
                    ev->mean[k] += d * ((double)n2 / nt);
                    ev->m2[k] += st[g].m2 + d * d * ((double)n1 * n2 / nt);
                }
                for (int c = 0; c < dim; c++) {
                    double* gm = ev->gradient_mean + k * dim + c;
                    double* gv = ev->gradient_m2 ? ev->gradient_m2 + k * dim + c : nullptr;
                    if (n1 == 0) { *gm = st[g].gmean[c]; if (gv) *gv = st[g].gm2[c]; }
                    else {
                        const double e = st[g].gmean[c] - *gm;
                        *gm += e * ((double)n2 / nt);
                        if (gv) *gv += st[g].gm2[c] + e * e * ((double)n1 * n2 / nt);
                    }
                }
                ev->count[k] = nt;
            }
        }
    };
    if (nThreads <= 1) work();
    else {
        std::vector<std::thread> th;
        for (int t = 0; t < nThreads; t++) th.emplace_back(work);
        for (auto& t : th) t.join();
    }
    return 0;
}

// ReverseWalkOnStarsSolver::solve's walks for all samples (reverse_walk_solver.h:304-338):
// totals [n_eval][6] added to; returns the number of walk steps
template <int D>
uint64_t rwsImpl(const zgpu_geometric_queries* gq, const zgpu_pde* pde, const zgpu_walk_settings* ws,
                 const zgpu_rws_samples* s, float normalOffset, float radiusClamp, float reg, uint64_t stream,
                 zgpu_rws_eval_points* ev, int nThreads) {
    Queries<D> q;
    q.absorbing = gq->absorbing ? (const Boundary<D>*)((Handle*)gq->absorbing)->b : nullptr;
    q.reflecting = gq->reflecting ? (const Boundary<D>*)((Handle*)gq->reflecting)->b : nullptr;
    for (int i = 0; i < D; i++) { q.domainMin[i] = gq->domain_min[i]; q.domainMax[i] = gq->domain_max[i]; }
    const bool selfNorm = gq->domain_is_watertight && pde->absorption_coeff == 0.0f &&
                          (!q.hasNonEmptyReflectingBoundary() || pde->are_robin_conditions_pure_neumann);
    RwsEval<D> e{ev->n, ev->pt, ev->normal, ev->type};
    nThreads = std::max(1, nThreads);
    std::vector<std::vector<double>> local(nThreads, std::vector<double>((size_t)ev->n * ZGPU_RWS_TOTALS, 0.0));
    std::vector<uint64_t> steps(nThreads, 0);
    std::atomic<int64_t> next{0};
    auto work = [&](int t) {
        Solver<D> sv{q, Pde<D>{pde}, *ws};
        for (;;) {
            const int64_t i = next.fetch_add(1);
            if (i >= s->n) break;
            const bool aligned = s->estimate_normal_aligned ? s->estimate_normal_aligned[i] != 0 : false;
            reverseWalkSample<D>(sv, load<D>(s->pt + i * D), load<D>(s->normal + i * D), s->type[i], aligned, s->pdf[i],
                                 s->contribution[i], s->dist_to_absorbing[i], s->seed[i], stream, e, normalOffset,
                                 radiusClamp, reg, selfNorm, local[t].data(), steps[t]);
        }
    };
    std::vector<std::thread> th;
    for (int t = 0; t < nThreads; t++) th.emplace_back(work, t);
    for (auto& t : th) t.join();
    uint64_t total = 0;
    for (int t = 0; t < nThreads; t++) {
        total += steps[t];
        for (size_t k = 0; k < local[t].size(); k++) ev->totals[k] += local[t][k];
    }
    return total;
}

extern "C" uint64_t orc_rws_solve(const zgpu_geometric_queries* gq, const zgpu_pde* pde, const zgpu_walk_settings* ws,
                                  const zgpu_rws_samples* s, float normalOffset, float radiusClamp, float reg,
                                  uint64_t stream, zgpu_rws_eval_points* ev, int nThreads) {
    return gq->dim == 2 ? rwsImpl<2>(gq, pde, ws, s, normalOffset, radiusClamp, reg, stream, ev, nThreads)
                        : rwsImpl<3>(gq, pde, ws, s, normalOffset, radiusClamp, reg, stream, ev, nThreads);
}
