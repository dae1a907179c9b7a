// oracle_geometry.h -- TEST INFRASTRUCTURE, NOT PRODUCT CODE (see oracle_core.h).
//
// Boundary geometry of the oracle: primitive routines restated from
// core/geometry_helpers.h, the reflectance primitives of
// utils/reflectance_boundary_bvh/geometry.h and robin_bounds.h, the float-bit ray offset
// of core/geometric_queries.h:175-207, plus brute-force and binary-SAH-BVH (leaf size 4,
// as reflectance_boundary_bvh/bvh.h:42) versions of every query the walk issues.
//
// FCPW (rohan-sawhney/fcpw, pinned commit unknown, absent from the reference mount)
// answers closest point, ray intersection, closest silhouette point, ball sampling and
// line of sight in the reference.  Its code is not available here, so those queries are
// restated from their published definitions:
//  * closest point / ray hit: exact geometric definitions; ties are broken by the lower
//    caller primitive index (brute force) -- the GPU traversal must agree except at ties;
//  * silhouettes: a vertex (2D) / edge (3D) is a silhouette from x when exactly one of its
//    two adjacent faces is front-facing (Walk on Stars, Sawhney et al. 2023, Sec. 4.2),
//    with degenerate cases (x on a face plane, x on the feature) resolved by the concavity
//    of the feature; features with one adjacent face are always silhouettes;
//  * ball sampling: a primitive overlapping the ball is chosen with probability
//    proportional to area * w(d^2) (w = the reference's branch-traversal weight,
//    utils/fcpw_geometric_queries.h:1391-1398, d = distance to the primitive), a point is
//    drawn uniformly on it and pdf = P(primitive)/area.  Any such pdf gives an unbiased
//    estimate of the reflecting-boundary integral, which is all the walk needs.
#pragma once

#include <array>
#include <map>
#include "oracle_core.h"

namespace orc {

// ---------------------------------------------------------------------------------------
// geometric_queries.h:154-207 -- robust ray-origin offset ("A Fast and Robust Method for
// Avoiding Self-Intersection", Wachter & Binder, Ray Tracing Gems 2019, ch. 6)
inline int floatAsInt(float a) { int b; std::memcpy(&b, &a, 4); return b; }
inline float intAsFloat(int a) { float b; std::memcpy(&b, &a, 4); return b; }
template <int D>
inline Vec<D> offsetPointAlongDirection(const Vec<D>& p, const Vec<D>& n) {
    const float origin = 1.0f / 32.0f;
    const float floatScale = 1.0f / 65536.0f;
    const float intScale = 256.0f;
    Vec<D> r;
    for (int i = 0; i < D; i++) {
        int nOffset = (int)(n[i] * intScale);
        float pOffset = intAsFloat(floatAsInt(p[i]) + (p[i] < 0 ? -nOffset : nOffset));
        r[i] = std::fabs(p[i]) < origin ? p[i] + floatScale * n[i] : pOffset;
    }
    return r;
}

// geometry_helpers.h:15-21, :77-81 (unnormalized normal, outward for CCW winding)
inline Vec<2> primNormal(const Vec<2>* p, bool normalize) {
    Vec<2> s = p[1] - p[0];
    Vec<2> n; n[0] = s[1]; n[1] = -s[0];
    return normalize ? normalized(n) : n;
}
inline Vec<3> primNormal(const Vec<3>* p, bool normalize) {
    Vec<3> n = cross3(p[1] - p[0], p[2] - p[0]);
    return normalize ? normalized(n) : n;
}
inline float primArea(const Vec<2>* p) { return norm(primNormal(p, false)); }
inline float primArea(const Vec<3>* p) { return 0.5f * norm(primNormal(p, false)); }

// geometry_helpers.h:28-49
inline float closestPointSegment(const Vec<2>& pa, const Vec<2>& pb, const Vec<2>& x, Vec<2>& pt) {
    Vec<2> u = pb - pa, v = x - pa;
    float c1 = dot(u, v);
    if (c1 <= 0.0f) { pt = pa; return norm(x - pa); }
    float c2 = dot(u, u);
    if (c2 <= c1) { pt = pb; return norm(x - pb); }
    float t = c1 / c2;
    pt = pa + u * t;
    return norm(x - pt);
}
inline float closestPointSegment3(const Vec<3>& pa, const Vec<3>& pb, const Vec<3>& x, Vec<3>& pt) {
    Vec<3> u = pb - pa, v = x - pa;
    float c1 = dot(u, v);
    if (c1 <= 0.0f) { pt = pa; return norm(x - pa); }
    float c2 = dot(u, u);
    if (c2 <= c1) { pt = pb; return norm(x - pb); }
    float t = c1 / c2;
    pt = pa + u * t;
    return norm(x - pt);
}
// geometry_helpers.h:94-161 (Ericson, Real-Time Collision Detection, 5.1.5)
inline float closestPointTriangle(const Vec<3>& pa, const Vec<3>& pb, const Vec<3>& pc, const Vec<3>& x, Vec<3>& pt) {
    Vec<3> ab = pb - pa, ac = pc - pa, ax = x - pa;
    float d1 = dot(ab, ax), d2 = dot(ac, ax);
    if (d1 <= 0.0f && d2 <= 0.0f) { pt = pa; return norm(x - pa); }
    Vec<3> bx = x - pb;
    float d3 = dot(ab, bx), d4 = dot(ac, bx);
    if (d3 >= 0.0f && d4 <= d3) { pt = pb; return norm(x - pb); }
    Vec<3> cx = x - pc;
    float d5 = dot(ab, cx), d6 = dot(ac, cx);
    if (d6 >= 0.0f && d5 <= d6) { pt = pc; return norm(x - pc); }
    float vc = d1 * d4 - d3 * d2;
    if (vc <= 0.0f && d1 >= 0.0f && d3 <= 0.0f) { float v = d1 / (d1 - d3); pt = pa + ab * v; return norm(x - pt); }
    float vb = d5 * d2 - d1 * d6;
    if (vb <= 0.0f && d2 >= 0.0f && d6 <= 0.0f) { float w = d2 / (d2 - d6); pt = pa + ac * w; return norm(x - pt); }
    float va = d3 * d6 - d5 * d4;
    if (va <= 0.0f && (d4 - d3) >= 0.0f && (d5 - d6) >= 0.0f) {
        float w = (d4 - d3) / ((d4 - d3) + (d5 - d6)); pt = pb + (pc - pb) * w; return norm(x - pt);
    }
    float denom = 1.0f / (va + vb + vc);
    float v = vb * denom, w = vc * denom;
    pt = pa + ab * v + ac * w;
    return norm(x - pt);
}
inline float closestPointPrim(const Vec<2>* p, const Vec<2>& x, Vec<2>& pt) { return closestPointSegment(p[0], p[1], x, pt); }
inline float closestPointPrim(const Vec<3>* p, const Vec<3>& x, Vec<3>& pt) { return closestPointTriangle(p[0], p[1], p[2], x, pt); }

// geometry_helpers.h:51-63, :163-180
inline float farthestPointPrim(const Vec<2>* p, const Vec<2>& x, Vec<2>& pt) {
    float da = norm2(x - p[0]), db = norm2(x - p[1]);
    if (da > db) { pt = p[0]; return std::sqrt(da); }
    pt = p[1]; return std::sqrt(db);
}
inline float farthestPointPrim(const Vec<3>* p, const Vec<3>& x, Vec<3>& pt) {
    float da = norm2(x - p[0]), db = norm2(x - p[1]), dc = norm2(x - p[2]);
    if (da >= db && da >= dc) { pt = p[0]; return std::sqrt(da); }
    if (db >= da && db >= dc) { pt = p[1]; return std::sqrt(db); }
    pt = p[2]; return std::sqrt(dc);
}

// geometry_helpers.h:65-75, :182-196 (uniform point on the primitive, pdf = 1/area)
inline Vec<2> samplePointOnPrim(const Vec<2>* p, const float* u, Vec<2>& n, float& pdf) {
    Vec<2> s = p[1] - p[0];
    Vec<2> pt = p[0] + s * u[0];
    n[0] = s[1]; n[1] = -s[0];
    float nn = norm(n);
    n = n / nn;
    pdf = 1.0f / nn;
    return pt;
}
inline Vec<3> samplePointOnPrim(const Vec<3>* p, const float* u, Vec<3>& n, float& pdf) {
    float u1 = std::sqrt(u[0]), u2 = u[1];
    float a = 1.0f - u1, b = u2 * u1, c = 1.0f - a - b;
    Vec<3> pt = p[0] * a + p[1] * b + p[2] * c;
    n = cross3(p[1] - p[0], p[2] - p[0]);
    float nn = norm(n);
    n = n / nn;
    pdf = 2.0f / nn;
    return pt;
}

// ray / primitive intersection: 2D segment by Cramer's rule, 3D by Moller-Trumbore
// ("Fast, Minimum Storage Ray/Triangle Intersection", 1997).  t in [0, tMax].
inline bool intersectPrim(const Vec<2>* p, const Vec<2>& o, const Vec<2>& d, float tMax, float& t) {
    Vec<2> e = p[1] - p[0];
    float denom = cross2(d, e);
    if (std::fabs(denom) < 1e-20f) return false;
    Vec<2> w = p[0] - o;
    float tt = cross2(w, e) / denom;
    float s = cross2(w, d) / denom;
    if (tt < 0.0f || tt > tMax || s < 0.0f || s > 1.0f) return false;
    t = tt;
    return true;
}
inline bool intersectPrim(const Vec<3>* p, const Vec<3>& o, const Vec<3>& d, float tMax, float& t) {
    Vec<3> e1 = p[1] - p[0], e2 = p[2] - p[0];
    Vec<3> pv = cross3(d, e2);
    float det = dot(e1, pv);
    if (std::fabs(det) < 1e-20f) return false;
    float inv = 1.0f / det;
    Vec<3> tv = o - p[0];
    float u = dot(tv, pv) * inv;
    if (u < 0.0f || u > 1.0f) return false;
    Vec<3> qv = cross3(tv, e1);
    float v = dot(d, qv) * inv;
    if (v < 0.0f || u + v > 1.0f) return false;
    float tt = dot(e2, qv) * inv;
    if (tt < 0.0f || tt > tMax) return false;
    t = tt;
    return true;
}

// silhouette tests (see header comment).  2D: the vertex joins a segment before it
// (normal nPrev) and one after it (normal nNext) in the winding order.
inline bool isSilhouetteVertex(const Vec<2>& nPrev, const Vec<2>& nNext, const Vec<2>& viewDir,
                               float d, bool flip, float precision) {
    float sign = flip ? -1.0f : 1.0f;
    if (d <= precision) return sign * cross2(nPrev, nNext) < -precision;  // x on a concave vertex
    Vec<2> u = viewDir / d;
    float d0 = dot(nPrev, u), d1 = dot(nNext, u);
    if (std::fabs(d0) <= precision) return sign * d1 > precision;
    if (std::fabs(d1) <= precision) return sign * d0 > precision;
    return d0 * d1 < 0.0f;
}
// 3D: edge pa->pb in the winding of the face with normal nA; nB is the neighbour's normal
inline bool isSilhouetteEdge(const Vec<3>& pa, const Vec<3>& pb, const Vec<3>& nA, const Vec<3>& nB,
                             const Vec<3>& viewDir, float d, bool flip, float precision) {
    float sign = flip ? -1.0f : 1.0f;
    if (d <= precision) {
        Vec<3> e = normalized(pb - pa);
        return sign * dot(e, cross3(nB, nA)) > precision;  // x on a concave edge
    }
    Vec<3> u = viewDir / d;
    float dA = dot(nA, u), dB = dot(nB, u);
    if (std::fabs(dA) <= precision) return sign * dB > precision;
    if (std::fabs(dB) <= precision) return sign * dA > precision;
    return dA * dB < 0.0f;
}

// reflectance_boundary_bvh/geometry.h:62-70
template <int D>
inline float closestPointPlane(const Vec<D>& p, const Vec<D>& n, const Vec<D>& x) {
    float t = dot(n, p - x) / dot(n, n);
    return std::fabs(t);
}
// robin_bounds.h:14-35
inline void robinStarRadiusBound(const Vec<2>& c, float& r2, float maxRobinCoeff, const Vec<2>& viewDirClosest,
                                 float closestPtDist, const Vec<2>& viewDirFarthest, float farthestPtDist,
                                 const Vec<2>& planePt, const Vec<2>& planeNormal) {
    float h = closestPointPlane<2>(planePt, planeNormal, c);
    if (h > 0.0f) {
        float cosUpper = std::fabs(dot(viewDirClosest / closestPtDist, planeNormal));
        float cosLower = std::fabs(dot(viewDirFarthest / farthestPtDist, planeNormal));
        float cosLine = std::sqrt(h * maxRobinCoeff) / 1.4142135623730950488f;
        float cosSeg = std::min(std::max(cosLine, cosLower), cosUpper);
        float cosSeg2 = cosSeg * cosSeg;
        float radius = (h / cosSeg) * std::exp(cosSeg2 / (h * maxRobinCoeff));
        r2 = std::min(r2, radius * radius);
    } else {
        r2 = std::min(r2, closestPtDist * closestPtDist);
    }
}
// robin_bounds.h:50-74
inline void robinStarRadiusBound(const Vec<3>& c, float& r2, float maxRobinCoeff, const Vec<3>& viewDirClosest,
                                 float closestPtDist, const Vec<3>& viewDirFarthest, float farthestPtDist,
                                 const Vec<3>& planePt, const Vec<3>& planeNormal) {
    float h = closestPointPlane<3>(planePt, planeNormal, c);
    if (h > 0.0f) {
        float cosUpper = std::fabs(dot(viewDirClosest / closestPtDist, planeNormal));
        float cosLower = std::fabs(dot(viewDirFarthest / farthestPtDist, planeNormal));
        float maxCos = std::sqrt(h * maxRobinCoeff);
        if (maxCos >= cosLower) {
            float cosPlane = maxCos / 1.7320508075688772935f;
            float cosTri = std::min(std::max(cosPlane, cosLower), cosUpper);
            float cosTri2 = cosTri * cosTri;
            float radius = h * h * maxRobinCoeff / (cosTri * (h * maxRobinCoeff - cosTri2));
            r2 = std::min(r2, radius * radius);
        }
    } else {
        r2 = std::min(r2, closestPtDist * closestPtDist);
    }
}

// branch traversal weight: |G_free,3D(max(sqrt(r2), 1e-2))| (fcpw_geometric_queries.h:1391-1398)
inline float branchWeight(float r2) {
    float r = std::max(std::sqrt(r2), 1e-2f);
    return std::fabs(1.0f / (4.0f * kPi * r));
}

// traversal work counters (per thread; summed by the solve driver): per query kind
// [0] closest point, [1] first ray hit, [2] line of sight, [3] star radius, [4] sampling
struct Counters { uint64_t calls[5] = {0}, nodes[5] = {0}, prims[5] = {0}; };
inline Counters& counters() { static thread_local Counters c; return c; }

template <int D>
struct Box {
    Vec<D> lo = Vec<D>::constant(kMaxFloat), hi = Vec<D>::constant(-kMaxFloat);
    void expand(const Vec<D>& p) { for (int i = 0; i < D; i++) { lo[i] = std::min(lo[i], p[i]); hi[i] = std::max(hi[i], p[i]); } }
    void expand(const Box& b) { expand(b.lo); expand(b.hi); }
    float dist2(const Vec<D>& x) const {
        float s = 0.0f;
        for (int i = 0; i < D; i++) { float d = std::max(std::max(lo[i] - x[i], 0.0f), x[i] - hi[i]); s += d * d; }
        return s;
    }
    float maxDist2(const Vec<D>& x) const {
        float s = 0.0f;
        for (int i = 0; i < D; i++) { float d = std::max(std::fabs(x[i] - lo[i]), std::fabs(x[i] - hi[i])); s += d * d; }
        return s;
    }
    float surface() const {
        Vec<D> e = hi - lo;
        if (D == 2) return 2.0f * (e[0] + e[1]);
        return 2.0f * (e[0] * e[1] + e[1] * e[2] + e[2] * e[0]);
    }
    bool rayOverlap(const Vec<D>& o, const Vec<D>& invD, float tMax) const {
        float t0 = 0.0f, t1 = tMax;
        for (int i = 0; i < D; i++) {
            float a = (lo[i] - o[i]) * invD[i], b = (hi[i] - o[i]) * invD[i];
            if (a > b) std::swap(a, b);
            t0 = std::max(t0, a); t1 = std::min(t1, b);
        }
        return t0 <= t1 * (1.0f + 2e-7f) + 1e-30f;
    }
};

template <int D>
struct Boundary {
    int kind = ZGPU_BOUNDARY_ABSORBING;
    std::vector<Vec<D>> pos;
    std::vector<std::array<int, D>> idx;
    // reflecting-boundary data per primitive (reflectance_boundary_bvh/geometry.h:30-35)
    std::vector<std::array<Vec<D>, D>> adjN;
    std::vector<std::array<uint8_t, D>> hasAdj, ignore;
    std::vector<float> kmin, kmax;
    // binary SAH BVH
    struct Node {
        Box<D> box; int left = -1, right = -1, start = 0, count = 0; float area = 0.0f;
        float axis[3] = {0, 0, 0}; float halfAngle = 3.14159265f;   // normal cone
        float kmin = 0.0f, kmax = 0.0f;                                  // Robin coefficient range
    };
    std::vector<Node> nodes;
    std::vector<int> order;
    bool useBvh = true;

    int nPrims() const { return (int)idx.size(); }
    void prim(int i, Vec<D>* p) const { for (int k = 0; k < D; k++) p[k] = pos[idx[i][k]]; }
    Vec<D> normalOf(int i) const { Vec<D> p[D]; prim(i, p); return primNormal(p, true); }
    float areaOf(int i) const { Vec<D> p[D]; prim(i, p); return primArea(p); }
    Box<D> boxOf(int i) const { Box<D> b; for (int k = 0; k < D; k++) b.expand(pos[idx[i][k]]); return b; }

    void buildAdjacency(bool solveDoubleSided, float silhouettePrecision);
    void buildBvh();
    void buildCones();
    // silhouette-candidate tree of a Neumann boundary (FCPW computeSilhouettes + its BVH):
    // one record per non-ignored vertex (2D) / edge (3D), deduplicated
    struct Feature { Vec<D> a, b, nA, nB; bool open; };
    std::vector<Feature> feats;
    std::vector<Node> fnodes;
    std::vector<int> forder;
    void buildFeatureTree();
    int buildFeatureRecursive(int start, int end, int depth);
    float featureRadius2(const Vec<D>& x, float r2, bool flip, float precision) const;
    bool coneMayHoldSilhouette(const Node& nd, const Vec<D>& x, float prec) const;
    bool robinVisit(const Node& nd, const Vec<D>& x, float r2, float& r2Min, float& r2Max) const;
    int buildRecursive(int start, int end, std::vector<Vec<D>>& centroids, int depth);

    // queries
    bool closestPoint(const Vec<D>& x, Vec<D>& pt, Vec<D>& n, float& d, int& primOut) const;
    bool intersect(const Vec<D>& o, const Vec<D>& dir, float tMax, Vec<D>& pt, Vec<D>& n, float& t, int& primOut,
                   int kind = 1) const;
    int countHits(const Vec<D>& o, const Vec<D>& dir, float tMax) const;
    bool occluded(const Vec<D>& a, const Vec<D>& b) const;
    void primStarRadius(int i, const Vec<D>& c, float& r2, bool flip, float precision) const;
    float starRadius(const Vec<D>& x, float minR, float maxR, float precision, bool flip) const;
    bool sample(const Vec<D>& x, float radius, const float* u, Vec<D>& pt, Vec<D>& n, float& pdf) const;
    double signedVolume() const;
};

// adjacency and silhouette-ignore flags: 2D fcpw_geometric_queries.h:745-799, 3D :892-973;
// ignore rule getIgnoreCandidateSilhouetteCallback :1029-1038
template <>
inline void Boundary<2>::buildAdjacency(bool solveDoubleSided, float silhouettePrecision) {
    int V = (int)pos.size(), L = nPrims();
    std::vector<std::array<int, 2>> vt(V, std::array<int, 2>{-1, -1});
    for (int i = 0; i < L; i++)
        for (int j = 0; j < 2; j++) vt[idx[i][j]][1 - j] = i;
    adjN.assign(L, {}); hasAdj.assign(L, {}); ignore.assign(L, {});
    for (int i = 0; i < L; i++) {
        Vec<2> n0 = normalOf(i);
        for (int j = 0; j < 2; j++) {
            int a = vt[idx[i][j]][j];
            if (a != -1) { hasAdj[i][j] = 1; adjN[i][j] = normalOf(a); }
            else { hasAdj[i][j] = 0; }
            if (hasAdj[i][j]) {
                float det = cross2(n0, adjN[i][j]) * (j == 0 ? 1.0f : -1.0f);
                ignore[i][j] = solveDoubleSided ? 0 : (det < silhouettePrecision ? 1 : 0);
            } else {
                ignore[i][j] = 0;
            }
        }
    }
}
template <>
inline void Boundary<3>::buildAdjacency(bool solveDoubleSided, float silhouettePrecision) {
    int T = nPrims();
    std::map<std::pair<int, int>, std::array<int, 2>> edges;
    for (int i = 0; i < T; i++)
        for (int j = 0; j < 3; j++) {
            int I = idx[i][j], J = idx[i][(j + 1) % 3];
            bool sw = false;
            if (I > J) { std::swap(I, J); sw = true; }
            auto it = edges.find({I, J});
            if (it == edges.end()) it = edges.emplace(std::make_pair(I, J), std::array<int, 2>{-1, -1}).first;
            it->second[sw ? 1 : 0] = i;
        }
    adjN.assign(T, {}); hasAdj.assign(T, {}); ignore.assign(T, {});
    for (int i = 0; i < T; i++) {
        Vec<3> n0 = normalOf(i);
        for (int j = 0; j < 3; j++) {
            int I = idx[i][j], J = idx[i][(j + 1) % 3];
            bool sw = false;
            if (I > J) { std::swap(I, J); sw = true; }
            int a = edges[{I, J}][sw ? 0 : 1];
            if (a != -1) { hasAdj[i][j] = 1; adjN[i][j] = normalOf(a); }
            else { hasAdj[i][j] = 0; }
            if (hasAdj[i][j]) {
                Vec<3> pa = pos[idx[i][j]], pb = pos[idx[i][(j + 1) % 3]];
                Vec<3> e = normalized(pb - pa);
                const Vec<3>& nj = adjN[i][j];
                float dihedral = std::atan2(dot(e, cross3(nj, n0)), dot(n0, nj));
                ignore[i][j] = solveDoubleSided ? 0 : (dihedral < silhouettePrecision ? 1 : 0);
            } else {
                ignore[i][j] = 0;
            }
        }
    }
}

template <int D>
int Boundary<D>::buildRecursive(int start, int end, std::vector<Vec<D>>& centroids, int depth) {
    int nodeIndex = (int)nodes.size();
    nodes.emplace_back();
    Box<D> box, cbox;
    float area = 0.0f;
    for (int i = start; i < end; i++) {
        box.expand(boxOf(order[i]));
        cbox.expand(centroids[order[i]]);
        area += areaOf(order[i]);
    }
    nodes[nodeIndex].box = box;
    nodes[nodeIndex].area = area;
    int n = end - start;
    if (n <= 4 || depth > 60) {
        nodes[nodeIndex].start = start; nodes[nodeIndex].count = n;
        return nodeIndex;
    }
    // binned SAH over centroids (16 bins per axis)
    const int B = 16;
    float bestCost = kMaxFloat; int bestAxis = -1, bestSplit = -1;
    for (int axis = 0; axis < D; axis++) {
        float lo = cbox.lo[axis], hi = cbox.hi[axis];
        if (hi - lo < 1e-12f) continue;
        Box<D> bb[B]; int cnt[B] = {0};
        for (int i = start; i < end; i++) {
            int b = std::min(B - 1, (int)(B * (centroids[order[i]][axis] - lo) / (hi - lo)));
            cnt[b]++; bb[b].expand(boxOf(order[i]));
        }
        Box<D> lb[B]; int lc[B]; Box<D> acc; int c = 0;
        for (int b = 0; b < B; b++) { acc.expand(bb[b]); c += cnt[b]; lb[b] = acc; lc[b] = c; }
        acc = Box<D>(); c = 0;
        for (int b = B - 1; b > 0; b--) {
            acc.expand(bb[b]); c += cnt[b];
            if (lc[b - 1] == 0 || c == 0) continue;
            float cost = lb[b - 1].surface() * lc[b - 1] + acc.surface() * c;
            if (cost < bestCost) { bestCost = cost; bestAxis = axis; bestSplit = b; }
        }
    }
    int mid;
    if (bestAxis < 0) {
        mid = start + n / 2;
    } else {
        float lo = cbox.lo[bestAxis], hi = cbox.hi[bestAxis];
        auto it = std::partition(order.begin() + start, order.begin() + end, [&](int p) {
            int b = std::min(B - 1, (int)(B * (centroids[p][bestAxis] - lo) / (hi - lo)));
            return b < bestSplit;
        });
        mid = (int)(it - order.begin());
        if (mid == start || mid == end) mid = start + n / 2;
    }
    int l = buildRecursive(start, mid, centroids, depth + 1);
    int r = buildRecursive(mid, end, centroids, depth + 1);
    nodes[nodeIndex].left = l; nodes[nodeIndex].right = r;
    return nodeIndex;
}

template <int D>
void Boundary<D>::buildBvh() {
    int P = nPrims();
    order.resize(P);
    for (int i = 0; i < P; i++) order[i] = i;
    nodes.clear();
    if (P == 0) return;
    std::vector<Vec<D>> centroids(P);
    for (int i = 0; i < P; i++) {
        Vec<D> c;
        for (int k = 0; k < D; k++) c = c + pos[idx[i][k]];
        centroids[i] = c / (float)D;
    }
    buildRecursive(0, P, centroids, 0);
}

// closest point (fcpw Aggregate::findClosestPoint as called at fcpw_geometric_queries.h:1074)
template <int D>
bool Boundary<D>::closestPoint(const Vec<D>& x, Vec<D>& ptOut, Vec<D>& nOut, float& dOut, int& primOut) const {
    float best = kMaxFloat; int bestPrim = -1; Vec<D> bestPt;
    Counters& C = counters();
    C.calls[0]++;
    auto test = [&](int i) {
        C.prims[0]++;
        Vec<D> p[D]; prim(i, p); Vec<D> q;
        float d = closestPointPrim(p, x, q);
        if (d < best || (d == best && i < bestPrim)) { best = d; bestPrim = i; bestPt = q; }
    };
    if (!useBvh || nodes.empty()) {
        for (int i = 0; i < nPrims(); i++) test(i);
    } else {
        int stack[128]; float sd[128]; int sp = 0;
        stack[sp] = 0; sd[sp] = nodes[0].box.dist2(x); sp++;
        while (sp > 0) {
            sp--; int ni = stack[sp]; float d2 = sd[sp];
            if (d2 > best * best) continue;
            const Node& nd = nodes[ni];
            C.nodes[0]++;
            if (nd.count > 0) { for (int k = 0; k < nd.count; k++) test(order[nd.start + k]); continue; }
            float dl = nodes[nd.left].box.dist2(x), dr = nodes[nd.right].box.dist2(x);
            if (dl <= dr) { stack[sp] = nd.right; sd[sp++] = dr; stack[sp] = nd.left; sd[sp++] = dl; }
            else { stack[sp] = nd.left; sd[sp++] = dl; stack[sp] = nd.right; sd[sp++] = dr; }
        }
    }
    if (bestPrim < 0) return false;
    ptOut = bestPt; nOut = normalOf(bestPrim); dOut = best; primOut = bestPrim;
    return true;
}

// first hit (fcpw Aggregate::intersect(ray) at fcpw_geometric_queries.h:1107, :1188)
template <int D>
bool Boundary<D>::intersect(const Vec<D>& o, const Vec<D>& dir, float tMax, Vec<D>& ptOut, Vec<D>& nOut, float& tOut, int& primOut,
                            int kind) const {
    float best = tMax; int bestPrim = -1;
    Counters& C = counters();
    C.calls[kind]++;
    auto test = [&](int i) {
        C.prims[kind]++;
        Vec<D> p[D]; prim(i, p); float t;
        if (intersectPrim(p, o, dir, best, t)) {
            if (bestPrim < 0 || t < best || (t == best && i < bestPrim)) { best = t; bestPrim = i; }
        }
    };
    if (!useBvh || nodes.empty()) {
        for (int i = 0; i < nPrims(); i++) test(i);
    } else {
        Vec<D> invD; for (int k = 0; k < D; k++) invD[k] = 1.0f / dir[k];
        int stack[128]; int sp = 0; stack[sp++] = 0;
        while (sp > 0) {
            int ni = stack[--sp];
            const Node& nd = nodes[ni];
            C.nodes[kind]++;
            if (!nd.box.rayOverlap(o, invD, best)) continue;
            if (nd.count > 0) { for (int k = 0; k < nd.count; k++) test(order[nd.start + k]); continue; }
            stack[sp++] = nd.right; stack[sp++] = nd.left;
        }
    }
    if (bestPrim < 0) return false;
    tOut = best; primOut = bestPrim; ptOut = o + dir * best; nOut = normalOf(bestPrim);
    return true;
}

template <int D>
int Boundary<D>::countHits(const Vec<D>& o, const Vec<D>& dir, float tMax) const {
    int hits = 0;
    for (int i = 0; i < nPrims(); i++) { Vec<D> p[D]; prim(i, p); float t; if (intersectPrim(p, o, dir, tMax, t)) hits++; }
    return hits;
}

// fcpw Aggregate::hasLineOfSight (fcpw_geometric_queries.h:1225): segment a->b blocked?
template <int D>
bool Boundary<D>::occluded(const Vec<D>& a, const Vec<D>& b) const {
    Vec<D> dir = b - a;
    float len = norm(dir);
    if (len <= 0.0f) return false;
    dir = dir / len;
    Vec<D> pt, n; float t; int pi;
    return intersect(a, dir, len, pt, n, t, pi, 2);
}

// reflectance_boundary_bvh/geometry.h:85-154 (2D) and :169-236 (3D)
template <>
inline void Boundary<2>::primStarRadius(int i, const Vec<2>& c, float& r2, bool flip, float precision) const {
    Vec<2> p[2]; prim(i, p);
    Vec<2> closest; float cd = closestPointPrim(p, c, closest);
    float cd2 = cd * cd;
    if (cd2 > r2) return;
    if (kmax[i] < kMaxFloat - kFcpwEpsilon) {
        Vec<2> n0 = primNormal(p, true);
        Vec<2> viewDirClosest = c - closest;
        for (int j = 0; j < 2; j++) {
            if (ignore[i][j]) continue;
            Vec<2> viewDir = c - p[j];
            float sd = norm(viewDir);
            bool sil = !hasAdj[i][j];
            if (!sil) sil = j == 0 ? isSilhouetteVertex(adjN[i][0], n0, viewDir, sd, flip, precision)
                                   : isSilhouetteVertex(n0, adjN[i][1], viewDir, sd, flip, precision);
            if (sil) r2 = std::min(r2, sd * sd);
        }
        if (kmax[i] > kFcpwEpsilon) {
            if (cd < kFcpwEpsilon) {
                r2 = cd;
            } else if (r2 > cd2) {
                Vec<2> far; float fd = farthestPointPrim(p, c, far);
                robinStarRadiusBound(c, r2, kmax[i], viewDirClosest, cd, c - far, fd, p[0], n0);
            }
        }
    } else {
        r2 = std::min(r2, cd2);
    }
}
template <>
inline void Boundary<3>::primStarRadius(int i, const Vec<3>& c, float& r2, bool flip, float precision) const {
    Vec<3> p[3]; prim(i, p);
    Vec<3> closest; float cd = closestPointPrim(p, c, closest);
    float cd2 = cd * cd;
    if (cd2 > r2) return;
    if (kmax[i] < kMaxFloat - kFcpwEpsilon) {
        Vec<3> n0 = primNormal(p, true);
        Vec<3> viewDirClosest = c - closest;
        for (int j = 0; j < 3; j++) {
            if (ignore[i][j]) continue;
            const Vec<3>& pj = p[j];
            const Vec<3>& pk = p[(j + 1) % 3];
            Vec<3> q; float sd = closestPointSegment3(pj, pk, c, q);
            Vec<3> viewDir = c - q;
            bool sil = !hasAdj[i][j];
            if (!sil) sil = isSilhouetteEdge(pj, pk, n0, adjN[i][j], viewDir, sd, flip, precision);
            if (sil) r2 = std::min(r2, sd * sd);
        }
        if (kmax[i] > kFcpwEpsilon) {
            if (cd < kFcpwEpsilon) {
                r2 = cd;
            } else if (r2 > cd2) {
                Vec<3> far; float fd = farthestPointPrim(p, c, far);
                robinStarRadiusBound(c, r2, kmax[i], viewDirClosest, cd, c - far, fd, p[0], n0);
            }
        }
    } else {
        r2 = std::min(r2, cd2);
    }
}


template <int D>
int Boundary<D>::buildFeatureRecursive(int start, int end, int depth) {
    int id = (int)fnodes.size();
    fnodes.emplace_back();
    Box<D> box, cbox;
    for (int i = start; i < end; i++) {
        const Feature& f = feats[forder[i]];
        box.expand(f.a); box.expand(f.b);
        cbox.expand(0.5f * (f.a + f.b));
    }
    fnodes[id].box = box;
    int n = end - start;
    if (n <= 4 || depth > 60) { fnodes[id].start = start; fnodes[id].count = n; return id; }
    int ax = 0;
    for (int i = 1; i < D; i++) if (cbox.hi[i] - cbox.lo[i] > cbox.hi[ax] - cbox.lo[ax]) ax = i;
    int mid = start + n / 2;
    std::nth_element(forder.begin() + start, forder.begin() + mid, forder.begin() + end, [&](int p, int q) {
        return feats[p].a[ax] + feats[p].b[ax] < feats[q].a[ax] + feats[q].b[ax];
    });
    int l = buildFeatureRecursive(start, mid, depth + 1);
    int r = buildFeatureRecursive(mid, end, depth + 1);
    fnodes[id].left = l; fnodes[id].right = r;
    return id;
}

template <int D>
void Boundary<D>::buildFeatureTree() {
    feats.clear(); fnodes.clear(); forder.clear();
    if (kind != ZGPU_BOUNDARY_NEUMANN) return;
    for (int i = 0; i < nPrims(); i++) {
        Vec<D> p[D]; prim(i, p);
        Vec<D> n0 = primNormal(p, true);
        for (int j = 0; j < D; j++) {
            if (ignore[i][j]) continue;
            Feature f;
            f.open = !hasAdj[i][j];
            if constexpr (D == 2) {
                f.a = p[j]; f.b = p[j];
                f.nA = j == 0 ? adjN[i][0] : n0;   // the segment before the vertex
                f.nB = j == 0 ? n0 : adjN[i][1];   // the segment after it
            } else {
                f.a = p[j]; f.b = p[(j + 1) % 3];
                f.nA = n0; f.nB = adjN[i][j];
            }
            // a feature shared by two faces is kept once (by the first face that lists it)
            bool dup = false;
            if (!f.open) {
                if constexpr (D == 2) dup = j == 1;   // each interior vertex: keep the copy of the segment it starts
                else dup = false;
            }
            if (!dup) feats.push_back(f);
        }
    }
    if constexpr (D == 3) {
        // dedupe shared edges by their sorted endpoint coordinates
        std::map<std::array<float, 6>, int> seen;
        std::vector<Feature> kept;
        for (auto& f : feats) {
            std::array<float, 6> k;
            bool ab = std::lexicographical_compare(f.a.v, f.a.v + 3, f.b.v, f.b.v + 3);
            for (int i = 0; i < 3; i++) { k[i] = ab ? f.a[i] : f.b[i]; k[3 + i] = ab ? f.b[i] : f.a[i]; }
            if (f.open || seen.emplace(k, 1).second) kept.push_back(f);
        }
        feats.swap(kept);
    }
    if (feats.empty()) return;
    forder.resize(feats.size());
    for (size_t i = 0; i < feats.size(); i++) forder[i] = (int)i;
    buildFeatureRecursive(0, (int)feats.size(), 0);
    // cones over the features' normals
    for (auto& nd : fnodes) {
        std::vector<int> stk = {(int)(&nd - &fnodes[0])};
        std::vector<Vec<D>> ns;
        bool open = false;
        while (!stk.empty()) {
            const Node& m = fnodes[stk.back()]; stk.pop_back();
            if (m.count == 0) { stk.push_back(m.left); stk.push_back(m.right); continue; }
            for (int k = 0; k < m.count; k++) {
                const Feature& f = feats[forder[m.start + k]];
                open = open || f.open;
                ns.push_back(f.nA); ns.push_back(f.nB);
            }
        }
        nd.kmax = 0.0f;
        if (open) { nd.halfAngle = kPi; continue; }
        double a[3] = {0, 0, 0};
        for (auto& n : ns) for (int i = 0; i < D; i++) a[i] += n[i];
        double l = std::sqrt(a[0] * a[0] + a[1] * a[1] + a[2] * a[2]);
        if (l < 1e-6) { nd.halfAngle = kPi; continue; }
        for (int i = 0; i < 3; i++) nd.axis[i] = (float)(a[i] / l);
        double h = 0.0;
        for (auto& n : ns) {
            double c = 0.0;
            for (int i = 0; i < D; i++) c += nd.axis[i] * n[i];
            h = std::max(h, std::acos(std::max(-1.0, std::min(1.0, c))));
        }
        nd.halfAngle = (float)std::min((double)kPi, h + 1e-4);
    }
}

// closest silhouette point within sqrt(r2) (FCPW findClosestSilhouettePoint, fcpw_geometric_queries.h:1264)
template <int D>
float Boundary<D>::featureRadius2(const Vec<D>& x, float r2, bool flip, float precision) const {
    if (fnodes.empty()) return r2;
    Counters& C = counters();
    int stack[128]; int sp = 0; stack[sp++] = 0;
    while (sp > 0) {
        const Node& nd = fnodes[stack[--sp]];
        C.nodes[3]++;
        if (nd.box.dist2(x) > r2) continue;
        if (!coneMayHoldSilhouette(nd, x, precision)) continue;
        if (nd.count > 0) {
            for (int k = 0; k < nd.count; k++) {
                const Feature& f = feats[forder[nd.start + k]];
                C.prims[3]++;
                bool sil = f.open;
                float d;
                if constexpr (D == 2) {
                    Vec<2> view = x - f.a;
                    d = norm(view);
                    if (d * d >= r2) continue;
                    if (!sil) sil = isSilhouetteVertex(f.nA, f.nB, view, d, flip, precision);
                } else {
                    Vec<3> q;
                    d = closestPointSegment3(f.a, f.b, x, q);
                    if (d * d >= r2) continue;
                    if (!sil) sil = isSilhouetteEdge(f.a, f.b, f.nA, f.nB, x - q, d, flip, precision);
                }
                if (sil) r2 = d * d;
            }
            continue;
        }
        float dl = fnodes[nd.left].box.dist2(x), dr = fnodes[nd.right].box.dist2(x);
        if (dl <= dr) { stack[sp++] = nd.right; stack[sp++] = nd.left; }
        else { stack[sp++] = nd.left; stack[sp++] = nd.right; }
    }
    return r2;
}

// computeStarRadiusForReflectingBoundary: Neumann (fcpw_geometric_queries.h:1254-1268) and
// Robin (:1277-1289, ReflectanceBvh::computeSquaredStarRadius bvh.h:414-506) in one rule:
// with kappa = 0 the reflectance primitives reduce to the closest-silhouette distance.
template <int D>
float Boundary<D>::starRadius(const Vec<D>& x, float minR, float maxR, float precision, bool flip) const {
    if (minR > maxR) return maxR;
    float r2 = maxR < kMaxFloat ? maxR * maxR : kMaxFloat;
    Counters& C = counters();
    C.calls[3]++;
    if (useBvh && kind == ZGPU_BOUNDARY_NEUMANN) return std::max(std::sqrt(featureRadius2(x, r2, flip, precision)), minR);
    if (!useBvh || nodes.empty()) {
        for (int i = 0; i < nPrims(); i++) primStarRadius(i, x, r2, flip, precision);
        C.prims[3] += nPrims();
    } else {
        // ReflectanceBvh::computeSquaredStarRadius (bvh.h:414-506): a node is entered with the
        // lower bound of its radius as key; a node without silhouettes also caps the radius
        int stack[128]; float key[128]; int sp = 0;
        float lo, hi;
        C.nodes[3]++;
        if (robinVisit(nodes[0], x, r2, lo, hi)) { stack[sp] = 0; key[sp] = lo; sp++; }
        while (sp > 0) {
            sp--;
            int ni = stack[sp];
            if (key[sp] > r2) continue;
            const Node& nd = nodes[ni];
            if (nd.count > 0) {
                for (int k = 0; k < nd.count; k++) primStarRadius(order[nd.start + k], x, r2, flip, precision);
                C.prims[3] += nd.count;
                continue;
            }
            float l0, h0, l1, h1;
            C.nodes[3] += 2;
            bool hit0 = robinVisit(nodes[nd.left], x, r2, l0, h0);
            if (hit0) r2 = std::min(r2, h0);
            bool hit1 = robinVisit(nodes[nd.right], x, r2, l1, h1);
            if (hit1) r2 = std::min(r2, h1);
            // farther child first, the closer one on top
            if (hit0 && hit1 && l1 < l0) { stack[sp] = nd.left; key[sp] = l0; sp++; stack[sp] = nd.right; key[sp] = l1; sp++; }
            else {
                if (hit1) { stack[sp] = nd.right; key[sp] = l1; sp++; }
                if (hit0) { stack[sp] = nd.left; key[sp] = l0; sp++; }
            }
        }
    }
    return std::max(std::sqrt(r2), minR);
}

// ReflectanceBvh::visitNode (bvh.h:369-412) with RobinBvhNodeBound (robin_bounds.h:110-154):
// false when the node cannot lower the radius; otherwise r2Min is the key it is entered with
// and r2Max a radius every primitive below it allows
template <int D>
bool Boundary<D>::robinVisit(const Node& nd, const Vec<D>& x, float r2, float& r2Min, float& r2Max) const {
    r2Min = nd.box.dist2(x);
    r2Max = nd.box.maxDist2(x);
    if (r2Min > r2) return false;
    if (nd.kmin >= kMaxFloat - kFcpwEpsilon) return true;          // perfectly absorbing subtree
    // angular range of the normals as seen from x (the view cone of the box's bounding sphere)
    bool silhouette = nd.halfAngle >= 0.5f * kPi;
    float lo = 0.0f, hi = 0.5f * kPi;
    if (!silhouette) {
        Vec<D> v;
        float rb2 = 0.0f;
        for (int i = 0; i < D; i++) {
            float h = 0.5f * (nd.box.hi[i] - nd.box.lo[i]);
            rb2 += h * h;
            v[i] = x[i] - 0.5f * (nd.box.lo[i] + nd.box.hi[i]);
        }
        float dv = norm(v);
        if (dv * dv <= rb2) silhouette = true;
        else {
            Vec<D> a;
            for (int i = 0; i < D; i++) a[i] = nd.axis[i];
            float theta = std::acos(std::min(std::max(dot(a, v) / dv, -1.0f), 1.0f));
            float spread = nd.halfAngle + std::asin(std::min(std::sqrt(rb2) / dv, 1.0f));
            lo = theta - spread;
            hi = theta + spread;
            silhouette = spread >= 0.5f * kPi || (lo <= 0.5f * kPi && 0.5f * kPi <= hi);
        }
    }
    if (silhouette) { r2Max = kMaxFloat; return true; }
    if (nd.kmax <= kFcpwEpsilon) return false;                       // perfectly reflecting, no silhouette
    float rMin = std::sqrt(r2Min), rMax = std::sqrt(r2Max);
    float minCos = std::min(std::fabs(std::cos(lo)), std::fabs(std::cos(hi)));
    if constexpr (D == 2) {
        float a = rMin * std::exp(minCos / (nd.kmax * rMax));
        float b = rMax * std::exp(1.0f / (nd.kmin * rMin));
        r2Min = a * a;
        r2Max = b * b;
    } else {
        if (rMax < minCos / nd.kmax) r2Min = kMaxFloat;
        else { float a = rMin / (1.0f - minCos / (nd.kmax * rMax)); r2Min = a * a; }
        if (rMin < 1.0f / nd.kmin) r2Max = kMaxFloat;
        else { float b = rMax / (1.0f - 1.0f / (nd.kmin * rMin)); r2Max = b * b; }
    }
    if (!(r2Min == r2Min)) r2Min = 0.0f;
    if (!(r2Max == r2Max)) r2Max = kMaxFloat;
    return true;
}

// weighted pick: returns index i with probability w[i]/sum(w), rescales u to [0,1) for reuse
inline int pickWeighted(const float* w, int n, float& u, float& prob) {
    float total = 0.0f;
    for (int k = 0; k < n; k++) total += w[k];
    if (!(total > 0.0f)) return -1;
    float acc = 0.0f;
    int last = -1; float lastAcc = 0.0f;
    for (int k = 0; k < n; k++) {
        if (w[k] <= 0.0f) continue;
        float p = w[k] / total;
        if (u < acc + p) {
            u = std::min(std::max((u - acc) / p, 0.0f), 0.99999994f);
            prob *= p;
            return k;
        }
        last = k; lastAcc = acc;
        acc += p;
    }
    float p = w[last] / total;
    u = std::min(std::max((u - lastAcc) / p, 0.0f), 0.99999994f);
    prob *= p;
    return last;
}

// sampleReflectingBoundary (fcpw_geometric_queries.h:1227-1242): see header comment
template <int D>
bool Boundary<D>::sample(const Vec<D>& x, float radius, const float* uIn, Vec<D>& ptOut, Vec<D>& nOut, float& pdfOut) const {
    float R2 = radius * radius;
    float u0 = uIn[0];
    float prob = 1.0f;
    int chosen = -1;
    Counters& C = counters();
    C.calls[4]++;
    auto primWeight = [&](int i) -> float {
        C.prims[4]++;
        Vec<D> p[D]; prim(i, p); Vec<D> q;
        float d = closestPointPrim(p, x, q);
        return (d * d <= R2) ? primArea(p) * branchWeight(d * d) : 0.0f;
    };
    if (!useBvh || nodes.empty()) {
        std::vector<float> w(nPrims());
        for (int i = 0; i < nPrims(); i++) w[i] = primWeight(i);
        chosen = pickWeighted(w.data(), nPrims(), u0, prob);
    } else {
        int ni = 0;
        if (nodes[0].box.dist2(x) > R2) return false;
        while (true) {
            const Node& nd = nodes[ni];
            C.nodes[4]++;
            if (nd.count > 0) {
                float w[8];
                for (int k = 0; k < nd.count; k++) w[k] = primWeight(order[nd.start + k]);
                int k = pickWeighted(w, nd.count, u0, prob);
                chosen = k < 0 ? -1 : order[nd.start + k];
                break;
            }
            float w[2];
            float dl = nodes[nd.left].box.dist2(x), dr = nodes[nd.right].box.dist2(x);
            w[0] = dl <= R2 ? nodes[nd.left].area * branchWeight(dl) : 0.0f;
            w[1] = dr <= R2 ? nodes[nd.right].area * branchWeight(dr) : 0.0f;
            int k = pickWeighted(w, 2, u0, prob);
            if (k < 0) return false;
            ni = k == 0 ? nd.left : nd.right;
        }
    }
    if (chosen < 0) return false;
    Vec<D> p[D]; prim(chosen, p);
    // the first random number chose the primitive; the others place the point on it
    float uu[2] = {uIn[1], D > 2 ? uIn[D - 1] : 0.0f};
    float primPdf;
    ptOut = samplePointOnPrim(p, uu, nOut, primPdf);
    pdfOut = prob * primPdf;
    return true;
}

// normal cone per node over the faces adjacent to its non-ignored silhouette features
// (halfAngle < 0: no candidate; pi: an open feature or a degenerate axis) and the Robin
// coefficient range of the subtree.  On a Robin boundary the cone covers every face of the
// subtree and its neighbours, as computeBoundingConeForPrimitives does
// (reflectance_boundary_bvh/bvh.h:210-262): the node bounds need the range of all normals.
template <int D>
void Boundary<D>::buildCones() {
    if (nodes.empty() || kind == ZGPU_BOUNDARY_ABSORBING) return;
    for (auto& nd : nodes) {
        std::vector<int> stk = {(int)(&nd - &nodes[0])};
        std::vector<Vec<D>> ns;
        bool open = false;
        const bool all = kind == ZGPU_BOUNDARY_ROBIN;
        float km = 0.0f, kn = all ? kMaxFloat : 0.0f;
        while (!stk.empty()) {
            const Node& m = nodes[stk.back()]; stk.pop_back();
            if (m.count == 0) { stk.push_back(m.left); stk.push_back(m.right); continue; }
            for (int k = 0; k < m.count; k++) {
                int i = order[m.start + k];
                km = std::max(km, kmax[i]);
                if (all) kn = std::min(kn, kmin[i]);
                bool any = all;
                for (int j = 0; j < D; j++) {
                    if (!all && ignore[i][j]) continue;
                    if (!hasAdj[i][j]) { open = true; continue; }
                    ns.push_back(adjN[i][j]);
                    any = true;
                }
                if (any) ns.push_back(normalOf(i));
            }
        }
        nd.kmax = km;
        nd.kmin = kn;
        if (open) { nd.halfAngle = kPi; continue; }
        if (ns.empty()) { nd.halfAngle = -1.0f; continue; }
        double a[3] = {0, 0, 0};
        for (auto& n : ns) for (int i = 0; i < D; i++) a[i] += n[i];
        double l = std::sqrt(a[0] * a[0] + a[1] * a[1] + a[2] * a[2]);
        if (l < 1e-6) { nd.halfAngle = kPi; continue; }
        for (int i = 0; i < 3; i++) nd.axis[i] = (float)(a[i] / l);
        double h = 0.0;
        for (auto& n : ns) {
            double c = 0.0;
            for (int i = 0; i < D; i++) c += nd.axis[i] * n[i];
            h = std::max(h, std::acos(std::max(-1.0, std::min(1.0, c))));
        }
        nd.halfAngle = (float)std::min((double)kPi, h + 1e-4);
    }
}

// all normal/view angles on one side of pi/2 (beyond the silhouette test's precision band)
// -> every face front-facing or every face back-facing -> no silhouette in the subtree
template <int D>
bool Boundary<D>::coneMayHoldSilhouette(const Node& nd, const Vec<D>& x, float prec) const {
    if (nd.halfAngle < 0.0f) return false;
    if (nd.halfAngle >= 0.5f * kPi) return true;
    Vec<D> c, v;
    float rb2 = 0.0f;
    for (int i = 0; i < D; i++) {
        c[i] = 0.5f * (nd.box.lo[i] + nd.box.hi[i]);
        float h = 0.5f * (nd.box.hi[i] - nd.box.lo[i]);
        rb2 += h * h;
        v[i] = x[i] - c[i];
    }
    float rb = std::sqrt(rb2) + prec;
    float dv = norm(v);
    if (dv <= rb) return true;
    Vec<D> a;
    for (int i = 0; i < D; i++) a[i] = nd.axis[i];
    float theta = std::acos(std::min(std::max(dot(a, v) / dv, -1.0f), 1.0f));
    float beta = std::asin(std::min(rb / dv, 1.0f));
    float margin = std::asin(std::min(prec, 1.0f)) + 1e-3f;
    float spread = beta + nd.halfAngle;
    return !(theta + spread < 0.5f * kPi - margin || theta - spread > 0.5f * kPi + margin);
}

// Aggregate::signedVolume (computeSignedVolume, fcpw_geometric_queries.h:431-458)
template <int D>
double Boundary<D>::signedVolume() const {
    double v = 0.0;
    for (int i = 0; i < nPrims(); i++) {
        Vec<D> p[D]; prim(i, p);
        if constexpr (D == 2) {
            v += 0.5 * ((double)p[0][0] * p[1][1] - (double)p[0][1] * p[1][0]);
        } else {
            double a0 = p[0][0], a1 = p[0][1], a2 = p[0][2];
            double b0 = p[1][0], b1 = p[1][1], b2 = p[1][2];
            double c0 = p[2][0], c1 = p[2][1], c2 = p[2][2];
            v += ((a1 * b2 - a2 * b1) * c0 + (a2 * b0 - a0 * b2) * c1 + (a0 * b1 - a1 * b0) * c2) / 6.0;
        }
    }
    return v;
}

}  // namespace orc
