// zgpu_scene.cuh -- device layout of a boundary (wide BVH + primitives) and the fused
// geometric queries the walk issues every step:
//   closest point           (FCPW findClosestPoint,    utils/fcpw_geometric_queries.h:1074)
//   first ray hit / any hit (FCPW intersect, hasLineOfSight, :1107, :1188, :1225)
//   star radius             (findClosestSilhouettePoint :1264 / ReflectanceBvh bvh.h:414-506)
//   boundary sampling       (FCPW intersect(sphere, randNums, branchWeight) :1233)
//
// Layout in HBM (all 16-byte aligned, read with 128-bit __ldg loads):
//   node  = 8 float4 = 128 B (one L2 sector quad), 4 children in SoA:
//           [i] = child lower bound on axis i, [D+i] = upper bound on axis i,
//           [2D] = child references (int bits), [2D+1] = child surface area (sampling weight)
//   child reference: >= 0 internal node, EMPTY, or leaf -(1 + (first << 3 | count-1))
//   prim  = 2D: 1 float4 (a.xy, b.xy); 3D: 3 float4 (a.xyz,-), (b.xyz,-), (c.xyz,-)
//   sil   = reflecting boundaries only; 2D: (nPrev.xy, nNext.xy), (flags, kmin, kmax, 0)
//           3D: (n0.xyz, flags), (n1.xyz, kmin), (n2.xyz, kmax) -- neighbour normals across
//           each edge j = (v_j, v_j+1), flags = hasAdj bits 0..2 | ignore bits 3..5
#pragma once

#include "zgpu_math.cuh"

namespace zg {

constexpr int kWidth = 4;
constexpr int kEmptyChild = 0x7fffffff;
constexpr int kMaxStack = 64;      // upper bound of the per-thread traversal stack (shared memory)
constexpr int kMaxWideDepth = 20;   // 3 * depth + 2 <= kMaxStack
// stack entries a traversal of a tree of the given wide depth can hold at once
// (a traversal holds at most width - 1 pushed siblings per level, plus slack)
inline int stackEntriesForDepth(int depth, int width = 4) {
    int e = (width - 1) * depth + 2;
    return e < 8 ? 8 : (e > kMaxStack ? kMaxStack : e);
}

// Per-thread traversal stack in shared memory: entry k of this thread at [k * stride + lane].
// Every query of a walk step reuses the same stack (they run one after another).
struct TravStack {
    int* node;
    float* key;
    int stride;
    int cap;
    ZG_D void put(int k, int n, float d) { node[k * stride] = n; key[k * stride] = d; }
    ZG_D int nodeAt(int k) const { return node[k * stride]; }
    ZG_D float keyAt(int k) const { return key[k * stride]; }
};

// device error word bits
constexpr uint32_t kErrStackOverflow = 1u;
constexpr uint32_t kErrSplitOverflow = 2u;
constexpr uint32_t kErrBudget = 4u;
constexpr uint32_t kErrBadInput = 8u;
constexpr uint32_t kErrCacheOverflow = 16u;

struct BoundaryView {
    const float4* nodes = nullptr;
    const float4* cones = nullptr;   // reflecting boundaries: 8 float4 per node (child cones, child max kappa)
    const float4* prims = nullptr;
    const float4* sil = nullptr;
    const int* primIndex = nullptr;
    int nNodes = 0;
    int nPrims = 0;
    int stackEntries = 8;   // traversal stack entries this tree needs (from its wide depth)
    // silhouette-candidate tree of a Neumann boundary (Robin boundaries use the primitives)
    const float4* silTree = nullptr;
    const float4* silCones = nullptr;
    const float4* silFeat = nullptr;
    int silNodes = 0;
    int robin = 0;
    int width = 4;          // children per node: 4, or 8 (3D absorbing boundaries)
};

ZG_HD bool isLeaf(int c) { return c < 0; }
ZG_HD int leafFirst(int c) { return (-c - 1) >> 3; }
ZG_HD int leafCount(int c) { return ((-c - 1) & 7) + 1; }
ZG_HD int makeLeaf(int first, int count) { return -(1 + ((first << 3) | (count - 1))); }

// A node of W children (W = 4 or 8) is 2W float4: with G = W / 4 groups of 4 children,
// float4 [i G + g] holds the lower bounds on axis i of children 4g .. 4g + 3, [(D + i) G + g]
// the upper bounds, [2 D G + g] the child references and [(2 D + 1) G + g] the areas.
template <int D, int W = 4>
struct WideNode {
    float lo[D][W], hi[D][W];
    int child[W];
};

template <int D, int W = 4>
ZG_D void loadNode(const BoundaryView& b, int n, WideNode<D, W>& w) {
    constexpr int G = W / 4;
    const float4* p = b.nodes + (size_t)n * (2 * W);
#pragma unroll
    for (int i = 0; i < D; i++) {
#pragma unroll
        for (int g = 0; g < G; g++) {
            float4 l = __ldg(p + i * G + g), h = __ldg(p + (D + i) * G + g);
            w.lo[i][4 * g] = l.x; w.lo[i][4 * g + 1] = l.y; w.lo[i][4 * g + 2] = l.z; w.lo[i][4 * g + 3] = l.w;
            w.hi[i][4 * g] = h.x; w.hi[i][4 * g + 1] = h.y; w.hi[i][4 * g + 2] = h.z; w.hi[i][4 * g + 3] = h.w;
        }
    }
#pragma unroll
    for (int g = 0; g < G; g++) {
        int4 c = __ldg(reinterpret_cast<const int4*>(p + 2 * D * G + g));
        w.child[4 * g] = c.x; w.child[4 * g + 1] = c.y; w.child[4 * g + 2] = c.z; w.child[4 * g + 3] = c.w;
    }
}
ZG_D float4 loadNodeArea(const BoundaryView& b, int n, int D) { return __ldg(b.nodes + (size_t)n * 8 + 2 * D + 1); }

template <int D, int W>
ZG_D float boxDist2(const WideNode<D, W>& w, int k, V<D> x) {
    float s = 0.0f;
#pragma unroll
    for (int i = 0; i < D; i++) {
        float d = fmaxf(fmaxf(w.lo[i][k] - x[i], 0.0f), x[i] - w.hi[i][k]);
        s += d * d;
    }
    return s;
}
// slab test: entry distance of the ray (o, invDir) into child k within [0, tMax], or inf
template <int D, int W>
ZG_D float boxRay(const WideNode<D, W>& w, int k, V<D> o, V<D> inv, float tMax) {
    float t0 = 0.0f, t1 = tMax;
#pragma unroll
    for (int i = 0; i < D; i++) {
        float a = (w.lo[i][k] - o[i]) * inv[i];
        float c = (w.hi[i][k] - o[i]) * inv[i];
        t0 = fmaxf(t0, fminf(a, c));
        t1 = fminf(t1, fmaxf(a, c));
    }
    return t0 <= t1 * 1.0000002f ? t0 : kFltMax;
}

// ---------------------------------------------------------------- primitive access
template <int D> struct Prim { V<D> p[D]; };
ZG_D Prim<2> loadPrim(const BoundaryView& b, int i, V<2>) {
    float4 q = __ldg(b.prims + i);
    Prim<2> r; r.p[0][0] = q.x; r.p[0][1] = q.y; r.p[1][0] = q.z; r.p[1][1] = q.w; return r;
}
ZG_D Prim<3> loadPrim(const BoundaryView& b, int i, V<3>) {
    Prim<3> r;
#pragma unroll
    for (int k = 0; k < 3; k++) {
        float4 q = __ldg(b.prims + 3 * (size_t)i + k);
        r.p[k][0] = q.x; r.p[k][1] = q.y; r.p[k][2] = q.z;
    }
    return r;
}
template <int D> ZG_D Prim<D> loadPrim(const BoundaryView& b, int i) { return loadPrim(b, i, V<D>()); }

// unnormalised normal (geometry_helpers.h:15-21, :77-81): outward for CCW winding
ZG_D V<2> primNormalRaw(const Prim<2>& t) { V<2> s = t.p[1] - t.p[0]; V<2> n; n[0] = s[1]; n[1] = -s[0]; return n; }
ZG_D V<3> primNormalRaw(const Prim<3>& t) { return cross3(t.p[1] - t.p[0], t.p[2] - t.p[0]); }
template <int D> ZG_D V<D> primNormal(const Prim<D>& t) { V<D> n = primNormalRaw(t); return (1.0f / len(n)) * n; }
ZG_D float primArea(const Prim<2>& t) { return len(primNormalRaw(t)); }
ZG_D float primArea(const Prim<3>& t) { return 0.5f * len(primNormalRaw(t)); }

// closest point on a segment (geometry_helpers.h:28-49)
template <int D>
ZG_D float closestOnSegment(V<D> a, V<D> b, V<D> x, V<D>& pt) {
    V<D> u = b - a, v = x - a;
    float c1 = dot(u, v);
    if (c1 <= 0.0f) { pt = a; return len(x - a); }
    float c2 = dot(u, u);
    if (c2 <= c1) { pt = b; return len(x - b); }
    pt = a + (c1 / c2) * u;
    return len(x - pt);
}
ZG_D float closestOnPrim(const Prim<2>& t, V<2> x, V<2>& pt) { return closestOnSegment<2>(t.p[0], t.p[1], x, pt); }
// closest point on a triangle by Voronoi regions (geometry_helpers.h:94-161; Ericson 5.1.5)
ZG_D float closestOnPrim(const Prim<3>& t, V<3> x, V<3>& pt) {
    V<3> a = t.p[0], b = t.p[1], c = t.p[2];
    V<3> ab = b - a, ac = c - a, ax = x - a;
    float d1 = dot(ab, ax), d2 = dot(ac, ax);
    if (d1 <= 0.0f && d2 <= 0.0f) { pt = a; return len(x - a); }
    V<3> bx = x - b;
    float d3 = dot(ab, bx), d4 = dot(ac, bx);
    if (d3 >= 0.0f && d4 <= d3) { pt = b; return len(x - b); }
    V<3> cx = x - c;
    float d5 = dot(ab, cx), d6 = dot(ac, cx);
    if (d6 >= 0.0f && d5 <= d6) { pt = c; return len(x - c); }
    float vc = d1 * d4 - d3 * d2;
    if (vc <= 0.0f && d1 >= 0.0f && d3 <= 0.0f) { float v = d1 / (d1 - d3); pt = a + v * ab; return len(x - pt); }
    float vb = d5 * d2 - d1 * d6;
    if (vb <= 0.0f && d2 >= 0.0f && d6 <= 0.0f) { float w = d2 / (d2 - d6); pt = a + w * ac; return len(x - pt); }
    float va = d3 * d6 - d5 * d4;
    if (va <= 0.0f && (d4 - d3) >= 0.0f && (d5 - d6) >= 0.0f) {
        float w = (d4 - d3) / ((d4 - d3) + (d5 - d6)); pt = b + w * (c - b); return len(x - pt);
    }
    float denom = 1.0f / (va + vb + vc);
    float v = vb * denom, w = vc * denom;
    pt = a + v * ab + w * ac;
    return len(x - pt);
}
ZG_D float farthestOnPrim(const Prim<2>& t, V<2> x, V<2>& pt) {
    float da = len2(x - t.p[0]), db = len2(x - t.p[1]);
    if (da > db) { pt = t.p[0]; return sqrtf(da); }
    pt = t.p[1]; return sqrtf(db);
}
ZG_D float farthestOnPrim(const Prim<3>& t, V<3> x, V<3>& pt) {
    float da = len2(x - t.p[0]), db = len2(x - t.p[1]), dc = len2(x - t.p[2]);
    if (da >= db && da >= dc) { pt = t.p[0]; return sqrtf(da); }
    if (db >= da && db >= dc) { pt = t.p[1]; return sqrtf(db); }
    pt = t.p[2]; return sqrtf(dc);
}
// ray / primitive: 2D segment by Cramer's rule, 3D Moller-Trumbore; t in [0, tMax]
ZG_D bool rayPrim(const Prim<2>& t, V<2> o, V<2> d, float tMax, float& tHit) {
    V<2> e = t.p[1] - t.p[0];
    float den = cross2(d, e);
    if (fabsf(den) < 1e-20f) return false;
    V<2> w = t.p[0] - o;
    float tt = cross2(w, e) / den;
    float s = cross2(w, d) / den;
    if (tt < 0.0f || tt > tMax || s < 0.0f || s > 1.0f) return false;
    tHit = tt;
    return true;
}
ZG_D bool rayPrim(const Prim<3>& t, V<3> o, V<3> d, float tMax, float& tHit) {
    V<3> e1 = t.p[1] - t.p[0], e2 = t.p[2] - t.p[0];
    V<3> pv = cross3(d, e2);
    float det = dot(e1, pv);
    if (fabsf(det) < 1e-20f) return false;
    float inv = 1.0f / det;
    V<3> tv = o - t.p[0];
    float u = dot(tv, pv) * inv;
    if (u < 0.0f || u > 1.0f) return false;
    V<3> qv = cross3(tv, e1);
    float v = dot(d, qv) * inv;
    if (v < 0.0f || u + v > 1.0f) return false;
    float tt = dot(e2, qv) * inv;
    if (tt < 0.0f || tt > tMax) return false;
    tHit = tt;
    return true;
}

// select among 4 register values by a runtime index (no local-memory array)
ZG_D int pick4(int k, int a0, int a1, int a2, int a3) { return k == 0 ? a0 : k == 1 ? a1 : k == 2 ? a2 : a3; }
ZG_D float pick4f(int k, float a0, float a1, float a2, float a3) { return k == 0 ? a0 : k == 1 ? a1 : k == 2 ? a2 : a3; }
// the same over W registers
template <int W, typename T>
ZG_D T pickW(int k, const T (&a)[W]) {
    if constexpr (W == 4) {
        return k == 0 ? a[0] : k == 1 ? a[1] : k == 2 ? a[2] : a[3];
    } else {
        T v = a[0];
#pragma unroll
        for (int j = 1; j < W; j++) v = k == j ? a[j] : v;
        return v;
    }
}

// ---------------------------------------------------------------- child ordering
// Up to W internal children sorted by key with a fixed network (constant indices keep the
// arrays in registers); invalid slots carry key = +inf.  W = 4: 5 comparators; W = 8: the
// 19-comparator network (Knuth, TAOCP 5.3.4).
template <int W = 4>
struct ChildOrderW {
    float k[W];
    int c[W];
    ZG_D void clear() {
#pragma unroll
        for (int i = 0; i < W; i++) { k[i] = kFltMax; c[i] = -1; }
    }
    ZG_D void cswap(int a, int b) {
        bool sw = k[b] < k[a];
        float tk = sw ? k[b] : k[a]; k[b] = sw ? k[a] : k[b]; k[a] = tk;
        int tc = sw ? c[b] : c[a]; c[b] = sw ? c[a] : c[b]; c[a] = tc;
    }
    ZG_D void sort() {
        if constexpr (W == 4) {
            cswap(0, 1); cswap(2, 3); cswap(0, 2); cswap(1, 3); cswap(1, 2);
        } else {
            cswap(0, 2); cswap(1, 3); cswap(4, 6); cswap(5, 7);
            cswap(0, 4); cswap(1, 5); cswap(2, 6); cswap(3, 7);
            cswap(0, 1); cswap(2, 3); cswap(4, 5); cswap(6, 7);
            cswap(2, 4); cswap(3, 5);
            cswap(1, 4); cswap(3, 6);
            cswap(1, 2); cswap(3, 4); cswap(5, 6);
        }
    }
};
using ChildOrder = ChildOrderW<4>;

// Loops over the W children of a node are either unrolled or kept as loops (COMPACT): the
// Walk on Stars kernel runs five traversals per step and is bound by instruction fetch under
// divergence, so its traversals (rays, silhouettes, and its closest points) take the compact
// form (measured +10% walk-steps/s on the 2D mixed workload); Walk on Spheres runs one
// traversal per step and keeps the unrolled closest-point form (the compact one measured
// -27% there).

// after sort(): descend into slot 0 now, push slots W-1 .. 1 (farthest first) when within bound
template <int W, bool COMPACT = false>
ZG_D int descendAndPush(ChildOrderW<W>& o, float bound, TravStack& S, int& sp, uint32_t& err) {
    if constexpr (COMPACT) {
#pragma unroll 1
        for (int i = W - 1; i >= 1; i--) {
            if (o.c[i] >= 0 && o.k[i] <= bound) {
                if (sp < S.cap) S.put(sp++, o.c[i], o.k[i]); else err |= kErrStackOverflow;
            }
        }
    } else {
#pragma unroll
        for (int i = W - 1; i >= 1; i--) {
            if (o.c[i] >= 0 && o.k[i] <= bound) {
                if (sp < S.cap) S.put(sp++, o.c[i], o.k[i]); else err |= kErrStackOverflow;
            }
        }
    }
    return (o.c[0] >= 0 && o.k[0] <= bound) ? o.c[0] : -1;
}

// pop the next entry still within bound (-1 when exhausted)
ZG_D int popWithin(float bound, TravStack& S, int& sp) {
    while (sp > 0) {
        --sp;
        if (S.keyAt(sp) <= bound) return S.nodeAt(sp);
    }
    return -1;
}

// ---------------------------------------------------------------- closest point
template <int D>
struct ClosestHit {
    float d;       // distance (kFltMax if none)
    int slot;      // leaf-order primitive slot (-1 if none)
    V<D> pt;
};

// seed >= 0: a primitive slot tested first, whose distance bounds the search from the start
// (the walk's previous closest primitive); the answer is the same primitive of least
// (distance, index) with or without it, as every comparison and pruning test is inclusive.
template <int D, int W, bool COMPACT>
__device__ __noinline__ ClosestHit<D> closestPointW(const BoundaryView& b, V<D> x, TravStack& S, uint32_t& err,
                                                    int seed) {
    ClosestHit<D> best; best.d = kFltMax; best.slot = -1; best.pt = vzero<D>();
    float best2 = kFltMax;
    int bestIdx = 0x7fffffff;
    if (b.nNodes == 0) return best;
    if (seed >= 0) {
        V<D> q;
        best.d = closestOnPrim(loadPrim<D>(b, seed), x, q);
        best.slot = seed; best.pt = q; best2 = best.d * best.d; bestIdx = __ldg(b.primIndex + seed);
    }
    int sp = 0;
    int node = 0;
    for (;;) {
        WideNode<D, W> w;
        loadNode<D, W>(b, node, w);
        ChildOrderW<W> ord; ord.clear();
        unsigned leaves = 0;
        float lk[W];
        if constexpr (COMPACT) {
#pragma unroll 1
        for (int k = 0; k < W; k++) {
            int c = w.child[k];
            float d2 = boxDist2<D>(w, k, x);
            lk[k] = d2;
            bool ok = c != kEmptyChild && d2 <= best2;
            if (ok && isLeaf(c)) leaves |= 1u << k;
            if (ok && !isLeaf(c)) { ord.k[k] = d2; ord.c[k] = c; }
        }
        } else {
#pragma unroll
        for (int k = 0; k < W; k++) {
            int c = w.child[k];
            float d2 = boxDist2<D>(w, k, x);
            lk[k] = d2;
            bool ok = c != kEmptyChild && d2 <= best2;
            if (ok && isLeaf(c)) leaves |= 1u << k;
            if (ok && !isLeaf(c)) { ord.k[k] = d2; ord.c[k] = c; }
        }
        }
        while (leaves) {
            int k = __ffs(leaves) - 1;
            leaves &= leaves - 1;
            if (pickW<W>(k, lk) > best2) continue;   // pruned by a closer hit
            int c = pickW<W>(k, w.child);
            int first = leafFirst(c), count = leafCount(c);
#pragma unroll 1
            for (int j = 0; j < count; j++) {
                Prim<D> t = loadPrim<D>(b, first + j);
                V<D> q;
                float d = closestOnPrim(t, x, q);
                int idx = __ldg(b.primIndex + first + j);
                if (d < best.d || (d == best.d && idx < bestIdx)) {
                    best.d = d; best.slot = first + j; best.pt = q; best2 = d * d; bestIdx = idx;
                }
            }
        }
        ord.sort();
        int next = descendAndPush<W, COMPACT>(ord, best2, S, sp, err);
        node = next >= 0 ? next : popWithin(best2, S, sp);
        if (node < 0) break;
    }
    return best;
}

// closest point on a boundary of either node width (8-wide trees exist for 3D only)
template <int D, bool COMPACT = false>
ZG_D ClosestHit<D> closestPoint(const BoundaryView& b, V<D> x, TravStack& S, uint32_t& err, int seed = -1) {
    if constexpr (D == 3) {
        if (b.width == 8) return closestPointW<D, 8, COMPACT>(b, x, S, err, seed);
    }
    return closestPointW<D, 4, COMPACT>(b, x, S, err, seed);
}

// ---------------------------------------------------------------- warp-cooperative closest point
// All 32 lanes of a warp answer one query together (the caller loops over the lanes that
// need one).  A greedy descent to the nearest leaf gives the first bound; then each round
// takes up to 8 stack entries and tests their 4 children in parallel (lane = 4 * entry +
// child), pushes internal children within the bound and gathers the primitives of leaf
// children, which are tested 32 at a time.  The bound only shrinks and every comparison is
// inclusive, so the answer -- the primitive of least (distance, index) -- is the one the
// per-thread traversal returns.  The per-warp stack holds kCoopStack entries; on overflow the
// query stops and kErrStackOverflow is raised.
constexpr int kCoopStack = 480;
constexpr int kCoopPrims = 256;       // 8 entries x 4 leaf children x up to 8 primitives
struct CoopWork {
    int node[kCoopStack];
    float key[kCoopStack];
    int prim[kCoopPrims];
};

// component c of a float4 (c uniform within a quad of lanes, varying across the warp)
ZG_D float comp4(float4 v, int c) { return c == 0 ? v.x : c == 1 ? v.y : c == 2 ? v.z : v.w; }
ZG_D int comp4i(int4 v, int c) { return c == 0 ? v.x : c == 1 ? v.y : c == 2 ? v.z : v.w; }

template <int D, int NW = 4>
ZG_D float childBoxDist2(const BoundaryView& b, int node, int c, V<D> x, int& child) {
    constexpr int G = NW / 4;
    const float4* p = b.nodes + (size_t)node * (2 * NW) + (c >> 2);
    const int cc = c & 3;
    float s = 0.0f;
#pragma unroll
    for (int i = 0; i < D; i++) {
        float lo = comp4(__ldg(p + i * G), cc), hi = comp4(__ldg(p + (D + i) * G), cc);
        float d = fmaxf(fmaxf(lo - x[i], 0.0f), x[i] - hi);
        s += d * d;
    }
    child = comp4i(__ldg(reinterpret_cast<const int4*>(p + 2 * D * G)), cc);
    return s;
}

// folds the lanes' (d, idx, slot) candidates into the warp's best (uniform result)
ZG_D void warpBest(float d, int idx, int slot, float& bestD, int& bestIdx, int& bestSlot) {
    unsigned dm = __reduce_min_sync(0xffffffffu, __float_as_uint(d));   // d >= 0: bits order as values
    float dmin = __uint_as_float(dm);
    int im = __reduce_min_sync(0xffffffffu, (unsigned)(d == dmin ? idx : 0x7fffffff));
    unsigned owner = __ballot_sync(0xffffffffu, d == dmin && idx == im);
    int smin = __shfl_sync(0xffffffffu, slot, __ffs(owner) - 1);
    if (dmin < bestD || (dmin == bestD && im < bestIdx)) { bestD = dmin; bestIdx = im; bestSlot = smin; }
}

template <int D, int NW>
__device__ __noinline__ void coopClosestW(const BoundaryView& b, V<D> x, CoopWork& W, int lane, float& outD,
                                          int& outSlot, uint32_t& err) {
    constexpr int kShift = NW == 8 ? 3 : 2;        // lane = NW * entry + child
    constexpr int kTake = 32 / NW;                 // stack entries per round
    float bestD = kFltMax, best2 = kFltMax;
    int bestIdx = 0x7fffffff, bestSlot = -1;
    outD = kFltMax; outSlot = -1;
    if (b.nNodes == 0) return;
    const int c = lane & (NW - 1);
    // greedy descent: follow the nearest child to a leaf and test its primitives
    {
        int node = 0;
        for (int guard = 0; guard < kMaxWideDepth + 2; guard++) {
            int child;
            float d2 = childBoxDist2<D, NW>(b, node, c, x, child);
            if (child == kEmptyChild) d2 = kFltMax;
            unsigned m = __reduce_min_sync(0xffffffffu, __float_as_uint(d2));
            int k = __ffs(__ballot_sync(0xffffffffu, __float_as_uint(d2) == m)) - 1;
            int pick = __shfl_sync(0xffffffffu, child, k);
            if (pick == kEmptyChild) break;
            if (!isLeaf(pick)) { node = pick; continue; }
            float d = kFltMax; int idx = 0x7fffffff, slot = -1;
            if (lane < leafCount(pick)) {
                slot = leafFirst(pick) + lane;
                V<D> q;
                d = closestOnPrim(loadPrim<D>(b, slot), x, q);
                idx = __ldg(b.primIndex + slot);
            }
            warpBest(d, idx, slot, bestD, bestIdx, bestSlot);
            best2 = bestD * bestD;
            break;
        }
    }
    if (lane == 0) { W.node[0] = 0; W.key[0] = 0.0f; }
    int sp = 1;
    __syncwarp();
    while (sp > 0) {
        const int take = min(kTake, sp);
        sp -= take;
        const int e = lane >> kShift;
        int node = -1;
        float key = kFltMax;
        if (e < take) { node = W.node[sp + e]; key = W.key[sp + e]; }
        __syncwarp();
        int child = kEmptyChild;
        float d2 = kFltMax;
        if (node >= 0 && key <= best2) d2 = childBoxDist2<D, NW>(b, node, c, x, child);
        const bool ok = child != kEmptyChild && d2 <= best2;
        const bool inner = ok && !isLeaf(child), leaf = ok && isLeaf(child);
        // push the internal children
        const unsigned im = __ballot_sync(0xffffffffu, inner);
        const int nIn = __popc(im);
        if (sp + nIn > kCoopStack) { err |= kErrStackOverflow; break; }
        if (inner) {
            int pos = sp + __popc(im & ((1u << lane) - 1u));
            W.node[pos] = child;
            W.key[pos] = d2;
        }
        sp += nIn;
        // gather the leaf primitives: exclusive scan of the leaf sizes
        int cnt = leaf ? leafCount(child) : 0;
        int incl = cnt;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            int v = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += v;
        }
        const int total = __shfl_sync(0xffffffffu, incl, 31);
        for (int j = 0; j < cnt; j++) W.prim[incl - cnt + j] = leafFirst(child) + j;
        __syncwarp();
        for (int base = 0; base < total; base += 32) {
            float d = kFltMax; int idx = 0x7fffffff, slot = -1;
            if (base + lane < total) {
                slot = W.prim[base + lane];
                V<D> q;
                d = closestOnPrim(loadPrim<D>(b, slot), x, q);
                idx = __ldg(b.primIndex + slot);
            }
            warpBest(d, idx, slot, bestD, bestIdx, bestSlot);
            best2 = bestD * bestD;
        }
        __syncwarp();
    }
    outD = bestD;
    outSlot = bestSlot;
}

template <int D>
ZG_D void coopClosest(const BoundaryView& b, V<D> x, CoopWork& W, int lane, float& outD, int& outSlot, uint32_t& err) {
    if constexpr (D == 3) {
        if (b.width == 8) { coopClosestW<D, 8>(b, x, W, lane, outD, outSlot, err); return; }
    }
    coopClosestW<D, 4>(b, x, W, lane, outD, outSlot, err);
}

// ---------------------------------------------------------------- first ray hit
template <int D>
struct RayHit {
    float t;
    int slot;
};
template <int D>
ZG_D V<D> safeInv(V<D> d) {
    V<D> r;
#pragma unroll
    for (int i = 0; i < D; i++) r[i] = 1.0f / d[i];
    return r;
}

// anyHit = true stops at the first intersection (line-of-sight queries)
template <int D, int W>
__device__ __noinline__ RayHit<D> intersectRayW(const BoundaryView& b, V<D> o, V<D> dir, float tMax, bool anyHit,
                                                TravStack& S, uint32_t& err) {
    RayHit<D> hit; hit.t = tMax; hit.slot = -1;
    int bestIdx = 0x7fffffff;
    if (b.nNodes == 0) return hit;
    V<D> inv = safeInv<D>(dir);
    int sp = 0;
    int node = 0;
    for (;;) {
        WideNode<D, W> w;
        loadNode<D, W>(b, node, w);
        ChildOrderW<W> ord; ord.clear();
        unsigned leaves = 0;
#pragma unroll 1
        for (int k = 0; k < W; k++) {
            int c = w.child[k];
            float tn = boxRay<D>(w, k, o, inv, hit.t);
            bool ok = c != kEmptyChild && tn != kFltMax;
            if (ok && isLeaf(c)) leaves |= 1u << k;
            if (ok && !isLeaf(c)) { ord.k[k] = tn; ord.c[k] = c; }
        }
        while (leaves) {
            int k = __ffs(leaves) - 1;
            leaves &= leaves - 1;
            int c = pickW<W>(k, w.child);
            int first = leafFirst(c), count = leafCount(c);
#pragma unroll 1
            for (int j = 0; j < count; j++) {
                Prim<D> t = loadPrim<D>(b, first + j);
                float th;
                if (rayPrim(t, o, dir, hit.t, th)) {
                    int idx = __ldg(b.primIndex + first + j);
                    if (hit.slot < 0 || th < hit.t || (th == hit.t && idx < bestIdx)) {
                        hit.t = th; hit.slot = first + j; bestIdx = idx;
                        if (anyHit) return hit;
                    }
                }
            }
        }
        ord.sort();
        int next = descendAndPush<W, true>(ord, hit.t, S, sp, err);
        node = next >= 0 ? next : popWithin(hit.t, S, sp);
        if (node < 0) break;
    }
    return hit;
}

// first hit (anyHit: any hit) on a boundary of either node width
template <int D>
ZG_D RayHit<D> intersectRay(const BoundaryView& b, V<D> o, V<D> dir, float tMax, bool anyHit, TravStack& S,
                            uint32_t& err) {
    if constexpr (D == 3) {
        if (b.width == 8) return intersectRayW<D, 8>(b, o, dir, tMax, anyHit, S, err);
    }
    return intersectRayW<D, 4>(b, o, dir, tMax, anyHit, S, err);
}

// number of hits within tMax (intersect...AllHits, used by insideDomain)
template <int D, int W>
__device__ __noinline__ int countHitsW(const BoundaryView& b, V<D> o, V<D> dir, float tMax, TravStack& S, uint32_t& err) {
    if (b.nNodes == 0) return 0;
    V<D> inv = safeInv<D>(dir);
    int sp = 1;
    S.put(0, 0, 0.0f);
    int hits = 0;
    while (sp > 0) {
        WideNode<D, W> w;
        loadNode<D, W>(b, S.nodeAt(--sp), w);
        unsigned leaves = 0;
#pragma unroll 1
        for (int k = 0; k < W; k++) {
            int c = w.child[k];
            if (c == kEmptyChild || boxRay<D>(w, k, o, inv, tMax) == kFltMax) continue;
            if (isLeaf(c)) leaves |= 1u << k;
            else if (sp < S.cap) S.put(sp++, c, 0.0f);
            else err |= kErrStackOverflow;
        }
        while (leaves) {
            int k = __ffs(leaves) - 1;
            leaves &= leaves - 1;
            int c = pickW<W>(k, w.child);
            int first = leafFirst(c), count = leafCount(c);
#pragma unroll 1
            for (int j = 0; j < count; j++) {
                float th;
                if (rayPrim(loadPrim<D>(b, first + j), o, dir, tMax, th)) hits++;
            }
        }
    }
    return hits;
}

template <int D>
ZG_D int countHits(const BoundaryView& b, V<D> o, V<D> dir, float tMax, TravStack& S, uint32_t& err) {
    if constexpr (D == 3) {
        if (b.width == 8) return countHitsW<D, 8>(b, o, dir, tMax, S, err);
    }
    return countHitsW<D, 4>(b, o, dir, tMax, S, err);
}

// ---------------------------------------------------------------- silhouettes
// A vertex (2D) / edge (3D) is a silhouette from x when exactly one of its two adjacent
// faces is front-facing; degenerate views (x on a face plane or on the feature itself)
// are resolved by the concavity of the feature.  sign = -1 views the other side.
ZG_D bool silhouetteVertex(V<2> nPrev, V<2> nNext, V<2> view, float d, bool flip, float prec) {
    float sign = flip ? -1.0f : 1.0f;
    if (d <= prec) return sign * cross2(nPrev, nNext) < -prec;
    V<2> u = (1.0f / d) * view;
    float d0 = dot(nPrev, u), d1 = dot(nNext, u);
    if (fabsf(d0) <= prec) return sign * d1 > prec;
    if (fabsf(d1) <= prec) return sign * d0 > prec;
    return d0 * d1 < 0.0f;
}
ZG_D bool silhouetteEdge(V<3> pa, V<3> pb, V<3> nA, V<3> nB, V<3> view, float d, bool flip, float prec) {
    float sign = flip ? -1.0f : 1.0f;
    if (d <= prec) {
        V<3> e = pb - pa;
        e = (1.0f / len(e)) * e;
        return sign * dot(e, cross3(nB, nA)) > prec;
    }
    V<3> u = (1.0f / d) * view;
    float dA = dot(nA, u), dB = dot(nB, u);
    if (fabsf(dA) <= prec) return sign * dB > prec;
    if (fabsf(dB) <= prec) return sign * dA > prec;
    return dA * dB < 0.0f;
}

// Robin reflectance bounds on the star radius (reflectance_boundary_bvh/robin_bounds.h:12-74)
ZG_D void robinBound(V<2> c, float& r2, float kmax, V<2> viewClosest, float cd, V<2> viewFar, float fd, V<2> planePt, V<2> n) {
    float h = fabsf(dot(n, planePt - c) / dot(n, n));
    if (h > 0.0f) {
        float cosUpper = fabsf(dot((1.0f / cd) * viewClosest, n));
        float cosLower = fabsf(dot((1.0f / fd) * viewFar, n));
        float cosLine = sqrtf(h * kmax) / 1.41421356237309504880f;
        float cs = fminf(fmaxf(cosLine, cosLower), cosUpper);
        float r = (h / cs) * expf(cs * cs / (h * kmax));
        r2 = fminf(r2, r * r);
    } else {
        r2 = fminf(r2, cd * cd);
    }
}
ZG_D void robinBound(V<3> c, float& r2, float kmax, V<3> viewClosest, float cd, V<3> viewFar, float fd, V<3> planePt, V<3> n) {
    float h = fabsf(dot(n, planePt - c) / dot(n, n));
    if (h > 0.0f) {
        float cosUpper = fabsf(dot((1.0f / cd) * viewClosest, n));
        float cosLower = fabsf(dot((1.0f / fd) * viewFar, n));
        float maxCos = sqrtf(h * kmax);
        if (maxCos >= cosLower) {
            float cosPlane = maxCos / 1.73205080756887729353f;
            float ct = fminf(fmaxf(cosPlane, cosLower), cosUpper);
            float r = h * h * kmax / (ct * (h * kmax - ct * ct));
            r2 = fminf(r2, r * r);
        }
    } else {
        r2 = fminf(r2, cd * cd);
    }
}

// per-primitive star radius (reflectance_boundary_bvh/geometry.h:85-154, :169-236)
ZG_D void primStarRadius(const BoundaryView& b, int slot, V<2> c, float& r2, bool flip, float prec) {
    Prim<2> t = loadPrim<2>(b, slot);
    V<2> closest;
    float cd = closestOnPrim(t, c, closest);
    float cd2 = cd * cd;
    if (cd2 > r2) return;
    float4 s0 = __ldg(b.sil + 2 * (size_t)slot), s1 = __ldg(b.sil + 2 * (size_t)slot + 1);
    float kmax = s1.z;
    if (kmax < kFltMax - kReflEps) {
        int flags = __float_as_int(s1.x);
        V<2> n0 = primNormal<2>(t);
        V<2> nPrev; nPrev[0] = s0.x; nPrev[1] = s0.y;
        V<2> nNext; nNext[0] = s0.z; nNext[1] = s0.w;
#pragma unroll
        for (int j = 0; j < 2; j++) {
            if (flags & (8 << j)) continue;   // ignored feature
            V<2> view = c - t.p[j];
            float sd = len(view);
            bool sil = !(flags & (1 << j));
            if (!sil) sil = j == 0 ? silhouetteVertex(nPrev, n0, view, sd, flip, prec)
                                   : silhouetteVertex(n0, nNext, view, sd, flip, prec);
            if (sil) r2 = fminf(r2, sd * sd);
        }
        if (kmax > kReflEps) {
            if (cd < kReflEps) {
                r2 = cd;
            } else if (r2 > cd2) {
                V<2> far;
                float fd = farthestOnPrim(t, c, far);
                robinBound(c, r2, kmax, c - closest, cd, c - far, fd, t.p[0], n0);
            }
        }
    } else {
        r2 = fminf(r2, cd2);
    }
}
ZG_D void primStarRadius(const BoundaryView& b, int slot, V<3> c, float& r2, bool flip, float prec) {
    Prim<3> t = loadPrim<3>(b, slot);
    V<3> closest;
    float cd = closestOnPrim(t, c, closest);
    float cd2 = cd * cd;
    if (cd2 > r2) return;
    float4 s[3];
#pragma unroll
    for (int k = 0; k < 3; k++) s[k] = __ldg(b.sil + 3 * (size_t)slot + k);
    float kmax = s[2].w;
    if (kmax < kFltMax - kReflEps) {
        int flags = __float_as_int(s[0].w);
        V<3> n0 = primNormal<3>(t);
#pragma unroll
        for (int j = 0; j < 3; j++) {
            if (flags & (8 << j)) continue;
            V<3> pj = t.p[j], pk = t.p[(j + 1) % 3];
            V<3> q;
            float sd = closestOnSegment<3>(pj, pk, c, q);
            bool sil = !(flags & (1 << j));
            if (!sil) {
                V<3> nj; nj[0] = s[j].x; nj[1] = s[j].y; nj[2] = s[j].z;
                sil = silhouetteEdge(pj, pk, n0, nj, c - q, sd, flip, prec);
            }
            if (sil) r2 = fminf(r2, sd * sd);
        }
        if (kmax > kReflEps) {
            if (cd < kReflEps) {
                r2 = cd;
            } else if (r2 > cd2) {
                V<3> far;
                float fd = farthestOnPrim(t, c, far);
                robinBound(c, r2, kmax, c - closest, cd, c - far, fd, t.p[0], n0);
            }
        }
    } else {
        r2 = fminf(r2, cd2);
    }
}

// Can the subtree of child k hold a silhouette feature seen from x?  All face normals of
// its candidate features lie within `halfAngle` of `axis`; the view directions from the
// child's bounding sphere (grown by the precision) lie within beta of the direction to its
// centre.  When every normal/view angle stays on one side of pi/2 (beyond the precision
// band of the silhouette test) all faces are front- or all back-facing: no silhouette.
template <int D>
ZG_D bool coneMayHoldSilhouette(float4 cone, const WideNode<D>& w, int k, V<D> x, float prec) {
    if (cone.w < 0.0f) return false;
    if (cone.w >= 1.5707963f) return true;
    V<D> v;
    float rb2 = 0.0f;
#pragma unroll
    for (int i = 0; i < D; i++) {
        float h = 0.5f * (w.hi[i][k] - w.lo[i][k]);
        rb2 += h * h;
        v[i] = x[i] - 0.5f * (w.lo[i][k] + w.hi[i][k]);
    }
    float rb = sqrtf(rb2) + prec;
    float dv2 = len2(v);
    if (dv2 <= rb * rb) return true;
    float inv = rsqrtf(dv2);
    V<D> a;
    a[0] = cone.x; a[1] = cone.y;
    if (D == 3) a[D - 1] = cone.z;
    float cosT = dot(a, v) * inv;                      // cos(theta)
    // spread = beta + halfAngle + margin with sin(beta) = rb/dv; margin covers the
    // |n.view| <= prec band of the silhouette test
    float A = cone.w + prec + 1e-3f;
    float sA, cA;
    __sincosf(A, &sA, &cA);
    float sB = fminf(rb * inv, 1.0f), cB = sqrtf(fmaxf(0.0f, 1.0f - sB * sB));
    if (cB * cA - sB * sA <= 0.0f) return true;        // spread >= pi/2
    float sinSpread = sB * cA + cB * sA;               // sin(spread) = cos(pi/2 - spread)
    return !(cosT > sinSpread || cosT < -sinSpread);   // all front-facing or all back-facing
}

// Angular range of the normals of child k's faces as seen from x: returns false when the
// range straddles pi/2 (a silhouette is possible); otherwise minAbsCos = |cos| of the range
// end nearest to pi/2 (reflectance_boundary_bvh/bvh.h:382-392 with FCPW's cone overlap).
template <int D>
ZG_D bool coneAngleRangeBox(float4 cone, const float* lo, const float* hi, V<D> x, float& minAbsCos) {
    if (cone.w < 0.0f) { minAbsCos = 1.0f; return true; }      // no silhouette candidate at all
    if (cone.w >= 1.5707963f) return false;
    V<D> v;
    float rb2 = 0.0f;
#pragma unroll
    for (int i = 0; i < D; i++) {
        float h = 0.5f * (hi[i] - lo[i]);
        rb2 += h * h;
        v[i] = x[i] - 0.5f * (lo[i] + hi[i]);
    }
    float dv2 = len2(v);
    if (dv2 <= rb2) return false;
    float inv = rsqrtf(dv2);
    V<D> a;
    a[0] = cone.x; a[1] = cone.y;
    if (D == 3) a[D - 1] = cone.z;
    float cosT = fminf(fmaxf(dot(a, v) * inv, -1.0f), 1.0f), sinT = sqrtf(fmaxf(0.0f, 1.0f - cosT * cosT));
    float sB = fminf(sqrtf(rb2) * inv, 1.0f), cB = sqrtf(fmaxf(0.0f, 1.0f - sB * sB));
    float sA, cA;
    __sincosf(cone.w, &sA, &cA);
    float cS = cB * cA - sB * sA, sS = sB * cA + cB * sA;   // cos / sin of spread = beta + halfAngle
    if (cS <= 0.0f) return false;
    float cHi = cosT * cS - sinT * sS;                      // cos(theta + spread)
    float cLo = cosT * cS + sinT * sS;                      // cos(theta - spread)
    if (cHi > 0.0f) { minAbsCos = cHi; return true; }       // every face front-facing
    if (cLo < 0.0f) { minAbsCos = -cLo; return true; }      // every face back-facing
    return false;
}
template <int D>
ZG_D bool coneAngleRange(float4 cone, const WideNode<D>& w, int k, V<D> x, float& minAbsCos) {
    float lo[D], hi[D];
#pragma unroll
    for (int i = 0; i < D; i++) { lo[i] = w.lo[i][k]; hi[i] = w.hi[i][k]; }
    return coneAngleRangeBox<D>(cone, lo, hi, x, minAbsCos);
}

// node bounds on the squared star radius of every primitive below a node without
// silhouettes (reflectance_boundary_bvh/robin_bounds.h:110-154), maxAbsCos = 1
ZG_D void robinNodeBounds(int D, float rMin, float rMax, float kmin, float kmax, float minCos, float& r2Min, float& r2Max) {
    if (D == 2) {
        float lo = rMin * expf(minCos / (kmax * rMax));
        float hi = rMax * expf(1.0f / (kmin * rMin));
        r2Min = lo * lo;
        r2Max = hi * hi;
    } else {
        if (rMax < minCos / kmax) r2Min = kFltMax;
        else { float lo = rMin / (1.0f - minCos / (kmax * rMax)); r2Min = lo * lo; }
        if (rMin < 1.0f / kmin) r2Max = kFltMax;
        else { float hi = rMax / (1.0f - 1.0f / (kmin * rMin)); r2Max = hi * hi; }
    }
    if (!(r2Min == r2Min)) r2Min = 0.0f;     // NaN -> no pruning
    if (!(r2Max == r2Max)) r2Max = kFltMax;
}

template <int D>
ZG_D float boxMaxDist2(const WideNode<D>& w, int k, V<D> x) {
    float s = 0.0f;
#pragma unroll
    for (int i = 0; i < D; i++) {
        float d = fmaxf(fabsf(x[i] - w.lo[i][k]), fabsf(x[i] - w.hi[i][k]));
        s += d * d;
    }
    return s;
}

// computeStarRadiusForReflectingBoundary: max(sqrt(min(maxR^2, silhouettes, Robin bounds)), minR)
// one silhouette-candidate record: 2D vertex (v, nPrev, nNext), 3D edge (a, b, nA, nB)
ZG_D void featureRadius(const BoundaryView& b, int slot, V<2> x, float& r2, bool flip, float prec) {
    float4 f0 = __ldg(b.silFeat + 2 * (size_t)slot), f1 = __ldg(b.silFeat + 2 * (size_t)slot + 1);
    V<2> view; view[0] = x[0] - f0.x; view[1] = x[1] - f0.y;
    float d2 = len2(view);
    if (d2 >= r2) return;
    float d = sqrtf(d2);
    bool sil = __float_as_int(f1.z) != 0;
    if (!sil) {
        V<2> nPrev; nPrev[0] = f0.z; nPrev[1] = f0.w;
        V<2> nNext; nNext[0] = f1.x; nNext[1] = f1.y;
        sil = silhouetteVertex(nPrev, nNext, view, d, flip, prec);
    }
    if (sil) r2 = d2;
}
ZG_D void featureRadius(const BoundaryView& b, int slot, V<3> x, float& r2, bool flip, float prec) {
    const float4* f = b.silFeat + 4 * (size_t)slot;
    float4 f0 = __ldg(f), f1 = __ldg(f + 1);
    V<3> pa; pa[0] = f0.x; pa[1] = f0.y; pa[2] = f0.z;
    V<3> pb; pb[0] = f1.x; pb[1] = f1.y; pb[2] = f1.z;
    V<3> q;
    float d = closestOnSegment<3>(pa, pb, x, q);
    if (d * d >= r2) return;
    bool sil = __float_as_int(f0.w) != 0;
    if (!sil) {
        float4 f2 = __ldg(f + 2), f3 = __ldg(f + 3);
        V<3> nA; nA[0] = f2.x; nA[1] = f2.y; nA[2] = f2.z;
        V<3> nB; nB[0] = f3.x; nB[1] = f3.y; nB[2] = f3.z;
        sil = silhouetteEdge(pa, pb, nA, nB, x - q, d, flip, prec);
    }
    if (sil) r2 = d * d;
}

// closest silhouette point of a Neumann boundary within sqrt(r2) (FCPW findClosestSilhouettePoint,
// fcpw_geometric_queries.h:1264): traversal of the candidate tree, cone-pruned
template <int D>
__device__ __noinline__ float silhouetteRadius2(const BoundaryView& b, V<D> x, float r2, bool flip, float prec,
                                                TravStack& S, uint32_t& err) {
    if (b.silNodes == 0) return r2;
    BoundaryView t = b;
    t.nodes = b.silTree;
    int sp = 0;
    int node = 0;
    for (;;) {
        WideNode<D> w;
        loadNode<D>(t, node, w);
        ChildOrder ord; ord.clear();
        unsigned leaves = 0;
#pragma unroll 1
        for (int k = 0; k < 4; k++) {
            int c = w.child[k];
            float d2 = boxDist2<D>(w, k, x);
            bool ok = c != kEmptyChild && d2 < r2 &&
                      coneMayHoldSilhouette<D>(__ldg(b.silCones + (size_t)node * 8 + k), w, k, x, prec);
            if (ok && isLeaf(c)) leaves |= 1u << k;
            if (ok && !isLeaf(c)) { ord.k[k] = d2; ord.c[k] = c; }
        }
        while (leaves) {
            int k = __ffs(leaves) - 1;
            leaves &= leaves - 1;
            int c = pick4(k, w.child[0], w.child[1], w.child[2], w.child[3]);
            int first = leafFirst(c), count = leafCount(c);
#pragma unroll 1
            for (int j = 0; j < count; j++) featureRadius(b, first + j, x, r2, flip, prec);
        }
        ord.sort();
        int next = descendAndPush<4, true>(ord, r2, S, sp, err);
        node = next >= 0 ? next : popWithin(r2, S, sp);
        if (node < 0) break;
    }
    return r2;
}

template <int D>
__device__ __noinline__ float starRadius(const BoundaryView& b, V<D> x, float minR, float maxR, float prec, bool flip,
                                         TravStack& S, uint32_t& err) {
    if (minR > maxR) return maxR;
    float r2 = maxR < kFltMax ? maxR * maxR : kFltMax;
    if (!b.robin) return fmaxf(sqrtf(silhouetteRadius2<D>(b, x, r2, flip, prec, S, err)), minR);
    if (b.nNodes > 0) {
        int sp = 0;
        int node = 0;
        for (;;) {
            WideNode<D> w;
            loadNode<D>(b, node, w);
            float4 km = b.cones ? __ldg(b.cones + (size_t)node * 8 + 4) : make_float4(kFltMax, kFltMax, kFltMax, kFltMax);
            float4 kn = b.cones ? __ldg(b.cones + (size_t)node * 8 + 5) : make_float4(0, 0, 0, 0);
            const float kmaxChild[4] = {km.x, km.y, km.z, km.w};
            const float kminChild[4] = {kn.x, kn.y, kn.z, kn.w};
            ChildOrder ord; ord.clear();
            unsigned leaves = 0;
#pragma unroll
            for (int k = 0; k < 4; k++) {
                int c = w.child[k];
                float d2 = boxDist2<D>(w, k, x);
                float key = d2;
                bool ok = c != kEmptyChild && d2 <= r2;
                if (ok && kminChild[k] >= kFltMax - kReflEps) {
                    // perfectly absorbing subtree: the farthest box point bounds the radius
                    r2 = fminf(r2, boxMaxDist2<D>(w, k, x));
                } else if (ok) {
                    float minCos;
                    if (coneAngleRange<D>(__ldg(b.cones + (size_t)node * 8 + k), w, k, x, minCos)) {
                        // no silhouette below: pure reflection contributes nothing, reflectance is bounded
                        if (kmaxChild[k] <= kReflEps) {
                            ok = false;
                        } else {
                            float r2Min, r2Max;
                            robinNodeBounds(D, sqrtf(d2), sqrtf(boxMaxDist2<D>(w, k, x)), kminChild[k], kmaxChild[k],
                                            minCos, r2Min, r2Max);
                            key = fmaxf(d2, r2Min);
                            ok = key <= r2;
                            if (ok) r2 = fminf(r2, r2Max);
                        }
                    }
                }
                if (ok && isLeaf(c)) leaves |= 1u << k;
                if (ok && !isLeaf(c)) { ord.k[k] = key; ord.c[k] = c; }
            }
            while (leaves) {
                int k = __ffs(leaves) - 1;
                leaves &= leaves - 1;
                int c = pick4(k, w.child[0], w.child[1], w.child[2], w.child[3]);
                int first = leafFirst(c), count = leafCount(c);
#pragma unroll 1
                for (int j = 0; j < count; j++) primStarRadius(b, first + j, x, r2, flip, prec);
            }
            ord.sort();
            int next = descendAndPush(ord, r2, S, sp, err);
            node = next >= 0 ? next : popWithin(r2, S, sp);
            if (node < 0) break;
        }
    }
    return fmaxf(sqrtf(r2), minR);
}

// Robin star radius answered by the whole warp (the caller loops over the lanes that need
// one); the rules are those of starRadius above.  Each round takes up to 8 stack entries and
// tests their 4 children in parallel: the children's upper bounds (perfectly absorbing
// subtrees, Robin node bounds) are folded into the radius by a warp minimum before their
// lower bounds are compared with it; internal children within the radius are pushed, leaf
// primitives are tested 32 at a time and their radii folded the same way.  A primitive never
// lowers the radius below its own closest distance, so the result does not depend on the
// order primitives are met in, up to the node upper bounds.
template <int D>
__device__ __noinline__ float coopRobinStarRadius(const BoundaryView& b, V<D> x, float minR, float maxR, float prec,
                                                  bool flip, CoopWork& W, int lane, uint32_t& err) {
    if (minR > maxR) return maxR;
    float r2 = maxR < kFltMax ? maxR * maxR : kFltMax;
    if (b.nNodes == 0) return fmaxf(sqrtf(r2), minR);
    const int c = lane & 3;
    if (lane == 0) { W.node[0] = 0; W.key[0] = 0.0f; }
    int sp = 1;
    __syncwarp();
    while (sp > 0) {
        const int take = min(8, sp);
        sp -= take;
        const int e = lane >> 2;
        int node = -1;
        float key = kFltMax;
        if (e < take) { node = W.node[sp + e]; key = W.key[sp + e]; }
        __syncwarp();
        int child = kEmptyChild;
        float ckey = kFltMax, cap = kFltMax;
        bool ok = false;
        if (node >= 0 && key <= r2) {
            const float4* p = b.nodes + (size_t)node * 8;
            float lo[D], hi[D], d2 = 0.0f, far2 = 0.0f;
#pragma unroll
            for (int i = 0; i < D; i++) {
                lo[i] = comp4(__ldg(p + i), c);
                hi[i] = comp4(__ldg(p + D + i), c);
                float dn = fmaxf(fmaxf(lo[i] - x[i], 0.0f), x[i] - hi[i]);
                float df = fmaxf(fabsf(x[i] - lo[i]), fabsf(x[i] - hi[i]));
                d2 += dn * dn;
                far2 += df * df;
            }
            child = comp4i(__ldg(reinterpret_cast<const int4*>(p + 2 * D)), c);
            if (child != kEmptyChild && d2 <= r2) {
                ok = true;
                ckey = d2;
                const float kmin = comp4(__ldg(b.cones + (size_t)node * 8 + 5), c);
                const float kmax = comp4(__ldg(b.cones + (size_t)node * 8 + 4), c);
                if (kmin >= kFltMax - kReflEps) {
                    cap = far2;                         // perfectly absorbing subtree
                } else {
                    float minCos;
                    if (coneAngleRangeBox<D>(__ldg(b.cones + (size_t)node * 8 + c), lo, hi, x, minCos)) {
                        if (kmax <= kReflEps) {
                            ok = false;                 // purely reflecting, no silhouette below
                        } else {
                            float r2Min, r2Max;
                            robinNodeBounds(D, sqrtf(d2), sqrtf(far2), kmin, kmax, minCos, r2Min, r2Max);
                            ckey = fmaxf(d2, r2Min);
                            cap = r2Max;
                        }
                    }
                }
            }
        }
        // upper bounds first (cap >= 0: float bits order as values), then the lower bounds
        if (!ok) cap = kFltMax;
        r2 = fminf(r2, __uint_as_float(__reduce_min_sync(0xffffffffu, __float_as_uint(cap))));
        ok = ok && ckey <= r2;
        const bool inner = ok && !isLeaf(child), leaf = ok && isLeaf(child);
        const unsigned im = __ballot_sync(0xffffffffu, inner);
        const int nIn = __popc(im);
        if (sp + nIn > kCoopStack) { err |= kErrStackOverflow; break; }
        if (inner) {
            int pos = sp + __popc(im & ((1u << lane) - 1u));
            W.node[pos] = child;
            W.key[pos] = ckey;
        }
        sp += nIn;
        int cnt = leaf ? leafCount(child) : 0;
        int incl = cnt;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            int v = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += v;
        }
        const int total = __shfl_sync(0xffffffffu, incl, 31);
        for (int j = 0; j < cnt; j++) W.prim[incl - cnt + j] = leafFirst(child) + j;
        __syncwarp();
        for (int base = 0; base < total; base += 32) {
            float mine = r2;
            if (base + lane < total) primStarRadius(b, W.prim[base + lane], x, mine, flip, prec);
            r2 = fminf(r2, __uint_as_float(__reduce_min_sync(0xffffffffu, __float_as_uint(mine))));
        }
        __syncwarp();
    }
    return fmaxf(sqrtf(r2), minR);
}

// ---------------------------------------------------------------- boundary sampling
// |G_free,3D(max(sqrt(r2), 1e-2))| (utils/fcpw_geometric_queries.h:1391-1398)
ZG_D float branchWeight(float r2) {
    float r = fmaxf(sqrtf(r2), 1e-2f);
    return 1.0f / (4.0f * kPi * r);
}
// weight of a primitive for boundary sampling: area * branchWeight(distance^2) inside the ball
template <int D>
ZG_D float samplingWeight(const Prim<D>& t, V<D> x, float R2) {
    V<D> q;
    float d = closestOnPrim(t, x, q);
    return d * d <= R2 ? primArea(t) * branchWeight(d * d) : 0.0f;
}

// Stochastic descent: children overlapping the ball are chosen with probability
// proportional to area * branchWeight(box distance^2), primitives in the leaf with
// area * branchWeight(distance^2); a point is drawn uniformly on the primitive and
// pdf = P(path) / area.  Unbiased for the boundary integral over the ball.  The first
// random number is reused across levels (rescaled to [0,1) after every choice).
template <int D>
__device__ __noinline__ bool sampleBoundary(const BoundaryView& b, V<D> x, float radius, const float* uIn, V<D>& pt,
                                            V<D>& n, float& pdf) {
    if (b.nNodes == 0) return false;
    const float R2 = radius * radius;
    float u0 = uIn[0];
    float prob = 1.0f;
    int node = 0;
#pragma unroll 1
    for (int depth = 0; depth < 64; depth++) {
        WideNode<D> w;
        loadNode<D>(b, node, w);
        float4 ar = loadNodeArea(b, node, D);
        float wt0, wt1, wt2, wt3;
        {
            float d0 = w.child[0] == kEmptyChild ? kFltMax : boxDist2<D>(w, 0, x);
            float d1 = w.child[1] == kEmptyChild ? kFltMax : boxDist2<D>(w, 1, x);
            float d2 = w.child[2] == kEmptyChild ? kFltMax : boxDist2<D>(w, 2, x);
            float d3 = w.child[3] == kEmptyChild ? kFltMax : boxDist2<D>(w, 3, x);
            wt0 = d0 <= R2 ? ar.x * branchWeight(d0) : 0.0f;
            wt1 = d1 <= R2 ? ar.y * branchWeight(d1) : 0.0f;
            wt2 = d2 <= R2 ? ar.z * branchWeight(d2) : 0.0f;
            wt3 = d3 <= R2 ? ar.w * branchWeight(d3) : 0.0f;
        }
        float total = wt0 + wt1 + wt2 + wt3;
        if (!(total > 0.0f)) return false;
        // choose child k: first k with u0 * total < cumulative weight (last positive on round-off)
        float target = u0 * total, acc = 0.0f, wk = 0.0f, before = 0.0f;
        int k = -1;
#pragma unroll
        for (int i = 0; i < 4; i++) {
            float wi = pick4f(i, wt0, wt1, wt2, wt3);
            if (wi > 0.0f && (k < 0 || target >= acc)) { k = i; wk = wi; before = acc; }
            acc += wi;
            if (k >= 0 && target < acc) break;
        }
        prob *= wk / total;
        u0 = fminf(fmaxf((target - before) / wk, 0.0f), 0.99999994f);
        int c = pick4(k, w.child[0], w.child[1], w.child[2], w.child[3]);
        if (!isLeaf(c)) { node = c; continue; }
        // leaf: total weight, then walk again to the chosen primitive
        int first = leafFirst(c), count = leafCount(c);
        float lt = 0.0f;
#pragma unroll 1
        for (int j = 0; j < count; j++) lt += samplingWeight<D>(loadPrim<D>(b, first + j), x, R2);
        if (!(lt > 0.0f)) return false;
        float lTarget = u0 * lt, lAcc = 0.0f, lw = 0.0f, lBefore = 0.0f;
        int pick = -1;
#pragma unroll 1
        for (int j = 0; j < count; j++) {
            float wj = samplingWeight<D>(loadPrim<D>(b, first + j), x, R2);
            if (wj > 0.0f && (pick < 0 || lTarget >= lAcc)) { pick = j; lw = wj; lBefore = lAcc; }
            lAcc += wj;
            if (pick >= 0 && lTarget < lAcc) break;
        }
        prob *= lw / lt;
        Prim<D> t = loadPrim<D>(b, first + pick);
        V<D> nr = primNormalRaw(t);
        float nn = len(nr);
        n = (1.0f / nn) * nr;
        if (D == 2) {
            pt = t.p[0] + uIn[1] * (t.p[1] - t.p[0]);
            pdf = prob / nn;
        } else {
            float u1 = sqrtf(uIn[1]), u2 = uIn[D - 1];
            float a = 1.0f - u1, bb = u2 * u1, cc = 1.0f - a - bb;
            pt = a * t.p[0] + bb * t.p[1] + cc * t.p[D - 1];
            pdf = prob * 2.0f / nn;
        }
        (void)lBefore;
        return true;
    }
    return false;
}

}  // namespace zg
