// zgpu_build.cpp -- boundary preprocessing on the host: feature adjacency and silhouette
// flags (utils/fcpw_geometric_queries.h:745-799 for 2D vertex tables, :892-973 for 3D
// edge maps, ignore rule :1029-1038), a binned-SAH binary BVH with leaves of <= 4
// primitives, and its collapse into the 4-wide, 128-byte node layout of zgpu_scene.cuh.
#include "zgpu_build.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <array>
#include <map>
#include <numeric>
#include <thread>
#include <unordered_map>

namespace zg {
namespace {

constexpr float kInf = 3.402823466e+38f;
constexpr int kEmpty = 0x7fffffff;
constexpr int kLeafMax = 4;

struct Box {
    float lo[3] = {kInf, kInf, kInf};
    float hi[3] = {-kInf, -kInf, -kInf};
    void grow(const float* p, int D) { for (int i = 0; i < D; i++) { lo[i] = std::min(lo[i], p[i]); hi[i] = std::max(hi[i], p[i]); } }
    void grow(const Box& b, int D) { grow(b.lo, D); grow(b.hi, D); }
    float half_area(int D) const {
        float e[3];
        for (int i = 0; i < D; i++) e[i] = std::max(0.0f, hi[i] - lo[i]);
        return D == 2 ? e[0] + e[1] : e[0] * e[1] + e[1] * e[2] + e[2] * e[0];
    }
};

struct BNode {
    Box box;
    int left = -1, right = -1, first = 0, count = 0;
    float area = 0.0f;
};

struct Builder {
    int D;
    std::vector<Box> pbox;
    std::vector<float> cent;   // [n*D]
    std::vector<float> parea;
    std::vector<int> order;
    std::vector<BNode> nodes;

    int build(int start, int end, int depth) {
        int id = (int)nodes.size();
        nodes.emplace_back();
        Box box, cbox;
        float area = 0.0f;
        for (int i = start; i < end; i++) {
            box.grow(pbox[order[i]], D);
            cbox.grow(&cent[(size_t)order[i] * D], D);
            area += parea[order[i]];
        }
        nodes[id].box = box;
        nodes[id].area = area;
        int n = end - start;
        if (n <= kLeafMax || depth > 40) {
            nodes[id].first = start;
            nodes[id].count = n;
            return id;
        }
        constexpr int B = 16;
        float best = kInf; int bestAxis = -1, bestSplit = -1;
        for (int ax = 0; ax < D; ax++) {
            float lo = cbox.lo[ax], hi = cbox.hi[ax];
            if (!(hi - lo > 1e-12f)) continue;
            float scale = B / (hi - lo);
            Box bb[B]; int cnt[B] = {0};
            for (int i = start; i < end; i++) {
                int p = order[i];
                int b = std::min(B - 1, (int)((cent[(size_t)p * D + ax] - lo) * scale));
                cnt[b]++; bb[b].grow(pbox[p], D);
            }
            float lArea[B]; int lCnt[B]; Box acc; int c = 0;
            for (int b = 0; b < B; b++) { acc.grow(bb[b], D); c += cnt[b]; lArea[b] = acc.half_area(D); lCnt[b] = c; }
            acc = Box(); c = 0;
            for (int b = B - 1; b > 0; b--) {
                acc.grow(bb[b], D); c += cnt[b];
                if (lCnt[b - 1] == 0 || c == 0) continue;
                float cost = lArea[b - 1] * lCnt[b - 1] + acc.half_area(D) * c;
                if (cost < best) { best = cost; bestAxis = ax; bestSplit = b; }
            }
        }
        int mid = start + n / 2;
        if (bestAxis >= 0) {
            float lo = cbox.lo[bestAxis], hi = cbox.hi[bestAxis];
            float scale = B / (hi - lo);
            auto it = std::partition(order.begin() + start, order.begin() + end, [&](int p) {
                return std::min(B - 1, (int)((cent[(size_t)p * D + bestAxis] - lo) * scale)) < bestSplit;
            });
            mid = (int)(it - order.begin());
        }
        if (mid == start || mid == end) {
            // degenerate split: median along the longest centroid axis
            int ax = 0;
            for (int i = 1; i < D; i++) if (cbox.hi[i] - cbox.lo[i] > cbox.hi[ax] - cbox.lo[ax]) ax = i;
            mid = start + n / 2;
            std::nth_element(order.begin() + start, order.begin() + mid, order.begin() + end,
                             [&](int a, int b) { return cent[(size_t)a * D + ax] < cent[(size_t)b * D + ax]; });
        }
        int l = build(start, mid, depth + 1);
        int r = build(mid, end, depth + 1);
        nodes[id].left = l;
        nodes[id].right = r;
        return id;
    }
};

int makeLeafRef(int first, int count) { return -(1 + ((first << 3) | (count - 1))); }

// Collapses the binary tree into nodes of `width` (4 or 8) children: 2 * width float4 per
// node, in the layout of zgpu_scene.cuh (per group of 4 children: lower bounds per axis,
// upper bounds per axis, child references, areas).
struct Collapser {
    int D;
    const std::vector<BNode>& bn;
    std::vector<float4>& out;
    int width = 4;
    int maxDepth = 0;
    std::vector<std::array<int, 8>> kidsOf;   // wide node -> binary node of each child (-1 empty)

    int emit(int b, int depth) {
        maxDepth = std::max(maxDepth, depth);
        const int stride = 2 * width, G = width / 4;
        int id = (int)(out.size() / stride);
        out.resize(out.size() + stride);
        kidsOf.push_back({-1, -1, -1, -1, -1, -1, -1, -1});
        // gather up to `width` children by opening the largest internal child
        std::vector<int> kids = {bn[b].left, bn[b].right};
        while ((int)kids.size() < width) {
            int pick = -1; float pa = -1.0f;
            for (int i = 0; i < (int)kids.size(); i++) {
                const BNode& k = bn[kids[i]];
                if (k.count == 0) { float a = k.box.half_area(D); if (a > pa) { pa = a; pick = i; } }
            }
            if (pick < 0) break;
            int k = kids[pick];
            kids.erase(kids.begin() + pick);
            kids.push_back(bn[k].left);
            kids.push_back(bn[k].right);
        }
        float lo[3][8], hi[3][8], area[8];
        int child[8];
        for (int c = 0; c < 8; c++) {
            for (int i = 0; i < 3; i++) { lo[i][c] = kInf; hi[i][c] = -kInf; }
            area[c] = 0.0f; child[c] = kEmpty;
        }
        for (int c = 0; c < (int)kids.size(); c++) kidsOf[id][c] = kids[c];
        for (int c = 0; c < (int)kids.size(); c++) {
            const BNode& k = bn[kids[c]];
            for (int i = 0; i < D; i++) { lo[i][c] = k.box.lo[i]; hi[i][c] = k.box.hi[i]; }
            area[c] = k.area;
            if (k.count > 0) child[c] = makeLeafRef(k.first, k.count);
        }
        for (int c = 0; c < (int)kids.size(); c++) {
            if (bn[kids[c]].count == 0) child[c] = emit(kids[c], depth + 1);
        }
        float4* p = &out[(size_t)id * stride];
        for (int g = 0; g < G; g++) {
            const int c0 = 4 * g;
            for (int i = 0; i < D; i++) {
                p[i * G + g] = make_float4(lo[i][c0], lo[i][c0 + 1], lo[i][c0 + 2], lo[i][c0 + 3]);
                p[(D + i) * G + g] = make_float4(hi[i][c0], hi[i][c0 + 1], hi[i][c0 + 2], hi[i][c0 + 3]);
            }
            int4 ci = make_int4(child[c0], child[c0 + 1], child[c0 + 2], child[c0 + 3]);
            std::memcpy(&p[2 * D * G + g], &ci, sizeof(int4));
            p[(2 * D + 1) * G + g] = make_float4(area[c0], area[c0 + 1], area[c0 + 2], area[c0 + 3]);
        }
        return id;
    }
};

inline void normal2(const float* a, const float* b, float* n) {
    float sx = b[0] - a[0], sy = b[1] - a[1];
    float l = std::sqrt(sx * sx + sy * sy);
    n[0] = sy / l; n[1] = -sx / l;
}
inline void normal3(const float* a, const float* b, const float* c, float* n) {
    float u[3] = {b[0] - a[0], b[1] - a[1], b[2] - a[2]}, v[3] = {c[0] - a[0], c[1] - a[1], c[2] - a[2]};
    float x = u[1] * v[2] - u[2] * v[1], y = u[2] * v[0] - u[0] * v[2], z = u[0] * v[1] - u[1] * v[0];
    float l = std::sqrt(x * x + y * y + z * z);
    n[0] = x / l; n[1] = y / l; n[2] = z / l;
}

// Normal cone over the silhouette candidates of a binary subtree: every normal of a face
// adjacent to a non-ignored feature lies within halfAngle of axis.  halfAngle < 0: no
// candidate in the subtree; halfAngle = pi: a feature with a single face (always a
// silhouette) or a degenerate axis.  With allNormals (Robin boundaries) the cone covers
// every face of the subtree and its neighbours, ignored features included, as the Robin
// star-radius bounds need the angular range of all normals
// (reflectance_boundary_bvh/bvh.h:210-262).
struct Cone { float axis[3] = {0, 0, 0}; float halfAngle = -1.0f; float kmax = 0.0f; float kmin = 0.0f; };

void coneOf(int D, const std::vector<BNode>& bn, int node, const std::vector<int>& order, const std::vector<float>& nrm,
            const std::vector<int>& adj, const std::vector<int>& flags, const float* kmaxArr, const float* kminArr,
            bool allNormals, Cone& out) {
    std::vector<int> stack = {node};
    std::vector<const float*> normals;
    bool open = false;
    float kmax = 0.0f, kmin = kmaxArr ? kInf : 0.0f;
    while (!stack.empty()) {
        int b = stack.back(); stack.pop_back();
        if (bn[b].count == 0) { stack.push_back(bn[b].left); stack.push_back(bn[b].right); continue; }
        for (int k = 0; k < bn[b].count; k++) {
            int i = order[bn[b].first + k];
            if (kmaxArr) kmax = std::max(kmax, kmaxArr[i]);
            if (kminArr) kmin = std::min(kmin, kminArr[i]);
            bool any = allNormals;
            for (int j = 0; j < D; j++) {
                if (!allNormals && (flags[i] & (8 << j))) continue;   // ignored feature
                if (!(flags[i] & (1 << j))) { open = true; continue; }
                normals.push_back(&nrm[(size_t)adj[(size_t)i * D + j] * D]);
                any = true;
            }
            if (any) normals.push_back(&nrm[(size_t)i * D]);
        }
    }
    out = Cone();
    out.kmax = kmax;
    out.kmin = kmin;
    if (open) { out.halfAngle = 3.14159265f; return; }
    if (normals.empty()) { out.halfAngle = -1.0f; return; }
    double a[3] = {0, 0, 0};
    for (const float* n : normals) for (int i = 0; i < D; i++) a[i] += n[i];
    double l = std::sqrt(a[0] * a[0] + a[1] * a[1] + a[2] * a[2]);
    if (l < 1e-6) { out.halfAngle = 3.14159265f; return; }
    for (int i = 0; i < 3; i++) out.axis[i] = (float)(a[i] / l);
    double h = 0.0;
    for (const float* n : normals) {
        double c = 0.0;
        for (int i = 0; i < D; i++) c += out.axis[i] * n[i];
        h = std::max(h, std::acos(std::max(-1.0, std::min(1.0, c))));
    }
    out.halfAngle = (float)std::min(3.14159265, h + 1e-4);
}


// Builds the wide tree over `n` items with the given boxes / centroids / weights; fills
// `order` (leaf slot -> item) and returns the collapsed nodes (+ per-wide-node binary kids).
struct WideTree {
    std::vector<float4> nodes;
    std::vector<std::array<int, 8>> kids;
    std::vector<BNode> bnodes;
    std::vector<int> order;
    int depth = 0;
};

void buildWideTree(int D, const std::vector<Box>& boxes, const std::vector<float>& cent, const std::vector<float>& weight,
                   WideTree& out) {
    int n = (int)boxes.size();
    Builder bld;
    bld.D = D;
    bld.pbox = boxes;
    bld.cent = cent;
    bld.parea = weight;
    bld.order.resize(n);
    std::iota(bld.order.begin(), bld.order.end(), 0);
    bld.nodes.reserve((size_t)2 * n / kLeafMax + 16);
    bld.build(0, n, 0);
    out.order = bld.order;
    out.bnodes = bld.nodes;
    if (bld.nodes[0].count > 0) {
        out.nodes.resize(8);
        for (int i = 0; i < D; i++) {
            out.nodes[i] = make_float4(bld.nodes[0].box.lo[i], kInf, kInf, kInf);
            out.nodes[D + i] = make_float4(bld.nodes[0].box.hi[i], -kInf, -kInf, -kInf);
        }
        int4 ci = make_int4(makeLeafRef(0, bld.nodes[0].count), kEmpty, kEmpty, kEmpty);
        std::memcpy(&out.nodes[2 * D], &ci, sizeof(int4));
        out.nodes[2 * D + 1] = make_float4(bld.nodes[0].area, 0, 0, 0);
        out.kids.push_back({0, -1, -1, -1, -1, -1, -1, -1});
        out.depth = 1;
        return;
    }
    Collapser col{D, out.bnodes, out.nodes};
    col.emit(0, 1);
    out.kids = col.kidsOf;
    out.depth = col.maxDepth;
}

// Normal cone over a set of unit normals (axis = normalised mean, half angle = max deviation).
void coneOverNormals(int D, const std::vector<const float*>& ns, bool open, float* axis, float& halfAngle) {
    axis[0] = axis[1] = axis[2] = 0.0f;
    if (open) { halfAngle = 3.14159265f; return; }
    if (ns.empty()) { halfAngle = -1.0f; return; }
    double a[3] = {0, 0, 0};
    for (const float* n : ns) for (int i = 0; i < D; i++) a[i] += n[i];
    double l = std::sqrt(a[0] * a[0] + a[1] * a[1] + a[2] * a[2]);
    if (l < 1e-6) { halfAngle = 3.14159265f; return; }
    for (int i = 0; i < 3; i++) axis[i] = (float)(a[i] / l);
    double h = 0.0;
    for (const float* n : ns) {
        double c = 0.0;
        for (int i = 0; i < D; i++) c += axis[i] * n[i];
        h = std::max(h, std::acos(std::max(-1.0, std::min(1.0, c))));
    }
    halfAngle = (float)std::min(3.14159265, h + 1e-4);
}

}  // namespace

bool buildBoundary(int D, const float* pos, int nV, const int* idx, int nP, int kind, const float* kmin,
                   const float* kmax, bool doubleSided, float silPrec, HostBoundary& hb, std::string& err, int width) {
    hb = HostBoundary();
    hb.dim = D; hb.kind = kind; hb.nPrims = nP; hb.width = width;
    if (width != 4 && !(width == 8 && D == 3 && kind == 0)) {
        err = "8-wide nodes are built for 3D absorbing boundaries only";
        return false;
    }
    if (D != 2 && D != 3) { err = "dim must be 2 or 3"; return false; }
    if (nP < 0 || nV < 0) { err = "negative sizes"; return false; }
    for (int i = 0; i < nP * D; i++)
        if (idx[i] < 0 || idx[i] >= nV) { err = "primitive index out of range"; return false; }
    if (nP == 0) return true;
    if (nP >= (1 << 27)) { err = "too many primitives"; return false; }

    // ---- per-primitive normals, adjacency, silhouette flags and Robin ranges
    std::vector<float> nrm((size_t)nP * D);
    for (int i = 0; i < nP; i++) {
        const float* a = pos + (size_t)idx[i * D] * D;
        const float* b = pos + (size_t)idx[i * D + 1] * D;
        if (D == 2) normal2(a, b, &nrm[(size_t)i * 2]);
        else normal3(a, b, pos + (size_t)idx[i * D + 2] * D, &nrm[(size_t)i * 3]);
    }
    std::vector<int> adj((size_t)nP * D, -1);
    if (D == 2) {
        // vertex -> (segment ending at it, segment starting at it)
        std::vector<int> endsAt(nV, -1), startsAt(nV, -1);
        for (int i = 0; i < nP; i++) { startsAt[idx[i * 2]] = i; endsAt[idx[i * 2 + 1]] = i; }
        for (int i = 0; i < nP; i++) { adj[i * 2] = endsAt[idx[i * 2]]; adj[i * 2 + 1] = startsAt[idx[i * 2 + 1]]; }
    } else {
        // directed edge (u,v) of face f is shared with the face holding (v,u)
        std::unordered_map<uint64_t, int> dir;
        dir.reserve((size_t)nP * 3 * 2);
        for (int i = 0; i < nP; i++)
            for (int j = 0; j < 3; j++) {
                uint64_t u = (uint32_t)idx[i * 3 + j], v = (uint32_t)idx[i * 3 + (j + 1) % 3];
                dir[(u << 32) | v] = i;
            }
        for (int i = 0; i < nP; i++)
            for (int j = 0; j < 3; j++) {
                uint64_t u = (uint32_t)idx[i * 3 + j], v = (uint32_t)idx[i * 3 + (j + 1) % 3];
                auto it = dir.find((v << 32) | u);
                adj[i * 3 + j] = it == dir.end() ? -1 : it->second;
            }
    }
    std::vector<int> flags(nP, 0);
    for (int i = 0; i < nP; i++) {
        int f = 0;
        for (int j = 0; j < D; j++) {
            int a = adj[(size_t)i * D + j];
            if (a < 0) continue;
            f |= 1 << j;
            bool ignore;
            if (D == 2) {
                const float* n0 = &nrm[(size_t)i * 2];
                const float* nj = &nrm[(size_t)a * 2];
                float det = (n0[0] * nj[1] - n0[1] * nj[0]) * (j == 0 ? 1.0f : -1.0f);
                ignore = !doubleSided && det < silPrec;
            } else {
                const float* n0 = &nrm[(size_t)i * 3];
                const float* nj = &nrm[(size_t)a * 3];
                const float* pa = pos + (size_t)idx[i * 3 + j] * 3;
                const float* pb = pos + (size_t)idx[i * 3 + (j + 1) % 3] * 3;
                float e[3] = {pb[0] - pa[0], pb[1] - pa[1], pb[2] - pa[2]};
                float el = std::sqrt(e[0] * e[0] + e[1] * e[1] + e[2] * e[2]);
                float c[3] = {nj[1] * n0[2] - nj[2] * n0[1], nj[2] * n0[0] - nj[0] * n0[2], nj[0] * n0[1] - nj[1] * n0[0]};
                float angle = std::atan2((e[0] * c[0] + e[1] * c[1] + e[2] * c[2]) / el,
                                         n0[0] * nj[0] + n0[1] * nj[1] + n0[2] * nj[2]);
                ignore = !doubleSided && angle < silPrec;
            }
            if (ignore) f |= 8 << j;
        }
        flags[i] = f;
    }

    // ---- BVH over primitive boxes
    Builder bld;
    bld.D = D;
    bld.pbox.resize(nP);
    bld.cent.assign((size_t)nP * D, 0.0f);
    bld.parea.resize(nP);
    for (int i = 0; i < nP; i++) {
        Box b;
        for (int k = 0; k < D; k++) {
            const float* p = pos + (size_t)idx[i * D + k] * D;
            b.grow(p, D);
            for (int a = 0; a < D; a++) bld.cent[(size_t)i * D + a] += p[a] / D;
        }
        bld.pbox[i] = b;
        const float* a = pos + (size_t)idx[i * D] * D;
        const float* bb = pos + (size_t)idx[i * D + 1] * D;
        if (D == 2) {
            bld.parea[i] = std::hypot(bb[0] - a[0], bb[1] - a[1]);
        } else {
            const float* c = pos + (size_t)idx[i * D + 2] * D;
            float u[3] = {bb[0] - a[0], bb[1] - a[1], bb[2] - a[2]}, v[3] = {c[0] - a[0], c[1] - a[1], c[2] - a[2]};
            float x = u[1] * v[2] - u[2] * v[1], y = u[2] * v[0] - u[0] * v[2], z = u[0] * v[1] - u[1] * v[0];
            bld.parea[i] = 0.5f * std::sqrt(x * x + y * y + z * z);
        }
    }
    bld.order.resize(nP);
    std::iota(bld.order.begin(), bld.order.end(), 0);
    bld.nodes.reserve((size_t)2 * nP / kLeafMax + 16);
    bld.build(0, nP, 0);

    // ---- wide layout
    if (bld.nodes[0].count > 0) {
        // tiny scene: a root whose single child is the leaf
        const int G = width / 4;
        hb.nodes.assign((size_t)2 * width, make_float4(0, 0, 0, 0));
        for (int g = 0; g < G; g++) {
            for (int i = 0; i < D; i++) {
                hb.nodes[i * G + g] = make_float4(g == 0 ? bld.nodes[0].box.lo[i] : kInf, kInf, kInf, kInf);
                hb.nodes[(D + i) * G + g] = make_float4(g == 0 ? bld.nodes[0].box.hi[i] : -kInf, -kInf, -kInf, -kInf);
            }
            int4 ci = make_int4(g == 0 ? makeLeafRef(0, bld.nodes[0].count) : kEmpty, kEmpty, kEmpty, kEmpty);
            std::memcpy(&hb.nodes[2 * D * G + g], &ci, sizeof(int4));
            hb.nodes[(2 * D + 1) * G + g] = make_float4(g == 0 ? bld.nodes[0].area : 0.0f, 0, 0, 0);
        }
        hb.depth = 1;
    } else {
        Collapser col{D, bld.nodes, hb.nodes};
        col.width = width;
        col.emit(0, 1);
        hb.depth = col.maxDepth;
        if (kind != 0) {
            hb.cones.assign(hb.nodes.size(), make_float4(0, 0, 0, -1));
            for (size_t w = 0; w < col.kidsOf.size(); w++) {
                float km[4] = {0, 0, 0, 0}, kn[4] = {0, 0, 0, 0};
                for (int c = 0; c < 4; c++) {
                    int b = col.kidsOf[w][c];
                    if (b < 0) continue;
                    Cone cone;
                    coneOf(D, bld.nodes, b, bld.order, nrm, adj, flags, kind == 2 ? kmax : nullptr,
                           kind == 2 ? kmin : nullptr, kind == 2, cone);
                    hb.cones[w * 8 + c] = make_float4(cone.axis[0], cone.axis[1], cone.axis[2], cone.halfAngle);
                    km[c] = cone.kmax;
                    kn[c] = cone.kmin;
                }
                hb.cones[w * 8 + 4] = make_float4(km[0], km[1], km[2], km[3]);
                hb.cones[w * 8 + 5] = make_float4(kn[0], kn[1], kn[2], kn[3]);
            }
        }
    }
    hb.nNodes = (int)(hb.nodes.size() / (2 * width));
    if (kind != 0 && hb.cones.empty()) {
        // single-leaf scene: an always-visit cone
        hb.cones.assign(8, make_float4(0, 0, 0, 3.14159265f));
        float km = 0.0f, kn = kind == 2 ? kInf : 0.0f;
        if (kind == 2 && kmax) for (int i = 0; i < nP; i++) { km = std::max(km, kmax[i]); kn = std::min(kn, kmin[i]); }
        hb.cones[4] = make_float4(km, 0, 0, 0);
        hb.cones[5] = make_float4(kn, 0, 0, 0);
    }

    // ---- primitives and silhouette data in leaf order
    hb.primIndex = bld.order;
    hb.prims.resize((size_t)nP * (D == 2 ? 1 : 3));
    bool reflecting = kind != 0;
    if (reflecting) hb.sil.resize((size_t)nP * (D == 2 ? 2 : 3));
    for (int s = 0; s < nP; s++) {
        int i = bld.order[s];
        if (D == 2) {
            const float* a = pos + (size_t)idx[i * 2] * 2;
            const float* b = pos + (size_t)idx[i * 2 + 1] * 2;
            hb.prims[s] = make_float4(a[0], a[1], b[0], b[1]);
        } else {
            for (int k = 0; k < 3; k++) {
                const float* p = pos + (size_t)idx[i * 3 + k] * 3;
                hb.prims[(size_t)s * 3 + k] = make_float4(p[0], p[1], p[2], 0.0f);
            }
        }
        if (!reflecting) continue;
        float lo = kind == 2 && kmin ? kmin[i] : 0.0f;
        float hi = kind == 2 && kmax ? kmax[i] : 0.0f;
        float fl;
        int f = flags[i];
        std::memcpy(&fl, &f, 4);
        float an[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
        for (int j = 0; j < D; j++) {
            int a = adj[(size_t)i * D + j];
            if (a >= 0) for (int k = 0; k < D; k++) an[j][k] = nrm[(size_t)a * D + k];
        }
        if (D == 2) {
            hb.sil[(size_t)s * 2] = make_float4(an[0][0], an[0][1], an[1][0], an[1][1]);
            hb.sil[(size_t)s * 2 + 1] = make_float4(fl, lo, hi, 0.0f);
        } else {
            hb.sil[(size_t)s * 3] = make_float4(an[0][0], an[0][1], an[0][2], fl);
            hb.sil[(size_t)s * 3 + 1] = make_float4(an[1][0], an[1][1], an[1][2], lo);
            hb.sil[(size_t)s * 3 + 2] = make_float4(an[2][0], an[2][1], an[2][2], hi);
        }
    }
    // signed volume (computeSignedVolume, utils/fcpw_geometric_queries.h:431-458)
    double vol = 0.0;
    for (int i = 0; i < nP; i++) {
        const float* a = pos + (size_t)idx[i * D] * D;
        const float* b = pos + (size_t)idx[i * D + 1] * D;
        if (D == 2) {
            vol += 0.5 * ((double)a[0] * b[1] - (double)a[1] * b[0]);
        } else {
            const float* c = pos + (size_t)idx[i * D + 2] * D;
            vol += (((double)a[1] * b[2] - (double)a[2] * b[1]) * c[0] + ((double)a[2] * b[0] - (double)a[0] * b[2]) * c[1] +
                    ((double)a[0] * b[1] - (double)a[1] * b[0]) * c[2]) / 6.0;
        }
    }
    // ---- silhouette-candidate tree (FCPW computeSilhouettes, fcpw_geometric_queries.h:631):
    // every non-ignored vertex / edge once (kept by the face with the lower index when it has
    // two faces), with the normals of its two faces
    if (reflecting) {
        struct Feature { float a[3], b[3], nA[3], nB[3]; bool open; };
        std::vector<Feature> feats;
        for (int i = 0; i < nP; i++) {
            for (int j = 0; j < D; j++) {
                if (flags[i] & (8 << j)) continue;
                int a = adj[(size_t)i * D + j];
                if (a >= 0 && a < i) continue;   // the other face holds this feature
                Feature f{};
                f.open = a < 0;
                const float* n0 = &nrm[(size_t)i * D];
                const float* na = a >= 0 ? &nrm[(size_t)a * D] : n0;
                if (D == 2) {
                    const float* v = pos + (size_t)idx[i * 2 + j] * 2;
                    for (int k = 0; k < 2; k++) { f.a[k] = v[k]; f.b[k] = v[k]; }
                    // j = 0: the vertex ends the neighbour and starts this segment
                    const float* nPrev = j == 0 ? na : n0;
                    const float* nNext = j == 0 ? n0 : na;
                    for (int k = 0; k < 2; k++) { f.nA[k] = nPrev[k]; f.nB[k] = nNext[k]; }
                } else {
                    const float* pa = pos + (size_t)idx[i * 3 + j] * 3;
                    const float* pb = pos + (size_t)idx[i * 3 + (j + 1) % 3] * 3;
                    for (int k = 0; k < 3; k++) { f.a[k] = pa[k]; f.b[k] = pb[k]; f.nA[k] = n0[k]; f.nB[k] = na[k]; }
                }
                feats.push_back(f);
            }
        }
        hb.silFeatures = (int)feats.size();
        if (!feats.empty()) {
            std::vector<Box> fb(feats.size());
            std::vector<float> fc(feats.size() * D), fw(feats.size(), 1.0f);
            for (size_t k = 0; k < feats.size(); k++) {
                fb[k].grow(feats[k].a, D);
                fb[k].grow(feats[k].b, D);
                for (int i = 0; i < D; i++) fc[k * D + i] = 0.5f * (feats[k].a[i] + feats[k].b[i]);
            }
            WideTree wt;
            buildWideTree(D, fb, fc, fw, wt);
            hb.silTree = wt.nodes;
            hb.silNodes = (int)(wt.nodes.size() / 8);
            hb.silDepth = wt.depth;
            hb.silCones.assign(wt.nodes.size(), make_float4(0, 0, 0, -1));
            for (size_t w = 0; w < wt.kids.size(); w++) {
                for (int c = 0; c < 4; c++) {
                    int b = wt.kids[w][c];
                    if (b < 0) continue;
                    std::vector<int> stk = {b};
                    std::vector<const float*> ns;
                    bool open = false;
                    while (!stk.empty()) {
                        const BNode& m = wt.bnodes[stk.back()]; stk.pop_back();
                        if (m.count == 0) { stk.push_back(m.left); stk.push_back(m.right); continue; }
                        for (int q = 0; q < m.count; q++) {
                            const Feature& f = feats[wt.order[m.first + q]];
                            if (f.open) open = true;
                            ns.push_back(f.nA);
                            ns.push_back(f.nB);
                        }
                    }
                    float axis[3], half;
                    coneOverNormals(D, ns, open, axis, half);
                    hb.silCones[w * 8 + c] = make_float4(axis[0], axis[1], axis[2], half);
                }
            }
            int per = D == 2 ? 2 : 4;
            hb.silFeat.resize(feats.size() * per);
            for (size_t s2 = 0; s2 < feats.size(); s2++) {
                const Feature& f = feats[wt.order[s2]];
                float fl;
                int flg = f.open ? 1 : 0;
                std::memcpy(&fl, &flg, 4);
                if (D == 2) {
                    hb.silFeat[s2 * 2] = make_float4(f.a[0], f.a[1], f.nA[0], f.nA[1]);
                    hb.silFeat[s2 * 2 + 1] = make_float4(f.nB[0], f.nB[1], fl, 0.0f);
                } else {
                    hb.silFeat[s2 * 4] = make_float4(f.a[0], f.a[1], f.a[2], fl);
                    hb.silFeat[s2 * 4 + 1] = make_float4(f.b[0], f.b[1], f.b[2], 0.0f);
                    hb.silFeat[s2 * 4 + 2] = make_float4(f.nA[0], f.nA[1], f.nA[2], 0.0f);
                    hb.silFeat[s2 * 4 + 3] = make_float4(f.nB[0], f.nB[1], f.nB[2], 0.0f);
                }
            }
        }
    }
    hb.signedVolume = (float)vol;
    return true;
}

}  // namespace zg
