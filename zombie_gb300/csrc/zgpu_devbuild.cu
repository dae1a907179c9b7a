// zgpu_devbuild.cu -- builds a boundary's 4-wide BVH on the device: absorbing boundaries, and
// reflecting (Neumann / Robin) boundaries with their normal cones, Robin coefficient ranges,
// silhouette flags and silhouette-candidate tree.
//
// The tree is the linear BVH of Karras, "Maximizing Parallelism in the Construction of BVHs,
// Octrees, and k-d Trees" (HPG 2012): items (primitives, or silhouette features) are ordered
// by the Morton code of their box centre (cub radix sort), the binary radix tree over the
// sorted codes is built with one thread per internal node, boxes are refitted bottom-up with
// one arrival counter per node, and the binary tree is collapsed level by level into the
// 4-wide, 128-byte node layout the host builder emits (zgpu_build.cpp): each wide node opens
// its largest internal children until it holds four, and a subtree of at most 4 items becomes
// a leaf reference to its contiguous range of the sorted items.
//
// Reflecting boundaries add, all on the device: face normals; face adjacency (2D: vertex
// tables; 3D: directed edges sorted by key and matched to their reverse by binary search, the
// highest face index winning on non-manifold edges as in the host's map); the silhouette
// ignore rule (utils/fcpw_geometric_queries.h:1029-1038); per-face silhouette records; normal
// cones merged bottom-up (axis = normalised sum of the normals below, half angle bounded by
// max over children of angle(axis, child axis) + child half angle, so a cone may be a little
// wider than the host's exact one, never narrower); Robin coefficient ranges; and the
// silhouette-candidate features (every non-ignored vertex / edge once) with their own tree.
// Queries are exact on any valid tree with conservative cones, so a device-built boundary
// answers like the host-built one (tests compare them); Morton order is a lower-quality split
// than the host's binned SAH.
#include <cub/device/device_radix_sort.cuh>
#include <cub/device/device_scan.cuh>

#include <cfloat>
#include <cstdint>
#include <vector>

#include "zgpu_internal.h"

namespace zg {
namespace {

constexpr int kEmpty = 0x7fffffff;
constexpr int kLeafMax = 4;
constexpr float kPiF = 3.14159265f;

struct BinNode {        // internal node of the binary radix tree
    int left, right;    // >= 0 internal index, < 0: -(leaf position + 1)
    int parent;         // internal index (-1 root)
    int first, count;   // range of sorted items
};

__device__ __forceinline__ uint32_t spread2(uint32_t v) {   // 16 bits -> every other bit
    v &= 0xffffu;
    v = (v | (v << 8)) & 0x00ff00ffu;
    v = (v | (v << 4)) & 0x0f0f0f0fu;
    v = (v | (v << 2)) & 0x33333333u;
    v = (v | (v << 1)) & 0x55555555u;
    return v;
}
__device__ __forceinline__ uint32_t spread3(uint32_t v) {   // 10 bits -> every third bit
    v &= 0x3ffu;
    v = (v | (v << 16)) & 0x030000ffu;
    v = (v | (v << 8)) & 0x0300f00fu;
    v = (v | (v << 4)) & 0x030c30c3u;
    v = (v | (v << 2)) & 0x09249249u;
    return v;
}

// ordered-int image of a float (for atomic min / max)
__device__ __forceinline__ int fkey(float f) { int i = __float_as_int(f); return i >= 0 ? i : i ^ 0x7fffffff; }
__device__ __forceinline__ float fval(int i) { return __int_as_float(i >= 0 ? i : i ^ 0x7fffffff); }

__device__ __forceinline__ void centreBounds(int D, const float* l, const float* h, int* sceneKey) {
    for (int j = 0; j < D; j++) {
        const float c = 0.5f * (l[j] + h[j]);
        atomicMin(sceneKey + j, fkey(c));
        atomicMax(sceneKey + 3 + j, fkey(c));
    }
}

// primitive boxes, areas (the SAH weight the host uses) and the bounds of the box centres
template <int D>
__global__ void primKernel(const float* __restrict__ pos, const int* __restrict__ idx, int n, float4* __restrict__ lo,
                           float4* __restrict__ hi, float* __restrict__ area, int* __restrict__ sceneKey) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float l[3] = {FLT_MAX, FLT_MAX, FLT_MAX}, h[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX}, v[3][3];
    for (int k = 0; k < D; k++) {
        const int vi = idx[i * D + k];
        for (int j = 0; j < D; j++) {
            v[k][j] = pos[(size_t)vi * D + j];
            l[j] = fminf(l[j], v[k][j]);
            h[j] = fmaxf(h[j], v[k][j]);
        }
    }
    lo[i] = make_float4(l[0], l[1], D == 3 ? l[2] : 0.0f, 0.0f);
    hi[i] = make_float4(h[0], h[1], D == 3 ? h[2] : 0.0f, 0.0f);
    if (D == 2) {
        area[i] = hypotf(v[1][0] - v[0][0], v[1][1] - v[0][1]);
    } else {
        const float ax = v[1][0] - v[0][0], ay = v[1][1] - v[0][1], az = v[1][2] - v[0][2];
        const float bx = v[2][0] - v[0][0], by = v[2][1] - v[0][1], bz = v[2][2] - v[0][2];
        const float cx = ay * bz - az * by, cy = az * bx - ax * bz, cz = ax * by - ay * bx;
        area[i] = 0.5f * sqrtf(cx * cx + cy * cy + cz * cz);
    }
    centreBounds(D, l, h, sceneKey);
}

template <int D>
__global__ void mortonKernel(const float4* __restrict__ lo, const float4* __restrict__ hi, int n,
                             const int* __restrict__ sceneKey, uint32_t* __restrict__ code, int* __restrict__ ids) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float c[3] = {0.5f * (lo[i].x + hi[i].x), 0.5f * (lo[i].y + hi[i].y), 0.5f * (lo[i].z + hi[i].z)};
    uint32_t q[3] = {0, 0, 0};
    const float scale = D == 2 ? 65535.0f : 1023.0f;
    for (int j = 0; j < D; j++) {
        const float a = fval(sceneKey[j]), b = fval(sceneKey[3 + j]);
        const float t = b > a ? (c[j] - a) / (b - a) : 0.5f;
        q[j] = (uint32_t)fminf(fmaxf(t * scale, 0.0f), scale);
    }
    code[i] = D == 2 ? (spread2(q[0]) | (spread2(q[1]) << 1)) : (spread3(q[0]) | (spread3(q[1]) << 1) | (spread3(q[2]) << 2));
    ids[i] = i;
}

// common prefix length of sorted keys i and j (ties broken by position), -1 outside [0, n)
__device__ __forceinline__ int delta(const uint32_t* code, int n, int i, int j) {
    if (j < 0 || j >= n) return -1;
    const uint32_t a = code[i], b = code[j];
    if (a == b) return 32 + __clz((uint32_t)i ^ (uint32_t)j);
    return __clz(a ^ b);
}

__global__ void radixTreeKernel(const uint32_t* __restrict__ code, int n, BinNode* __restrict__ nodes,
                                int* __restrict__ leafParent) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n - 1) return;
    const int d = delta(code, n, i, i + 1) > delta(code, n, i, i - 1) ? 1 : -1;
    const int dmin = delta(code, n, i, i - d);
    int lmax = 2;
    while (delta(code, n, i, i + lmax * d) > dmin) lmax <<= 1;
    int l = 0;
    for (int t = lmax >> 1; t >= 1; t >>= 1)
        if (delta(code, n, i, i + (l + t) * d) > dmin) l += t;
    const int j = i + l * d;
    const int dnode = delta(code, n, i, j);
    int s = 0;
    for (int t = (l + 1) >> 1;; t = (t + 1) >> 1) {
        if (delta(code, n, i, i + (s + t) * d) > dnode) s += t;
        if (t == 1) break;
    }
    const int gamma = i + s * d + min(d, 0);
    const int first = min(i, j), last = max(i, j);
    BinNode& nd = nodes[i];
    nd.first = first;
    nd.count = last - first + 1;
    if (first == gamma) { nd.left = -(gamma + 1); leafParent[gamma] = i; }
    else { nd.left = gamma; nodes[gamma].parent = i; }
    if (last == gamma + 1) { nd.right = -(gamma + 2); leafParent[gamma + 1] = i; }
    else { nd.right = gamma + 1; nodes[gamma + 1].parent = i; }
    if (i == 0) nd.parent = -1;
}

// boxes and areas bottom-up: the second child to arrive at a node computes it
__global__ void refitKernel(const int* __restrict__ ids, const float4* __restrict__ plo, const float4* __restrict__ phi,
                            const float* __restrict__ parea, int n, const BinNode* __restrict__ nodes,
                            const int* __restrict__ leafParent, float4* nlo, float4* nhi, float* narea,
                            int* arrive) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= n) return;
    int node = leafParent[s];
    while (node >= 0) {
        __threadfence();
        if (atomicAdd(arrive + node, 1) == 0) return;
        const BinNode nd = nodes[node];
        float4 l[2], h[2];
        float a[2];
        const int kids[2] = {nd.left, nd.right};
        for (int k = 0; k < 2; k++) {
            if (kids[k] < 0) {
                const int p = ids[-kids[k] - 1];
                l[k] = plo[p]; h[k] = phi[p]; a[k] = parea[p];
            } else {
                l[k] = __ldcg(nlo + kids[k]); h[k] = __ldcg(nhi + kids[k]); a[k] = __ldcg(narea + kids[k]);
            }
        }
        nlo[node] = make_float4(fminf(l[0].x, l[1].x), fminf(l[0].y, l[1].y), fminf(l[0].z, l[1].z), 0.0f);
        nhi[node] = make_float4(fmaxf(h[0].x, h[1].x), fmaxf(h[0].y, h[1].y), fmaxf(h[0].z, h[1].z), 0.0f);
        narea[node] = a[0] + a[1];
        node = nd.parent;
    }
}

// ---------------------------------------------------------------------- normal cones
// A cone: axis.xyz + half angle in w (< 0: no normal below, pi: open feature or degenerate
// axis), the unnormalised sum of the normals below, and the Robin coefficient range.
struct ConeArrays {
    float4* axis;   // per item / per internal node
    float4* sum;    // xyz: sum of normals, w: number of normals
    float2* k;      // (kmin, kmax)
};

__device__ __forceinline__ float angleBetween(float4 a, float4 b) {
    const float c = a.x * b.x + a.y * b.y + a.z * b.z;
    return acosf(fminf(fmaxf(c, -1.0f), 1.0f));
}

// merges two cones into a cone that holds both
__device__ void mergeCones(const float4 a[2], const float4 s[2], const float2 k[2], float4& axis, float4& sum, float2& kr) {
    kr = make_float2(fminf(k[0].x, k[1].x), fmaxf(k[0].y, k[1].y));
    const bool none0 = a[0].w < 0.0f, none1 = a[1].w < 0.0f;
    sum = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    if (none0 && none1) { axis = make_float4(0.0f, 0.0f, 0.0f, -1.0f); return; }
    for (int c = 0; c < 2; c++)
        if (a[c].w >= 0.0f) { sum.x += s[c].x; sum.y += s[c].y; sum.z += s[c].z; sum.w += s[c].w; }
    if (a[0].w >= kPiF || a[1].w >= kPiF) { axis = make_float4(0.0f, 0.0f, 0.0f, kPiF); return; }
    const float l = sqrtf(sum.x * sum.x + sum.y * sum.y + sum.z * sum.z);
    if (l < 1e-6f) { axis = make_float4(0.0f, 0.0f, 0.0f, kPiF); return; }
    axis = make_float4(sum.x / l, sum.y / l, sum.z / l, 0.0f);
    float h = 0.0f;
    for (int c = 0; c < 2; c++)
        if (a[c].w >= 0.0f) h = fmaxf(h, angleBetween(axis, a[c]) + a[c].w);
    axis.w = fminf(kPiF, h + 2e-5f);     // covers the rounding of the float angles
}

// cones of the internal nodes bottom-up (second arrival computes), like refitKernel
__global__ void coneRefitKernel(const int* __restrict__ ids, ConeArrays item, int n, const BinNode* __restrict__ nodes,
                                const int* __restrict__ leafParent, ConeArrays node, int* arrive) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= n) return;
    int at = leafParent[s];
    while (at >= 0) {
        __threadfence();
        if (atomicAdd(arrive + at, 1) == 0) return;
        const BinNode nd = nodes[at];
        float4 a[2], sm[2];
        float2 k[2];
        const int kids[2] = {nd.left, nd.right};
        for (int c = 0; c < 2; c++) {
            if (kids[c] < 0) {
                const int p = ids[-kids[c] - 1];
                a[c] = item.axis[p]; sm[c] = item.sum[p]; k[c] = item.k[p];
            } else {
                a[c] = __ldcg(node.axis + kids[c]); sm[c] = __ldcg(node.sum + kids[c]);
                k[c] = __ldcg(node.k + kids[c]);
            }
        }
        float4 ax, su;
        float2 kr;
        mergeCones(a, sm, k, ax, su, kr);
        node.axis[at] = ax; node.sum[at] = su; node.k[at] = kr;
        at = nd.parent;
    }
}

// the child cones of every wide node (rows 0-3), child max and min Robin coefficients (rows
// 4 and 5) from the binary node (or single item) behind each child
__global__ void wideConeKernel(const int* __restrict__ wideKids, int nWide, const int* __restrict__ ids, ConeArrays item,
                               ConeArrays node, float4* __restrict__ cones) {
    const int w = blockIdx.x * blockDim.x + threadIdx.x;
    if (w >= nWide) return;
    float km[4] = {0, 0, 0, 0}, kn[4] = {0, 0, 0, 0};
    for (int c = 0; c < 4; c++) {
        const int r = wideKids[w * 4 + c];
        float4 ax = make_float4(0.0f, 0.0f, 0.0f, -1.0f);
        if (r != kEmpty) {
            float2 k;
            if (r >= 0) { ax = node.axis[r]; k = node.k[r]; }
            else { const int p = ids[-r - 1]; ax = item.axis[p]; k = item.k[p]; }
            kn[c] = k.x; km[c] = k.y;
        }
        cones[(size_t)w * 8 + c] = ax;
    }
    cones[(size_t)w * 8 + 4] = make_float4(km[0], km[1], km[2], km[3]);
    cones[(size_t)w * 8 + 5] = make_float4(kn[0], kn[1], kn[2], kn[3]);
    cones[(size_t)w * 8 + 6] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    cones[(size_t)w * 8 + 7] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
}

__device__ __forceinline__ float halfArea(float4 l, float4 h, int D) {
    const float x = h.x - l.x, y = h.y - l.y, z = h.z - l.z;
    return D == 2 ? x + y : x * y + y * z + z * x;
}

// One level of the collapse: frontier entry k is binary node bin[k] emitted as wide node wide[k].
// wideKids (optional) records the binary reference behind each wide child.
template <int D>
__global__ void collapseKernel(const int* __restrict__ frontierBin, const int* __restrict__ frontierWide, int nFront,
                               const BinNode* __restrict__ nodes, const int* __restrict__ ids,
                               const float4* __restrict__ plo, const float4* __restrict__ phi,
                               const float* __restrict__ parea, const float4* __restrict__ nlo,
                               const float4* __restrict__ nhi, const float* __restrict__ narea, float4* __restrict__ out,
                               int* __restrict__ wideKids, int* __restrict__ nextBin, int* __restrict__ nextWide,
                               int* __restrict__ counters) {
    const int f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= nFront) return;
    const int b = frontierBin[f], w = frontierWide[f];
    // children as binary refs (>= 0 internal, < 0 leaf); open the largest internal child
    // that holds more than kLeafMax items until there are four
    int kid[4] = {nodes[b].left, nodes[b].right, 0, 0};
    int nk = 2;
    while (nk < 4) {
        int pick = -1;
        float best = -1.0f;
        for (int k = 0; k < nk; k++) {
            if (kid[k] < 0 || nodes[kid[k]].count <= kLeafMax) continue;
            const float a = halfArea(nlo[kid[k]], nhi[kid[k]], D);
            if (a > best) { best = a; pick = k; }
        }
        if (pick < 0) break;
        const int open = kid[pick];
        kid[pick] = nodes[open].left;
        kid[nk++] = nodes[open].right;
    }
    float lo[3][4], hi[3][4], area[4];
    int child[4];
    for (int c = 0; c < 4; c++) {
        for (int i = 0; i < 3; i++) { lo[i][c] = FLT_MAX; hi[i][c] = -FLT_MAX; }
        area[c] = 0.0f;
        child[c] = kEmpty;
        if (wideKids) wideKids[(size_t)w * 4 + c] = c < nk ? kid[c] : kEmpty;
    }
    for (int c = 0; c < nk; c++) {
        float4 l, h;
        if (kid[c] < 0) {
            const int s = -kid[c] - 1, p = ids[s];
            l = plo[p]; h = phi[p]; area[c] = parea[p];
            child[c] = makeLeaf(s, 1);
        } else {
            const BinNode nd = nodes[kid[c]];
            l = nlo[kid[c]]; h = nhi[kid[c]]; area[c] = narea[kid[c]];
            if (nd.count <= kLeafMax) {
                child[c] = makeLeaf(nd.first, nd.count);
            } else {
                const int id = atomicAdd(counters + 0, 1);      // wide node id
                const int slot = atomicAdd(counters + 1, 1);    // next frontier slot
                nextBin[slot] = kid[c];
                nextWide[slot] = id;
                child[c] = id;
            }
        }
        lo[0][c] = l.x; lo[1][c] = l.y; lo[2][c] = l.z;
        hi[0][c] = h.x; hi[1][c] = h.y; hi[2][c] = h.z;
    }
    float4* p = out + (size_t)w * 8;
    for (int i = 0; i < D; i++) {
        p[i] = make_float4(lo[i][0], lo[i][1], lo[i][2], lo[i][3]);
        p[D + i] = make_float4(hi[i][0], hi[i][1], hi[i][2], hi[i][3]);
    }
    int4 ci = make_int4(child[0], child[1], child[2], child[3]);
    p[2 * D] = *reinterpret_cast<float4*>(&ci);
    p[2 * D + 1] = make_float4(area[0], area[1], area[2], area[3]);
    for (int i = 2 * D + 2; i < 8; i++) p[i] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
}

// primitives in leaf order and their caller indices
template <int D>
__global__ void gatherKernel(const float* __restrict__ pos, const int* __restrict__ idx, const int* __restrict__ ids,
                             int n, float4* __restrict__ prims, int* __restrict__ primIndex) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= n) return;
    const int i = ids[s];
    primIndex[s] = i;
    if (D == 2) {
        const int a = idx[2 * i], b = idx[2 * i + 1];
        prims[s] = make_float4(pos[2 * a], pos[2 * a + 1], pos[2 * b], pos[2 * b + 1]);
    } else {
        for (int k = 0; k < 3; k++) {
            const int v = idx[3 * i + k];
            prims[(size_t)s * 3 + k] = make_float4(pos[3 * v], pos[3 * v + 1], pos[3 * v + 2], 0.0f);
        }
    }
}

// ------------------------------------------------------------ reflecting boundaries
// face normals (segment: (dy, -dx) / len; triangle: (b - a) x (c - a) / |.|)
template <int D>
__global__ void normalKernel(const float* __restrict__ pos, const int* __restrict__ idx, int n, float* __restrict__ nrm) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float* a = pos + (size_t)idx[i * D] * D;
    const float* b = pos + (size_t)idx[i * D + 1] * D;
    if (D == 2) {
        const float sx = b[0] - a[0], sy = b[1] - a[1], l = sqrtf(sx * sx + sy * sy);
        nrm[2 * i] = sy / l; nrm[2 * i + 1] = -sx / l;
    } else {
        const float* c = pos + (size_t)idx[i * 3 + 2] * 3;
        const float u[3] = {b[0] - a[0], b[1] - a[1], b[2] - a[2]}, v[3] = {c[0] - a[0], c[1] - a[1], c[2] - a[2]};
        const float x = u[1] * v[2] - u[2] * v[1], y = u[2] * v[0] - u[0] * v[2], z = u[0] * v[1] - u[1] * v[0];
        const float l = sqrtf(x * x + y * y + z * z);
        nrm[3 * i] = x / l; nrm[3 * i + 1] = y / l; nrm[3 * i + 2] = z / l;
    }
}

// 2D: the segments starting / ending at each vertex (the highest index on a shared vertex)
__global__ void vertexTableKernel(const int* __restrict__ idx, int n, int* startsAt, int* endsAt) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    atomicMax(startsAt + idx[2 * i], i);
    atomicMax(endsAt + idx[2 * i + 1], i);
}
__global__ void adjacency2Kernel(const int* __restrict__ idx, int n, const int* __restrict__ startsAt,
                                 const int* __restrict__ endsAt, int* __restrict__ adj) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    adj[2 * i] = endsAt[idx[2 * i]];
    adj[2 * i + 1] = startsAt[idx[2 * i + 1]];
}

// 3D: directed edge (u, v) of face f, keyed u << 32 | v
__global__ void edgeKeyKernel(const int* __restrict__ idx, int n, unsigned long long* __restrict__ key,
                              int* __restrict__ face) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= 3 * n) return;
    const int i = e / 3, j = e % 3;
    const unsigned long long u = (uint32_t)idx[3 * i + j], v = (uint32_t)idx[3 * i + (j + 1) % 3];
    key[e] = (u << 32) | v;
    face[e] = i;
}
// the face holding the reverse edge (v, u): the last of the equal keys in the stable sort
__global__ void adjacency3Kernel(const int* __restrict__ idx, int n, const unsigned long long* __restrict__ key,
                                 const int* __restrict__ face, int* __restrict__ adj) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= 3 * n) return;
    const int i = e / 3, j = e % 3;
    const unsigned long long u = (uint32_t)idx[3 * i + j], v = (uint32_t)idx[3 * i + (j + 1) % 3];
    const unsigned long long want = (v << 32) | u;
    int lo = 0, hi = 3 * n;          // first position with key > want
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (key[mid] <= want) lo = mid + 1; else hi = mid;
    }
    adj[e] = (lo > 0 && key[lo - 1] == want) ? face[lo - 1] : -1;
}

// bit j: feature j has a neighbour; bit 3 + j: feature j is ignored (not a silhouette
// candidate: utils/fcpw_geometric_queries.h:1029-1038)
template <int D>
__global__ void flagKernel(const float* __restrict__ pos, const int* __restrict__ idx, const float* __restrict__ nrm,
                           const int* __restrict__ adj, int n, bool doubleSided, float prec, int* __restrict__ flags) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    int f = 0;
    for (int j = 0; j < D; j++) {
        const int a = adj[(size_t)i * D + j];
        if (a < 0) continue;
        f |= 1 << j;
        bool ignore;
        const float* n0 = nrm + (size_t)i * D;
        const float* nj = nrm + (size_t)a * D;
        if (D == 2) {
            const float det = (n0[0] * nj[1] - n0[1] * nj[0]) * (j == 0 ? 1.0f : -1.0f);
            ignore = !doubleSided && det < prec;
        } else {
            const float* pa = pos + (size_t)idx[i * 3 + j] * 3;
            const float* pb = pos + (size_t)idx[i * 3 + (j + 1) % 3] * 3;
            const float e[3] = {pb[0] - pa[0], pb[1] - pa[1], pb[2] - pa[2]};
            const float el = sqrtf(e[0] * e[0] + e[1] * e[1] + e[2] * e[2]);
            const float c[3] = {nj[1] * n0[2] - nj[2] * n0[1], nj[2] * n0[0] - nj[0] * n0[2], nj[0] * n0[1] - nj[1] * n0[0]};
            const float angle = atan2f((e[0] * c[0] + e[1] * c[1] + e[2] * c[2]) / el,
                                       n0[0] * nj[0] + n0[1] * nj[1] + n0[2] * nj[2]);
            ignore = !doubleSided && angle < prec;
        }
        if (ignore) f |= 8 << j;
    }
    flags[i] = f;
}

// cone of one item over the normals it brings: a face its own normal and those of its
// non-ignored neighbours (every neighbour for Robin boundaries); an open feature makes it pi
template <int D>
__global__ void faceConeKernel(const float* __restrict__ nrm, const int* __restrict__ adj, const int* __restrict__ flags,
                               const float* __restrict__ kmin, const float* __restrict__ kmax, int n, bool allNormals,
                               ConeArrays out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float* list[4];
    int m = 0;
    bool open = false, any = allNormals;
    for (int j = 0; j < D; j++) {
        if (!allNormals && (flags[i] & (8 << j))) continue;
        if (!(flags[i] & (1 << j))) { open = true; continue; }
        list[m++] = nrm + (size_t)adj[(size_t)i * D + j] * D;
        any = true;
    }
    if (any) list[m++] = nrm + (size_t)i * D;
    out.k[i] = make_float2(kmin ? kmin[i] : 0.0f, kmax ? kmax[i] : 0.0f);
    float4 s = make_float4(0.0f, 0.0f, 0.0f, (float)m);
    for (int q = 0; q < m; q++) { s.x += list[q][0]; s.y += list[q][1]; if (D == 3) s.z += list[q][2]; }
    out.sum[i] = s;
    if (open) { out.axis[i] = make_float4(0.0f, 0.0f, 0.0f, kPiF); return; }
    if (m == 0) { out.axis[i] = make_float4(0.0f, 0.0f, 0.0f, -1.0f); return; }
    const float l = sqrtf(s.x * s.x + s.y * s.y + s.z * s.z);
    if (l < 1e-6f) { out.axis[i] = make_float4(0.0f, 0.0f, 0.0f, kPiF); return; }
    float4 ax = make_float4(s.x / l, s.y / l, s.z / l, 0.0f);
    float h = 0.0f;
    for (int q = 0; q < m; q++) {
        const float4 nq = make_float4(list[q][0], list[q][1], D == 3 ? list[q][2] : 0.0f, 0.0f);
        h = fmaxf(h, angleBetween(ax, nq));
    }
    ax.w = fminf(kPiF, h + 1e-4f);
    out.axis[i] = ax;
}

// per-face silhouette records in leaf order: neighbour normals, flags, Robin range
template <int D>
__global__ void silRecordKernel(const int* __restrict__ ids, const float* __restrict__ nrm, const int* __restrict__ adj,
                                const int* __restrict__ flags, const float* __restrict__ kmin,
                                const float* __restrict__ kmax, int n, float4* __restrict__ sil) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= n) return;
    const int i = ids[s];
    float an[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
    for (int j = 0; j < D; j++) {
        const int a = adj[(size_t)i * D + j];
        if (a >= 0) for (int k = 0; k < D; k++) an[j][k] = nrm[(size_t)a * D + k];
    }
    const float fl = __int_as_float(flags[i]);
    const float lo = kmin ? kmin[i] : 0.0f, hi = kmax ? kmax[i] : 0.0f;
    if (D == 2) {
        sil[(size_t)s * 2] = make_float4(an[0][0], an[0][1], an[1][0], an[1][1]);
        sil[(size_t)s * 2 + 1] = make_float4(fl, lo, hi, 0.0f);
    } else {
        sil[(size_t)s * 3] = make_float4(an[0][0], an[0][1], an[0][2], fl);
        sil[(size_t)s * 3 + 1] = make_float4(an[1][0], an[1][1], an[1][2], lo);
        sil[(size_t)s * 3 + 2] = make_float4(an[2][0], an[2][1], an[2][2], hi);
    }
}

// silhouette-candidate features: every non-ignored vertex (2D) / edge (3D), kept by the face
// with the lower index when two faces share it (FCPW computeSilhouettes)
template <int D>
__device__ __forceinline__ bool keepsFeature(const int* adj, const int* flags, int i, int j) {
    if (flags[i] & (8 << j)) return false;
    const int a = adj[(size_t)i * D + j];
    return !(a >= 0 && a < i);
}
template <int D>
__global__ void featureCountKernel(const int* __restrict__ adj, const int* __restrict__ flags, int n, int* __restrict__ count) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    int c = 0;
    for (int j = 0; j < D; j++) c += keepsFeature<D>(adj, flags, i, j);
    count[i] = c;
}
// feature records (a, b, nA, nB; a.w = 1 for an open feature) in face order, their boxes
template <int D>
__global__ void featureEmitKernel(const float* __restrict__ pos, const int* __restrict__ idx, const float* __restrict__ nrm,
                                  const int* __restrict__ adj, const int* __restrict__ flags, const int* __restrict__ offset,
                                  int n, float4* __restrict__ fa, float4* __restrict__ fb, float4* __restrict__ fnA,
                                  float4* __restrict__ fnB, float4* __restrict__ lo, float4* __restrict__ hi,
                                  float* __restrict__ weight, int* __restrict__ sceneKey) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    int out = offset[i];
    for (int j = 0; j < D; j++) {
        if (!keepsFeature<D>(adj, flags, i, j)) continue;
        const int a = adj[(size_t)i * D + j];
        const float* n0 = nrm + (size_t)i * D;
        const float* na = a >= 0 ? nrm + (size_t)a * D : n0;
        float pa[3] = {0, 0, 0}, pb[3] = {0, 0, 0}, nA[3] = {0, 0, 0}, nB[3] = {0, 0, 0};
        if (D == 2) {
            const float* v = pos + (size_t)idx[i * 2 + j] * 2;
            pa[0] = pb[0] = v[0]; pa[1] = pb[1] = v[1];
            const float* nPrev = j == 0 ? na : n0;      // j = 0: the vertex ends the neighbour
            const float* nNext = j == 0 ? n0 : na;
            nA[0] = nPrev[0]; nA[1] = nPrev[1]; nB[0] = nNext[0]; nB[1] = nNext[1];
        } else {
            const float* p0 = pos + (size_t)idx[i * 3 + j] * 3;
            const float* p1 = pos + (size_t)idx[i * 3 + (j + 1) % 3] * 3;
            for (int k = 0; k < 3; k++) { pa[k] = p0[k]; pb[k] = p1[k]; nA[k] = n0[k]; nB[k] = na[k]; }
        }
        fa[out] = make_float4(pa[0], pa[1], pa[2], a < 0 ? 1.0f : 0.0f);
        fb[out] = make_float4(pb[0], pb[1], pb[2], 0.0f);
        fnA[out] = make_float4(nA[0], nA[1], nA[2], 0.0f);
        fnB[out] = make_float4(nB[0], nB[1], nB[2], 0.0f);
        const float l[3] = {fminf(pa[0], pb[0]), fminf(pa[1], pb[1]), fminf(pa[2], pb[2])};
        const float h[3] = {fmaxf(pa[0], pb[0]), fmaxf(pa[1], pb[1]), fmaxf(pa[2], pb[2])};
        lo[out] = make_float4(l[0], l[1], l[2], 0.0f);
        hi[out] = make_float4(h[0], h[1], h[2], 0.0f);
        weight[out] = 1.0f;
        centreBounds(D, l, h, sceneKey);
        out++;
    }
}
// a feature's cone over its two face normals (pi for an open feature)
__global__ void featureConeKernel(const float4* __restrict__ fa, const float4* __restrict__ fnA,
                                  const float4* __restrict__ fnB, int n, ConeArrays out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float4 a = fnA[i], b = fnB[i];
    out.k[i] = make_float2(0.0f, 0.0f);
    out.sum[i] = make_float4(a.x + b.x, a.y + b.y, a.z + b.z, 2.0f);
    if (fa[i].w != 0.0f) { out.axis[i] = make_float4(0.0f, 0.0f, 0.0f, kPiF); return; }
    const float sx = a.x + b.x, sy = a.y + b.y, sz = a.z + b.z, l = sqrtf(sx * sx + sy * sy + sz * sz);
    if (l < 1e-6f) { out.axis[i] = make_float4(0.0f, 0.0f, 0.0f, kPiF); return; }
    float4 ax = make_float4(sx / l, sy / l, sz / l, 0.0f);
    ax.w = fminf(kPiF, fmaxf(angleBetween(ax, a), angleBetween(ax, b)) + 1e-4f);
    out.axis[i] = ax;
}
// feature records in the candidate tree's leaf order (2D: 2 float4, 3D: 4 float4)
template <int D>
__global__ void featureGatherKernel(const int* __restrict__ ids, const float4* __restrict__ fa,
                                    const float4* __restrict__ fb, const float4* __restrict__ fnA,
                                    const float4* __restrict__ fnB, int n, float4* __restrict__ out) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= n) return;
    const int k = ids[s];
    const float4 a = fa[k], b = fb[k], nA = fnA[k], nB = fnB[k];
    const float fl = __int_as_float(a.w != 0.0f ? 1 : 0);
    if (D == 2) {
        out[(size_t)s * 2] = make_float4(a.x, a.y, nA.x, nA.y);
        out[(size_t)s * 2 + 1] = make_float4(nB.x, nB.y, fl, 0.0f);
    } else {
        out[(size_t)s * 4] = make_float4(a.x, a.y, a.z, fl);
        out[(size_t)s * 4 + 1] = make_float4(b.x, b.y, b.z, 0.0f);
        out[(size_t)s * 4 + 2] = make_float4(nA.x, nA.y, nA.z, 0.0f);
        out[(size_t)s * 4 + 3] = make_float4(nB.x, nB.y, nB.z, 0.0f);
    }
}

template <typename T>
struct DevBuf {
    T* p = nullptr;
    DevBuf() = default;
    DevBuf(const DevBuf&) = delete;
    DevBuf& operator=(const DevBuf&) = delete;
    ~DevBuf() { if (p) cudaFree(p); }
    cudaError_t alloc(size_t n) { return cudaMalloc(&p, sizeof(T) * (n ? n : 1)); }
    T* release() { T* r = p; p = nullptr; return r; }
};

#define ZB(expr) do { cudaError_t e_ = (expr); if (e_ != cudaSuccess) return e_; } while (0)

// the binary tree over n items with boxes (lo, hi), weights and centre bounds sceneKey
struct BinaryTree {
    int n = 0;
    DevBuf<int> ids;          // sorted position -> item
    DevBuf<BinNode> bin;      // n - 1 internal nodes
    DevBuf<float4> nlo, nhi;
    DevBuf<float> narea;
    DevBuf<int> leafParent;
};

cudaError_t buildBinary(int D, const float4* lo, const float4* hi, const float* area, const int* sceneKey, int n,
                        cudaStream_t s, BinaryTree& t) {
    const int T = 256, G = (n + T - 1) / T;
    t.n = n;
    DevBuf<uint32_t> code, codeSorted;
    DevBuf<int> ids;
    ZB(code.alloc(n)); ZB(codeSorted.alloc(n)); ZB(ids.alloc(n)); ZB(t.ids.alloc(n));
    if (D == 2) mortonKernel<2><<<G, T, 0, s>>>(lo, hi, n, sceneKey, code.p, ids.p);
    else mortonKernel<3><<<G, T, 0, s>>>(lo, hi, n, sceneKey, code.p, ids.p);
    ZB(cudaGetLastError());
    size_t tmpBytes = 0;
    ZB(cub::DeviceRadixSort::SortPairs(nullptr, tmpBytes, code.p, codeSorted.p, ids.p, t.ids.p, n, 0, 32, s));
    DevBuf<unsigned char> tmp;
    ZB(tmp.alloc(tmpBytes));
    ZB(cub::DeviceRadixSort::SortPairs(tmp.p, tmpBytes, code.p, codeSorted.p, ids.p, t.ids.p, n, 0, 32, s));
    const int nInner = n - 1;
    DevBuf<int> arrive;
    ZB(t.bin.alloc(nInner)); ZB(t.nlo.alloc(nInner)); ZB(t.nhi.alloc(nInner)); ZB(t.narea.alloc(nInner));
    ZB(t.leafParent.alloc(n)); ZB(arrive.alloc(nInner));
    ZB(cudaMemsetAsync(t.leafParent.p, 0xff, sizeof(int) * n, s));    // -1: the single-item root
    ZB(cudaMemsetAsync(arrive.p, 0, sizeof(int) * (nInner ? nInner : 1), s));
    if (nInner > 0) {
        radixTreeKernel<<<(nInner + T - 1) / T, T, 0, s>>>(codeSorted.p, n, t.bin.p, t.leafParent.p);
        ZB(cudaGetLastError());
        refitKernel<<<G, T, 0, s>>>(t.ids.p, lo, hi, area, n, t.bin.p, t.leafParent.p, t.nlo.p, t.nhi.p, t.narea.p,
                                    arrive.p);
        ZB(cudaGetLastError());
    }
    return cudaStreamSynchronize(s);    // the local buffers above are freed on return
}

// The wide tree: nodes (8 float4 each) and, when asked for, the binary reference behind each
// wide child (4 per node).  A single item becomes a root whose first child is the leaf.
cudaError_t collapseWide(int D, const BinaryTree& t, const float4* lo, const float4* hi, const float* area,
                         cudaStream_t s, float4** outNodes, int* outCount, int* outDepth, int** outWideKids) {
    const int T = 256, n = t.n, nInner = n - 1;
    const int cap = nInner > 0 ? nInner : 1;       // at most one wide node per internal binary node
    DevBuf<float4> nodes;
    DevBuf<int> kids;
    ZB(nodes.alloc((size_t)8 * cap));
    if (outWideKids) ZB(kids.alloc((size_t)4 * cap));
    int depth = 1, nNodes = 1;
    if (nInner == 0) {
        std::vector<float4> root(8, make_float4(0, 0, 0, 0));
        float4 l, h;
        float a;
        ZB(cudaMemcpyAsync(&l, lo, sizeof(float4), cudaMemcpyDeviceToHost, s));
        ZB(cudaMemcpyAsync(&h, hi, sizeof(float4), cudaMemcpyDeviceToHost, s));
        ZB(cudaMemcpyAsync(&a, area, sizeof(float), cudaMemcpyDeviceToHost, s));
        ZB(cudaStreamSynchronize(s));
        const float lv[3] = {l.x, l.y, l.z}, hv[3] = {h.x, h.y, h.z};
        for (int i = 0; i < D; i++) {
            root[i] = make_float4(lv[i], FLT_MAX, FLT_MAX, FLT_MAX);
            root[D + i] = make_float4(hv[i], -FLT_MAX, -FLT_MAX, -FLT_MAX);
        }
        int4 ci = make_int4(makeLeaf(0, 1), kEmpty, kEmpty, kEmpty);
        root[2 * D] = *reinterpret_cast<float4*>(&ci);
        root[2 * D + 1] = make_float4(a, 0, 0, 0);
        ZB(cudaMemcpyAsync(nodes.p, root.data(), sizeof(float4) * 8, cudaMemcpyHostToDevice, s));
        const int k4[4] = {-1, kEmpty, kEmpty, kEmpty};     // the item at sorted position 0
        if (outWideKids) ZB(cudaMemcpyAsync(kids.p, k4, sizeof(k4), cudaMemcpyHostToDevice, s));
        ZB(cudaStreamSynchronize(s));
    } else {
        DevBuf<int> fb0, fw0, fb1, fw1, counters;
        ZB(fb0.alloc(cap)); ZB(fw0.alloc(cap)); ZB(fb1.alloc(cap)); ZB(fw1.alloc(cap)); ZB(counters.alloc(2));
        const int zero[2] = {0, 0};
        ZB(cudaMemcpyAsync(fb0.p, zero, sizeof(int), cudaMemcpyHostToDevice, s));
        ZB(cudaMemcpyAsync(fw0.p, zero, sizeof(int), cudaMemcpyHostToDevice, s));
        int hostCount[2] = {1, 0};
        ZB(cudaMemcpyAsync(counters.p, hostCount, sizeof(hostCount), cudaMemcpyHostToDevice, s));
        int nFront = 1;
        int *cb = fb0.p, *cw = fw0.p, *nb = fb1.p, *nw = fw1.p;
        while (nFront > 0) {
            if (depth > kMaxWideDepth) return cudaErrorNotSupported;
            const int zeroSlot = 0;
            ZB(cudaMemcpyAsync(counters.p + 1, &zeroSlot, sizeof(int), cudaMemcpyHostToDevice, s));
            if (D == 2)
                collapseKernel<2><<<(nFront + T - 1) / T, T, 0, s>>>(cb, cw, nFront, t.bin.p, t.ids.p, lo, hi, area,
                                                                    t.nlo.p, t.nhi.p, t.narea.p, nodes.p, kids.p, nb,
                                                                    nw, counters.p);
            else
                collapseKernel<3><<<(nFront + T - 1) / T, T, 0, s>>>(cb, cw, nFront, t.bin.p, t.ids.p, lo, hi, area,
                                                                    t.nlo.p, t.nhi.p, t.narea.p, nodes.p, kids.p, nb,
                                                                    nw, counters.p);
            ZB(cudaGetLastError());
            ZB(cudaMemcpyAsync(hostCount, counters.p, sizeof(hostCount), cudaMemcpyDeviceToHost, s));
            ZB(cudaStreamSynchronize(s));
            nFront = hostCount[1];
            nNodes = hostCount[0];
            if (nFront > 0) depth++;
            std::swap(cb, nb);
            std::swap(cw, nw);
        }
    }
    *outNodes = nodes.release();
    *outCount = nNodes;
    *outDepth = depth;
    if (outWideKids) *outWideKids = kids.release();
    return cudaSuccess;
}

// cones of the internal nodes from the item cones, then the wide nodes' cone blocks
cudaError_t wideCones(const BinaryTree& t, ConeArrays item, const int* wideKids, int nWide, cudaStream_t s,
                      float4** outCones) {
    const int T = 256, n = t.n, nInner = n - 1;
    DevBuf<float4> axis, sum, cones;
    DevBuf<float2> k;
    DevBuf<int> arrive;
    ZB(axis.alloc(nInner)); ZB(sum.alloc(nInner)); ZB(k.alloc(nInner)); ZB(arrive.alloc(nInner));
    ZB(cones.alloc((size_t)8 * nWide));
    ConeArrays node{axis.p, sum.p, k.p};
    if (nInner > 0) {
        ZB(cudaMemsetAsync(arrive.p, 0, sizeof(int) * nInner, s));
        coneRefitKernel<<<(n + T - 1) / T, T, 0, s>>>(t.ids.p, item, n, t.bin.p, t.leafParent.p, node, arrive.p);
        ZB(cudaGetLastError());
    }
    wideConeKernel<<<(nWide + T - 1) / T, T, 0, s>>>(wideKids, nWide, t.ids.p, item, node, cones.p);
    ZB(cudaGetLastError());
    ZB(cudaStreamSynchronize(s));
    *outCones = cones.release();
    return cudaSuccess;
}

// the contiguous range of sorted points behind every wide child (first, count): internal
// binary nodes give their range, single items their position
__global__ void childRangeKernel(const int* __restrict__ wideKids, int nWide, const BinNode* __restrict__ bin,
                                 int2* __restrict__ ranges) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= 4 * nWide) return;
    const int r = wideKids[k];
    int2 v = make_int2(0, 0);
    if (r != kEmpty) v = r >= 0 ? make_int2(bin[r].first, bin[r].count) : make_int2(-r - 1, 1);
    ranges[k] = v;
}

// points as zero-extent boxes (unit weight), with their bounds
template <int D>
__global__ void pointBoxKernel(const float* __restrict__ pts, int n, float4* __restrict__ lo, float4* __restrict__ hi,
                               float* __restrict__ weight, int* __restrict__ sceneKey) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float p[3] = {0.0f, 0.0f, 0.0f};
    for (int j = 0; j < D; j++) p[j] = pts[(size_t)i * D + j];
    lo[i] = hi[i] = make_float4(p[0], p[1], p[2], 0.0f);
    weight[i] = 1.0f;
    centreBounds(D, p, p, sceneKey);
}

cudaError_t initSceneKey(int* key, cudaStream_t s) {
    static const int init[6] = {0x7fffffff, 0x7fffffff, 0x7fffffff, (int)0x80000000, (int)0x80000000, (int)0x80000000};
    ZB(cudaMemcpyAsync(key, init, sizeof(init), cudaMemcpyHostToDevice, s));
    return cudaStreamSynchronize(s);
}

}  // namespace

// A 4-wide BVH over n device-resident points for radius searches; order maps leaf slots to
// point indices.
cudaError_t buildPointBvhOnDevice(int D, const float* pts, int n, cudaStream_t s, float4** outNodes, int* outCount,
                                  int* outDepth, int** outOrder, int2** outRanges) {
    *outNodes = nullptr; *outCount = 0; *outDepth = 0; *outOrder = nullptr; *outRanges = nullptr;
    if (n <= 0) return cudaSuccess;
    const int T = 256, G = (n + T - 1) / T;
    DevBuf<float4> lo, hi;
    DevBuf<float> w;
    DevBuf<int> sceneKey;
    ZB(lo.alloc(n)); ZB(hi.alloc(n)); ZB(w.alloc(n)); ZB(sceneKey.alloc(6));
    ZB(initSceneKey(sceneKey.p, s));
    if (D == 2) pointBoxKernel<2><<<G, T, 0, s>>>(pts, n, lo.p, hi.p, w.p, sceneKey.p);
    else pointBoxKernel<3><<<G, T, 0, s>>>(pts, n, lo.p, hi.p, w.p, sceneKey.p);
    ZB(cudaGetLastError());
    BinaryTree tree;
    ZB(buildBinary(D, lo.p, hi.p, w.p, sceneKey.p, n, s, tree));
    DevBuf<int> kids;
    ZB(collapseWide(D, tree, lo.p, hi.p, w.p, s, outNodes, outCount, outDepth, &kids.p));
    DevBuf<int2> ranges;
    ZB(ranges.alloc((size_t)4 * *outCount));
    childRangeKernel<<<(4 * *outCount + T - 1) / T, T, 0, s>>>(kids.p, *outCount, tree.bin.p, ranges.p);
    ZB(cudaGetLastError());
    ZB(cudaStreamSynchronize(s));
    *outOrder = tree.ids.release();
    *outRanges = ranges.release();
    return cudaSuccess;
}

// Builds on the device from device-resident positions / indices.  Absorbing boundaries fill
// nodes, prims and primIndex; reflecting boundaries (kind 1 Neumann, 2 Robin with kmin/kmax
// per primitive in device memory) also cones, sil and the silhouette-candidate tree.  All
// outputs are device arrays owned by the caller (cudaFree); cudaErrorNotSupported when a tree
// is deeper than the traversal stack.
cudaError_t buildBoundaryOnDevice(int D, const float* pos, int nV, const int* idx, int nP, int kind, const float* kmin,
                                  const float* kmax, bool doubleSided, float prec, cudaStream_t s, DeviceBuilt& out) {
    out = DeviceBuilt();
    if (nP <= 0) return cudaSuccess;
    const int T = 256, G = (nP + T - 1) / T;
    DevBuf<float4> plo, phi;
    DevBuf<float> parea;
    DevBuf<int> sceneKey;
    ZB(plo.alloc(nP)); ZB(phi.alloc(nP)); ZB(parea.alloc(nP)); ZB(sceneKey.alloc(6));
    ZB(initSceneKey(sceneKey.p, s));
    if (D == 2) primKernel<2><<<G, T, 0, s>>>(pos, idx, nP, plo.p, phi.p, parea.p, sceneKey.p);
    else primKernel<3><<<G, T, 0, s>>>(pos, idx, nP, plo.p, phi.p, parea.p, sceneKey.p);
    ZB(cudaGetLastError());
    BinaryTree tree;
    ZB(buildBinary(D, plo.p, phi.p, parea.p, sceneKey.p, nP, s, tree));
    const bool reflecting = kind != 0;
    DevBuf<float4> nodes, prims, cones, sil, silTree, silCones, silFeat;
    DevBuf<int> primIndex, wideKids;
    int nNodes = 0, depth = 0;
    ZB(collapseWide(D, tree, plo.p, phi.p, parea.p, s, &nodes.p, &nNodes, &depth, reflecting ? &wideKids.p : nullptr));
    ZB(prims.alloc((size_t)nP * (D == 2 ? 1 : 3))); ZB(primIndex.alloc(nP));
    if (D == 2) gatherKernel<2><<<G, T, 0, s>>>(pos, idx, tree.ids.p, nP, prims.p, primIndex.p);
    else gatherKernel<3><<<G, T, 0, s>>>(pos, idx, tree.ids.p, nP, prims.p, primIndex.p);
    ZB(cudaGetLastError());
    int silNodes = 0, silDepth = 0, nFeat = 0;
    if (reflecting) {
        // normals, adjacency, flags
        DevBuf<float> nrm;
        DevBuf<int> adj, flags;
        ZB(nrm.alloc((size_t)nP * D)); ZB(adj.alloc((size_t)nP * D)); ZB(flags.alloc(nP));
        if (D == 2) normalKernel<2><<<G, T, 0, s>>>(pos, idx, nP, nrm.p);
        else normalKernel<3><<<G, T, 0, s>>>(pos, idx, nP, nrm.p);
        ZB(cudaGetLastError());
        if (D == 2) {
            DevBuf<int> startsAt, endsAt;
            ZB(startsAt.alloc(nV)); ZB(endsAt.alloc(nV));
            ZB(cudaMemsetAsync(startsAt.p, 0xff, sizeof(int) * nV, s));
            ZB(cudaMemsetAsync(endsAt.p, 0xff, sizeof(int) * nV, s));
            vertexTableKernel<<<G, T, 0, s>>>(idx, nP, startsAt.p, endsAt.p);
            adjacency2Kernel<<<G, T, 0, s>>>(idx, nP, startsAt.p, endsAt.p, adj.p);
            ZB(cudaGetLastError());
            ZB(cudaStreamSynchronize(s));
        } else {
            const int nE = 3 * nP, GE = (nE + T - 1) / T;
            DevBuf<unsigned long long> key, keySorted;
            DevBuf<int> face, faceSorted;
            ZB(key.alloc(nE)); ZB(keySorted.alloc(nE)); ZB(face.alloc(nE)); ZB(faceSorted.alloc(nE));
            edgeKeyKernel<<<GE, T, 0, s>>>(idx, nP, key.p, face.p);
            ZB(cudaGetLastError());
            size_t tmpBytes = 0;
            ZB(cub::DeviceRadixSort::SortPairs(nullptr, tmpBytes, key.p, keySorted.p, face.p, faceSorted.p, nE, 0, 64, s));
            DevBuf<unsigned char> tmp;
            ZB(tmp.alloc(tmpBytes));
            ZB(cub::DeviceRadixSort::SortPairs(tmp.p, tmpBytes, key.p, keySorted.p, face.p, faceSorted.p, nE, 0, 64, s));
            adjacency3Kernel<<<GE, T, 0, s>>>(idx, nP, keySorted.p, faceSorted.p, adj.p);
            ZB(cudaGetLastError());
            ZB(cudaStreamSynchronize(s));
        }
        if (D == 2) flagKernel<2><<<G, T, 0, s>>>(pos, idx, nrm.p, adj.p, nP, doubleSided, prec, flags.p);
        else flagKernel<3><<<G, T, 0, s>>>(pos, idx, nrm.p, adj.p, nP, doubleSided, prec, flags.p);
        ZB(cudaGetLastError());
        const float* kn = kind == 2 ? kmin : nullptr;
        const float* kx = kind == 2 ? kmax : nullptr;
        // cones of the primitive tree
        DevBuf<float4> iaxis, isum;
        DevBuf<float2> ik;
        ZB(iaxis.alloc(nP)); ZB(isum.alloc(nP)); ZB(ik.alloc(nP));
        ConeArrays item{iaxis.p, isum.p, ik.p};
        if (D == 2) faceConeKernel<2><<<G, T, 0, s>>>(nrm.p, adj.p, flags.p, kn, kx, nP, kind == 2, item);
        else faceConeKernel<3><<<G, T, 0, s>>>(nrm.p, adj.p, flags.p, kn, kx, nP, kind == 2, item);
        ZB(cudaGetLastError());
        ZB(wideCones(tree, item, wideKids.p, nNodes, s, &cones.p));
        // per-face silhouette records
        ZB(sil.alloc((size_t)nP * (D == 2 ? 2 : 3)));
        if (D == 2) silRecordKernel<2><<<G, T, 0, s>>>(tree.ids.p, nrm.p, adj.p, flags.p, kn, kx, nP, sil.p);
        else silRecordKernel<3><<<G, T, 0, s>>>(tree.ids.p, nrm.p, adj.p, flags.p, kn, kx, nP, sil.p);
        ZB(cudaGetLastError());
        // silhouette-candidate features and their tree
        DevBuf<int> count, offset;
        ZB(count.alloc(nP)); ZB(offset.alloc(nP));
        if (D == 2) featureCountKernel<2><<<G, T, 0, s>>>(adj.p, flags.p, nP, count.p);
        else featureCountKernel<3><<<G, T, 0, s>>>(adj.p, flags.p, nP, count.p);
        ZB(cudaGetLastError());
        size_t scanBytes = 0;
        ZB(cub::DeviceScan::ExclusiveSum(nullptr, scanBytes, count.p, offset.p, nP, s));
        DevBuf<unsigned char> scanTmp;
        ZB(scanTmp.alloc(scanBytes));
        ZB(cub::DeviceScan::ExclusiveSum(scanTmp.p, scanBytes, count.p, offset.p, nP, s));
        int last[2];
        ZB(cudaMemcpyAsync(&last[0], offset.p + nP - 1, sizeof(int), cudaMemcpyDeviceToHost, s));
        ZB(cudaMemcpyAsync(&last[1], count.p + nP - 1, sizeof(int), cudaMemcpyDeviceToHost, s));
        ZB(cudaStreamSynchronize(s));
        nFeat = last[0] + last[1];
        if (nFeat > 0) {
            const int GF = (nFeat + T - 1) / T;
            DevBuf<float4> fa, fb, fnA, fnB, flo, fhi;
            DevBuf<float> fw;
            ZB(fa.alloc(nFeat)); ZB(fb.alloc(nFeat)); ZB(fnA.alloc(nFeat)); ZB(fnB.alloc(nFeat));
            ZB(flo.alloc(nFeat)); ZB(fhi.alloc(nFeat)); ZB(fw.alloc(nFeat));
            ZB(initSceneKey(sceneKey.p, s));
            if (D == 2)
                featureEmitKernel<2><<<G, T, 0, s>>>(pos, idx, nrm.p, adj.p, flags.p, offset.p, nP, fa.p, fb.p, fnA.p,
                                                    fnB.p, flo.p, fhi.p, fw.p, sceneKey.p);
            else
                featureEmitKernel<3><<<G, T, 0, s>>>(pos, idx, nrm.p, adj.p, flags.p, offset.p, nP, fa.p, fb.p, fnA.p,
                                                    fnB.p, flo.p, fhi.p, fw.p, sceneKey.p);
            ZB(cudaGetLastError());
            BinaryTree ft;
            ZB(buildBinary(D, flo.p, fhi.p, fw.p, sceneKey.p, nFeat, s, ft));
            DevBuf<int> fKids;
            ZB(collapseWide(D, ft, flo.p, fhi.p, fw.p, s, &silTree.p, &silNodes, &silDepth, &fKids.p));
            DevBuf<float4> faxis, fsum;
            DevBuf<float2> fk;
            ZB(faxis.alloc(nFeat)); ZB(fsum.alloc(nFeat)); ZB(fk.alloc(nFeat));
            ConeArrays fitem{faxis.p, fsum.p, fk.p};
            featureConeKernel<<<GF, T, 0, s>>>(fa.p, fnA.p, fnB.p, nFeat, fitem);
            ZB(cudaGetLastError());
            ZB(wideCones(ft, fitem, fKids.p, silNodes, s, &silCones.p));
            ZB(silFeat.alloc((size_t)nFeat * (D == 2 ? 2 : 4)));
            if (D == 2) featureGatherKernel<2><<<GF, T, 0, s>>>(ft.ids.p, fa.p, fb.p, fnA.p, fnB.p, nFeat, silFeat.p);
            else featureGatherKernel<3><<<GF, T, 0, s>>>(ft.ids.p, fa.p, fb.p, fnA.p, fnB.p, nFeat, silFeat.p);
            ZB(cudaGetLastError());
        }
    }
    ZB(cudaStreamSynchronize(s));
    out.nodes = nodes.release(); out.nNodes = nNodes; out.depth = depth;
    out.prims = prims.release(); out.primIndex = primIndex.release();
    out.cones = cones.release(); out.sil = sil.release();
    out.silTree = silTree.release(); out.silCones = silCones.release(); out.silFeat = silFeat.release();
    out.silNodes = silNodes; out.silDepth = silDepth; out.silFeatures = nFeat;
    return cudaSuccess;
}
#undef ZB

}  // namespace zg
