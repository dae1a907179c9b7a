// zgpu_devbuild.cu -- builds an absorbing boundary's 4-wide BVH on the device.
//
// The construction is the linear BVH of Karras, "Maximizing Parallelism in the Construction
// of BVHs, Octrees, and k-d Trees" (HPG 2012): primitives are ordered by the Morton code of
// their centroid (cub radix sort), the binary radix tree over the sorted codes is built with
// one thread per internal node, boxes are refitted bottom-up with one arrival counter per
// node, and the binary tree is collapsed level by level into the same 4-wide, 128-byte node
// layout the host builder emits (zgpu_build.cpp): each wide node opens its largest internal
// children until it holds four, and a subtree of at most 4 primitives becomes a leaf
// reference to its contiguous range of the sorted primitives.  Queries are exact on any
// valid tree, so a device-built tree answers like the host-built one (tests compare them);
// Morton order is a lower-quality split than the host's binned SAH.
#include <cub/device/device_radix_sort.cuh>

#include <cfloat>
#include <cstdint>
#include <vector>

#include "zgpu_internal.h"

namespace zg {
namespace {

constexpr int kEmpty = 0x7fffffff;
constexpr int kLeafMax = 4;

struct BinNode {        // internal node of the binary radix tree
    int left, right;    // >= 0 internal index, < 0: -(leaf position + 1)
    int parent;         // internal index (-1 root)
    int first, count;   // range of sorted primitives
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
    for (int j = 0; j < D; j++) {      // bounds of the centroids
        const float c = 0.5f * (l[j] + h[j]);
        atomicMin(sceneKey + j, fkey(c));
        atomicMax(sceneKey + 3 + j, fkey(c));
    }
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

__device__ __forceinline__ float halfArea(float4 l, float4 h, int D) {
    const float x = h.x - l.x, y = h.y - l.y, z = h.z - l.z;
    return D == 2 ? x + y : x * y + y * z + z * x;
}

// One level of the collapse: frontier entry k is binary node bin[k] emitted as wide node wide[k].
template <int D>
__global__ void collapseKernel(const int* __restrict__ frontierBin, const int* __restrict__ frontierWide, int nFront,
                               const BinNode* __restrict__ nodes, const int* __restrict__ ids,
                               const float4* __restrict__ plo, const float4* __restrict__ phi,
                               const float* __restrict__ parea, const float4* __restrict__ nlo,
                               const float4* __restrict__ nhi, const float* __restrict__ narea, float4* __restrict__ out,
                               int* __restrict__ nextBin, int* __restrict__ nextWide, int* __restrict__ counters) {
    const int f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= nFront) return;
    const int b = frontierBin[f], w = frontierWide[f];
    // children as binary refs (>= 0 internal, < 0 leaf); open the largest internal child
    // that holds more than kLeafMax primitives until there are four
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

template <typename T>
struct DevBuf {
    T* p = nullptr;
    ~DevBuf() { if (p) cudaFree(p); }
    cudaError_t alloc(size_t n) { return cudaMalloc(&p, sizeof(T) * (n ? n : 1)); }
};

}  // namespace

// Builds on the device; outputs are device arrays owned by the caller (cudaFree).
// Returns cudaSuccess and the wide depth, or an error.
cudaError_t buildWideBvhOnDevice(int D, const float* pos, const int* idx, int nP, cudaStream_t s, float4** outNodes,
                                 int* outNodeCount, float4** outPrims, int** outPrimIndex, int* outDepth) {
    *outNodes = nullptr; *outPrims = nullptr; *outPrimIndex = nullptr; *outNodeCount = 0; *outDepth = 0;
    if (nP <= 0) return cudaSuccess;
    cudaError_t e;
#define ZB(expr) do { e = (expr); if (e != cudaSuccess) return e; } while (0)
    const int T = 256, G = (nP + T - 1) / T;
    DevBuf<float4> plo, phi;
    DevBuf<float> parea;
    DevBuf<int> sceneKey, ids, idsSorted, leafParent, arrive, counters, fb0, fw0, fb1, fw1;
    DevBuf<uint32_t> code, codeSorted;
    ZB(plo.alloc(nP)); ZB(phi.alloc(nP)); ZB(parea.alloc(nP)); ZB(sceneKey.alloc(6));
    const int init[6] = {0x7fffffff, 0x7fffffff, 0x7fffffff, (int)0x80000000, (int)0x80000000, (int)0x80000000};
    int hostInit[6];
    for (int j = 0; j < 6; j++) hostInit[j] = init[j];
    ZB(cudaMemcpyAsync(sceneKey.p, hostInit, sizeof(hostInit), cudaMemcpyHostToDevice, s));
    if (D == 2) primKernel<2><<<G, T, 0, s>>>(pos, idx, nP, plo.p, phi.p, parea.p, sceneKey.p);
    else primKernel<3><<<G, T, 0, s>>>(pos, idx, nP, plo.p, phi.p, parea.p, sceneKey.p);
    ZB(cudaGetLastError());
    ZB(code.alloc(nP)); ZB(codeSorted.alloc(nP)); ZB(ids.alloc(nP)); ZB(idsSorted.alloc(nP));
    if (D == 2) mortonKernel<2><<<G, T, 0, s>>>(plo.p, phi.p, nP, sceneKey.p, code.p, ids.p);
    else mortonKernel<3><<<G, T, 0, s>>>(plo.p, phi.p, nP, sceneKey.p, code.p, ids.p);
    ZB(cudaGetLastError());
    size_t tmpBytes = 0;
    ZB(cub::DeviceRadixSort::SortPairs(nullptr, tmpBytes, code.p, codeSorted.p, ids.p, idsSorted.p, nP, 0, 32, s));
    DevBuf<unsigned char> tmp;
    ZB(tmp.alloc(tmpBytes));
    ZB(cub::DeviceRadixSort::SortPairs(tmp.p, tmpBytes, code.p, codeSorted.p, ids.p, idsSorted.p, nP, 0, 32, s));
    const int nInner = nP - 1;
    DevBuf<BinNode> bin;
    DevBuf<float4> nlo, nhi;
    DevBuf<float> narea;
    ZB(bin.alloc(nInner)); ZB(nlo.alloc(nInner)); ZB(nhi.alloc(nInner)); ZB(narea.alloc(nInner));
    ZB(leafParent.alloc(nP)); ZB(arrive.alloc(nInner));
    ZB(cudaMemsetAsync(leafParent.p, 0xff, sizeof(int) * nP, s));    // -1: the single-primitive root
    ZB(cudaMemsetAsync(arrive.p, 0, sizeof(int) * (nInner ? nInner : 1), s));
    if (nInner > 0) {
        radixTreeKernel<<<(nInner + T - 1) / T, T, 0, s>>>(codeSorted.p, nP, bin.p, leafParent.p);
        ZB(cudaGetLastError());
        refitKernel<<<G, T, 0, s>>>(idsSorted.p, plo.p, phi.p, parea.p, nP, bin.p, leafParent.p, nlo.p, nhi.p, narea.p,
                                    arrive.p);
        ZB(cudaGetLastError());
    }
    // wide nodes: at most one per internal binary node (plus the root of a 1-primitive scene)
    const int cap = nInner > 0 ? nInner : 1;
    float4* nodes = nullptr;
    ZB(cudaMalloc(&nodes, sizeof(float4) * 8 * (size_t)cap));
    int depth = 1, nNodes = 1;
    if (nInner == 0) {
        // a single primitive: one root whose first child is the leaf
        std::vector<float4> root(8, make_float4(0, 0, 0, 0));
        float4 l, h;
        ZB(cudaMemcpyAsync(&l, plo.p, sizeof(float4), cudaMemcpyDeviceToHost, s));
        ZB(cudaMemcpyAsync(&h, phi.p, sizeof(float4), cudaMemcpyDeviceToHost, s));
        float a;
        ZB(cudaMemcpyAsync(&a, parea.p, sizeof(float), cudaMemcpyDeviceToHost, s));
        ZB(cudaStreamSynchronize(s));
        const float lv[3] = {l.x, l.y, l.z}, hv[3] = {h.x, h.y, h.z};
        for (int i = 0; i < D; i++) {
            root[i] = make_float4(lv[i], FLT_MAX, FLT_MAX, FLT_MAX);
            root[D + i] = make_float4(hv[i], -FLT_MAX, -FLT_MAX, -FLT_MAX);
        }
        int4 ci = make_int4(makeLeaf(0, 1), kEmpty, kEmpty, kEmpty);
        root[2 * D] = *reinterpret_cast<float4*>(&ci);
        root[2 * D + 1] = make_float4(a, 0, 0, 0);
        ZB(cudaMemcpyAsync(nodes, root.data(), sizeof(float4) * 8, cudaMemcpyHostToDevice, s));
    } else {
        ZB(fb0.alloc(cap)); ZB(fw0.alloc(cap)); ZB(fb1.alloc(cap)); ZB(fw1.alloc(cap)); ZB(counters.alloc(2));
        const int zero[2] = {0, 0};
        ZB(cudaMemcpyAsync(fb0.p, zero, sizeof(int), cudaMemcpyHostToDevice, s));
        ZB(cudaMemcpyAsync(fw0.p, zero, sizeof(int), cudaMemcpyHostToDevice, s));
        int hostCount[2] = {1, 0};
        ZB(cudaMemcpyAsync(counters.p, hostCount, sizeof(hostCount), cudaMemcpyHostToDevice, s));
        int nFront = 1;
        int *cb = fb0.p, *cw = fw0.p, *nb = fb1.p, *nw = fw1.p;
        while (nFront > 0) {
            if (depth > kMaxWideDepth) { cudaFree(nodes); return cudaErrorNotSupported; }
            const int zeroSlot = 0;
            ZB(cudaMemcpyAsync(counters.p + 1, &zeroSlot, sizeof(int), cudaMemcpyHostToDevice, s));
            if (D == 2)
                collapseKernel<2><<<(nFront + T - 1) / T, T, 0, s>>>(cb, cw, nFront, bin.p, idsSorted.p, plo.p, phi.p,
                                                                    parea.p, nlo.p, nhi.p, narea.p, nodes, nb, nw,
                                                                    counters.p);
            else
                collapseKernel<3><<<(nFront + T - 1) / T, T, 0, s>>>(cb, cw, nFront, bin.p, idsSorted.p, plo.p, phi.p,
                                                                    parea.p, nlo.p, nhi.p, narea.p, nodes, nb, nw,
                                                                    counters.p);
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
    float4* prims = nullptr;
    int* primIndex = nullptr;
    if (cudaMalloc(&prims, sizeof(float4) * (size_t)nP * (D == 2 ? 1 : 3)) != cudaSuccess ||
        cudaMalloc(&primIndex, sizeof(int) * (size_t)nP) != cudaSuccess) {
        cudaFree(nodes); cudaFree(prims); cudaFree(primIndex);
        return cudaErrorMemoryAllocation;
    }
    if (D == 2) gatherKernel<2><<<G, T, 0, s>>>(pos, idx, idsSorted.p, nP, prims, primIndex);
    else gatherKernel<3><<<G, T, 0, s>>>(pos, idx, idsSorted.p, nP, prims, primIndex);
    e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) { cudaFree(nodes); cudaFree(prims); cudaFree(primIndex); return e; }
    *outNodes = nodes; *outNodeCount = nNodes; *outPrims = prims; *outPrimIndex = primIndex; *outDepth = depth;
    return cudaSuccess;
#undef ZB
}

}  // namespace zg
