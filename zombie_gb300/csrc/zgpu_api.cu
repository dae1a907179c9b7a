// zgpu_api.cu -- implementation of the C ABI declared in include/zgpu.h.
//
// Host-memory arrays are staged through device scratch owned by the context (the
// end-to-end path); device-memory arrays are used in place.  Every kernel of a context
// runs on its stream; entry points return after the stream has drained.
#include <cfloat>
#include <cstdarg>
#include <cstdio>
#include <algorithm>
#include <cstring>
#include <map>
#include <string>
#include <vector>

#include "zgpu_build.h"
#include "zgpu_internal.h"

using namespace zg;

namespace {

thread_local std::string gLastError;

int fail(int code, const char* fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    gLastError = buf;
    return code;
}

#define ZG_CUDA(call)                                                                          \
    do {                                                                                       \
        cudaError_t e_ = (call);                                                               \
        if (e_ != cudaSuccess)                                                                 \
            return fail(e_ == cudaErrorMemoryAllocation ? ZGPU_ERR_OUT_OF_MEMORY : ZGPU_ERR_CUDA, \
                        "%s failed: %s", #call, cudaGetErrorString(e_));                       \
    } while (0)

struct Buf {
    void* p = nullptr;
    size_t bytes = 0;
};

cudaError_t ensure(Buf& b, size_t bytes) {
    if (bytes == 0) bytes = 16;
    if (b.bytes >= bytes) return cudaSuccess;
    if (b.p) cudaFree(b.p);
    b.p = nullptr;
    b.bytes = 0;
    size_t grow = bytes + bytes / 4;
    cudaError_t e = cudaMalloc(&b.p, grow);
    if (e == cudaSuccess) b.bytes = grow;
    return e;
}

}  // namespace

struct zgpu_context {
    int device = 0;
    int numSMs = 0;
    cudaStream_t stream = nullptr;
    cudaEvent_t ev[4] = {nullptr, nullptr, nullptr, nullptr};
    // scratch (indexed by role)
    enum { kPt, kNormal, kType, kEq, kDist, kNWalks, kSeed, kFsr, kAligned, kMean, kM2, kN, kLen, kSplits,
           kWalkStart, kFlags, kNPrev, kAccSum, kAccSq, kAccN, kAccLen, kAccSplits, kBlockSums, kCounters,
           kQ0, kQ1, kQ2, kQ3, kQ4, kQ5, kQ6, kQ7, kQ8, kQ9, kQ10, kQ11, kSplitScratch, kCacheRec, kSceneTable, kSceneId,
           kDistRefl, kGMean, kGM2, kGN, kAccGrad, kAccGradSq, kAccGradN, kDirDeriv, kFirstSrc, kDeriv, kAccFirstSrc,
           kAccDeriv, kB0, kB1, kB2, kB3, kB4, kB5, kB6, kB7, kB8, kB9, kB10, kB11, kB12, kB13, kB14, kB15, kB16, kB17,
           kB18, kB19, kWaveA, kWaveB, kWaveKey, kWaveRank, kWaveCount, kWaveOffset, kWaveCtr, kNumBufs };
    Buf bufs[kNumBufs];
    unsigned long long* hostCounters = nullptr;   // pinned: counters + error word
    // use_graph: the captured prepare/scan/walk/finalize sequence, replayed while the solve's
    // parameters (pointers, sizes, settings) are those it was captured with
    cudaGraphExec_t graphExec = nullptr;
    std::vector<unsigned char> graphKey;
    // use_graph on the wavefront: one captured chunk of kWaveCheck iterations, replayed
    // between the host's live-count checks while its parameters are those it was captured with
    cudaGraphExec_t waveGraphExec = nullptr;
    std::vector<unsigned char> waveGraphKey;
    // autotuner results by scene signature
    std::map<std::string, zgpu_solve_options> tuned;
    std::vector<Buf> gridBufs;   // device copies of host-memory PDE grids
    long long lastLaunches = 0;  // kernel launches of the last solve (zgpu_last_solve_launches)
};

struct zgpu_boundary {
    zgpu_context* ctx = nullptr;
    int dim = 2;
    int kind = 0;
    int nPrims = 0;
    int nNodes = 0;
    int depth = 0;
    float signedVolume = 0.0f;
    float4* nodes = nullptr;
    float4* cones = nullptr;
    float4* prims = nullptr;
    float4* silTree = nullptr;
    float4* silCones = nullptr;
    float4* silFeat = nullptr;
    float4* sil = nullptr;
    int* primIndex = nullptr;
    std::vector<int> primIndexHost;   // leaf slot -> caller index (for coefficient updates)
    BoundaryView view;
    int queryMode = ZGPU_QUERY_MODE_AUTO;   // batched closest-point / Robin star-radius queries
    // 3D absorbing boundaries built on the host keep their mesh, from which an 8-wide twin of
    // the tree is built on first use (zgpu_solve_options.bvh_width = 8, the autotuner)
    std::vector<float> hostPos;
    std::vector<int> hostIdx;
    zgpu_boundary* twin8 = nullptr;
};

namespace {

// Stages `count` elements of `elem` bytes from caller memory to device; returns the device pointer.
template <typename T>
int stageIn(zgpu_context* ctx, int role, const T* src, size_t count, int memory, const T** out) {
    if (!src) { *out = nullptr; return ZGPU_OK; }
    if (memory == ZGPU_MEM_DEVICE) { *out = src; return ZGPU_OK; }
    ZG_CUDA(ensure(ctx->bufs[role], count * sizeof(T)));
    ZG_CUDA(cudaMemcpyAsync(ctx->bufs[role].p, src, count * sizeof(T), cudaMemcpyHostToDevice, ctx->stream));
    *out = (const T*)ctx->bufs[role].p;
    return ZGPU_OK;
}
template <typename T>
int stageInOut(zgpu_context* ctx, int role, T* src, size_t count, int memory, T** out) {
    const T* c = nullptr;
    int st = stageIn<T>(ctx, role, src, count, memory, &c);
    *out = const_cast<T*>(c);
    return st;
}
template <typename T>
int stageOut(zgpu_context* ctx, const T* dev, T* dst, size_t count, int memory) {
    if (!dst || memory == ZGPU_MEM_DEVICE) return ZGPU_OK;
    ZG_CUDA(cudaMemcpyAsync(dst, dev, count * sizeof(T), cudaMemcpyDeviceToHost, ctx->stream));
    return ZGPU_OK;
}
template <typename T>
int scratch(zgpu_context* ctx, int role, size_t count, T** out) {
    ZG_CUDA(ensure(ctx->bufs[role], count * sizeof(T)));
    *out = (T*)ctx->bufs[role].p;
    return ZGPU_OK;
}

#define ZG_TRY(x) do { int s_ = (x); if (s_ != ZGPU_OK) return s_; } while (0)

int checkBoundary(zgpu_boundary* b, int dim, const char* what) {
    if (!b) return ZGPU_OK;
    if (b->dim != dim) return fail(ZGPU_ERR_INVALID_ARG, "%s boundary has dim %d, queries have dim %d", what, b->dim, dim);
    return ZGPU_OK;
}

int checkField(int kind, const zgpu_grid& g, int D, const char* name) {
    if (kind < ZGPU_FIELD_ZERO || kind > ZGPU_FIELD_GRID) return fail(ZGPU_ERR_INVALID_ARG, "%s: unknown field kind %d", name, kind);
    if (kind != ZGPU_FIELD_GRID) return ZGPU_OK;
    if (!g.values) return fail(ZGPU_ERR_INVALID_ARG, "%s: grid has no values", name);
    int64_t cells = 1;
    for (int i = 0; i < D; i++) {
        if (g.shape[i] < 1) return fail(ZGPU_ERR_INVALID_ARG, "%s: grid shape[%d] = %d must be >= 1", name, i, g.shape[i]);
        if (!(g.grid_max[i] > g.grid_min[i])) return fail(ZGPU_ERR_INVALID_ARG, "%s: grid_max[%d] must exceed grid_min[%d]", name, i, i);
        cells *= g.shape[i];
        if (cells > ((int64_t)1 << 40)) return fail(ZGPU_ERR_INVALID_ARG, "%s: grid has too many cells", name);
    }
    return ZGPU_OK;
}

int64_t gridCells(const zgpu_grid& g, int D) {
    int64_t c = 1;
    for (int i = 0; i < D; i++) c *= g.shape[i];
    return c;
}

}  // namespace

namespace zg {
// the PDE's fields: kinds, grid shapes and boxes, and where the grid values live
int checkPdeFields(const zgpu_pde* pde, int D, bool hostGrids) {
    ZG_TRY(checkField(pde->source_kind, pde->source_grid, D, "source"));
    ZG_TRY(checkField(pde->dirichlet_kind, pde->dirichlet_grid, D, "dirichlet"));
    ZG_TRY(checkField(pde->robin_kind, pde->robin_grid, D, "robin"));
    ZG_TRY(checkField(pde->robin_coeff_kind, pde->robin_coeff_grid, D, "robin_coeff"));
    if (pde->robin_coeff_kind == ZGPU_FIELD_ANALYTIC) return fail(ZGPU_ERR_UNSUPPORTED, "robin_coeff must be ZERO, CONSTANT or GRID");
    const bool grids = pde->source_kind == ZGPU_FIELD_GRID || pde->dirichlet_kind == ZGPU_FIELD_GRID ||
                       pde->robin_kind == ZGPU_FIELD_GRID || pde->robin_coeff_kind == ZGPU_FIELD_GRID;
    if (grids && pde->memory != ZGPU_MEM_DEVICE && (!hostGrids || pde->memory != ZGPU_MEM_HOST))
        return fail(ZGPU_ERR_INVALID_ARG, hostGrids ? "pde.memory must be ZGPU_MEM_HOST or ZGPU_MEM_DEVICE"
                                                    : "grid values must be in device memory here");
    return ZGPU_OK;
}
}  // namespace zg

// internal accessors used by the allocation-free entry point (zgpu_static.cu) and the cache
namespace zg {
void setLastError(const char* msg) { gLastError = msg; }
int contextDevice(const zgpu_context* ctx) { return ctx->device; }
bool boundaryView(const zgpu_boundary* b, BoundaryView* view, int* dim, int* kind) {
    if (!b) return false;
    *view = b->view; *dim = b->dim; *kind = b->kind;
    return true;
}
}  // namespace zg

extern "C" {

int zgpu_abi_version(void) { return ZGPU_ABI_VERSION; }

const char* zgpu_last_error(void) { return gLastError.c_str(); }

int zgpu_context_create(int device, zgpu_context** out) {
    if (!out) return fail(ZGPU_ERR_INVALID_ARG, "out is NULL");
    *out = nullptr;
    int n = 0;
    ZG_CUDA(cudaGetDeviceCount(&n));
    if (device < 0 || device >= n) return fail(ZGPU_ERR_INVALID_ARG, "device %d out of range (%d devices)", device, n);
    ZG_CUDA(cudaSetDevice(device));
    zgpu_context* c = new zgpu_context();
    c->device = device;
    cudaDeviceGetAttribute(&c->numSMs, cudaDevAttrMultiProcessorCount, device);
    cudaError_t e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
    for (int i = 0; i < 4 && e == cudaSuccess; i++) e = cudaEventCreate(&c->ev[i]);
    if (e == cudaSuccess) e = cudaMallocHost((void**)&c->hostCounters, sizeof(unsigned long long) * 16);
    if (e != cudaSuccess) {
        zgpu_context_destroy(c);
        return fail(ZGPU_ERR_CUDA, "context creation failed: %s", cudaGetErrorString(e));
    }
    *out = c;
    return ZGPU_OK;
}

int zgpu_context_destroy(zgpu_context* c) {
    if (!c) return ZGPU_OK;
    cudaSetDevice(c->device);
    if (c->stream) cudaStreamSynchronize(c->stream);
    for (auto& b : c->bufs) if (b.p) cudaFree(b.p);
    for (auto& b : c->gridBufs) if (b.p) cudaFree(b.p);
    for (auto& e : c->ev) if (e) cudaEventDestroy(e);
    if (c->hostCounters) cudaFreeHost(c->hostCounters);
    if (c->graphExec) cudaGraphExecDestroy(c->graphExec);
    if (c->waveGraphExec) cudaGraphExecDestroy(c->waveGraphExec);
    if (c->stream) cudaStreamDestroy(c->stream);
    delete c;
    return ZGPU_OK;
}

int zgpu_context_synchronize(zgpu_context* c) {
    if (!c) return fail(ZGPU_ERR_INVALID_ARG, "context is NULL");
    ZG_CUDA(cudaStreamSynchronize(c->stream));
    return ZGPU_OK;
}

void* zgpu_context_stream(zgpu_context* c) { return c ? (void*)c->stream : nullptr; }

int zgpu_boundary_create(zgpu_context* ctx, int dim, const float* positions, int n_vertices, const int* indices,
                         int n_prims, int kind, const float* min_robin, const float* max_robin,
                         int solve_double_sided, float silhouette_precision, int bvh_width, zgpu_boundary** out) {
    if (!ctx || !out) return fail(ZGPU_ERR_INVALID_ARG, "context/out is NULL");
    *out = nullptr;
    if (dim != 2 && dim != 3) return fail(ZGPU_ERR_INVALID_ARG, "dim must be 2 or 3, got %d", dim);
    if (kind < ZGPU_BOUNDARY_ABSORBING || kind > ZGPU_BOUNDARY_ROBIN) return fail(ZGPU_ERR_INVALID_ARG, "unknown boundary kind %d", kind);
    if (bvh_width == 0) bvh_width = 4;
    if (bvh_width != 4 && bvh_width != 8) return fail(ZGPU_ERR_INVALID_ARG, "bvh_width must be 4 or 8, got %d", bvh_width);
    if (bvh_width == 8 && (dim != 3 || kind != ZGPU_BOUNDARY_ABSORBING))
        return fail(ZGPU_ERR_UNSUPPORTED, "8-wide nodes are built for 3D absorbing boundaries only");
    if (n_prims > 0 && (!positions || !indices)) return fail(ZGPU_ERR_INVALID_ARG, "positions/indices are NULL");
    if (kind == ZGPU_BOUNDARY_ROBIN && n_prims > 0 && (!min_robin || !max_robin))
        return fail(ZGPU_ERR_INVALID_ARG, "Robin boundary needs min/max Robin coefficients per primitive");
    HostBoundary hb;
    std::string err;
    if (!buildBoundary(dim, positions, n_vertices, indices, n_prims, kind, min_robin, max_robin,
                       solve_double_sided != 0, silhouette_precision, hb, err, bvh_width))
        return fail(ZGPU_ERR_INVALID_ARG, "boundary build: %s", err.c_str());
    if (hb.depth > kMaxWideDepth || hb.silDepth > kMaxWideDepth || (bvh_width - 1) * hb.depth + 2 > kMaxStack)
        return fail(ZGPU_ERR_UNSUPPORTED, "boundary BVH depth %d/%d exceeds the traversal stack (max %d entries)",
                    hb.depth, hb.silDepth, kMaxStack);
    ZG_CUDA(cudaSetDevice(ctx->device));
    zgpu_boundary* b = new zgpu_boundary();
    b->ctx = ctx; b->dim = dim; b->kind = kind; b->nPrims = n_prims; b->nNodes = hb.nNodes; b->depth = hb.depth;
    b->signedVolume = hb.signedVolume;
    b->primIndexHost = hb.primIndex;
    auto upload = [&](void** dst, const void* src, size_t bytes) -> cudaError_t {
        if (bytes == 0) return cudaSuccess;
        cudaError_t e = cudaMalloc(dst, bytes);
        if (e != cudaSuccess) return e;
        return cudaMemcpy(*dst, src, bytes, cudaMemcpyHostToDevice);
    };
    cudaError_t e = upload((void**)&b->nodes, hb.nodes.data(), hb.nodes.size() * sizeof(float4));
    if (e == cudaSuccess) e = upload((void**)&b->cones, hb.cones.data(), hb.cones.size() * sizeof(float4));
    if (e == cudaSuccess) e = upload((void**)&b->prims, hb.prims.data(), hb.prims.size() * sizeof(float4));
    if (e == cudaSuccess) e = upload((void**)&b->sil, hb.sil.data(), hb.sil.size() * sizeof(float4));
    if (e == cudaSuccess) e = upload((void**)&b->primIndex, hb.primIndex.data(), hb.primIndex.size() * sizeof(int));
    if (e == cudaSuccess) e = upload((void**)&b->silTree, hb.silTree.data(), hb.silTree.size() * sizeof(float4));
    if (e == cudaSuccess) e = upload((void**)&b->silCones, hb.silCones.data(), hb.silCones.size() * sizeof(float4));
    if (e == cudaSuccess) e = upload((void**)&b->silFeat, hb.silFeat.data(), hb.silFeat.size() * sizeof(float4));
    if (e != cudaSuccess) {
        zgpu_boundary_destroy(b);
        return fail(e == cudaErrorMemoryAllocation ? ZGPU_ERR_OUT_OF_MEMORY : ZGPU_ERR_CUDA, "boundary upload: %s",
                    cudaGetErrorString(e));
    }
    b->view.nodes = b->nodes; b->view.cones = b->cones; b->view.prims = b->prims; b->view.sil = b->sil; b->view.primIndex = b->primIndex;
    b->view.nNodes = b->nNodes; b->view.nPrims = b->nPrims;
    b->view.stackEntries = std::max(stackEntriesForDepth(b->depth, bvh_width), stackEntriesForDepth(hb.silDepth));
    b->view.width = bvh_width;
    b->view.silTree = b->silTree; b->view.silCones = b->silCones; b->view.silFeat = b->silFeat;
    b->view.silNodes = hb.silNodes;
    b->view.robin = kind == ZGPU_BOUNDARY_ROBIN;
    if (dim == 3 && kind == ZGPU_BOUNDARY_ABSORBING && bvh_width == 4 && n_prims > 0) {
        b->hostPos.assign(positions, positions + (size_t)n_vertices * 3);
        b->hostIdx.assign(indices, indices + (size_t)n_prims * 3);
    }
    *out = b;
    return ZGPU_OK;
}

int zgpu_boundary_create_on_device(zgpu_context* ctx, int dim, const float* positions, int n_vertices,
                                   const int* indices, int n_prims, int kind, const float* min_robin,
                                   const float* max_robin, int solve_double_sided, float silhouette_precision,
                                   int memory, zgpu_boundary** out) {
    if (!ctx || !out) return fail(ZGPU_ERR_INVALID_ARG, "context/out is NULL");
    *out = nullptr;
    if (dim != 2 && dim != 3) return fail(ZGPU_ERR_INVALID_ARG, "dim must be 2 or 3, got %d", dim);
    if (kind < ZGPU_BOUNDARY_ABSORBING || kind > ZGPU_BOUNDARY_ROBIN) return fail(ZGPU_ERR_INVALID_ARG, "unknown boundary kind %d", kind);
    if (n_prims < 0 || n_vertices < 0) return fail(ZGPU_ERR_INVALID_ARG, "negative sizes");
    if (n_prims >= (1 << 27)) return fail(ZGPU_ERR_INVALID_ARG, "too many primitives");
    if (n_prims > 0 && (!positions || !indices)) return fail(ZGPU_ERR_INVALID_ARG, "positions/indices are NULL");
    if (kind == ZGPU_BOUNDARY_ROBIN && n_prims > 0 && (!min_robin || !max_robin))
        return fail(ZGPU_ERR_INVALID_ARG, "Robin boundary needs min/max Robin coefficients per primitive");
    if (memory != ZGPU_MEM_HOST && memory != ZGPU_MEM_DEVICE) return fail(ZGPU_ERR_INVALID_ARG, "unknown memory space");
    ZG_CUDA(cudaSetDevice(ctx->device));
    cudaStream_t s = ctx->stream;
    // host copies: index validation and the signed volume (computeSignedVolume,
    // utils/fcpw_geometric_queries.h:431-458)
    std::vector<float> hp((size_t)n_vertices * dim);
    std::vector<int> hi((size_t)n_prims * dim);
    if (memory == ZGPU_MEM_HOST) {
        std::memcpy(hp.data(), positions, hp.size() * sizeof(float));
        std::memcpy(hi.data(), indices, hi.size() * sizeof(int));
    } else {
        ZG_CUDA(cudaMemcpy(hp.data(), positions, hp.size() * sizeof(float), cudaMemcpyDeviceToHost));
        ZG_CUDA(cudaMemcpy(hi.data(), indices, hi.size() * sizeof(int), cudaMemcpyDeviceToHost));
    }
    for (int v : hi)
        if (v < 0 || v >= n_vertices) return fail(ZGPU_ERR_INVALID_ARG, "index %d outside [0, %d)", v, n_vertices);
    double vol = 0.0;
    for (int i = 0; i < n_prims; i++) {
        const float* a = &hp[(size_t)hi[(size_t)i * dim] * dim];
        const float* b = &hp[(size_t)hi[(size_t)i * dim + 1] * dim];
        if (dim == 2) {
            vol += 0.5 * ((double)a[0] * b[1] - (double)a[1] * b[0]);
        } else {
            const float* c = &hp[(size_t)hi[(size_t)i * dim + 2] * dim];
            vol += (((double)a[1] * b[2] - (double)a[2] * b[1]) * c[0] + ((double)a[2] * b[0] - (double)a[0] * b[2]) * c[1] +
                    ((double)a[0] * b[1] - (double)a[1] * b[0]) * c[2]) / 6.0;
        }
    }
    // inputs on the device
    const bool robin = kind == ZGPU_BOUNDARY_ROBIN;
    const float* dp = positions;
    const int* di = indices;
    const float* dkn = robin ? min_robin : nullptr;
    const float* dkx = robin ? max_robin : nullptr;
    std::vector<void*> staged;
    auto stage = [&](const void* src, size_t bytes, const void** dst) -> cudaError_t {
        void* p = nullptr;
        cudaError_t e = cudaMalloc(&p, bytes ? bytes : 16);
        if (e != cudaSuccess) return e;
        staged.push_back(p);
        *dst = p;
        return cudaMemcpy(p, src, bytes, cudaMemcpyHostToDevice);
    };
    auto freeStaged = [&]() { for (void* p : staged) cudaFree(p); };
    cudaError_t e = cudaSuccess;
    if (memory == ZGPU_MEM_HOST && n_prims > 0) {
        e = stage(hp.data(), hp.size() * sizeof(float), (const void**)&dp);
        if (e == cudaSuccess) e = stage(hi.data(), hi.size() * sizeof(int), (const void**)&di);
        if (e == cudaSuccess && robin) e = stage(min_robin, (size_t)n_prims * sizeof(float), (const void**)&dkn);
        if (e == cudaSuccess && robin) e = stage(max_robin, (size_t)n_prims * sizeof(float), (const void**)&dkx);
        if (e != cudaSuccess) { freeStaged(); return fail(ZGPU_ERR_OUT_OF_MEMORY, "staging: %s", cudaGetErrorString(e)); }
    }
    DeviceBuilt db;
    e = buildBoundaryOnDevice(dim, dp, n_vertices, di, n_prims, kind, dkn, dkx, solve_double_sided != 0,
                              silhouette_precision, s, db);
    freeStaged();
    auto release = [&]() {
        cudaFree(db.nodes); cudaFree(db.cones); cudaFree(db.prims); cudaFree(db.sil); cudaFree(db.primIndex);
        cudaFree(db.silTree); cudaFree(db.silCones); cudaFree(db.silFeat);
    };
    if (e == cudaErrorNotSupported)
        return fail(ZGPU_ERR_UNSUPPORTED, "device-built BVH deeper than the traversal stack (%d levels); build on the host",
                    kMaxWideDepth);
    if (e != cudaSuccess) {
        release();
        return fail(e == cudaErrorMemoryAllocation ? ZGPU_ERR_OUT_OF_MEMORY : ZGPU_ERR_CUDA, "device BVH build: %s",
                    cudaGetErrorString(e));
    }
    zgpu_boundary* b = new zgpu_boundary();
    b->ctx = ctx; b->dim = dim; b->kind = kind; b->nPrims = n_prims; b->nNodes = db.nNodes;
    b->depth = db.depth; b->signedVolume = (float)vol;
    b->nodes = db.nodes; b->cones = db.cones; b->prims = db.prims; b->sil = db.sil; b->primIndex = db.primIndex;
    b->silTree = db.silTree; b->silCones = db.silCones; b->silFeat = db.silFeat;
    if (robin && n_prims > 0) {
        // leaf slot -> caller index, for coefficient updates
        b->primIndexHost.resize(n_prims);
        if (cudaMemcpy(b->primIndexHost.data(), db.primIndex, sizeof(int) * n_prims, cudaMemcpyDeviceToHost) != cudaSuccess) {
            zgpu_boundary_destroy(b);
            return fail(ZGPU_ERR_CUDA, "device BVH build: reading the primitive order");
        }
    }
    b->view.nodes = b->nodes; b->view.cones = b->cones; b->view.prims = b->prims; b->view.sil = b->sil;
    b->view.primIndex = b->primIndex;
    b->view.nNodes = b->nNodes; b->view.nPrims = n_prims;
    b->view.stackEntries = stackEntriesForDepth(std::max(std::max(db.depth, db.silDepth), 1));
    b->view.silTree = b->silTree; b->view.silCones = b->silCones; b->view.silFeat = b->silFeat;
    b->view.silNodes = db.silNodes;
    b->view.robin = robin;
    *out = b;
    return ZGPU_OK;
}

int zgpu_boundary_destroy(zgpu_boundary* b) {
    if (!b) return ZGPU_OK;
    if (b->ctx) cudaSetDevice(b->ctx->device);
    if (b->twin8) zgpu_boundary_destroy(b->twin8);
    cudaFree(b->silTree); cudaFree(b->silCones); cudaFree(b->silFeat);
    cudaFree(b->nodes); cudaFree(b->cones); cudaFree(b->prims); cudaFree(b->sil); cudaFree(b->primIndex);
    delete b;
    return ZGPU_OK;
}

int zgpu_boundary_update_robin_coefficients(zgpu_boundary* b, const float* min_robin, const float* max_robin) {
    if (!b || !min_robin || !max_robin) return fail(ZGPU_ERR_INVALID_ARG, "NULL argument");
    if (b->kind != ZGPU_BOUNDARY_ROBIN) return fail(ZGPU_ERR_INVALID_ARG, "not a Robin boundary");
    if (b->nPrims == 0) return ZGPU_OK;
    int per = b->dim == 2 ? 2 : 3;
    std::vector<float4> sil((size_t)b->nPrims * per);
    ZG_CUDA(cudaMemcpy(sil.data(), b->sil, sil.size() * sizeof(float4), cudaMemcpyDeviceToHost));
    for (int s = 0; s < b->nPrims; s++) {
        int i = b->primIndexHost[s];
        if (b->dim == 2) { sil[(size_t)s * 2 + 1].y = min_robin[i]; sil[(size_t)s * 2 + 1].z = max_robin[i]; }
        else { sil[(size_t)s * 3 + 1].w = min_robin[i]; sil[(size_t)s * 3 + 2].w = max_robin[i]; }
    }
    ZG_CUDA(cudaMemcpy(b->sil, sil.data(), sil.size() * sizeof(float4), cudaMemcpyHostToDevice));
    // refit the per-child coefficient ranges of the wide nodes (rows 4 and 5 of each node's
    // cone block), as updateCoefficientValues refits its nodes (reflectance_boundary_bvh/bvh.h:345-367)
    std::vector<float4> nodes((size_t)b->nNodes * 8), cones((size_t)b->nNodes * 8);
    ZG_CUDA(cudaMemcpy(nodes.data(), b->nodes, nodes.size() * sizeof(float4), cudaMemcpyDeviceToHost));
    ZG_CUDA(cudaMemcpy(cones.data(), b->cones, cones.size() * sizeof(float4), cudaMemcpyDeviceToHost));
    const int D = b->dim;
    auto range = [&](auto&& self, int c, float& lo, float& hi) -> void {
        lo = FLT_MAX; hi = 0.0f;
        if (c == kEmptyChild) return;
        if (isLeaf(c)) {
            for (int j = 0; j < leafCount(c); j++) {
                int i = b->primIndexHost[leafFirst(c) + j];
                lo = std::min(lo, min_robin[i]);
                hi = std::max(hi, max_robin[i]);
            }
            return;
        }
        int4 kids;
        std::memcpy(&kids, &nodes[(size_t)c * 8 + 2 * D], sizeof(int4));
        const int k4[4] = {kids.x, kids.y, kids.z, kids.w};
        float l4[4], h4[4];
        for (int k = 0; k < 4; k++) {
            self(self, k4[k], l4[k], h4[k]);
            lo = std::min(lo, l4[k]);
            hi = std::max(hi, h4[k]);
        }
        cones[(size_t)c * 8 + 4] = make_float4(h4[0], h4[1], h4[2], h4[3]);
        cones[(size_t)c * 8 + 5] = make_float4(l4[0], l4[1], l4[2], l4[3]);
    };
    float lo, hi;
    range(range, 0, lo, hi);
    ZG_CUDA(cudaMemcpy(b->cones, cones.data(), cones.size() * sizeof(float4), cudaMemcpyHostToDevice));
    return ZGPU_OK;
}

int zgpu_boundary_info(zgpu_boundary* b, int64_t* n_nodes, int32_t* depth, int64_t* node_bytes, int64_t* prim_bytes) {
    if (!b) return fail(ZGPU_ERR_INVALID_ARG, "boundary is NULL");
    if (n_nodes) *n_nodes = b->nNodes;
    if (depth) *depth = b->depth;
    if (node_bytes) *node_bytes = (int64_t)b->nNodes * 32 * b->view.width;
    if (prim_bytes) *prim_bytes = (int64_t)b->nPrims * (b->dim == 2 ? 16 : 48);
    return ZGPU_OK;
}

int zgpu_boundary_signed_volume(zgpu_boundary* b, float* out) {
    if (!b || !out) return fail(ZGPU_ERR_INVALID_ARG, "NULL argument");
    *out = b->signedVolume;
    return ZGPU_OK;
}

// ------------------------------------------------------------------ batched queries
#define ZG_QUERY_PROLOGUE()                                                             \
    if (!b) return fail(ZGPU_ERR_INVALID_ARG, "boundary is NULL");                       \
    if (n < 0) return fail(ZGPU_ERR_INVALID_ARG, "negative query count");               \
    if (memory != ZGPU_MEM_HOST && memory != ZGPU_MEM_DEVICE)                          \
        return fail(ZGPU_ERR_INVALID_ARG, "unknown memory space %d", memory);           \
    zgpu_context* ctx = b->ctx;                                                         \
    ZG_CUDA(cudaSetDevice(ctx->device));                                                \
    const int D = b->dim;                                                               \
    unsigned int* errw = nullptr;                                                       \
    ZG_TRY(scratch<unsigned int>(ctx, zgpu_context::kCounters, 16, &errw));             \
    ZG_CUDA(cudaMemsetAsync(errw, 0, sizeof(unsigned int), ctx->stream));

static int queryEpilogue(zgpu_context* ctx, unsigned int* errw) {
    ZG_CUDA(cudaMemcpyAsync(ctx->hostCounters, errw, sizeof(unsigned int), cudaMemcpyDeviceToHost, ctx->stream));
    ZG_CUDA(cudaStreamSynchronize(ctx->stream));
    unsigned int e = *(unsigned int*)ctx->hostCounters;
    if (e) return fail(ZGPU_ERR_DEVICE_STATE, "device error word 0x%x (traversal stack overflow)", e);
    return ZGPU_OK;
}

int zgpu_boundary_set_query_mode(zgpu_boundary* b, int mode) {
    if (!b) return fail(ZGPU_ERR_INVALID_ARG, "boundary is NULL");
    if (mode != ZGPU_QUERY_MODE_AUTO && mode != ZGPU_QUERY_MODE_LANE && mode != ZGPU_QUERY_MODE_WARP)
        return fail(ZGPU_ERR_INVALID_ARG, "unknown query mode %d", mode);
    b->queryMode = mode;
    return ZGPU_OK;
}

int zgpu_query_closest_point(zgpu_boundary* b, int64_t n, const float* x, int compute_signed, float* out_pt,
                             float* out_normal, float* out_dist, int32_t* out_prim, int memory) {
    ZG_QUERY_PROLOGUE();
    if (n == 0) return ZGPU_OK;
    if (!x) return fail(ZGPU_ERR_INVALID_ARG, "x is NULL");
    const float* dx; float *dpt, *dn, *dd; int* dp;
    ZG_TRY(stageIn<float>(ctx, zgpu_context::kQ0, x, (size_t)n * D, memory, &dx));
    if (memory == ZGPU_MEM_DEVICE) { dpt = out_pt; dn = out_normal; dd = out_dist; dp = out_prim; }
    else {
        ZG_TRY(scratch<float>(ctx, zgpu_context::kQ1, (size_t)n * D, &dpt));
        ZG_TRY(scratch<float>(ctx, zgpu_context::kQ2, (size_t)n * D, &dn));
        ZG_TRY(scratch<float>(ctx, zgpu_context::kQ3, (size_t)n, &dd));
        ZG_TRY(scratch<int>(ctx, zgpu_context::kQ4, (size_t)n, &dp));
    }
    if (b->queryMode == ZGPU_QUERY_MODE_WARP)
        ZG_CUDA(launchClosestCoop(b->view, D, n, dx, compute_signed, dpt, dn, dd, dp, errw, ctx->stream));
    else
        ZG_CUDA(launchClosest(b->view, D, n, dx, compute_signed, dpt, dn, dd, dp, errw, ctx->stream));
    ZG_TRY(stageOut<float>(ctx, dpt, out_pt, (size_t)n * D, memory));
    ZG_TRY(stageOut<float>(ctx, dn, out_normal, (size_t)n * D, memory));
    ZG_TRY(stageOut<float>(ctx, dd, out_dist, (size_t)n, memory));
    ZG_TRY(stageOut<int>(ctx, dp, out_prim, (size_t)n, memory));
    return queryEpilogue(ctx, errw);
}

int zgpu_query_intersect(zgpu_boundary* b, int64_t n, const float* origin, const float* normal, const float* dir,
                         const float* t_max, const int32_t* on_boundary, int32_t* out_hit, float* out_pt,
                         float* out_normal, float* out_dist, int32_t* out_prim, int memory) {
    ZG_QUERY_PROLOGUE();
    if (n == 0) return ZGPU_OK;
    if (!origin || !dir || !t_max || !out_hit) return fail(ZGPU_ERR_INVALID_ARG, "NULL required argument");
    if (on_boundary && !normal) return fail(ZGPU_ERR_INVALID_ARG, "on_boundary needs normals");
    const float *dO, *dN, *dD, *dT; const int* dOnb;
    ZG_TRY(stageIn<float>(ctx, zgpu_context::kQ0, origin, (size_t)n * D, memory, &dO));
    ZG_TRY(stageIn<float>(ctx, zgpu_context::kQ1, normal, (size_t)n * D, memory, &dN));
    ZG_TRY(stageIn<float>(ctx, zgpu_context::kQ2, dir, (size_t)n * D, memory, &dD));
    ZG_TRY(stageIn<float>(ctx, zgpu_context::kQ3, t_max, (size_t)n, memory, &dT));
    ZG_TRY(stageIn<int>(ctx, zgpu_context::kQ4, on_boundary, (size_t)n, memory, &dOnb));
    int *dHit, *dPrim; float *dPt, *dNr, *dDist;
    if (memory == ZGPU_MEM_DEVICE) { dHit = out_hit; dPt = out_pt; dNr = out_normal; dDist = out_dist; dPrim = out_prim; }
    else {
        ZG_TRY(scratch<int>(ctx, zgpu_context::kQ5, (size_t)n, &dHit));
        ZG_TRY(scratch<float>(ctx, zgpu_context::kQ6, (size_t)n * D, &dPt));
        ZG_TRY(scratch<float>(ctx, zgpu_context::kQ7, (size_t)n * D, &dNr));
        ZG_TRY(scratch<float>(ctx, zgpu_context::kQ8, (size_t)n, &dDist));
        ZG_TRY(scratch<int>(ctx, zgpu_context::kQ9, (size_t)n, &dPrim));
    }
    ZG_CUDA(launchIntersect(b->view, D, n, dO, dN, dD, dT, dOnb, dHit, dPt, dNr, dDist, dPrim, errw, ctx->stream));
    ZG_TRY(stageOut<int>(ctx, dHit, out_hit, (size_t)n, memory));
    ZG_TRY(stageOut<float>(ctx, dPt, out_pt, (size_t)n * D, memory));
    ZG_TRY(stageOut<float>(ctx, dNr, out_normal, (size_t)n * D, memory));
    ZG_TRY(stageOut<float>(ctx, dDist, out_dist, (size_t)n, memory));
    ZG_TRY(stageOut<int>(ctx, dPrim, out_prim, (size_t)n, memory));
    return queryEpilogue(ctx, errw);
}

int zgpu_query_count_hits(zgpu_boundary* b, int64_t n, const float* origin, const float* dir, const float* t_max,
                          int32_t* out_count, int memory) {
    ZG_QUERY_PROLOGUE();
    if (n == 0) return ZGPU_OK;
    if (!origin || !dir || !t_max || !out_count) return fail(ZGPU_ERR_INVALID_ARG, "NULL required argument");
    const float *dO, *dD, *dT; int* dOut;
    ZG_TRY(stageIn<float>(ctx, zgpu_context::kQ0, origin, (size_t)n * D, memory, &dO));
    ZG_TRY(stageIn<float>(ctx, zgpu_context::kQ1, dir, (size_t)n * D, memory, &dD));
    ZG_TRY(stageIn<float>(ctx, zgpu_context::kQ2, t_max, (size_t)n, memory, &dT));
    if (memory == ZGPU_MEM_DEVICE) dOut = out_count; else ZG_TRY(scratch<int>(ctx, zgpu_context::kQ3, (size_t)n, &dOut));
    ZG_CUDA(launchCountHits(b->view, D, n, dO, dD, dT, dOut, errw, ctx->stream));
    ZG_TRY(stageOut<int>(ctx, dOut, out_count, (size_t)n, memory));
    return queryEpilogue(ctx, errw);
}

int zgpu_query_star_radius(zgpu_boundary* b, int64_t n, const float* x, const float* min_radius,
                           const float* max_radius, float silhouette_precision, const int32_t* flip,
                           float* out_radius, int memory) {
    ZG_QUERY_PROLOGUE();
    if (n == 0) return ZGPU_OK;
    if (!x || !min_radius || !max_radius || !out_radius) return fail(ZGPU_ERR_INVALID_ARG, "NULL required argument");
    if (b->kind == ZGPU_BOUNDARY_ABSORBING) return fail(ZGPU_ERR_INVALID_ARG, "star radius needs a reflecting boundary");
    const float *dx, *dmin, *dmax; const int* dflip; float* dout;
    ZG_TRY(stageIn<float>(ctx, zgpu_context::kQ0, x, (size_t)n * D, memory, &dx));
    ZG_TRY(stageIn<float>(ctx, zgpu_context::kQ1, min_radius, (size_t)n, memory, &dmin));
    ZG_TRY(stageIn<float>(ctx, zgpu_context::kQ2, max_radius, (size_t)n, memory, &dmax));
    ZG_TRY(stageIn<int>(ctx, zgpu_context::kQ3, flip, (size_t)n, memory, &dflip));
    if (memory == ZGPU_MEM_DEVICE) dout = out_radius; else ZG_TRY(scratch<float>(ctx, zgpu_context::kQ4, (size_t)n, &dout));
    if (b->queryMode == ZGPU_QUERY_MODE_WARP && b->kind == ZGPU_BOUNDARY_ROBIN)
        ZG_CUDA(launchStarRadiusCoop(b->view, D, n, dx, dmin, dmax, silhouette_precision, dflip, dout, errw, ctx->stream));
    else
        ZG_CUDA(launchStarRadius(b->view, D, n, dx, dmin, dmax, silhouette_precision, dflip, dout, errw, ctx->stream));
    ZG_TRY(stageOut<float>(ctx, dout, out_radius, (size_t)n, memory));
    return queryEpilogue(ctx, errw);
}

int zgpu_query_occluded(zgpu_boundary* b, int64_t n, const float* xi, const float* xj, const float* ni,
                        const float* nj, const int32_t* offset_i, const int32_t* offset_j, int32_t* out_occluded,
                        int memory) {
    ZG_QUERY_PROLOGUE();
    if (n == 0) return ZGPU_OK;
    if (!xi || !xj || !out_occluded) return fail(ZGPU_ERR_INVALID_ARG, "NULL required argument");
    if ((offset_i && !ni) || (offset_j && !nj)) return fail(ZGPU_ERR_INVALID_ARG, "offsets need normals");
    const float *dxi, *dxj, *dni, *dnj; const int *doi, *doj; int* dout;
    ZG_TRY(stageIn<float>(ctx, zgpu_context::kQ0, xi, (size_t)n * D, memory, &dxi));
    ZG_TRY(stageIn<float>(ctx, zgpu_context::kQ1, xj, (size_t)n * D, memory, &dxj));
    ZG_TRY(stageIn<float>(ctx, zgpu_context::kQ2, ni, (size_t)n * D, memory, &dni));
    ZG_TRY(stageIn<float>(ctx, zgpu_context::kQ3, nj, (size_t)n * D, memory, &dnj));
    ZG_TRY(stageIn<int>(ctx, zgpu_context::kQ4, offset_i, (size_t)n, memory, &doi));
    ZG_TRY(stageIn<int>(ctx, zgpu_context::kQ5, offset_j, (size_t)n, memory, &doj));
    if (memory == ZGPU_MEM_DEVICE) dout = out_occluded; else ZG_TRY(scratch<int>(ctx, zgpu_context::kQ6, (size_t)n, &dout));
    ZG_CUDA(launchOccluded(b->view, D, n, dxi, dxj, dni, dnj, doi, doj, dout, errw, ctx->stream));
    ZG_TRY(stageOut<int>(ctx, dout, out_occluded, (size_t)n, memory));
    return queryEpilogue(ctx, errw);
}

int zgpu_query_sample_boundary(zgpu_boundary* b, int64_t n, const float* x, const float* radius,
                               const float* rand_nums, int32_t* out_found, float* out_pt, float* out_normal,
                               float* out_pdf, int memory) {
    ZG_QUERY_PROLOGUE();
    if (n == 0) return ZGPU_OK;
    if (!x || !radius || !rand_nums || !out_found || !out_pt || !out_normal || !out_pdf)
        return fail(ZGPU_ERR_INVALID_ARG, "NULL required argument");
    if (b->view.width != 4) return fail(ZGPU_ERR_UNSUPPORTED, "boundary sampling needs a 4-wide tree");
    const float *dx, *dr, *du; int* dfound; float *dpt, *dn, *dpdf;
    ZG_TRY(stageIn<float>(ctx, zgpu_context::kQ0, x, (size_t)n * D, memory, &dx));
    ZG_TRY(stageIn<float>(ctx, zgpu_context::kQ1, radius, (size_t)n, memory, &dr));
    ZG_TRY(stageIn<float>(ctx, zgpu_context::kQ2, rand_nums, (size_t)n * D, memory, &du));
    if (memory == ZGPU_MEM_DEVICE) { dfound = out_found; dpt = out_pt; dn = out_normal; dpdf = out_pdf; }
    else {
        ZG_TRY(scratch<int>(ctx, zgpu_context::kQ3, (size_t)n, &dfound));
        ZG_TRY(scratch<float>(ctx, zgpu_context::kQ4, (size_t)n * D, &dpt));
        ZG_TRY(scratch<float>(ctx, zgpu_context::kQ5, (size_t)n * D, &dn));
        ZG_TRY(scratch<float>(ctx, zgpu_context::kQ6, (size_t)n, &dpdf));
    }
    ZG_CUDA(launchSample(b->view, D, n, dx, dr, du, dfound, dpt, dn, dpdf, ctx->stream));
    ZG_TRY(stageOut<int>(ctx, dfound, out_found, (size_t)n, memory));
    ZG_TRY(stageOut<float>(ctx, dpt, out_pt, (size_t)n * D, memory));
    ZG_TRY(stageOut<float>(ctx, dn, out_normal, (size_t)n * D, memory));
    ZG_TRY(stageOut<float>(ctx, dpdf, out_pdf, (size_t)n, memory));
    return queryEpilogue(ctx, errw);
}

// -------------------------------------------------------------------------- solve
}  // extern "C"

namespace {

// zgpu_solve and zgpu_solve_cached: cache == NULL runs the plain walk
// checks one scene (queries, PDE, settings) of a solve
int checkScene(const zgpu_geometric_queries* q, const zgpu_pde* pde, const zgpu_walk_settings* ws, int D) {
    if (q->dim != D) return fail(ZGPU_ERR_INVALID_ARG, "queries dim must be %d, got %d", D, q->dim);
    ZG_TRY(checkBoundary(q->absorbing, D, "absorbing"));
    ZG_TRY(checkBoundary(q->reflecting, D, "reflecting"));
    if (q->reflecting && q->reflecting->kind == ZGPU_BOUNDARY_ABSORBING)
        return fail(ZGPU_ERR_INVALID_ARG, "reflecting slot holds an absorbing boundary");
    if (q->absorbing && q->absorbing->kind != ZGPU_BOUNDARY_ABSORBING)
        return fail(ZGPU_ERR_INVALID_ARG, "absorbing slot holds a reflecting boundary");
    if (ws->max_walk_length <= 0) return fail(ZGPU_ERR_INVALID_ARG, "max_walk_length must be positive");
    if (!(ws->epsilon_shell_for_absorbing_boundary >= 0.0f)) return fail(ZGPU_ERR_INVALID_ARG, "epsilon shell must be >= 0");
    if (!(ws->splitting_threshold > 0.0f)) return fail(ZGPU_ERR_INVALID_ARG, "splitting threshold must be > 0");
    if (!(pde->absorption_coeff >= 0.0f)) return fail(ZGPU_ERR_INVALID_ARG, "absorption coefficient must be >= 0");
    ZG_TRY(zg::checkPdeFields(pde, D, true));
    if (pde->solution.n_terms < 0 || pde->solution.n_terms > ZGPU_MAX_TERMS)
        return fail(ZGPU_ERR_INVALID_ARG, "analytic solution has %d terms (max %d)", pde->solution.n_terms, ZGPU_MAX_TERMS);
    return ZGPU_OK;
}

namespace {
// Grids given in host memory are copied into device buffers of the context (four fields x
// two orientations per scene) and the descriptor is pointed at the copies.
int stageGrids(zgpu_context* ctx, zgpu_pde& pde, int D, int scene) {
    if (pde.memory != ZGPU_MEM_HOST) return ZGPU_OK;
    const int kinds[4] = {pde.source_kind, pde.dirichlet_kind, pde.robin_kind, pde.robin_coeff_kind};
    zgpu_grid* grids[4] = {&pde.source_grid, &pde.dirichlet_grid, &pde.robin_grid, &pde.robin_coeff_grid};
    for (int f = 0; f < 4; f++) {
        if (kinds[f] != ZGPU_FIELD_GRID) continue;
        const size_t bytes = (size_t)gridCells(*grids[f], D) * sizeof(float);
        const float** src[2] = {&grids[f]->values, &grids[f]->values_aligned};
        for (int a = 0; a < 2; a++) {
            if (!*src[a]) continue;
            const size_t slot = ((size_t)scene * 4 + f) * 2 + a;
            if (ctx->gridBufs.size() <= slot) ctx->gridBufs.resize(slot + 1);
            ZG_CUDA(ensure(ctx->gridBufs[slot], bytes));
            ZG_CUDA(cudaMemcpyAsync(ctx->gridBufs[slot].p, *src[a], bytes, cudaMemcpyHostToDevice, ctx->stream));
            *src[a] = (const float*)ctx->gridBufs[slot].p;
        }
    }
    pde.memory = ZGPU_MEM_DEVICE;
    return ZGPU_OK;
}
}  // namespace

SceneDesc sceneOf(const zgpu_geometric_queries* q, const zgpu_pde* pde, const zgpu_walk_settings* ws) {
    SceneDesc d;
    std::memset(&d, 0, sizeof(d));
    d.hasAbs = q->absorbing && q->absorbing->nPrims > 0;
    d.hasRefl = q->reflecting && q->reflecting->nPrims > 0;
    if (d.hasAbs) d.absorbing = q->absorbing->view;
    if (d.hasRefl) d.reflecting = q->reflecting->view;
    for (int i = 0; i < 3; i++) { d.domainMin[i] = q->domain_min[i]; d.domainMax[i] = q->domain_max[i]; }
    d.ws = *ws;
    d.pde = *pde;
    return d;
}

// The 8-wide twin of a 3D absorbing boundary (the boundary itself if it is 8-wide), built
// from the boundary's host copy of its mesh on first use.
int wideTwin(zgpu_boundary* b, zgpu_boundary** out) {
    if (b->view.width == 8) { *out = b; return ZGPU_OK; }
    if (!b->twin8) {
        if (b->hostIdx.empty())
            return fail(ZGPU_ERR_UNSUPPORTED, "bvh_width 8 needs a 3D absorbing boundary built on the host");
        zgpu_boundary* t = nullptr;
        ZG_TRY(zgpu_boundary_create(b->ctx, 3, b->hostPos.data(), (int)(b->hostPos.size() / 3), b->hostIdx.data(),
                                    (int)(b->hostIdx.size() / 3), ZGPU_BOUNDARY_ABSORBING, nullptr, nullptr, 0, 0.0f, 8,
                                    &t));
        t->queryMode = b->queryMode;
        b->twin8 = t;
    }
    *out = b->twin8;
    return ZGPU_OK;
}

// zgpu_solve, zgpu_solve_cached and zgpu_solve_batched.  nScenes > 1: points->scene_id
// selects each point's row of q / pde / ws.
// The sorted-wavefront walk loop (zgpu_wave.cuh): iterations of sort, refill and the step
// kernels over a pool of walk records until no walk is left.  The host reads the
// live count every kWaveCheck iterations (the iterations between run on an empty pool).
#ifndef ZG_WAVE_POOL_LOG2
#define ZG_WAVE_POOL_LOG2 23
#endif
constexpr long long kWavePool = 1LL << ZG_WAVE_POOL_LOG2;
constexpr int kWaveCheck = 8;
#ifndef ZG_WAVE_DRAIN_FACTOR
#define ZG_WAVE_DRAIN_FACTOR 1
#endif

int runWave(zgpu_context* ctx, const SolveParams& P0, int D, cudaStream_t s, bool useGraph, long long* launches) {
    using C = zgpu_context;
    SolveParams P = P0;
    P.splitStack = nullptr;   // no split scratch: a split reports kErrSplitOverflow
    long long total = 0;
    ZG_CUDA(cudaMemcpyAsync(&total, P.walkStart + P.nPoints, sizeof(long long), cudaMemcpyDeviceToHost, s));
    ZG_CUDA(cudaStreamSynchronize(s));
    if (total <= 0) return ZGPU_OK;
    const long long pool = std::min(total, kWavePool);
    const int vec = waveRecordVec(D);
    WaveParams w;
    float4 *a = nullptr, *b = nullptr;
    ZG_TRY(scratch<float4>(ctx, C::kWaveA, (size_t)pool * vec, &a));
    ZG_TRY(scratch<float4>(ctx, C::kWaveB, (size_t)pool * vec, &b));
    ZG_TRY(scratch<uint32_t>(ctx, C::kWaveKey, (size_t)pool, &w.key));
    ZG_TRY(scratch<uint32_t>(ctx, C::kWaveRank, (size_t)pool, &w.rank));
    ZG_TRY(scratch<uint32_t>(ctx, C::kWaveCount, (size_t)kWaveCells, &w.count));
    ZG_TRY(scratch<uint32_t>(ctx, C::kWaveOffset, (size_t)kWaveCells + 1, &w.offset));
    ZG_TRY(scratch<long long>(ctx, C::kWaveCtr, kWaveCtrs, &w.ctr));
    ZG_CUDA(cudaMemsetAsync(w.count, 0, kWaveCells * sizeof(uint32_t), s));
    ZG_CUDA(cudaMemsetAsync(w.ctr, 0, kWaveCtrs * sizeof(long long), s));
    w.pool = pool;
    const bool batched = P.sceneId != nullptr;
    const bool screened = batched ? P.batchScreened != 0 : P.sc.pde.absorption_coeff > 0.0f;
    const int blocks = ctx->numSMs * waveBlocksPerSM(D, P.solver, screened, batched);
    // the sort's cells: one Morton grid over the domain box; a batched solve puts the scene id
    // above a coarser grid over each scene's own box, within the same 2^16 cells
    w.axisBits = D == 2 ? kWaveBits2D : kWaveBits3D;
    w.sceneMask = 0u;
    if (batched) {
        int sceneBits = 0;
        while (sceneBits < 16 && (1LL << sceneBits) < (long long)P.nScenes) sceneBits++;
        w.axisBits = std::min(w.axisBits, (16 - sceneBits) / D);
        w.sceneMask = (uint32_t)((1u << sceneBits) - 1u);
    }
    // a slot holds one walk for at most max_walk_length + 1 iterations, so every walk has
    // started after ceil(total / pool) such periods and ended one period later
    const double periods = (double)((total + pool - 1) / pool + 1);
    const double maxIter = periods * ((double)P.sc.ws.max_walk_length + 1.0) + 2.0 * kWaveCheck;
    // the tail: once every walk has started and at most this many records are live (one per
    // resident thread of the step kernels), the drain kernel runs them to their ends
    const long long drainAt = (long long)blocks * 128 * ZG_WAVE_DRAIN_FACTOR;
    // a chunk of kWaveCheck iterations (an even number: the buffers are where they started
    // after it), launched one by one or replayed from its captured graph
    auto chunk = [&]() -> cudaError_t {
        float4* cs = a;
        float4* cd = b;
        for (int k = 0; k < kWaveCheck; k++) {
            w.src = cs;
            w.dst = cd;
            cudaError_t e = launchWaveIteration(P, w, D, blocks, ctx->numSMs, s);
            if (e != cudaSuccess) return e;
            std::swap(cs, cd);
        }
        return cudaSuccess;
    };
    if (useGraph) {
        std::vector<unsigned char> key(sizeof(SolveParams) + sizeof(WaveParams) + 2 * sizeof(int));
        WaveParams wk = w;
        wk.src = a;
        wk.dst = b;
        const int dims[2] = {D, blocks};
        std::memcpy(key.data(), &P, sizeof(P));
        std::memcpy(key.data() + sizeof(P), &wk, sizeof(wk));
        std::memcpy(key.data() + sizeof(P) + sizeof(wk), dims, sizeof(dims));
        if (!ctx->waveGraphExec || ctx->waveGraphKey != key) {
            if (ctx->waveGraphExec) { cudaGraphExecDestroy(ctx->waveGraphExec); ctx->waveGraphExec = nullptr; }
            cudaGraph_t g = nullptr;
            ZG_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeRelaxed));
            cudaError_t e = chunk();
            cudaError_t e2 = cudaStreamEndCapture(s, &g);
            if (e == cudaSuccess) e = e2;
            if (e == cudaSuccess) e = cudaGraphInstantiate(&ctx->waveGraphExec, g, 0);
            if (g) cudaGraphDestroy(g);
            ZG_CUDA(e);
            ctx->waveGraphKey = key;
        }
    }
    static_assert(kWaveCheck % 2 == 0, "a chunk leaves the records in the buffer it started from");
    *launches = 0;
    for (long long it = 0;;) {
        if (useGraph) ZG_CUDA(cudaGraphLaunch(ctx->waveGraphExec, s));
        else ZG_CUDA(chunk());
        it += kWaveCheck;
        *launches += (long long)kWaveCheck * waveLaunchesPerIteration(P.solver);
        long long c[kWaveCtrs];
        ZG_CUDA(cudaMemcpyAsync(c, w.ctr, sizeof(c), cudaMemcpyDeviceToHost, s));
        ZG_CUDA(cudaStreamSynchronize(s));
        const long long live = c[kWaveLive];
        if (live == 0) break;
        if (c[kWaveNext] >= total && live <= drainAt) {
            w.dst = a;   // the records the last iteration left (a chunk ends where it began)
            ZG_CUDA(launchWaveDrain(P, w, D, blocks, s));
            *launches += 1;
            break;
        }
        if ((double)it > maxIter)
            return fail(ZGPU_ERR_DEVICE_STATE, "the wavefront schedule still had %lld live walks after %lld iterations",
                        live, it);
    }
    return ZGPU_OK;
}

int solveImpl(zgpu_context* ctx, int solver, int nScenes, const zgpu_geometric_queries* q, const zgpu_pde* pde,
              const zgpu_walk_settings* ws, const zgpu_sample_points* pts, zgpu_sample_statistics* stats,
              const zgpu_solve_options* opt, zgpu_cache* cache, float cacheMinDist, zgpu_solve_report* report) {
    if (!ctx || !q || !pde || !ws || !pts || !stats) return fail(ZGPU_ERR_INVALID_ARG, "NULL required argument");
    if (solver != ZGPU_SOLVER_WALK_ON_SPHERES && solver != ZGPU_SOLVER_WALK_ON_STARS)
        return fail(ZGPU_ERR_INVALID_ARG, "unknown solver %d", solver);
    const int D = q->dim;
    if (D != 2 && D != 3) return fail(ZGPU_ERR_INVALID_ARG, "queries dim must be 2 or 3, got %d", D);
    if (nScenes < 1) return fail(ZGPU_ERR_INVALID_ARG, "n_scenes must be >= 1");
    const bool batched = nScenes > 1 || (pts->scene_id != nullptr);
    if (batched && cache) return fail(ZGPU_ERR_UNSUPPORTED, "the neural cache serves single-scene solves");
    if (batched && pts->n > 0 && !pts->scene_id) return fail(ZGPU_ERR_INVALID_ARG, "scene_id is required with n_scenes > 1");
    for (int k = 0; k < nScenes; k++) ZG_TRY(checkScene(q + k, pde + k, ws + k, D));
    if (pts->n < 0) return fail(ZGPU_ERR_INVALID_ARG, "negative point count");
    if (pts->memory != stats->memory) return fail(ZGPU_ERR_INVALID_ARG, "points and statistics must share a memory space");
    if (pts->memory != ZGPU_MEM_HOST && pts->memory != ZGPU_MEM_DEVICE) return fail(ZGPU_ERR_INVALID_ARG, "unknown memory space");
    if (pts->n > 0 && (!pts->pt || !pts->dist_to_absorbing || !pts->n_walks || !pts->seed))
        return fail(ZGPU_ERR_INVALID_ARG, "pt, dist_to_absorbing, n_walks and seed are required");
    if (!stats->solution_mean || !stats->solution_m2 || !stats->n_solution_estimates || !stats->total_walk_length ||
        !stats->total_splits)
        return fail(ZGPU_ERR_INVALID_ARG, "statistics arrays are required");
    zgpu_geometric_queries qWide;
    if (opt && opt->bvh_width != 0 && opt->bvh_width != 4) {
        if (opt->bvh_width != 8) return fail(ZGPU_ERR_INVALID_ARG, "bvh_width must be 0, 4 or 8");
        if (batched) return fail(ZGPU_ERR_UNSUPPORTED, "bvh_width 8 serves single-scene solves");
        if (q->absorbing && q->absorbing->nPrims > 0) {
            qWide = *q;
            ZG_TRY(wideTwin(q->absorbing, &qWide.absorbing));
            q = &qWide;
        }
    }

    ZG_CUDA(cudaSetDevice(ctx->device));
    const int64_t n = pts->n;
    const int mem = pts->memory;
    cudaStream_t s = ctx->stream;
    SolveParams P;
    std::memset(&P, 0, sizeof(P));
    P.solver = solver;
    P.sc = sceneOf(q, pde, ws);
    ZG_TRY(stageGrids(ctx, P.sc.pde, D, 0));
    P.nPoints = n;
    using C = zgpu_context;
    int sceneStack = 8;
    if (batched) {
        // the scene table and each point's row in it
        std::vector<SceneDesc> table(nScenes);
        for (int k = 0; k < nScenes; k++) {
            table[k] = sceneOf(q + k, pde + k, ws + k);
            ZG_TRY(stageGrids(ctx, table[k].pde, D, k));
            if (table[k].hasAbs) sceneStack = std::max(sceneStack, table[k].absorbing.stackEntries);
            if (table[k].hasRefl) sceneStack = std::max(sceneStack, table[k].reflecting.stackEntries);
            P.batchScreened |= pde[k].absorption_coeff > 0.0f;
        }
        SceneDesc* dTable = nullptr;
        ZG_TRY(scratch<SceneDesc>(ctx, C::kSceneTable, (size_t)nScenes, &dTable));
        ZG_CUDA(cudaMemcpyAsync(dTable, table.data(), sizeof(SceneDesc) * nScenes, cudaMemcpyHostToDevice, s));
        P.scenes = dTable;
        P.nScenes = nScenes;
        ZG_TRY(stageIn<int>(ctx, C::kSceneId, pts->scene_id, (size_t)n, mem, &P.sceneId));
    }
    ZG_TRY(stageIn<float>(ctx, C::kPt, pts->pt, (size_t)n * D, mem, &P.pt));
    ZG_TRY(stageIn<float>(ctx, C::kNormal, pts->normal, (size_t)n * D, mem, &P.normal));
    ZG_TRY(stageIn<int>(ctx, C::kType, pts->type, (size_t)n, mem, &P.type));
    ZG_TRY(stageIn<int>(ctx, C::kEq, pts->estimation_quantity, (size_t)n, mem, &P.eq));
    ZG_TRY(stageIn<float>(ctx, C::kDist, pts->dist_to_absorbing, (size_t)n, mem, &P.distAbs));
    ZG_TRY(stageIn<int>(ctx, C::kNWalks, pts->n_walks, (size_t)n, mem, &P.nWalks));
    ZG_TRY(stageIn<uint64_t>(ctx, C::kSeed, pts->seed, (size_t)n, mem, &P.seed));
    ZG_TRY(stageIn<int>(ctx, C::kAligned, pts->estimate_normal_aligned, (size_t)n, mem, &P.aligned));
    if (pts->first_sphere_radius) {
        ZG_TRY(stageInOut<float>(ctx, C::kFsr, pts->first_sphere_radius, (size_t)n, mem, &P.fsr));
        P.fsrPersistent = 1;
    } else {
        ZG_TRY(scratch<float>(ctx, C::kFsr, (size_t)n, &P.fsr));
        P.fsrPersistent = 0;
    }
    ZG_TRY(stageInOut<double>(ctx, C::kMean, stats->solution_mean, (size_t)n, mem, &P.statMean));
    ZG_TRY(stageInOut<double>(ctx, C::kM2, stats->solution_m2, (size_t)n, mem, &P.statM2));
    ZG_TRY(stageInOut<int>(ctx, C::kN, stats->n_solution_estimates, (size_t)n, mem, &P.statN));
    ZG_TRY(stageInOut<long long>(ctx, C::kLen, (long long*)stats->total_walk_length, (size_t)n, mem, &P.statLen));
    ZG_TRY(stageInOut<long long>(ctx, C::kSplits, (long long*)stats->total_splits, (size_t)n, mem, &P.statSplits));
    // estimateSolutionAndGradient: needs the gradient statistics arrays
    const bool gradients = stats->gradient_mean && stats->n_gradient_estimates && pts->estimation_quantity;
    if (gradients) {
        ZG_TRY(stageInOut<double>(ctx, C::kGMean, stats->gradient_mean, (size_t)n * D, mem, &P.statGradMean));
        ZG_TRY(stageInOut<double>(ctx, C::kGM2, stats->gradient_m2, (size_t)n * D, mem, &P.statGradM2));
        ZG_TRY(stageInOut<int>(ctx, C::kGN, stats->n_gradient_estimates, (size_t)n, mem, &P.statGradN));
        ZG_TRY(stageIn<float>(ctx, C::kDistRefl, pts->dist_to_reflecting, (size_t)n, mem, &P.distRefl));
        ZG_TRY(scratch<double>(ctx, C::kAccGrad, (size_t)n * D, &P.accGrad));
        ZG_TRY(scratch<double>(ctx, C::kAccGradSq, (size_t)n * D, &P.accGradSq));
        ZG_TRY(scratch<int>(ctx, C::kAccGradN, (size_t)n, &P.accGradN));
        ZG_TRY(stageIn<float>(ctx, C::kDirDeriv, pts->direction_for_derivative, (size_t)n * D, mem, &P.dirDeriv));
        if (stats->total_first_source_contribution) {
            ZG_TRY(stageInOut<double>(ctx, C::kFirstSrc, stats->total_first_source_contribution, (size_t)n, mem, &P.statFirstSrc));
            ZG_TRY(scratch<double>(ctx, C::kAccFirstSrc, (size_t)n, &P.accFirstSrc));
        }
        if (stats->total_derivative_contribution) {
            ZG_TRY(stageInOut<double>(ctx, C::kDeriv, stats->total_derivative_contribution, (size_t)n, mem, &P.statDeriv));
            ZG_TRY(scratch<double>(ctx, C::kAccDeriv, (size_t)n, &P.accDeriv));
        }
    }
    long long* blockSums = nullptr;
    ZG_TRY(scratch<long long>(ctx, C::kWalkStart, (size_t)n + 1, &P.walkStart));
    ZG_TRY(scratch<int>(ctx, C::kFlags, (size_t)n, &P.pointFlags));
    ZG_TRY(scratch<int>(ctx, C::kNPrev, (size_t)n, &P.nPrev));
    ZG_TRY(scratch<double>(ctx, C::kAccSum, (size_t)n, &P.accSum));
    ZG_TRY(scratch<double>(ctx, C::kAccSq, (size_t)n, &P.accSq));
    ZG_TRY(scratch<int>(ctx, C::kAccN, (size_t)n, &P.accN));
    ZG_TRY(scratch<long long>(ctx, C::kAccLen, (size_t)n, &P.accLen));
    ZG_TRY(scratch<long long>(ctx, C::kAccSplits, (size_t)n, &P.accSplits));
    ZG_TRY(scratch<long long>(ctx, C::kBlockSums, scanScratchElems(n), &blockSums));
    ZG_TRY(scratch<unsigned long long>(ctx, C::kCounters, 16, &P.counters));
    P.errorWord = (unsigned int*)(P.counters + 8);
    ZG_CUDA(cudaMemsetAsync(P.counters, 0, 16 * sizeof(unsigned long long), s));

    int threads = opt && opt->block_size > 0 ? opt->block_size : 128;
    if (threads % 32 != 0 || threads > 128) return fail(ZGPU_ERR_INVALID_ARG, "block_size must be a multiple of 32 and <= 128");
    P.stackEntries = sceneStack;
    if (P.sc.hasAbs) P.stackEntries = std::max(P.stackEntries, P.sc.absorbing.stackEntries);
    if (P.sc.hasRefl) P.stackEntries = std::max(P.stackEntries, P.sc.reflecting.stackEntries);
    // Walk on Spheres on a large scene: each closest-point query is answered by a whole warp
    // (per-query work varies by orders of magnitude between walks, which idles the lanes of
    // a one-lane-per-query traversal); the walk kernel then needs no per-thread stack
    const int queryMode = opt ? opt->query_mode : 0;
    if (opt && opt->step_budget < 0) return fail(ZGPU_ERR_INVALID_ARG, "step_budget must be >= 0");
    P.stepBudget = opt ? opt->step_budget : 0;
    if (queryMode < 0 || queryMode > 2) return fail(ZGPU_ERR_INVALID_ARG, "query_mode must be 0, 1 or 2");
    const int walkStackEntries = P.stackEntries;
    if (solver == ZGPU_SOLVER_WALK_ON_SPHERES && P.sc.hasAbs && !batched)
        P.coop = queryMode == 2 || (queryMode == 0 && D == 3 && q->absorbing->nPrims >= kCoopMinPrims);
    // Walk on Stars with a Robin boundary: its star radius visits thousands of primitives from
    // interior points under the reflectance bounds, the case the warp-wide traversal serves
    if (solver == ZGPU_SOLVER_WALK_ON_STARS && P.sc.hasRefl && q->reflecting->kind == ZGPU_BOUNDARY_ROBIN && !batched)
        P.coopStar = queryMode == 2 || (queryMode == 0 && D == 3 && q->reflecting->nPrims >= kCoopStarMinPrims);
    // the walk loop's schedule: the sorted wavefront serves solution solves (one scene or a
    // batch) without neural cache, split scratch or warp-wide queries; with use_graph it
    // replays its iterations from a captured graph
    const int schedule = opt ? opt->schedule : ZGPU_SCHEDULE_AUTO;
    if (schedule < ZGPU_SCHEDULE_AUTO || schedule > ZGPU_SCHEDULE_WAVEFRONT)
        return fail(ZGPU_ERR_INVALID_ARG, "schedule must be 0, 1 or 2");
    bool scenesServe = true;   // every scene: non-negative Robin coefficients, no splitting
    for (int k = 0; k < nScenes; k++)
        scenesServe = scenesServe && pde[k].are_robin_coeffs_nonnegative && ws[k].splitting_threshold >= 2.0f;
    const bool waveServes = !gradients && !cache && queryMode != ZGPU_QUERY_MODE_WARP && scenesServe;
    if (schedule == ZGPU_SCHEDULE_WAVEFRONT && !waveServes)
        return fail(ZGPU_ERR_UNSUPPORTED, "the wavefront schedule serves solutions only, without cache or warp-wide "
                                          "queries, with non-negative Robin coefficients and splitting_threshold >= 2");
    const bool waveAuto = D == 2 && solver == ZGPU_SOLVER_WALK_ON_STARS;
    const bool useWave = waveServes && (schedule == ZGPU_SCHEDULE_WAVEFRONT || (schedule == ZGPU_SCHEDULE_AUTO && waveAuto));
    if (useWave) P.coop = P.coopStar = 0;
    if (P.coop) P.stackEntries = 0;
    int perSM = opt && opt->blocks_per_sm > 0 ? opt->blocks_per_sm
                                              : walkKernelMaxBlocksPerSM(D, solver, threads, P);
    P.stackEntries = walkStackEntries;
    int blocks = ctx->numSMs * perSM;
    ZG_TRY(scratch<float4>(ctx, C::kSplitScratch, (size_t)blocks * threads * 3 * kSplitStack, &P.splitStack));

    // kernel launches of this solve: prepare, the walk-id scan (3 kernels, 1 without points),
    // the walk kernel or the wavefront iterations (6 kernels each, 5 for Walk on Spheres) and
    // its drain, the cache pass, finalize
    long long waveLaunches = 0;
    ctx->lastLaunches = 0;
    ZG_CUDA(cudaEventRecord(ctx->ev[0], s));
    if (opt && opt->use_graph && !cache && !useWave) {
        // the four launches as one CUDA graph: re-captured when anything they read changed
        SolveParams Pwalk = P;
        if (Pwalk.coop) Pwalk.stackEntries = 0;
        std::vector<unsigned char> key(sizeof(SolveParams) * 2 + 4 * sizeof(int64_t));
        const int64_t dims[4] = {(int64_t)D, (int64_t)blocks, (int64_t)threads, (int64_t)(intptr_t)blockSums};
        std::memcpy(key.data(), &P, sizeof(P));
        std::memcpy(key.data() + sizeof(P), &Pwalk, sizeof(P));
        std::memcpy(key.data() + 2 * sizeof(P), dims, sizeof(dims));
        if (!ctx->graphExec || ctx->graphKey != key) {
            if (ctx->graphExec) { cudaGraphExecDestroy(ctx->graphExec); ctx->graphExec = nullptr; }
            cudaGraph_t g = nullptr;
            ZG_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeRelaxed));
            cudaError_t e = launchPrepare(P, D, s);
            if (e == cudaSuccess) e = launchScan(P.walkStart, n, blockSums, s);
            if (e == cudaSuccess && n > 0) e = launchWalk(Pwalk, D, blocks, threads, s);
            if (e == cudaSuccess) e = launchFinalize(Pwalk, D, s);
            cudaError_t e2 = cudaStreamEndCapture(s, &g);
            if (e == cudaSuccess) e = e2;
            if (e == cudaSuccess) e = cudaGraphInstantiate(&ctx->graphExec, g, 0);
            if (g) cudaGraphDestroy(g);
            ZG_CUDA(e);
            ctx->graphKey = key;
        }
        ZG_CUDA(cudaEventRecord(ctx->ev[1], s));
        ZG_CUDA(cudaGraphLaunch(ctx->graphExec, s));
        ZG_CUDA(cudaEventRecord(ctx->ev[2], s));
    } else {
    ZG_CUDA(launchPrepare(P, D, s));
    ZG_CUDA(launchScan(P.walkStart, n, blockSums, s));
    if (cache) {
        // one record per walk at most (no splitting): size the buffer by the walk count
        long long totalWalks = 0;
        ZG_CUDA(cudaMemcpyAsync(&totalWalks, P.walkStart + n, sizeof(long long), cudaMemcpyDeviceToHost, s));
        ZG_CUDA(cudaStreamSynchronize(s));
        P.cacheCap = std::max(1LL, totalWalks);
        ZG_TRY(scratch<float4>(ctx, C::kCacheRec, (size_t)P.cacheCap * 2, &P.cacheRec));
        P.cacheMinDist = cacheMinDist;
    }
    ZG_CUDA(cudaEventRecord(ctx->ev[1], s));
    if (P.coop) P.stackEntries = 0;     // the prepare kernel above used the per-thread stacks
    if (n > 0) {
        if (useWave) ZG_TRY(runWave(ctx, P, D, s, opt && opt->use_graph, &waveLaunches));
        else ZG_CUDA(launchWalk(P, D, blocks, threads, s));
    }
    if (cache && n > 0)
        ZG_CUDA(launchCacheAccumulate(cache, P.cacheRec, P.counters + kCtrCache, P.cacheCap, P.accSum, P.accSq,
                                      P.accN, P.accLen, P.errorWord, s));
    ZG_CUDA(cudaEventRecord(ctx->ev[2], s));
    ZG_CUDA(launchFinalize(P, D, s));
    }
    ZG_CUDA(cudaEventRecord(ctx->ev[3], s));
    ctx->lastLaunches = n > 0 ? 5 + (useWave ? waveLaunches : 1) + (cache ? 1 : 0) : 1;
    ZG_TRY(stageOut<double>(ctx, P.statMean, stats->solution_mean, (size_t)n, mem));
    ZG_TRY(stageOut<double>(ctx, P.statM2, stats->solution_m2, (size_t)n, mem));
    ZG_TRY(stageOut<int>(ctx, P.statN, stats->n_solution_estimates, (size_t)n, mem));
    ZG_TRY(stageOut<long long>(ctx, P.statLen, (long long*)stats->total_walk_length, (size_t)n, mem));
    ZG_TRY(stageOut<long long>(ctx, P.statSplits, (long long*)stats->total_splits, (size_t)n, mem));
    if (P.fsrPersistent) ZG_TRY(stageOut<float>(ctx, P.fsr, pts->first_sphere_radius, (size_t)n, mem));
    if (gradients) {
        ZG_TRY(stageOut<double>(ctx, P.statGradMean, stats->gradient_mean, (size_t)n * D, mem));
        if (stats->gradient_m2) ZG_TRY(stageOut<double>(ctx, P.statGradM2, stats->gradient_m2, (size_t)n * D, mem));
        ZG_TRY(stageOut<int>(ctx, P.statGradN, stats->n_gradient_estimates, (size_t)n, mem));
        if (P.statFirstSrc) ZG_TRY(stageOut<double>(ctx, P.statFirstSrc, stats->total_first_source_contribution, (size_t)n, mem));
        if (P.statDeriv) ZG_TRY(stageOut<double>(ctx, P.statDeriv, stats->total_derivative_contribution, (size_t)n, mem));
    }
    ZG_CUDA(cudaMemcpyAsync(ctx->hostCounters, P.counters, 9 * sizeof(unsigned long long), cudaMemcpyDeviceToHost, s));
    ZG_CUDA(cudaMemcpyAsync(ctx->hostCounters + 12, P.walkStart + n, sizeof(long long), cudaMemcpyDeviceToHost, s));
    ZG_CUDA(cudaStreamSynchronize(s));
    unsigned int errWord = (unsigned int)(ctx->hostCounters[8] & 0xffffffffu);
    if (report) {
        std::memset(report, 0, sizeof(*report));
        report->total_steps = ctx->hostCounters[kCtrSteps];
        report->escaped_walks = ctx->hostCounters[kCtrEscaped];
        report->exceeded_walks = ctx->hostCounters[kCtrExceeded];
        report->rr_terminated = ctx->hostCounters[kCtrRR];
        report->total_walks = ctx->hostCounters[12];
        report->error_word = errWord;
        report->cache_terminated = cache ? std::min<unsigned long long>(ctx->hostCounters[kCtrCache], P.cacheCap) : 0;
        cudaEventElapsedTime(&report->kernel_ms, ctx->ev[1], ctx->ev[2]);
        cudaEventElapsedTime(&report->total_ms, ctx->ev[0], ctx->ev[3]);
    }
    if (errWord & kErrBudget)
        return fail(ZGPU_ERR_TIMEOUT_BUDGET, "a walk state exceeded step_budget = %lld loop iterations; its walk was "
                                             "dropped", (long long)P.stepBudget);
    if (errWord)
        return fail(ZGPU_ERR_DEVICE_STATE,
                    "device error word 0x%x (1: traversal stack, 2: split stack, 8: scene id outside the table, "
                    "16: cache record overflow)", errWord);
    return ZGPU_OK;
}

}  // namespace

extern "C" {

int zgpu_last_solve_launches(zgpu_context* ctx, int64_t* launches) {
    if (!ctx || !launches) return fail(ZGPU_ERR_INVALID_ARG, "NULL required argument");
    *launches = ctx->lastLaunches;
    return ZGPU_OK;
}

int zgpu_solve(zgpu_context* ctx, int solver, const zgpu_geometric_queries* q, const zgpu_pde* pde,
               const zgpu_walk_settings* ws, const zgpu_sample_points* pts, zgpu_sample_statistics* stats,
               const zgpu_solve_options* opt, zgpu_solve_report* report) {
    return solveImpl(ctx, solver, 1, q, pde, ws, pts, stats, opt, nullptr, 0.0f, report);
}

int zgpu_solve_cached(zgpu_context* ctx, int solver, const zgpu_geometric_queries* q, const zgpu_pde* pde,
                      const zgpu_walk_settings* ws, const zgpu_sample_points* pts, zgpu_sample_statistics* stats,
                      const zgpu_solve_options* opt, zgpu_cache* cache, float min_distance, zgpu_solve_report* report) {
    if (!cache) return fail(ZGPU_ERR_INVALID_ARG, "cache is NULL (use zgpu_solve for the plain walk)");
    if (!ctx || !q || !ws) return fail(ZGPU_ERR_INVALID_ARG, "NULL required argument");
    if (cacheDim(cache) != q->dim) return fail(ZGPU_ERR_INVALID_ARG, "cache dim %d does not match queries dim %d",
                                              cacheDim(cache), q->dim);
    if (!(min_distance > 0.0f)) return fail(ZGPU_ERR_INVALID_ARG, "min_distance must be > 0");
    if (ws->splitting_threshold < FLT_MAX)
        return fail(ZGPU_ERR_UNSUPPORTED, "walk splitting is not supported with the cache (splitting_threshold must be FLT_MAX)");
    if (cacheStream(cache) != ctx->stream) return fail(ZGPU_ERR_INVALID_ARG, "cache belongs to another context");
    return solveImpl(ctx, solver, 1, q, pde, ws, pts, stats, opt, cache, min_distance, report);
}

// Autotuner: times candidate launch configurations on a stride sample of the points and
// keeps the fastest (walk steps per kernel millisecond) per scene signature.
int zgpu_autotune(zgpu_context* ctx, int solver, const zgpu_geometric_queries* q, const zgpu_pde* pde,
                  const zgpu_walk_settings* ws, const zgpu_sample_points* pts, int32_t sample_points,
                  int32_t sample_walks, zgpu_solve_options* out, float* best_rate) {
    if (!ctx || !q || !pde || !ws || !pts || !out) return fail(ZGPU_ERR_INVALID_ARG, "NULL required argument");
    if (pts->n <= 0) return fail(ZGPU_ERR_INVALID_ARG, "autotuning needs points");
    if (sample_points <= 0 || sample_walks <= 0) return fail(ZGPU_ERR_INVALID_ARG, "sample sizes must be positive");
    const int D = q->dim;
    if (D != 2 && D != 3) return fail(ZGPU_ERR_INVALID_ARG, "queries dim must be 2 or 3");
    auto lg = [](int64_t v) { int b = 0; while (v > 1) { v >>= 1; b++; } return b; };
    char sig[160];
    std::snprintf(sig, sizeof(sig), "D%d s%d a%d r%d k%d x%d", D, solver,
                  lg(q->absorbing ? q->absorbing->nPrims : 0), lg(q->reflecting ? q->reflecting->nPrims : 0),
                  q->reflecting ? q->reflecting->kind : -1, pde->absorption_coeff > 0.0f ? 1 : 0);
    auto it = ctx->tuned.find(sig);
    if (it != ctx->tuned.end()) { *out = it->second; if (best_rate) *best_rate = -1.0f; return ZGPU_OK; }
    // stride sample of the points, staged on the host
    const int64_t n = pts->n;
    const int64_t m = std::min<int64_t>(n, sample_points);
    const int64_t stride = n / m;
    auto pull = [&](const void* src, size_t elem, std::vector<unsigned char>& all) -> int {
        all.assign((size_t)n * elem, 0);
        if (!src) { all.clear(); return ZGPU_OK; }
        if (pts->memory == ZGPU_MEM_DEVICE) { ZG_CUDA(cudaMemcpy(all.data(), src, all.size(), cudaMemcpyDeviceToHost)); }
        else std::memcpy(all.data(), src, all.size());
        return ZGPU_OK;
    };
    std::vector<unsigned char> aPt, aN, aT, aD, aS, aA;
    ZG_TRY(pull(pts->pt, sizeof(float) * D, aPt));
    ZG_TRY(pull(pts->normal, sizeof(float) * D, aN));
    ZG_TRY(pull(pts->type, sizeof(int32_t), aT));
    ZG_TRY(pull(pts->dist_to_absorbing, sizeof(float), aD));
    ZG_TRY(pull(pts->seed, sizeof(uint64_t), aS));
    ZG_TRY(pull(pts->estimate_normal_aligned, sizeof(int32_t), aA));
    auto pick = [&](const std::vector<unsigned char>& all, size_t elem) {
        std::vector<unsigned char> o;
        if (all.empty()) return o;
        o.resize((size_t)m * elem);
        for (int64_t i = 0; i < m; i++) std::memcpy(&o[(size_t)i * elem], &all[(size_t)(i * stride) * elem], elem);
        return o;
    };
    std::vector<unsigned char> sPt = pick(aPt, sizeof(float) * D), sN = pick(aN, sizeof(float) * D),
                               sT = pick(aT, 4), sD = pick(aD, 4), sS = pick(aS, 8), sA = pick(aA, 4);
    std::vector<int32_t> nw((size_t)m, sample_walks), cnt((size_t)m);
    std::vector<double> mean((size_t)m), m2((size_t)m);
    std::vector<long long> len((size_t)m), spl((size_t)m);
    zgpu_sample_points sp;
    std::memset(&sp, 0, sizeof(sp));
    sp.n = m; sp.memory = ZGPU_MEM_HOST;
    sp.pt = (const float*)sPt.data();
    sp.normal = sN.empty() ? nullptr : (const float*)sN.data();
    sp.type = sT.empty() ? nullptr : (const int32_t*)sT.data();
    sp.dist_to_absorbing = (const float*)sD.data();
    sp.seed = (const uint64_t*)sS.data();
    sp.estimate_normal_aligned = sA.empty() ? nullptr : (const int32_t*)sA.data();
    sp.n_walks = nw.data();
    zgpu_sample_statistics st;
    std::memset(&st, 0, sizeof(st));
    st.memory = ZGPU_MEM_HOST;
    st.solution_mean = mean.data(); st.solution_m2 = m2.data(); st.n_solution_estimates = cnt.data();
    st.total_walk_length = (int64_t*)len.data(); st.total_splits = (int64_t*)spl.data();
    // query modes worth sweeping: warp-wide closest points (Walk on Spheres) and warp-wide
    // Robin star radii (Walk on Stars)
    const bool sweepQuery = (solver == ZGPU_SOLVER_WALK_ON_SPHERES && q->absorbing && q->absorbing->nPrims > 0) ||
                            (solver == ZGPU_SOLVER_WALK_ON_STARS && q->reflecting && q->reflecting->nPrims > 0 &&
                             q->reflecting->kind == ZGPU_BOUNDARY_ROBIN);
    const int threadsC[3] = {32, 64, 128};
    const int perSMC[3] = {0, 2, 4};
    // node widths: 8-wide trees for 3D absorbing boundaries with a host copy of their mesh
    const bool sweepWidth = D == 3 && q->absorbing && q->absorbing->nPrims > 0 &&
                            (q->absorbing->view.width == 8 || !q->absorbing->hostIdx.empty());
    zgpu_solve_options best;
    std::memset(&best, 0, sizeof(best));
    double bestRate = -1.0;
    for (int wi = 0; wi < (sweepWidth ? 2 : 1); wi++)
    for (int qm = sweepQuery ? 1 : 0; qm <= (sweepQuery ? 2 : 0); qm++)
        for (int ti = 0; ti < 3; ti++)
            for (int pi = 0; pi < 3; pi++) {
                zgpu_solve_options o;
                std::memset(&o, 0, sizeof(o));
                o.block_size = threadsC[ti];
                o.blocks_per_sm = perSMC[pi];
                o.query_mode = qm;
                o.bvh_width = wi == 0 ? 4 : 8;
                // the knobs are the persistent kernel's; the sample is too small to measure the
                // wavefront, whose iterations are launch-bound until the pool fills
                o.schedule = ZGPU_SCHEDULE_PERSISTENT;
                double rate = 0.0;
                for (int rep = 0; rep < 2; rep++) {
                    std::fill(cnt.begin(), cnt.end(), 0);
                    std::fill(mean.begin(), mean.end(), 0.0);
                    std::fill(m2.begin(), m2.end(), 0.0);
                    std::fill(len.begin(), len.end(), 0);
                    std::fill(spl.begin(), spl.end(), 0);
                    zgpu_solve_report r;
                    int stt = solveImpl(ctx, solver, 1, q, pde, ws, &sp, &st, &o, nullptr, 0.0f, &r);
                    if (stt != ZGPU_OK) return stt;
                    if (r.kernel_ms > 0.0f) rate = std::max(rate, (double)r.total_steps / r.kernel_ms);
                }
                if (rate > bestRate) { bestRate = rate; best = o; }
            }
    best.schedule = ZGPU_SCHEDULE_AUTO;   // solves keep the automatic schedule
    ctx->tuned[sig] = best;
    *out = best;
    if (best_rate) *best_rate = (float)(bestRate * 1e3);
    return ZGPU_OK;
}

int zgpu_solve_batched(zgpu_context* ctx, int solver, int n_scenes, const zgpu_geometric_queries* queries,
                       const zgpu_pde* pdes, const zgpu_walk_settings* settings, const zgpu_sample_points* points,
                       zgpu_sample_statistics* stats, const zgpu_solve_options* options, zgpu_solve_report* report) {
    if (n_scenes == 1 && (!points || !points->scene_id))
        return zgpu_solve(ctx, solver, queries, pdes, settings, points, stats, options, report);
    return solveImpl(ctx, solver, n_scenes, queries, pdes, settings, points, stats, options, nullptr, 0.0f, report);
}

}  // extern "C"

// ------------------------------------------------------------------ PDE fields, BVC
int zgpu_pde_evaluate(zgpu_context* ctx, int dim, const zgpu_pde* pde, int64_t n, const float* x, const float* normal,
                      const int32_t* aligned, int memory, float* out_source, float* out_dirichlet, float* out_robin,
                      float* out_robin_coeff) {
    if (!ctx || !pde) return fail(ZGPU_ERR_INVALID_ARG, "NULL required argument");
    if (dim != 2 && dim != 3) return fail(ZGPU_ERR_INVALID_ARG, "dim must be 2 or 3, got %d", dim);
    if (n < 0 || (n > 0 && !x)) return fail(ZGPU_ERR_INVALID_ARG, "points");
    if (memory != ZGPU_MEM_HOST && memory != ZGPU_MEM_DEVICE) return fail(ZGPU_ERR_INVALID_ARG, "unknown memory space");
    ZG_TRY(zg::checkPdeFields(pde, dim, true));
    if (n == 0) return ZGPU_OK;
    ZG_CUDA(cudaSetDevice(ctx->device));
    using C = zgpu_context;
    zgpu_pde dp = *pde;
    ZG_TRY(stageGrids(ctx, dp, dim, 0));
    const float *dx, *dn;
    const int* da;
    ZG_TRY(stageIn<float>(ctx, C::kB0, x, (size_t)n * dim, memory, &dx));
    ZG_TRY(stageIn<float>(ctx, C::kB1, normal, (size_t)n * dim, memory, &dn));
    ZG_TRY(stageIn<int>(ctx, C::kB2, aligned, (size_t)n, memory, &da));
    float* outs[4] = {out_source, out_dirichlet, out_robin, out_robin_coeff};
    float* dOut[4] = {nullptr, nullptr, nullptr, nullptr};
    for (int k = 0; k < 4; k++) {
        if (!outs[k]) continue;
        if (memory == ZGPU_MEM_DEVICE) dOut[k] = outs[k];
        else ZG_TRY(scratch<float>(ctx, C::kB3 + k, (size_t)n, &dOut[k]));
    }
    ZG_CUDA(launchPdeEvaluate(dim, dp, n, dx, dn, da, dOut[0], dOut[1], dOut[2], dOut[3], ctx->stream));
    for (int k = 0; k < 4; k++)
        if (outs[k] && memory == ZGPU_MEM_HOST)
            ZG_CUDA(cudaMemcpyAsync(outs[k], dOut[k], sizeof(float) * n, cudaMemcpyDeviceToHost, ctx->stream));
    ZG_CUDA(cudaStreamSynchronize(ctx->stream));
    return ZGPU_OK;
}

int zgpu_bvc_splat(zgpu_context* ctx, int dim, const zgpu_pde* pde, const zgpu_bvc_samples* samples, float radius_clamp,
                   float kernel_regularization, float robin_coeff_cutoff_for_normal_derivative,
                   float cutoff_dist_to_absorbing_boundary, float cutoff_dist_to_reflecting_boundary,
                   zgpu_bvc_eval_points* ev, int memory) {
    if (!ctx || !pde || !samples || !ev) return fail(ZGPU_ERR_INVALID_ARG, "NULL required argument");
    if (dim != 2 && dim != 3) return fail(ZGPU_ERR_INVALID_ARG, "dim must be 2 or 3, got %d", dim);
    if (memory != ZGPU_MEM_HOST && memory != ZGPU_MEM_DEVICE) return fail(ZGPU_ERR_INVALID_ARG, "unknown memory space");
    if (samples->n < 0 || ev->n < 0) return fail(ZGPU_ERR_INVALID_ARG, "negative sizes");
    if (samples->n > 0 && (!samples->pt || !samples->normal || !samples->pdf || !samples->type || !samples->solution ||
                           !samples->normal_derivative || !samples->contribution))
        return fail(ZGPU_ERR_INVALID_ARG, "sample arrays pt, normal, pdf, type, solution, normal_derivative and "
                                          "contribution are required");
    if (ev->n > 0 && (!ev->pt || !ev->dist_to_absorbing || !ev->mean || !ev->m2 || !ev->count || !ev->gradient_mean))
        return fail(ZGPU_ERR_INVALID_ARG, "evaluation arrays pt, dist_to_absorbing, mean, m2, count and gradient_mean "
                                          "are required");
    if (!(pde->absorption_coeff >= 0.0f)) return fail(ZGPU_ERR_INVALID_ARG, "absorption coefficient must be >= 0");
    if (samples->n == 0 || ev->n == 0) return ZGPU_OK;
    if (samples->n >= ((int64_t)1 << 40) || ev->n >= ((int64_t)1 << 40)) return fail(ZGPU_ERR_INVALID_ARG, "too many points");
    ZG_CUDA(cudaSetDevice(ctx->device));
    using C = zgpu_context;
    const int64_t ns = samples->n, ne = ev->n;
    BvcSplatParams p;
    std::memset(&p, 0, sizeof(p));
    p.nSamples = ns;
    ZG_TRY(stageIn<float>(ctx, C::kB0, samples->pt, (size_t)ns * dim, memory, &p.pt));
    ZG_TRY(stageIn<float>(ctx, C::kB1, samples->normal, (size_t)ns * dim, memory, &p.normal));
    ZG_TRY(stageIn<float>(ctx, C::kB2, samples->pdf, (size_t)ns, memory, &p.pdf));
    ZG_TRY(stageIn<int>(ctx, C::kB3, samples->type, (size_t)ns, memory, &p.type));
    ZG_TRY(stageIn<int>(ctx, C::kB4, samples->estimate_normal_aligned, (size_t)ns, memory, &p.aligned));
    ZG_TRY(stageIn<float>(ctx, C::kB5, samples->solution, (size_t)ns, memory, &p.solution));
    ZG_TRY(stageIn<float>(ctx, C::kB6, samples->normal_derivative, (size_t)ns, memory, &p.normalDerivative));
    ZG_TRY(stageIn<float>(ctx, C::kB7, samples->contribution, (size_t)ns, memory, &p.contribution));
    ZG_TRY(stageIn<float>(ctx, C::kB8, samples->robin_coeff, (size_t)ns, memory, &p.robinCoeff));
    p.nEval = ne;
    ZG_TRY(stageIn<float>(ctx, C::kB9, ev->pt, (size_t)ne * dim, memory, &p.evalPt));
    ZG_TRY(stageIn<int>(ctx, C::kB10, ev->type, (size_t)ne, memory, &p.evalType));
    ZG_TRY(stageIn<float>(ctx, C::kB11, ev->dist_to_absorbing, (size_t)ne, memory, &p.evalDistA));
    ZG_TRY(stageIn<float>(ctx, C::kB12, ev->dist_to_reflecting, (size_t)ne, memory, &p.evalDistR));
    const size_t ng = (size_t)ne * ZGPU_BVC_GROUPS;
    ZG_TRY(stageInOut<double>(ctx, C::kB13, ev->mean, ng, memory, &p.mean));
    ZG_TRY(stageInOut<double>(ctx, C::kB14, ev->m2, ng, memory, &p.m2));
    ZG_TRY(stageInOut<int>(ctx, C::kB15, ev->count, ng, memory, &p.count));
    ZG_TRY(stageInOut<double>(ctx, C::kB16, ev->gradient_mean, ng * dim, memory, &p.gradMean));
    if (ev->gradient_m2) ZG_TRY(stageInOut<double>(ctx, C::kB17, ev->gradient_m2, ng * dim, memory, &p.gradM2));
    p.sqrtLambda = std::sqrt(pde->absorption_coeff);
    p.radiusClamp = radius_clamp;
    p.regularization = kernel_regularization;
    p.robinCutoff = robin_coeff_cutoff_for_normal_derivative;
    p.cutoffA = cutoff_dist_to_absorbing_boundary;
    p.cutoffR = cutoff_dist_to_reflecting_boundary;
    // the statistic groups present in the cache: one launch each
    std::vector<int32_t> ht((size_t)ns), ha;
    if (memory == ZGPU_MEM_HOST) std::memcpy(ht.data(), samples->type, sizeof(int32_t) * ns);
    else ZG_CUDA(cudaMemcpy(ht.data(), samples->type, sizeof(int32_t) * ns, cudaMemcpyDeviceToHost));
    if (samples->estimate_normal_aligned) {
        ha.resize((size_t)ns);
        if (memory == ZGPU_MEM_HOST) std::memcpy(ha.data(), samples->estimate_normal_aligned, sizeof(int32_t) * ns);
        else ZG_CUDA(cudaMemcpy(ha.data(), samples->estimate_normal_aligned, sizeof(int32_t) * ns, cudaMemcpyDeviceToHost));
    }
    bool present[ZGPU_BVC_GROUPS] = {false, false, false, false, false};
    for (int64_t j = 0; j < ns; j++) {
        const int t = ht[j], al = ha.empty() ? 0 : ha[j];
        const int g = t == ZGPU_SAMPLE_ON_ABSORBING_BOUNDARY ? (al ? ZGPU_BVC_ABSORBING_ALIGNED : ZGPU_BVC_ABSORBING)
                    : t == ZGPU_SAMPLE_ON_REFLECTING_BOUNDARY ? (al ? ZGPU_BVC_REFLECTING_ALIGNED : ZGPU_BVC_REFLECTING)
                    : ZGPU_BVC_SOURCE;
        present[g] = true;
    }
    const int splits = bvcSplitCount(ne, ns, ctx->numSMs);
    if (splits > 1) ZG_TRY(scratch<double>(ctx, C::kB18, (size_t)splits * ne * (3 + 2 * dim), &p.partial));
    for (int g = 0; g < ZGPU_BVC_GROUPS; g++) {
        if (!present[g]) continue;
        p.group = g;
        ZG_CUDA(launchBvcSplat(dim, pde->absorption_coeff > 0.0f, p, splits, ctx->stream));
    }
    ZG_TRY(stageOut<double>(ctx, p.mean, ev->mean, ng, memory));
    ZG_TRY(stageOut<double>(ctx, p.m2, ev->m2, ng, memory));
    ZG_TRY(stageOut<int>(ctx, p.count, ev->count, ng, memory));
    ZG_TRY(stageOut<double>(ctx, p.gradMean, ev->gradient_mean, ng * dim, memory));
    if (ev->gradient_m2) ZG_TRY(stageOut<double>(ctx, p.gradM2, ev->gradient_m2, ng * dim, memory));
    ZG_CUDA(cudaStreamSynchronize(ctx->stream));
    return ZGPU_OK;
}

// ------------------------------------------------------------------ reverse walk on stars
int zgpu_rws_solve(zgpu_context* ctx, const zgpu_geometric_queries* q, const zgpu_pde* pde, const zgpu_walk_settings* ws,
                   const zgpu_rws_samples* samples, float normal_offset_for_absorbing_boundary, float radius_clamp,
                   float kernel_regularization, uint64_t stream, zgpu_rws_eval_points* ev, int memory,
                   zgpu_solve_report* report) {
    if (!ctx || !q || !pde || !ws || !samples || !ev) return fail(ZGPU_ERR_INVALID_ARG, "NULL required argument");
    const int D = q->dim;
    if (D != 2 && D != 3) return fail(ZGPU_ERR_INVALID_ARG, "queries dim must be 2 or 3, got %d", D);
    ZG_TRY(checkScene(q, pde, ws, D));
    if (memory != ZGPU_MEM_HOST && memory != ZGPU_MEM_DEVICE) return fail(ZGPU_ERR_INVALID_ARG, "unknown memory space");
    if (samples->n < 0 || ev->n < 0) return fail(ZGPU_ERR_INVALID_ARG, "negative sizes");
    if (samples->n > 0 && (!samples->pt || !samples->normal || !samples->type || !samples->pdf || !samples->contribution ||
                           !samples->dist_to_absorbing || !samples->seed))
        return fail(ZGPU_ERR_INVALID_ARG, "sample arrays pt, normal, type, pdf, contribution, dist_to_absorbing and "
                                          "seed are required");
    if (ev->n > 0 && (!ev->pt || !ev->totals)) return fail(ZGPU_ERR_INVALID_ARG, "evaluation arrays pt and totals are required");
    if (!(normal_offset_for_absorbing_boundary > 0.0f))
        return fail(ZGPU_ERR_INVALID_ARG, "normal_offset_for_absorbing_boundary must be > 0");
    if (samples->n >= ((int64_t)1 << 40) || ev->n >= ((int64_t)1 << 30)) return fail(ZGPU_ERR_INVALID_ARG, "too many points");
    if (report) std::memset(report, 0, sizeof(*report));
    if (samples->n == 0 || ev->n == 0) return ZGPU_OK;
    ZG_CUDA(cudaSetDevice(ctx->device));
    using C = zgpu_context;
    cudaStream_t s = ctx->stream;
    const int64_t ns = samples->n, ne = ev->n;
    RwsParams P;
    std::memset(&P, 0, sizeof(P));
    P.sc = sceneOf(q, pde, ws);
    ZG_TRY(stageGrids(ctx, P.sc.pde, D, 0));
    P.nSamples = ns;
    ZG_TRY(stageIn<float>(ctx, C::kB0, samples->pt, (size_t)ns * D, memory, &P.pt));
    ZG_TRY(stageIn<float>(ctx, C::kB1, samples->normal, (size_t)ns * D, memory, &P.normal));
    ZG_TRY(stageIn<int>(ctx, C::kB2, samples->type, (size_t)ns, memory, &P.type));
    ZG_TRY(stageIn<int>(ctx, C::kB3, samples->estimate_normal_aligned, (size_t)ns, memory, &P.aligned));
    ZG_TRY(stageIn<float>(ctx, C::kB4, samples->pdf, (size_t)ns, memory, &P.pdf));
    ZG_TRY(stageIn<float>(ctx, C::kB5, samples->contribution, (size_t)ns, memory, &P.contribution));
    ZG_TRY(stageIn<float>(ctx, C::kB6, samples->dist_to_absorbing, (size_t)ns, memory, &P.distAbs));
    ZG_TRY(stageIn<uint64_t>(ctx, C::kB7, samples->seed, (size_t)ns, memory, &P.seed));
    P.stream = stream;
    P.nEval = ne;
    ZG_TRY(stageIn<float>(ctx, C::kB9, ev->pt, (size_t)ne * D, memory, &P.evalPt));
    ZG_TRY(stageIn<float>(ctx, C::kB10, ev->normal, (size_t)ne * D, memory, &P.evalNormal));
    ZG_TRY(stageIn<int>(ctx, C::kB11, ev->type, (size_t)ne, memory, &P.evalType));
    ZG_TRY(stageInOut<double>(ctx, C::kB13, ev->totals, (size_t)ne * ZGPU_RWS_TOTALS, memory, &P.totals));
    // the evaluation points' tree for the per-step radius searches
    float4* evalNodes = nullptr;
    int* evalOrder = nullptr;
    int2* evalRanges = nullptr;
    int nEvalNodes = 0, evalDepth = 0;
    cudaError_t e = buildPointBvhOnDevice(D, P.evalPt, (int)ne, s, &evalNodes, &nEvalNodes, &evalDepth, &evalOrder,
                                          &evalRanges);
    auto freeTree = [&]() { cudaFree(evalNodes); cudaFree(evalOrder); cudaFree(evalRanges); };
    if (e != cudaSuccess) {
        freeTree();
        if (e == cudaErrorNotSupported) return fail(ZGPU_ERR_UNSUPPORTED, "evaluation-point tree too deep");
        return fail(ZGPU_ERR_CUDA, "evaluation-point tree: %s", cudaGetErrorString(e));
    }
    P.evalNodes = evalNodes;
    P.evalOrder = evalOrder;
    P.evalRanges = evalRanges;
    P.evalDepth = evalDepth;
    P.normalOffset = normal_offset_for_absorbing_boundary;
    P.radiusClamp = radius_clamp;
    P.regularization = kernel_regularization;
    P.selfNormalize = q->domain_is_watertight && pde->absorption_coeff == 0.0f &&
                      (!P.sc.hasRefl || pde->are_robin_conditions_pure_neumann);
    P.stackEntries = 8;
    if (P.sc.hasAbs) P.stackEntries = std::max(P.stackEntries, P.sc.absorbing.stackEntries);
    if (P.sc.hasRefl) P.stackEntries = std::max(P.stackEntries, P.sc.reflecting.stackEntries);
    unsigned long long* counters = nullptr;
    if (int st = scratch<unsigned long long>(ctx, C::kCounters, 16, &counters)) { freeTree(); return st; }
    P.counters = counters;
    P.errorWord = (unsigned int*)(counters + 8);
    e = cudaMemsetAsync(counters, 0, 16 * sizeof(unsigned long long), s);
    if (e == cudaSuccess) e = cudaEventRecord(ctx->ev[1], s);
    if (e == cudaSuccess) e = launchReverseWalks(D, pde->absorption_coeff > 0.0f, P, ctx->numSMs * 4, s);
    if (e == cudaSuccess) e = cudaEventRecord(ctx->ev[2], s);
    if (e != cudaSuccess) { freeTree(); return fail(ZGPU_ERR_CUDA, "reverse walks: %s", cudaGetErrorString(e)); }
    int st = stageOut<double>(ctx, P.totals, ev->totals, (size_t)ne * ZGPU_RWS_TOTALS, memory);
    if (st == ZGPU_OK) {
        e = cudaMemcpyAsync(ctx->hostCounters, counters, 9 * sizeof(unsigned long long), cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) st = fail(ZGPU_ERR_CUDA, "reverse walks: %s", cudaGetErrorString(e));
    }
    freeTree();
    if (st != ZGPU_OK) return st;
    const unsigned int errWord = (unsigned int)(ctx->hostCounters[8] & 0xffffffffu);
    if (report) {
        report->total_steps = ctx->hostCounters[0];
        report->total_walks = ctx->hostCounters[1];
        report->error_word = errWord;
        cudaEventElapsedTime(&report->kernel_ms, ctx->ev[1], ctx->ev[2]);
        report->total_ms = report->kernel_ms;
    }
    if (errWord) return fail(ZGPU_ERR_DEVICE_STATE, "reverse walks: device error word 0x%x", errWord);
    return ZGPU_OK;
}
