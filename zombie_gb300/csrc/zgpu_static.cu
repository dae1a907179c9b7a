// zgpu_static.cu -- zgpu_solve_static: the solve entry point that allocates nothing.
//
// For callers that must not allocate device memory (a plug-in whose host owns the GPU memory
// budget, a real-time loop that forbids cudaMalloc after start-up).  All scratch of the
// prepare / scan / walk / finalize kernels lives in gStaticScratch below, a fixed
// file-scope array that every GPU loading the library holds until exit.  Host code cannot
// pass `gStaticScratch` itself to a kernel (in host code the name is a host-side shadow, not
// a device address), so the device address is looked up once per device with
// cudaGetSymbolAddress, with that device current.  Every call shares the array; calls that
// overlap on the GPU race.  The looked-up address is kept for the life of the process: it
// assumes the device's primary context lives until exit (after cudaDeviceReset the module is
// loaded again and the kept address is stale).
//
// Limits: solution estimates only (no gradient statistics), one scene (no scene_id), no walk
// splitting.  A throughput that would split (thr > splitting_threshold = FLT_MAX, i.e. thr
// overflowed to inf) raises the device error word instead of storing a split state.
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <mutex>

#include "zgpu_internal.h"

namespace {

static __device__ __align__(256) unsigned char gStaticScratch[ZGPU_STATIC_SCRATCH_BYTES];

constexpr int kMaxDevices = 64;
std::mutex gSetupMutex;
unsigned char* gScratchAddr[kMaxDevices] = {nullptr};

int fail(int code, const char* fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    zg::setLastError(buf);
    return code;
}

// device address of gStaticScratch on the current device, looked up on first use
int scratchAddress(int device, unsigned char** out) {
    if (device < 0 || device >= kMaxDevices) return fail(ZGPU_ERR_INVALID_ARG, "device %d out of range", device);
    std::lock_guard<std::mutex> lock(gSetupMutex);
    if (!gScratchAddr[device]) {
        void* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, gStaticScratch);
        if (e != cudaSuccess || !p)
            return fail(ZGPU_ERR_CUDA, "cudaGetSymbolAddress(static scratch) failed: %s", cudaGetErrorString(e));
        gScratchAddr[device] = (unsigned char*)p;
    }
    *out = gScratchAddr[device];
    return ZGPU_OK;
}

// carves 256-byte-aligned sub-arrays out of the static scratch
struct Carver {
    unsigned char* base;
    size_t used = 0;
    template <typename T>
    T* take(size_t count) {
        size_t off = (used + 255) & ~size_t(255);
        used = off + count * sizeof(T);
        return (T*)(base + off);
    }
};

}  // namespace

extern "C" int zgpu_solve_static(void* stream, int solver, const zgpu_geometric_queries* q, const zgpu_pde* pde,
                                 const zgpu_walk_settings* ws, const zgpu_sample_points* pts,
                                 zgpu_sample_statistics* stats, zgpu_solve_report* report) {
    using namespace zg;
    if (!q || !pde || !ws || !pts || !stats) return fail(ZGPU_ERR_INVALID_ARG, "NULL required argument");
    if (solver != ZGPU_SOLVER_WALK_ON_SPHERES && solver != ZGPU_SOLVER_WALK_ON_STARS)
        return fail(ZGPU_ERR_INVALID_ARG, "unknown solver %d", solver);
    const int D = q->dim;
    if (D != 2 && D != 3) return fail(ZGPU_ERR_INVALID_ARG, "queries dim must be 2 or 3, got %d", D);
    const int64_t n = pts->n;
    if (n < 0 || n > ZGPU_STATIC_MAX_POINTS)
        return fail(ZGPU_ERR_INVALID_ARG, "zgpu_solve_static takes at most %d points (got %lld); use zgpu_solve",
                    ZGPU_STATIC_MAX_POINTS, (long long)n);
    if (pts->memory != ZGPU_MEM_DEVICE || stats->memory != ZGPU_MEM_DEVICE)
        return fail(ZGPU_ERR_INVALID_ARG, "zgpu_solve_static needs points and statistics in device memory");
    if (n > 0 && (!pts->pt || !pts->dist_to_absorbing || !pts->n_walks || !pts->seed))
        return fail(ZGPU_ERR_INVALID_ARG, "pt, dist_to_absorbing, n_walks and seed are required");
    if (!stats->solution_mean || !stats->solution_m2 || !stats->n_solution_estimates || !stats->total_walk_length ||
        !stats->total_splits)
        return fail(ZGPU_ERR_INVALID_ARG, "statistics arrays are required");
    // solution estimates of one scene only: gradient moments and a scene table would need
    // scratch (and staging) this entry point does not have
    if (stats->gradient_mean || stats->gradient_m2 || stats->n_gradient_estimates)
        return fail(ZGPU_ERR_UNSUPPORTED, "zgpu_solve_static estimates solutions only: pass no gradient statistics");
    if (pts->scene_id)
        return fail(ZGPU_ERR_UNSUPPORTED, "zgpu_solve_static solves one scene: scene_id must be NULL");
    if (!(ws->splitting_threshold >= 3.402823466e+38f))
        return fail(ZGPU_ERR_INVALID_ARG, "zgpu_solve_static does not split walks: splitting_threshold must be FLT_MAX");
    if (ws->max_walk_length <= 0 || !(ws->epsilon_shell_for_absorbing_boundary >= 0.0f) || !(pde->absorption_coeff >= 0.0f))
        return fail(ZGPU_ERR_INVALID_ARG, "invalid walk settings or absorption coefficient");
    // grids must already be on the device: this entry point copies nothing
    if (int st = checkPdeFields(pde, D, false)) return st;
    if (pde->solution.n_terms < 0 || pde->solution.n_terms > ZGPU_MAX_TERMS)
        return fail(ZGPU_ERR_INVALID_ARG, "analytic solution has %d terms (max %d)", pde->solution.n_terms, ZGPU_MAX_TERMS);

    SolveParams P;
    std::memset(&P, 0, sizeof(P));
    P.solver = solver;
    int bdim = 0, bkind = 0;
    if (q->absorbing) {
        BoundaryView v;
        if (!boundaryView(q->absorbing, &v, &bdim, &bkind) || bdim != D || bkind != ZGPU_BOUNDARY_ABSORBING)
            return fail(ZGPU_ERR_INVALID_ARG, "absorbing boundary does not match the queries");
        if (v.nPrims > 0) { P.sc.hasAbs = 1; P.sc.absorbing = v; }
    }
    if (q->reflecting) {
        BoundaryView v;
        if (!boundaryView(q->reflecting, &v, &bdim, &bkind) || bdim != D || bkind == ZGPU_BOUNDARY_ABSORBING)
            return fail(ZGPU_ERR_INVALID_ARG, "reflecting boundary does not match the queries");
        if (v.nPrims > 0) { P.sc.hasRefl = 1; P.sc.reflecting = v; }
    }
    for (int i = 0; i < 3; i++) { P.sc.domainMin[i] = q->domain_min[i]; P.sc.domainMax[i] = q->domain_max[i]; }
    P.sc.ws = *ws;
    P.sc.pde = *pde;
    P.nPoints = n;
    P.pt = pts->pt; P.normal = pts->normal; P.type = pts->type; P.eq = pts->estimation_quantity;
    P.distAbs = pts->dist_to_absorbing; P.nWalks = pts->n_walks; P.seed = pts->seed;
    P.aligned = pts->estimate_normal_aligned;
    P.statMean = stats->solution_mean; P.statM2 = stats->solution_m2; P.statN = stats->n_solution_estimates;
    P.statLen = (long long*)stats->total_walk_length; P.statSplits = (long long*)stats->total_splits;
    P.splitStack = nullptr;   // no split slots: the walk kernel reports a split instead of storing it
    P.stackEntries = 8;
    if (P.sc.hasAbs) P.stackEntries = P.sc.absorbing.stackEntries > P.stackEntries ? P.sc.absorbing.stackEntries : P.stackEntries;
    if (P.sc.hasRefl) P.stackEntries = P.sc.reflecting.stackEntries > P.stackEntries ? P.sc.reflecting.stackEntries : P.stackEntries;

    int device = 0;
    cudaError_t e = cudaGetDevice(&device);
    if (e != cudaSuccess) return fail(ZGPU_ERR_CUDA, "cudaGetDevice: %s", cudaGetErrorString(e));
    unsigned char* base = nullptr;
    int st = scratchAddress(device, &base);
    if (st != ZGPU_OK) return st;

    // carve the scratch: counters first (cleared every call), then the per-point arrays
    Carver cv{base};
    P.counters = cv.take<unsigned long long>(16);
    P.errorWord = (unsigned int*)(P.counters + 8);
    P.walkStart = cv.take<long long>((size_t)n + 1);
    P.pointFlags = cv.take<int>((size_t)n);
    P.nPrev = cv.take<int>((size_t)n);
    P.accSum = cv.take<double>((size_t)n);
    P.accSq = cv.take<double>((size_t)n);
    P.accN = cv.take<int>((size_t)n);
    P.accLen = cv.take<long long>((size_t)n);
    P.accSplits = cv.take<long long>((size_t)n);
    if (pts->first_sphere_radius) { P.fsr = pts->first_sphere_radius; P.fsrPersistent = 1; }
    else { P.fsr = cv.take<float>((size_t)n); P.fsrPersistent = 0; }
    long long* blockSums = cv.take<long long>(scanScratchElems(n));
    if (cv.used > ZGPU_STATIC_SCRATCH_BYTES)
        return fail(ZGPU_ERR_INVALID_ARG, "static scratch too small for %lld points", (long long)n);

    cudaStream_t s = (cudaStream_t)stream;
    int numSMs = 0;
    cudaDeviceGetAttribute(&numSMs, cudaDevAttrMultiProcessorCount, device);
    const int threads = 128;
    int perSM = walkKernelMaxBlocksPerSM(D, solver, threads, P);
    int blocks = numSMs * perSM;

    // the accumulators are cleared by the prepare kernel; the counters and error word here
    if ((e = cudaMemsetAsync(P.counters, 0, 16 * sizeof(unsigned long long), s)) != cudaSuccess)
        return fail(ZGPU_ERR_CUDA, "clearing static counters: %s", cudaGetErrorString(e));
    if ((e = launchPrepare(P, D, s)) != cudaSuccess ||
        (e = launchScan(P.walkStart, n, blockSums, s)) != cudaSuccess ||
        (n > 0 && (e = launchWalk(P, D, blocks, threads, s)) != cudaSuccess) ||
        (e = launchFinalize(P, D, s)) != cudaSuccess)
        return fail(ZGPU_ERR_CUDA, "kernel launch: %s", cudaGetErrorString(e));
    unsigned long long ctr[9] = {0};
    long long totalWalks = 0;
    if ((e = cudaMemcpyAsync(ctr, P.counters, sizeof(ctr), cudaMemcpyDeviceToHost, s)) != cudaSuccess ||
        (e = cudaMemcpyAsync(&totalWalks, P.walkStart + n, sizeof(long long), cudaMemcpyDeviceToHost, s)) != cudaSuccess ||
        (e = cudaStreamSynchronize(s)) != cudaSuccess)
        return fail(ZGPU_ERR_CUDA, "reading back counters: %s", cudaGetErrorString(e));
    unsigned int errWord = (unsigned int)(ctr[8] & 0xffffffffu);
    if (report) {
        std::memset(report, 0, sizeof(*report));
        report->total_steps = ctr[kCtrSteps];
        report->escaped_walks = ctr[kCtrEscaped];
        report->exceeded_walks = ctr[kCtrExceeded];
        report->rr_terminated = ctr[kCtrRR];
        report->total_walks = (uint64_t)totalWalks;
        report->error_word = errWord;
    }
    if (errWord) return fail(ZGPU_ERR_DEVICE_STATE, "device error word 0x%x", errWord);
    return ZGPU_OK;
}
