// zgpu_internal.h -- declarations shared by the kernels (zgpu_walk.cu) and the C ABI
// implementation (zgpu_api.cu).
#pragma once

#include <cuda_runtime.h>
#include "zgpu_scene.cuh"

namespace zg {

// walk completion codes (WalkCompletionCode, point_estimation/common.h:132-137)
enum : int { kReached = 0, kRussianRoulette = 1, kExceeded = 2, kEscaped = 3 };

// counters[] slots
enum : int { kCtrNext = 0, kCtrSteps = 1, kCtrEscaped = 2, kCtrExceeded = 3, kCtrRR = 4, kCtrWalks = 5, kCtrCache = 6,
             kCtrCount = 8 };

// per-point flags written by the prepare kernel
enum : int { kPointBoundaryValue = 1, kPointFlip = 2, kPointGradient = 4 };

// what a walk needs of its problem: boundaries, domain box, settings and PDE
struct SceneDesc {
    int hasAbs, hasRefl;
    BoundaryView absorbing, reflecting;
    float domainMin[3], domainMax[3];
    zgpu_walk_settings ws;
    zgpu_pde pde;
};

struct SolveParams {
    int solver;
    SceneDesc sc;               // the problem of a single-scene solve
    const SceneDesc* scenes;    // batched solve: the scene table (device memory) ...
    const int* sceneId;         // ... and each point's row in it (NULL: single scene)
    int nScenes;
    int batchScreened;          // some scene of the table has an absorption coefficient > 0
    int64_t nPoints;
    // sample points (device)
    const float* pt;
    const float* normal;
    const int* type;
    const int* eq;
    const float* distAbs;
    const int* nWalks;
    const uint64_t* seed;
    const int* aligned;
    float* fsr;
    int fsrPersistent;          // 1: fsr is the caller's array (reuse when n_prev > 0)
    // statistics (device, caller-owned)
    double* statMean;
    double* statM2;
    int* statN;
    double* statGradMean;       // [n][D] (estimateSolutionAndGradient points)
    double* statGradM2;
    int* statGradN;
    const float* distRefl;      // gradient points of Walk on Stars: distance to the reflecting boundary
    const float* dirDeriv;      // [n][D] directionForDerivative (NULL: the first axis)
    double* statFirstSrc;       // running sums of first source contributions (NULL: not kept)
    double* statDeriv;          // running sums of directional derivative contributions
    long long* statLen;
    long long* statSplits;
    // scratch
    long long* walkStart;       // nPoints + 1
    int* pointFlags;            // nPoints
    int* nPrev;                 // nPoints: statN before this call
    double* accSum;
    double* accSq;
    int* accN;
    long long* accLen;
    long long* accSplits;
    double* accGrad;            // [n][D] sums and sums of squares of gradient estimates
    double* accGradSq;
    int* accGradN;
    double* accFirstSrc;        // this call's sums of the two above (NULL when not kept)
    double* accDeriv;
    unsigned long long* counters;
    unsigned int* errorWord;
    float4* splitStack;         // walk threads x kSplitStack x 3 float4
    int stackEntries;           // shared-memory traversal stack entries per thread
    // neural cache: walks end at their first position after a step that lies at least
    // cacheMinDist from the boundary (0 = off) and leave a record (2 float4: position and
    // throughput; partial estimate, point, walk length) for the cache pass
    float cacheMinDist;
    float4* cacheRec;
    long long cacheCap;
    // Walk on Spheres: closest-point queries answered by the whole warp (CoopWork per warp in
    // shared memory after the per-thread stacks)
    int coop;
    // Walk on Stars on a Robin boundary: star radii answered by the whole warp
    int coopStar;
    // cap on loop iterations per walk state (0: none); a walk that reaches it is dropped and
    // kErrBudget raised
    long long stepBudget;
};

// the sorted-wavefront Walk on Stars schedule (zgpu_wave.cuh): its pool of walk records and
// the sort's scratch (device memory)
struct WaveParams {
    const float4* src;        // records of the previous iteration
    float4* dst;              // records of this iteration (sorted, then refilled)
    uint32_t* key;            // [pool] Morton cell of each record of src (kWaveCells: free)
    uint32_t* rank;           // [pool] the record's place in its cell
    uint32_t* count;          // [kWaveCells] records per cell (zeroed by the scan)
    uint32_t* offset;         // [kWaveCells + 1] first slot of each cell in dst
    long long* ctr;           // [0] next walk id, [1] sorted live records, [2] first new id, [3] live slots,
                              // [4] live slots of the previous iteration
    long long pool;           // records per buffer
    int axisBits;             // sort grid: 2^axisBits cells per axis (per scene of a batched solve)
    uint32_t sceneMask;       // batched solves: scene id bits above the cell (mask of the id)
};

enum : int { kWaveNext = 0, kWaveSorted = 1, kWaveFirstNew = 2, kWaveLive = 3, kWavePrevLive = 4, kWaveCtrs = 8 };
// cells of the sort: a 2^kWaveBits2D square grid in 2D, 2^kWaveBits3D cubed in 3D
#ifndef ZG_WAVE_BITS_2D
#define ZG_WAVE_BITS_2D 8
#endif
constexpr int kWaveBits2D = ZG_WAVE_BITS_2D;
constexpr int kWaveBits3D = 5;
constexpr int kWaveCells = 1 << (2 * kWaveBits2D > 3 * kWaveBits3D ? 2 * kWaveBits2D : 3 * kWaveBits3D);

constexpr int kSplitStack = 8;
// Walk on Spheres in 3D answers closest-point queries with a whole warp from this many
// absorbing primitives on (query_mode 0)
constexpr int kCoopMinPrims = 20000;
// Walk on Stars in 3D answers Robin star radii with a whole warp from this many primitives
constexpr int kCoopStarMinPrims = 4096;

// kernels / launchers (zgpu_walk.cu)
cudaError_t launchPrepare(const SolveParams& p, int dim, cudaStream_t s);
cudaError_t launchScan(long long* data, int64_t n, long long* blockSums, cudaStream_t s);
cudaError_t launchWalk(const SolveParams& p, int dim, int blocks, int threads, cudaStream_t s);
cudaError_t launchFinalize(const SolveParams& p, int dim, cudaStream_t s);
// one iteration of the sorted-wavefront walk loop (zgpu_wave.cuh); blocks: of the step
// kernels (numSMs x waveBlocksPerSM)
cudaError_t launchWaveIteration(const SolveParams& p, const WaveParams& w, int dim, int blocks, int numSMs, cudaStream_t s);
// the live records of w.dst to the end of their walks (the wavefront's tail)
cudaError_t launchWaveDrain(const SolveParams& p, const WaveParams& w, int dim, int blocks, cudaStream_t s);
int waveBlocksPerSM(int dim, int solver, bool screened, bool batched);
int waveRecordVec(int dim);
int waveLaunchesPerIteration(int solver);
int walkKernelMaxBlocksPerSM(int dim, int solver, int threads, const SolveParams& p);
// validates a PDE's field kinds and grids (hostGrids: grid values may be in host memory)
int checkPdeFields(const zgpu_pde* pde, int D, bool hostGrids);
// neural cache pass over the walk records (zgpu_cache.cu)
cudaError_t launchCacheAccumulate(const zgpu_cache* c, const float4* rec, const unsigned long long* recCount,
                                  int64_t cap, double* accSum, double* accSq, int* accN, long long* accLen,
                                  unsigned int* errw, cudaStream_t s);
int cacheDim(const zgpu_cache* c);
cudaStream_t cacheStream(const zgpu_cache* c);
int contextDevice(const zgpu_context* ctx);
size_t scanScratchElems(int64_t n);

// device-side LBVH build of an absorbing boundary's 4-wide tree (zgpu_devbuild.cu)
// a boundary built on the device (zgpu_devbuild.cu): device arrays owned by the receiver
struct DeviceBuilt {
    float4* nodes = nullptr;
    float4* cones = nullptr;       // reflecting boundaries
    float4* prims = nullptr;
    float4* sil = nullptr;         // reflecting boundaries
    int* primIndex = nullptr;
    float4* silTree = nullptr;     // reflecting boundaries with silhouette candidates
    float4* silCones = nullptr;
    float4* silFeat = nullptr;
    int nNodes = 0, depth = 0, silNodes = 0, silDepth = 0, silFeatures = 0;
};
// pos [nV * D], idx [nP * D], kmin / kmax [nP] (Robin) in device memory; kind 0 absorbing,
// 1 Neumann, 2 Robin.  cudaErrorNotSupported: a tree deeper than the traversal stack.
cudaError_t buildBoundaryOnDevice(int D, const float* pos, int nV, const int* idx, int nP, int kind, const float* kmin,
                                  const float* kmax, bool doubleSided, float prec, cudaStream_t s, DeviceBuilt& out);

// Boundary Value Caching splat (zgpu_bvc.cu): device arrays of one cache and of the
// evaluation points, one statistic group per launch
struct BvcSplatParams {
    int64_t nSamples;
    const float* pt;
    const float* normal;
    const float* pdf;
    const int* type;
    const int* aligned;
    const float* solution;
    const float* normalDerivative;
    const float* contribution;
    const float* robinCoeff;
    int64_t nEval;
    const float* evalPt;
    const int* evalType;
    const float* evalDistA;
    const float* evalDistR;
    double* mean;
    double* m2;
    int* count;
    double* gradMean;
    double* gradM2;
    float sqrtLambda, radiusClamp, regularization, robinCutoff, cutoffA, cutoffR;
    int group;
    // cache split across grid.y: splitChunk samples per block row; partial moments
    // [split][eval][3 + 2 dim] merged by a second kernel (NULL: one split, merged in place)
    int64_t splitChunk;
    double* partial;
};
// splits of the cache for nEval points on numSMs SMs; the partial buffer needs
// splits * nEval * (3 + 2 dim) doubles when splits > 1
int bvcSplitCount(int64_t nEval, int64_t nSamples, int numSMs);
cudaError_t launchBvcSplat(int D, bool screened, const BvcSplatParams& p, int splits, cudaStream_t s);
cudaError_t launchPdeEvaluate(int D, const zgpu_pde& pde, int64_t n, const float* x, const float* nrm, const int* aligned,
                              float* src, float* dir, float* rob, float* kap, cudaStream_t s);

// a 4-wide BVH over points (reverse walks' radius searches, zgpu_devbuild.cu): nodes as the
// boundary trees', order[sorted slot] = point index; device arrays owned by the receiver
cudaError_t buildPointBvhOnDevice(int D, const float* pts, int n, cudaStream_t s, float4** nodes, int* nNodes,
                                  int* depth, int** order, int2** childRanges);

// reverse Walk on Stars (zgpu_rws.cu)
struct RwsParams {
    SceneDesc sc;
    int64_t nSamples;
    const float* pt;
    const float* normal;
    const int* type;
    const int* aligned;
    const float* pdf;
    const float* contribution;
    const float* distAbs;
    const uint64_t* seed;
    uint64_t stream;
    int64_t nEval;
    const float* evalPt;
    const float* evalNormal;
    const int* evalType;
    double* totals;
    const float4* evalNodes;       // point BVH over the evaluation points
    const int* evalOrder;
    const int2* evalRanges;        // per wide child: (first sorted slot, count)
    int evalDepth;
    float normalOffset, radiusClamp, regularization;
    int selfNormalize;
    int stackEntries;
    unsigned long long* counters;  // [0] steps, [1] walks
    unsigned int* errorWord;
};
cudaError_t launchReverseWalks(int D, bool screened, const RwsParams& p, int blocks, cudaStream_t s);

// accessors into the C ABI objects (zgpu_api.cu)
void setLastError(const char* msg);
bool boundaryView(const zgpu_boundary* b, BoundaryView* view, int* dim, int* kind);

// batched query kernels
cudaError_t launchClosest(const BoundaryView& b, int dim, int64_t n, const float* x, int computeSigned,
                          float* pt, float* nrm, float* dist, int* prim, unsigned int* err, cudaStream_t s);
cudaError_t launchIntersect(const BoundaryView& b, int dim, int64_t n, const float* o, const float* nrmIn,
                            const float* dir, const float* tmax, const int* onb, int* hit, float* pt, float* nrm,
                            float* dist, int* prim, unsigned int* err, cudaStream_t s);
cudaError_t launchCountHits(const BoundaryView& b, int dim, int64_t n, const float* o, const float* dir,
                            const float* tmax, int* out, unsigned int* err, cudaStream_t s);
cudaError_t launchStarRadius(const BoundaryView& b, int dim, int64_t n, const float* x, const float* minR,
                             const float* maxR, float prec, const int* flip, float* out, unsigned int* err,
                             cudaStream_t s);
// the same queries answered by one warp per query (closest points; Robin star radii)
cudaError_t launchClosestCoop(const BoundaryView& b, int dim, int64_t n, const float* x, int computeSigned,
                              float* pt, float* nrm, float* dist, int* prim, unsigned int* err, cudaStream_t s);
cudaError_t launchStarRadiusCoop(const BoundaryView& b, int dim, int64_t n, const float* x, const float* minR,
                                 const float* maxR, float prec, const int* flip, float* out, unsigned int* err,
                                 cudaStream_t s);
cudaError_t launchOccluded(const BoundaryView& b, int dim, int64_t n, const float* xi, const float* xj,
                           const float* ni, const float* nj, const int* oi, const int* oj, int* out,
                           unsigned int* err, cudaStream_t s);
cudaError_t launchSample(const BoundaryView& b, int dim, int64_t n, const float* x, const float* r, const float* u,
                         int* found, float* pt, float* nrm, float* pdf, cudaStream_t s);

}  // namespace zg
