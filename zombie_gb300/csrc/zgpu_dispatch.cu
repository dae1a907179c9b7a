// zgpu_dispatch.cu -- dimension dispatch of the kernel launchers and the walk-id scan.
#include "zgpu_wave.cuh"

namespace zg {

extern template struct Launch<2>;
extern template struct Launch<3>;
extern template struct WalkLaunch<2, ZGPU_SOLVER_WALK_ON_SPHERES>;
extern template struct WalkLaunch<2, ZGPU_SOLVER_WALK_ON_STARS>;
extern template struct WalkLaunch<3, ZGPU_SOLVER_WALK_ON_SPHERES>;
extern template struct WalkLaunch<3, ZGPU_SOLVER_WALK_ON_STARS>;
extern template struct WaveLaunch<2, ZGPU_SOLVER_WALK_ON_SPHERES>;
extern template struct WaveLaunch<2, ZGPU_SOLVER_WALK_ON_STARS>;
extern template struct WaveLaunch<3, ZGPU_SOLVER_WALK_ON_SPHERES>;
extern template struct WaveLaunch<3, ZGPU_SOLVER_WALK_ON_STARS>;

namespace detail {
// ------------------------------------------------------------------------- scan
constexpr int kScanBlock = 1024;

__global__ void scanBlocks(long long* data, int64_t n, long long* blockSums) {
    __shared__ long long s[kScanBlock];
    int64_t i = (int64_t)blockIdx.x * kScanBlock + threadIdx.x;
    long long v = i < n ? data[i] : 0;
    s[threadIdx.x] = v;
    __syncthreads();
    for (int off = 1; off < kScanBlock; off <<= 1) {
        long long t = threadIdx.x >= off ? s[threadIdx.x - off] : 0;
        __syncthreads();
        s[threadIdx.x] += t;
        __syncthreads();
    }
    if (i < n) data[i] = s[threadIdx.x] - v;   // exclusive
    if (threadIdx.x == kScanBlock - 1) blockSums[blockIdx.x] = s[threadIdx.x];
}
// single block: exclusive scan of the block sums in chunks, writes the grand total to data[n]
__global__ void scanSums(long long* blockSums, int64_t nb, long long* data, int64_t n) {
    __shared__ long long s[kScanBlock];
    __shared__ long long carry;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    for (int64_t base = 0; base < nb; base += kScanBlock) {
        int64_t i = base + threadIdx.x;
        long long v = i < nb ? blockSums[i] : 0;
        s[threadIdx.x] = v;
        __syncthreads();
        for (int off = 1; off < kScanBlock; off <<= 1) {
            long long t = threadIdx.x >= off ? s[threadIdx.x - off] : 0;
            __syncthreads();
            s[threadIdx.x] += t;
            __syncthreads();
        }
        if (i < nb) blockSums[i] = carry + s[threadIdx.x] - v;
        __syncthreads();
        if (threadIdx.x == kScanBlock - 1) carry += s[threadIdx.x];
        __syncthreads();
    }
    if (threadIdx.x == 0) data[n] = carry;
}
__global__ void scanAdd(long long* data, int64_t n, const long long* blockSums) {
    int64_t i = (int64_t)blockIdx.x * kScanBlock + threadIdx.x;
    if (i < n) data[i] += blockSums[blockIdx.x];
}

}  // namespace detail

cudaError_t launchPrepare(const SolveParams& p, int dim, cudaStream_t s) {
    return dim == 2 ? Launch<2>::prepare(p, s) : Launch<3>::prepare(p, s);
}
size_t scanScratchElems(int64_t n) { return (size_t)((n + detail::kScanBlock - 1) / detail::kScanBlock) + 1; }
cudaError_t launchScan(long long* data, int64_t n, long long* blockSums, cudaStream_t s) {
    int64_t nb = (n + detail::kScanBlock - 1) / detail::kScanBlock;
    if (nb > 0) detail::scanBlocks<<<(unsigned)nb, detail::kScanBlock, 0, s>>>(data, n, blockSums);
    detail::scanSums<<<1, detail::kScanBlock, 0, s>>>(blockSums, nb, data, n);
    if (nb > 0) detail::scanAdd<<<(unsigned)nb, detail::kScanBlock, 0, s>>>(data, n, blockSums);
    return cudaGetLastError();
}
cudaError_t launchWalk(const SolveParams& p, int dim, int blocks, int threads, cudaStream_t s) {
    bool wos = p.solver == ZGPU_SOLVER_WALK_ON_SPHERES;
    if (dim == 2) return wos ? WalkLaunch<2, ZGPU_SOLVER_WALK_ON_SPHERES>::walk(p, blocks, threads, s)
                             : WalkLaunch<2, ZGPU_SOLVER_WALK_ON_STARS>::walk(p, blocks, threads, s);
    return wos ? WalkLaunch<3, ZGPU_SOLVER_WALK_ON_SPHERES>::walk(p, blocks, threads, s)
               : WalkLaunch<3, ZGPU_SOLVER_WALK_ON_STARS>::walk(p, blocks, threads, s);
}
#define ZG_WAVE_DISPATCH(dim, solver, CALL)                                                          \
    ((dim) == 2 ? ((solver) == ZGPU_SOLVER_WALK_ON_SPHERES ? WaveLaunch<2, ZGPU_SOLVER_WALK_ON_SPHERES>::CALL \
                                                          : WaveLaunch<2, ZGPU_SOLVER_WALK_ON_STARS>::CALL)   \
                : ((solver) == ZGPU_SOLVER_WALK_ON_SPHERES ? WaveLaunch<3, ZGPU_SOLVER_WALK_ON_SPHERES>::CALL \
                                                          : WaveLaunch<3, ZGPU_SOLVER_WALK_ON_STARS>::CALL))
cudaError_t launchWaveIteration(const SolveParams& p, const WaveParams& w, int dim, int blocks, int numSMs, cudaStream_t s) {
    return ZG_WAVE_DISPATCH(dim, p.solver, iterate(p, w, blocks, numSMs, s));
}
cudaError_t launchWaveDrain(const SolveParams& p, const WaveParams& w, int dim, int blocks, cudaStream_t s) {
    return ZG_WAVE_DISPATCH(dim, p.solver, drain(p, w, blocks, s));
}
int waveBlocksPerSM(int dim, int solver, bool screened, bool batched) {
    return ZG_WAVE_DISPATCH(dim, solver, blocksPerSM(screened, batched));
}
int waveRecordVec(int dim) { return dim == 2 ? WaveLaunch<2, ZGPU_SOLVER_WALK_ON_STARS>::kVec : WaveLaunch<3, ZGPU_SOLVER_WALK_ON_STARS>::kVec; }
int waveLaunchesPerIteration(int solver) {
    return solver == ZGPU_SOLVER_WALK_ON_SPHERES ? WaveLaunch<2, ZGPU_SOLVER_WALK_ON_SPHERES>::kLaunches
                                                 : WaveLaunch<2, ZGPU_SOLVER_WALK_ON_STARS>::kLaunches;
}
#undef ZG_WAVE_DISPATCH
int walkKernelMaxBlocksPerSM(int dim, int solver, int threads, const SolveParams& p) {
    const bool wos = solver == ZGPU_SOLVER_WALK_ON_SPHERES;
    const size_t smem = walkSmemBytes(p, threads);
    if (dim == 2) return wos ? WalkLaunch<2, ZGPU_SOLVER_WALK_ON_SPHERES>::maxBlocksPerSM(p, threads, smem)
                             : WalkLaunch<2, ZGPU_SOLVER_WALK_ON_STARS>::maxBlocksPerSM(p, threads, smem);
    return wos ? WalkLaunch<3, ZGPU_SOLVER_WALK_ON_SPHERES>::maxBlocksPerSM(p, threads, smem)
               : WalkLaunch<3, ZGPU_SOLVER_WALK_ON_STARS>::maxBlocksPerSM(p, threads, smem);
}
cudaError_t launchFinalize(const SolveParams& p, int dim, cudaStream_t s) {
    return dim == 2 ? Launch<2>::finalize(p, s) : Launch<3>::finalize(p, s);
}
cudaError_t launchClosest(const BoundaryView& b, int dim, int64_t n, const float* x, int computeSigned, float* pt,
                          float* nrm, float* dist, int* prim, unsigned int* err, cudaStream_t s) {
    return dim == 2 ? Launch<2>::closest(b, n, x, computeSigned, pt, nrm, dist, prim, err, s)
                    : Launch<3>::closest(b, n, x, computeSigned, pt, nrm, dist, prim, err, s);
}
cudaError_t launchClosestCoop(const BoundaryView& b, int dim, int64_t n, const float* x, int computeSigned, float* pt,
                              float* nrm, float* dist, int* prim, unsigned int* err, cudaStream_t s) {
    return dim == 2 ? Launch<2>::closestCoop(b, n, x, computeSigned, pt, nrm, dist, prim, err, s)
                    : Launch<3>::closestCoop(b, n, x, computeSigned, pt, nrm, dist, prim, err, s);
}
cudaError_t launchStarRadiusCoop(const BoundaryView& b, int dim, int64_t n, const float* x, const float* minR,
                                 const float* maxR, float prec, const int* flip, float* out, unsigned int* err,
                                 cudaStream_t s) {
    return dim == 2 ? Launch<2>::starRadiusCoop(b, n, x, minR, maxR, prec, flip, out, err, s)
                    : Launch<3>::starRadiusCoop(b, n, x, minR, maxR, prec, flip, out, err, s);
}
cudaError_t launchIntersect(const BoundaryView& b, int dim, int64_t n, const float* o, const float* nrmIn,
                            const float* dir, const float* tmax, const int* onb, int* hit, float* pt, float* nrm,
                            float* dist, int* prim, unsigned int* err, cudaStream_t s) {
    return dim == 2 ? Launch<2>::intersect(b, n, o, nrmIn, dir, tmax, onb, hit, pt, nrm, dist, prim, err, s)
                    : Launch<3>::intersect(b, n, o, nrmIn, dir, tmax, onb, hit, pt, nrm, dist, prim, err, s);
}
cudaError_t launchCountHits(const BoundaryView& b, int dim, int64_t n, const float* o, const float* dir,
                            const float* tmax, int* out, unsigned int* err, cudaStream_t s) {
    return dim == 2 ? Launch<2>::countHits(b, n, o, dir, tmax, out, err, s) : Launch<3>::countHits(b, n, o, dir, tmax, out, err, s);
}
cudaError_t launchStarRadius(const BoundaryView& b, int dim, int64_t n, const float* x, const float* minR,
                             const float* maxR, float prec, const int* flip, float* out, unsigned int* err,
                             cudaStream_t s) {
    return dim == 2 ? Launch<2>::starRadius(b, n, x, minR, maxR, prec, flip, out, err, s)
                    : Launch<3>::starRadius(b, n, x, minR, maxR, prec, flip, out, err, s);
}
cudaError_t launchOccluded(const BoundaryView& b, int dim, int64_t n, const float* xi, const float* xj,
                           const float* ni, const float* nj, const int* oi, const int* oj, int* out,
                           unsigned int* err, cudaStream_t s) {
    return dim == 2 ? Launch<2>::occluded(b, n, xi, xj, ni, nj, oi, oj, out, err, s)
                    : Launch<3>::occluded(b, n, xi, xj, ni, nj, oi, oj, out, err, s);
}
cudaError_t launchSample(const BoundaryView& b, int dim, int64_t n, const float* x, const float* r, const float* u,
                         int* found, float* pt, float* nrm, float* pdf, cudaStream_t s) {
    return dim == 2 ? Launch<2>::sample(b, n, x, r, u, found, pt, nrm, pdf, s)
                    : Launch<3>::sample(b, n, x, r, u, found, pt, nrm, pdf, s);
}

}  // namespace zg
