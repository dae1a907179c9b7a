// zgpu_wave.cuh -- the sorted-wavefront schedule of the walk loop (Walk on Stars and Walk on Spheres).
//
// The persistent walk kernel gives every lane one walk from start to end: after a few steps
// the 32 walks of a warp are spread over the domain, their traversals visit unrelated tree
// nodes, and the warp runs each query as long as its slowest lane.  This schedule keeps a
// pool of walk states as fixed-size records in device memory instead and runs the walk loop
// as iterations of six launches:
//   1. waveKeyKernel: each live record's Morton cell of its position (a 2^kWaveBits2D square
//      grid in 2D, 2^kWaveBits3D cubed in 3D, over the domain box; a batched solve puts the
//      scene id above a coarser grid over the scene's own box) and its rank within the cell
//      (one atomicAdd on the cell's count per group of warp lanes sharing the cell);
//   2. waveScanKernel (one block): exclusive sum of the cell counts, the pool's live count,
//      and the range of new walk ids that fills the free slots;
//   3. waveScatterKernel: copies each live record to its cell's range of the other buffer, so
//      the pool is ordered by cell and the warps of the next two kernels run neighbouring
//      walks, whose traversals share their nodes;
//   4. waveRefillKernel: starts new walks (consecutive ids, so consecutive walks of a point)
//      in the slots after the sorted records, up to the new live count;
//   5.-6. wavePhaseKernel<0> and <1>: one Walk on Stars step over the live slots, split at
//      the star radius (Walker::waveRadius / waveAdvance); Walk on Spheres runs its step as
//      one kernel, wavePhaseKernel<2> (Walker::waveStepWoS).
// Once every walk has started and no more live records are left than the step kernels have
// resident threads, waveDrainKernel runs each remaining record to the end of its walk in a
// loop: the walks finishing last would otherwise take hundreds of iterations of launches.
// A walk's random numbers and arithmetic are those of the persistent kernel; only the order
// in which walks finish, and so the order of the FP64 sums per point, differs.
// A step reads its record four times and writes it three times (key, scatter, two phases):
// about 0.5 KB of HBM traffic per walk step in 2D, which buys coherent queries.
#pragma once

#include "zgpu_kernels.cuh"

namespace zg {

constexpr int kWaveScanThreads = 1024;
// resident blocks per SM the step kernels are compiled for (48 registers); measured on the
// default 2D Walk on Stars workload: 10 ahead of 8 (-1.4%) and 6 (-3%)
#ifndef ZG_WAVE_MIN_BLOCKS
#define ZG_WAVE_MIN_BLOCKS 10
#endif

namespace detail {

ZG_D uint32_t spreadBits2(uint32_t v) {   // up to 16 bits -> every second bit
    v = (v | (v << 8)) & 0x00FF00FFu;
    v = (v | (v << 4)) & 0x0F0F0F0Fu;
    v = (v | (v << 2)) & 0x33333333u;
    v = (v | (v << 1)) & 0x55555555u;
    return v;
}
ZG_D uint32_t spreadBits3(uint32_t v) {   // 5 bits -> every third of 15
    v = (v | (v << 8)) & 0x100Fu;
    v = (v | (v << 4)) & 0x10C3u;
    v = (v | (v << 2)) & 0x1249u;
    return v;
}

// Morton cell of x in a 2^bits-per-axis grid over the scene's domain box
template <int D>
ZG_D uint32_t waveCell(const SceneDesc& sc, const float* x, int bits) {
    const float cells = (float)(1 << bits);
    uint32_t c[D];
#pragma unroll
    for (int i = 0; i < D; i++) {
        const float ext = sc.domainMax[i] - sc.domainMin[i];
        float t = ext > 0.0f ? (x[i] - sc.domainMin[i]) * (cells / ext) : 0.0f;
        t = fminf(fmaxf(t, 0.0f), cells - 1.0f);   // NaN -> 0
        c[i] = (uint32_t)t;
    }
    if (D == 2) return spreadBits2(c[0]) | (spreadBits2(c[1]) << 1);
    return spreadBits3(c[0]) | (spreadBits3(c[1]) << 1) | (spreadBits3(c[D - 1]) << 2);
}

// cell and in-cell rank of the records [0, live) of src; lanes of a warp that share a cell
// (most of them: the records are in cell order from the previous sort) take their ranks
// from one atomicAdd.  A batched solve's key is its scene above the cell in the scene's box.
template <int D, int SOLVER, bool BATCHED>
__global__ void __launch_bounds__(256) waveKeyKernel(const __grid_constant__ SolveParams P, const WaveParams W) {
    using WalkerT = Walker<D, ZGPU_SOLVER_WALK_ON_STARS, false, false, false>;
    constexpr int vec = WalkerT::kWaveVec, pw = WalkerT::kWavePointWord;
    const long long live = W.ctr[kWaveLive];
    const int lane = threadIdx.x & 31;
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long base = (long long)blockIdx.x * blockDim.x + (threadIdx.x & ~31); base < live; base += stride) {
        const long long i = base + lane;
        uint32_t k = kWaveCells;
        if (i < live) {
            const float4* r = W.src + i * vec;
            const float4 q = r[pw / 4];
            const float pwv[4] = {q.x, q.y, q.z, q.w};
            const int point = __float_as_int(pwv[pw % 4]);
            if (point >= 0) {
                const float4 a = r[0];
                const float x[3] = {a.x, a.y, a.z};
                if constexpr (BATCHED) {
                    const int scene = __ldg(P.sceneId + point);
                    k = ((uint32_t)scene & W.sceneMask) << (D * W.axisBits) | waveCell<D>(P.scenes[scene], x, W.axisBits);
                } else {
                    k = waveCell<D>(P.sc, x, W.axisBits);
                }
            }
        }
        const unsigned peers = __match_any_sync(kFull, k);
        const int leader = __ffs(peers) - 1;
        uint32_t first = 0;
        if (lane == leader && k < kWaveCells) first = atomicAdd(W.count + k, (uint32_t)__popc(peers));
        first = __shfl_sync(kFull, first, leader);
        if (i < live) {
            W.key[i] = k;
            W.rank[i] = first + __popc(peers & ((1u << lane) - 1u));
        }
    }
}

// one block: exclusive sum of the cell counts, then the refill range (a template only so that
// each translation unit's instance stays its own)
template <int D, int SOLVER>
__global__ void __launch_bounds__(kWaveScanThreads) waveScanKernel(const __grid_constant__ SolveParams P, const WaveParams W) {
    constexpr int n = kWaveCells;
    constexpr int per4 = n / kWaveScanThreads / 4;   // uint4 per thread
    static_assert(per4 >= 1 && per4 * 4 * kWaveScanThreads == n, "cells per scan thread");
    __shared__ uint32_t warpSum[kWaveScanThreads / 32];
    const int t = threadIdx.x, lane = t & 31, wid = t >> 5;
    const uint4* cnt4 = reinterpret_cast<const uint4*>(W.count) + (size_t)t * per4;
    uint32_t s = 0;
#pragma unroll
    for (int j = 0; j < per4; j++) { const uint4 c = cnt4[j]; s += c.x + c.y + c.z + c.w; }
    uint32_t incl = s;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t v = __shfl_up_sync(kFull, incl, o);
        if (lane >= o) incl += v;
    }
    if (lane == 31) warpSum[wid] = incl;
    __syncthreads();
    if (wid == 0) {
        uint32_t w = warpSum[lane];
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t v = __shfl_up_sync(kFull, w, o);
            if (lane >= o) w += v;
        }
        warpSum[lane] = w;   // inclusive over warps
    }
    __syncthreads();
    uint32_t run = incl - s + (wid > 0 ? warpSum[wid - 1] : 0u);
    uint4* off4 = reinterpret_cast<uint4*>(W.offset) + (size_t)t * per4;
    uint4* zero4 = reinterpret_cast<uint4*>(W.count) + (size_t)t * per4;
#pragma unroll
    for (int j = 0; j < per4; j++) {
        const uint4 c = cnt4[j];
        uint4 o;
        o.x = run; run += c.x;
        o.y = run; run += c.y;
        o.z = run; run += c.z;
        o.w = run; run += c.w;
        off4[j] = o;
        zero4[j] = make_uint4(0u, 0u, 0u, 0u);
    }
    if (t == kWaveScanThreads - 1) {
        const long long sorted = (long long)run;   // every live record has a cell
        W.offset[n] = run;
        const long long total = __ldg(P.walkStart + P.nPoints);
        const long long next = W.ctr[kWaveNext];
        long long fresh = W.pool - sorted;
        if (fresh > total - next) fresh = total - next;
        if (fresh < 0) fresh = 0;
        W.ctr[kWavePrevLive] = W.ctr[kWaveLive];
        W.ctr[kWaveSorted] = sorted;
        W.ctr[kWaveFirstNew] = next;
        W.ctr[kWaveNext] = next + fresh;
        W.ctr[kWaveLive] = sorted + fresh;
    }
}

template <int D, int SOLVER>
__global__ void __launch_bounds__(256) waveScatterKernel(const WaveParams W) {
    using WalkerT = Walker<D, ZGPU_SOLVER_WALK_ON_STARS, false, false, false>;
    constexpr int vec = WalkerT::kWaveVec;
    const long long n = W.ctr[kWavePrevLive];
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const uint32_t k = W.key[i];
        if (k >= kWaveCells) continue;
        const long long d = (long long)W.offset[k] + W.rank[i];
        const float4* r = W.src + i * vec;
        float4* o = W.dst + d * vec;
#pragma unroll
        for (int v = 0; v < vec; v++) o[v] = r[v];
    }
}

// new walks in the slots [sorted, live) after the sorted records (slots from live on are
// never read: every kernel stops at the live count)
template <int D, int SOLVER, bool SCREENED, bool BATCHED>
__global__ void __launch_bounds__(kWalkThreads) waveRefillKernel(const __grid_constant__ SolveParams P, const WaveParams W) {
    using WalkerT = Walker<D, SOLVER, SCREENED, BATCHED, false>;
    constexpr int vec = WalkerT::kWaveVec;
    int stackNode[kMaxStack];
    float stackKey[kMaxStack];
    TravStack S{stackNode, stackKey, 1, P.stackEntries};
    WalkerT walker(P, S);
    walker.splitSlots = nullptr;
    const long long sorted = W.ctr[kWaveSorted], live = W.ctr[kWaveLive], first = W.ctr[kWaveFirstNew];
    const int lane = threadIdx.x & 31;
    const long long warps = (long long)gridDim.x * (blockDim.x >> 5);
    for (long long lo = sorted + ((long long)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5)) * 32; lo < live;
         lo += warps * 32) {
        // the point of the warp's first new walk, then each lane's by a short forward scan
        const long long id0 = first + (lo - sorted);
        const int p0 = warpFindPoint(P, id0, lane);
        const long long slot = lo + lane;
        if (slot < live) {
            const long long id = first + (slot - sorted);
            int p = p0;
            while (__ldg(P.walkStart + p + 1) <= id) p++;
            walker.start(id, p);
            walker.waveStore(W.dst + slot * vec);
        }
    }
}

// PHASE 0 / 1: the two kernels of a Walk on Stars step; 2: a Walk on Spheres step
template <int D, int SOLVER, bool SCREENED, bool BATCHED, int PHASE>
__global__ void __launch_bounds__(kWalkThreads, ZG_WAVE_MIN_BLOCKS) wavePhaseKernel(const __grid_constant__ SolveParams P,
                                                                                      const WaveParams W) {
    using WalkerT = Walker<D, SOLVER, SCREENED, BATCHED, false>;
    constexpr int vec = WalkerT::kWaveVec, pw = WalkerT::kWavePointWord;
    int stackNode[kMaxStack];
    float stackKey[kMaxStack];
    TravStack S{stackNode, stackKey, 1, P.stackEntries};
    WalkerT walker(P, S);
    walker.splitSlots = nullptr;
    const long long live = W.ctr[kWaveLive];
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < live; i += (long long)gridDim.x * blockDim.x) {
        float4* r = W.dst + i * vec;
        if (reinterpret_cast<const int*>(r)[pw] < 0) continue;
        walker.waveLoad(r);
        bool alive;
        if constexpr (PHASE == 0) alive = walker.waveRadius();
        else if constexpr (PHASE == 1) alive = walker.waveAdvance();
        else alive = walker.waveStepWoS();
        if (alive) walker.waveStore(r);
        else reinterpret_cast<int*>(r)[pw] = -1;
    }
    unsigned long long v[4] = {walker.steps, walker.escaped, walker.exceeded, walker.rr};
#pragma unroll
    for (int k = 0; k < 4; k++)
        for (int o = 16; o > 0; o >>= 1) v[k] += __shfl_xor_sync(kFull, v[k], o);
    uint32_t e = walker.err;
    for (int o = 16; o > 0; o >>= 1) e |= __shfl_xor_sync(kFull, e, o);
    if ((threadIdx.x & 31) == 0) {
        if (v[0]) atomicAdd(P.counters + kCtrSteps, v[0]);
        if (v[1]) atomicAdd(P.counters + kCtrEscaped, v[1]);
        if (v[2]) atomicAdd(P.counters + kCtrExceeded, v[2]);
        if (v[3]) atomicAdd(P.counters + kCtrRR, v[3]);
        if (e) atomicOr(P.errorWord, e);
    }
}

// the tail: once every walk has started and the live records are few, each thread runs its
// records to the end of their walks (no sort, no per-step launch); the same step members,
// so the same walks
template <int D, int SOLVER, bool SCREENED, bool BATCHED>
__global__ void __launch_bounds__(kWalkThreads, ZG_WAVE_MIN_BLOCKS) waveDrainKernel(const __grid_constant__ SolveParams P,
                                                                                      const WaveParams W) {
    using WalkerT = Walker<D, SOLVER, SCREENED, BATCHED, false>;
    constexpr int vec = WalkerT::kWaveVec, pw = WalkerT::kWavePointWord;
    int stackNode[kMaxStack];
    float stackKey[kMaxStack];
    TravStack S{stackNode, stackKey, 1, P.stackEntries};
    WalkerT walker(P, S);
    walker.splitSlots = nullptr;
    const long long live = W.ctr[kWaveLive];
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < live; i += (long long)gridDim.x * blockDim.x) {
        const float4* r = W.dst + i * vec;
        if (reinterpret_cast<const int*>(r)[pw] < 0) continue;
        walker.waveLoad(r);
        if constexpr (SOLVER == ZGPU_SOLVER_WALK_ON_STARS) {
            while (walker.waveRadius() && walker.waveAdvance()) {}
        } else {
            while (walker.waveStepWoS()) {}
        }
    }
    unsigned long long v[4] = {walker.steps, walker.escaped, walker.exceeded, walker.rr};
#pragma unroll
    for (int k = 0; k < 4; k++)
        for (int o = 16; o > 0; o >>= 1) v[k] += __shfl_xor_sync(kFull, v[k], o);
    uint32_t e = walker.err;
    for (int o = 16; o > 0; o >>= 1) e |= __shfl_xor_sync(kFull, e, o);
    if ((threadIdx.x & 31) == 0) {
        if (v[0]) atomicAdd(P.counters + kCtrSteps, v[0]);
        if (v[1]) atomicAdd(P.counters + kCtrEscaped, v[1]);
        if (v[2]) atomicAdd(P.counters + kCtrExceeded, v[2]);
        if (v[3]) atomicAdd(P.counters + kCtrRR, v[3]);
        if (e) atomicOr(P.errorWord, e);
    }
}

}  // namespace detail

// launchers of one wavefront iteration, instantiated with each solver's walk kernels
template <int D, int SOLVER>
struct WaveLaunch {
    static constexpr bool kStars = SOLVER == ZGPU_SOLVER_WALK_ON_STARS;
    static constexpr int kVec = detail::Walker<D, SOLVER, false, false, false>::kWaveVec;
    static constexpr int kStepKernels = kStars ? 2 : 1;
    static constexpr int kLaunches = 4 + kStepKernels;   // per iteration
    template <bool SCREENED, bool BATCHED>
    static const void* phaseOf(int k) {
        if constexpr (!kStars) return (const void*)detail::wavePhaseKernel<D, SOLVER, SCREENED, BATCHED, 2>;
        else return k == 0 ? (const void*)detail::wavePhaseKernel<D, SOLVER, SCREENED, BATCHED, 0>
                           : (const void*)detail::wavePhaseKernel<D, SOLVER, SCREENED, BATCHED, 1>;
    }
    static const void* phase(bool screened, bool batched, int k) {
        if (batched) return screened ? phaseOf<true, true>(k) : phaseOf<false, true>(k);
        return screened ? phaseOf<true, false>(k) : phaseOf<false, false>(k);
    }
    template <bool SCREENED, bool BATCHED>
    static void refill(const SolveParams& p, const WaveParams& w, int numSMs, cudaStream_t s) {
        detail::waveRefillKernel<D, SOLVER, SCREENED, BATCHED><<<numSMs * 8, detail::kWalkThreads, 0, s>>>(p, w);
    }
    template <bool SCREENED, bool BATCHED>
    static void drainWith(const SolveParams& p, const WaveParams& w, int blocks, cudaStream_t s) {
        detail::waveDrainKernel<D, SOLVER, SCREENED, BATCHED><<<blocks, detail::kWalkThreads, 0, s>>>(p, w);
    }
    static bool screenedOf(const SolveParams& p) {
        return p.sceneId ? p.batchScreened != 0 : p.sc.pde.absorption_coeff > 0.0f;
    }
    static int blocksPerSM(bool screened, bool batched) {
        int best = 1 << 30;
        for (int k = 0; k < kStepKernels; k++) {
            int b = 0;
            if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, phase(screened, batched, k), detail::kWalkThreads, 0) != cudaSuccess) b = 1;
            best = b < best ? b : best;
        }
        return best > 0 ? best : 1;
    }
    static cudaError_t iterate(const SolveParams& p, const WaveParams& w, int blocks, int numSMs, cudaStream_t s) {
        const bool screened = screenedOf(p), batched = p.sceneId != nullptr;
        const int sortBlocks = numSMs * 8;
        if (batched) detail::waveKeyKernel<D, SOLVER, true><<<sortBlocks, 256, 0, s>>>(p, w);
        else detail::waveKeyKernel<D, SOLVER, false><<<sortBlocks, 256, 0, s>>>(p, w);
        detail::waveScanKernel<D, SOLVER><<<1, kWaveScanThreads, 0, s>>>(p, w);
        detail::waveScatterKernel<D, SOLVER><<<sortBlocks, 256, 0, s>>>(w);
        if (batched) { if (screened) refill<true, true>(p, w, numSMs, s); else refill<false, true>(p, w, numSMs, s); }
        else { if (screened) refill<true, false>(p, w, numSMs, s); else refill<false, false>(p, w, numSMs, s); }
        void* args[] = {const_cast<SolveParams*>(&p), const_cast<WaveParams*>(&w)};
        for (int k = 0; k < kStepKernels; k++) {
            cudaError_t e = cudaLaunchKernel(phase(screened, batched, k), dim3(blocks), dim3(detail::kWalkThreads), args, 0, s);
            if (e != cudaSuccess) return e;
        }
        return cudaGetLastError();
    }
    // the records [0, live) of w.dst to the end of their walks
    static cudaError_t drain(const SolveParams& p, const WaveParams& w, int blocks, cudaStream_t s) {
        const bool screened = screenedOf(p), batched = p.sceneId != nullptr;
        if (batched) { if (screened) drainWith<true, true>(p, w, blocks, s); else drainWith<false, true>(p, w, blocks, s); }
        else { if (screened) drainWith<true, false>(p, w, blocks, s); else drainWith<false, false>(p, w, blocks, s); }
        return cudaGetLastError();
    }
};

}  // namespace zg
