// zgpu_cache.cu -- neural cache kernels (training, inference, walk-record accumulation,
// Adam) and their C ABI (include/zgpu.h, zgpu_cache_*).  See zgpu_cache.cuh for the tile
// scheme.  The cache has no counterpart in the reference.
#include <cfloat>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <random>
#include <vector>

#include "zgpu_cache.cuh"
#include "zgpu_internal.h"
#include "zgpu_umma.cuh"

using namespace zg;
using namespace zg::cache;

namespace {

// shared-memory carve-up of the training kernel (byte offsets, 16-byte aligned)
constexpr size_t align16(size_t b) { return (b + 15) & ~size_t(15); }
constexpr size_t kOffW = 0;
constexpr size_t kOffE = align16(kOffW + sizeof(SharedWeights));                        // 4 x 2 x [16][kS32]
constexpr size_t kOffET = align16(kOffE + sizeof(__nv_bfloat16) * kWarps * 2 * kRows * kS32);   // [32][kS64]
constexpr size_t kOffH1T = align16(kOffET + sizeof(__nv_bfloat16) * kInputs * kS64);    // [64][kS64]
constexpr size_t kOffDZ2T = align16(kOffH1T + sizeof(__nv_bfloat16) * kHidden * kS64);
constexpr size_t kOffDZ1T = align16(kOffDZ2T + sizeof(__nv_bfloat16) * kHidden * kS64);
constexpr size_t kOffDE = align16(kOffDZ1T + sizeof(__nv_bfloat16) * kHidden * kS64);   // 4 x [16][33] f32
constexpr size_t kOffX = align16(kOffDE + sizeof(float) * kWarps * kRows * 33);          // 4 x [16][3] f32
constexpr size_t kTrainSmem = align16(kOffX + sizeof(float) * kWarps * kRows * 3);
// inference kernel: weights + per-warp encoding tiles + positions
constexpr size_t kEvalOffE = align16(sizeof(SharedWeights));
constexpr size_t kEvalOffX = align16(kEvalOffE + sizeof(__nv_bfloat16) * kWarps * 2 * kRows * kS32);
constexpr size_t kEvalSmem = align16(kEvalOffX + sizeof(float) * kWarps * kRows * 3);

ZG_D __nv_bfloat16 bf(float v) { return __float2bfloat16_rn(v); }

// Fused forward + backward over count points (indices (offset + j) mod n); gradients of the
// loss invBatch * sum (y - t)^2 are accumulated into G.
template <int D>
__global__ void __launch_bounds__(kWarps * 32, 1)
trainKernel(const Net N, const Grads G, const float* __restrict__ x, const float* __restrict__ target, int64_t n,
            int64_t offset, int64_t count, float invBatch) {
    extern __shared__ __align__(16) unsigned char smem[];
    SharedWeights& S = *reinterpret_cast<SharedWeights*>(smem + kOffW);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int g = lane >> 2, t = lane & 3;
    __nv_bfloat16* E = reinterpret_cast<__nv_bfloat16*>(smem + kOffE) + warp * 2 * kRows * kS32;
    __nv_bfloat16* eT = reinterpret_cast<__nv_bfloat16*>(smem + kOffET);
    __nv_bfloat16* h1T = reinterpret_cast<__nv_bfloat16*>(smem + kOffH1T);
    __nv_bfloat16* dz2T = reinterpret_cast<__nv_bfloat16*>(smem + kOffDZ2T);
    __nv_bfloat16* dz1T = reinterpret_cast<__nv_bfloat16*>(smem + kOffDZ1T);
    float* deS = reinterpret_cast<float*>(smem + kOffDE) + warp * kRows * 33;
    float (*xs)[3] = reinterpret_cast<float (*)[3]>(smem + kOffX) + warp * kRows;
    loadWeights(N, S, true);
    __syncthreads();

    float gW2[8][4], gW1[4][4];
#pragma unroll
    for (int i = 0; i < 8; i++) for (int e = 0; e < 4; e++) gW2[i][e] = 0.0f;
#pragma unroll
    for (int i = 0; i < 4; i++) for (int e = 0; e < 4; e++) gW1[i][e] = 0.0f;
    float pw3[16], pb2[16], pb1[16];
#pragma unroll
    for (int i = 0; i < 16; i++) { pw3[i] = 0.0f; pb2[i] = 0.0f; pb1[i] = 0.0f; }
    float pb3 = 0.0f;
    double ploss = 0.0;
    const int pcol = warp * kRows;   // this warp's columns in the transposed tiles

    for (int64_t base = (int64_t)blockIdx.x * kBlockRows; base < count; base += (int64_t)gridDim.x * kBlockRows) {
        const int64_t r0 = base + pcol;
        const int nValid = (int)max((int64_t)0, min((int64_t)kRows, count - r0));
        if (lane < kRows) {
#pragma unroll
            for (int i = 0; i < 3; i++)
                xs[lane][i] = (lane < nValid && i < D) ? __ldg(x + ((offset + r0 + lane) % n) * D + i) : 0.0f;
        }
        __syncwarp();
        encodeTile<D>(N, xs, nValid, E, lane);
        __syncwarp();
        float h1[8][4], h2[8][4];
        float2 y = forwardTile(S, E, h1, h2, lane);
        // loss and output gradient for rows g and g + 8
        float r0v = 0.0f, r1v = 0.0f;
        if (g < nValid) r0v = y.x - __ldg(target + (offset + r0 + g) % n);
        if (g + 8 < nValid) r1v = y.y - __ldg(target + (offset + r0 + g + 8) % n);
        const float dy0 = 2.0f * r0v * invBatch, dy1 = 2.0f * r1v * invBatch;
        if (t == 0) { ploss += (double)r0v * r0v + (double)r1v * r1v; pb3 += dy0 + dy1; }
        // h1 (BF16, as the forward pass used it) into the transposed tile
#pragma unroll
        for (int nt = 0; nt < 8; nt++) {
            const int c = 8 * nt + 2 * t;
            h1T[c * kS64 + pcol + g] = bf(h1[nt][0]);
            h1T[(c + 1) * kS64 + pcol + g] = bf(h1[nt][1]);
            h1T[c * kS64 + pcol + g + 8] = bf(h1[nt][2]);
            h1T[(c + 1) * kS64 + pcol + g + 8] = bf(h1[nt][3]);
        }
        // output layer backward: dz2 = dy w3 relu'(z2)
        float dz2[8][4];
#pragma unroll
        for (int nt = 0; nt < 8; nt++) {
            const int c = 8 * nt + 2 * t;
            const float wa = S.w3[c], wb = S.w3[c + 1];
            pw3[2 * nt] += dy0 * h2[nt][0] + dy1 * h2[nt][2];
            pw3[2 * nt + 1] += dy0 * h2[nt][1] + dy1 * h2[nt][3];
            dz2[nt][0] = h2[nt][0] > 0.0f ? dy0 * wa : 0.0f;
            dz2[nt][1] = h2[nt][1] > 0.0f ? dy0 * wb : 0.0f;
            dz2[nt][2] = h2[nt][2] > 0.0f ? dy1 * wa : 0.0f;
            dz2[nt][3] = h2[nt][3] > 0.0f ? dy1 * wb : 0.0f;
            pb2[2 * nt] += dz2[nt][0] + dz2[nt][2];
            pb2[2 * nt + 1] += dz2[nt][1] + dz2[nt][3];
            dz2T[c * kS64 + pcol + g] = bf(dz2[nt][0]);
            dz2T[(c + 1) * kS64 + pcol + g] = bf(dz2[nt][1]);
            dz2T[c * kS64 + pcol + g + 8] = bf(dz2[nt][2]);
            dz2T[(c + 1) * kS64 + pcol + g + 8] = bf(dz2[nt][3]);
        }
        // dh1 = dz2 W2 (B operand from W2^T), then dz1 = dh1 relu'(z1)
        float dz1[8][4];
#pragma unroll
        for (int nt = 0; nt < 8; nt++) for (int e = 0; e < 4; e++) dz1[nt][e] = 0.0f;
#pragma unroll
        for (int kt = 0; kt < 4; kt++) {
            uint32_t a0 = pack2(dz2[2 * kt][0], dz2[2 * kt][1]), a1 = pack2(dz2[2 * kt][2], dz2[2 * kt][3]);
            uint32_t a2 = pack2(dz2[2 * kt + 1][0], dz2[2 * kt + 1][1]), a3 = pack2(dz2[2 * kt + 1][2], dz2[2 * kt + 1][3]);
#pragma unroll
            for (int nt = 0; nt < 8; nt++) {
                const __nv_bfloat16* w = S.W2T + (8 * nt + g) * kS64 + 16 * kt + 2 * t;
                mma16816(dz1[nt], a0, a1, a2, a3, ld32(w), ld32(w + 8));
            }
        }
#pragma unroll
        for (int nt = 0; nt < 8; nt++) {
            const int c = 8 * nt + 2 * t;
#pragma unroll
            for (int e = 0; e < 4; e++) dz1[nt][e] = h1[nt][e] > 0.0f ? dz1[nt][e] : 0.0f;
            pb1[2 * nt] += dz1[nt][0] + dz1[nt][2];
            pb1[2 * nt + 1] += dz1[nt][1] + dz1[nt][3];
            dz1T[c * kS64 + pcol + g] = bf(dz1[nt][0]);
            dz1T[(c + 1) * kS64 + pcol + g] = bf(dz1[nt][1]);
            dz1T[c * kS64 + pcol + g + 8] = bf(dz1[nt][2]);
            dz1T[(c + 1) * kS64 + pcol + g + 8] = bf(dz1[nt][3]);
        }
        // de = dz1 W1 (B operand from W1^T): gradient of the encoding
        float de[4][4];
#pragma unroll
        for (int nt = 0; nt < 4; nt++) for (int e = 0; e < 4; e++) de[nt][e] = 0.0f;
#pragma unroll
        for (int kt = 0; kt < 4; kt++) {
            uint32_t a0 = pack2(dz1[2 * kt][0], dz1[2 * kt][1]), a1 = pack2(dz1[2 * kt][2], dz1[2 * kt][3]);
            uint32_t a2 = pack2(dz1[2 * kt + 1][0], dz1[2 * kt + 1][1]), a3 = pack2(dz1[2 * kt + 1][2], dz1[2 * kt + 1][3]);
#pragma unroll
            for (int nt = 0; nt < 4; nt++) {
                const __nv_bfloat16* w = S.W1T + (8 * nt + g) * kS64 + 16 * kt + 2 * t;
                mma16816(de[nt], a0, a1, a2, a3, ld32(w), ld32(w + 8));
            }
        }
#pragma unroll
        for (int nt = 0; nt < 4; nt++) {
            const int c = 8 * nt + 2 * t;
            deS[g * 33 + c] = de[nt][0];
            deS[g * 33 + c + 1] = de[nt][1];
            deS[(g + 8) * 33 + c] = de[nt][2];
            deS[(g + 8) * 33 + c + 1] = de[nt][3];
        }
        // encoding tile transposed for dW1
        for (int k = lane; k < kRows * kInputs; k += 32) {
            int p = k / kInputs, f = k % kInputs;
            eT[f * kS64 + pcol + p] = E[p * kS32 + f];
        }
        __syncwarp();
        // scatter the encoding gradient into the table (same (point, level) split as encoding)
        {
            const int p = lane & 15;
#pragma unroll 1
            for (int s = 0; s < 8; s++) {
                const int l = (lane >> 4) + 2 * s;
                if (p >= nValid || l >= N.levels) continue;
                uint32_t idx[1 << D];
                float w[1 << D];
                levelCorners<D>(N, l, xs[p], idx, w);
                const float d0 = deS[p * 33 + 2 * l], d1 = deS[p * 33 + 2 * l + 1];
                float2* tg = G.table + ((size_t)l << N.log2T);
#pragma unroll
                for (int c = 0; c < (1 << D); c++) atomicAdd(tg + idx[c], make_float2(w[c] * d0, w[c] * d1));
            }
        }
        __syncthreads();
        // weight gradients over the block's 64 points: warp w owns output rows 16w..16w+15
#pragma unroll
        for (int kt = 0; kt < 4; kt++) {
            const __nv_bfloat16* A = dz2T + (16 * warp + g) * kS64 + 16 * kt + 2 * t;
            uint32_t a0 = ld32(A), a1 = ld32(A + 8 * kS64), a2 = ld32(A + 8), a3 = ld32(A + 8 * kS64 + 8);
#pragma unroll
            for (int nt = 0; nt < 8; nt++) {
                const __nv_bfloat16* B = h1T + (8 * nt + g) * kS64 + 16 * kt + 2 * t;
                mma16816(gW2[nt], a0, a1, a2, a3, ld32(B), ld32(B + 8));
            }
            const __nv_bfloat16* A1 = dz1T + (16 * warp + g) * kS64 + 16 * kt + 2 * t;
            uint32_t c0 = ld32(A1), c1 = ld32(A1 + 8 * kS64), c2 = ld32(A1 + 8), c3 = ld32(A1 + 8 * kS64 + 8);
#pragma unroll
            for (int nt = 0; nt < 4; nt++) {
                const __nv_bfloat16* B = eT + (8 * nt + g) * kS64 + 16 * kt + 2 * t;
                mma16816(gW1[nt], c0, c1, c2, c3, ld32(B), ld32(B + 8));
            }
        }
        __syncthreads();
    }

    // flush: weight gradients (each element owned by one lane of one warp per block)
#pragma unroll
    for (int nt = 0; nt < 8; nt++)
#pragma unroll
        for (int e = 0; e < 4; e++) {
            int row = 16 * warp + g + 8 * (e >> 1), col = 8 * nt + 2 * t + (e & 1);
            atomicAdd(G.W2 + row * kHidden + col, gW2[nt][e]);
        }
#pragma unroll
    for (int nt = 0; nt < 4; nt++)
#pragma unroll
        for (int e = 0; e < 4; e++) {
            int row = 16 * warp + g + 8 * (e >> 1), col = 8 * nt + 2 * t + (e & 1);
            atomicAdd(G.W1 + row * kInputs + col, gW1[nt][e]);
        }
    // per-column partials: reduce over the 8 row groups (lanes with equal t)
#pragma unroll
    for (int i = 0; i < 16; i++) {
        for (int o = 4; o < 32; o <<= 1) {
            pw3[i] += __shfl_xor_sync(0xffffffffu, pw3[i], o);
            pb2[i] += __shfl_xor_sync(0xffffffffu, pb2[i], o);
            pb1[i] += __shfl_xor_sync(0xffffffffu, pb1[i], o);
        }
    }
    if (g == 0) {
#pragma unroll
        for (int nt = 0; nt < 8; nt++)
#pragma unroll
            for (int q = 0; q < 2; q++) {
                int col = 8 * nt + 2 * t + q;
                atomicAdd(G.w3 + col, pw3[2 * nt + q]);
                atomicAdd(G.b2 + col, pb2[2 * nt + q]);
                atomicAdd(G.b1 + col, pb1[2 * nt + q]);
            }
    }
    for (int o = 16; o > 0; o >>= 1) {
        pb3 += __shfl_xor_sync(0xffffffffu, pb3, o);
        ploss += __shfl_xor_sync(0xffffffffu, ploss, o);
    }
    if (lane == 0) {
        atomicAdd(G.b3, pb3);
        atomicAdd(G.loss, ploss);
    }
}

// Inference over records.  Mode 0: positions x [n][D] -> y [n].  Mode 1: walk records
// (cache-terminated walks, 2 float4 each: (x, throughput), (partial estimate, point, length))
// -> the walk total partial + throughput * cache(x) is accumulated into the point's sums.
template <int D, int MODE>
__global__ void __launch_bounds__(kWarps * 32)
evalKernel(const Net N, const float* __restrict__ x, float* __restrict__ y, int64_t n, const float4* __restrict__ rec,
           const unsigned long long* __restrict__ recCount, double* accSum, double* accSq, int* accN, long long* accLen) {
    extern __shared__ __align__(16) unsigned char smem[];
    SharedWeights& S = *reinterpret_cast<SharedWeights*>(smem);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int g = lane >> 2, t = lane & 3;
    __nv_bfloat16* E = reinterpret_cast<__nv_bfloat16*>(smem + kEvalOffE) + warp * 2 * kRows * kS32;
    float (*xs)[3] = reinterpret_cast<float (*)[3]>(smem + kEvalOffX) + warp * kRows;
    loadWeights(N, S, false);
    __syncthreads();
    const int64_t total = MODE == 1 ? (int64_t)min((unsigned long long)n, *recCount) : n;
    const int64_t tiles = (total + kRows - 1) / kRows;
    for (int64_t tile = (int64_t)blockIdx.x * kWarps + warp; tile < tiles; tile += (int64_t)gridDim.x * kWarps) {
        const int64_t r0 = tile * kRows;
        const int nValid = (int)min((int64_t)kRows, total - r0);
        if (lane < kRows) {
            if (MODE == 0) {
#pragma unroll
                for (int i = 0; i < 3; i++) xs[lane][i] = (lane < nValid && i < D) ? __ldg(x + (r0 + lane) * D + i) : 0.0f;
            } else {
                float4 a = lane < nValid ? __ldg(rec + 2 * (r0 + lane)) : make_float4(0, 0, 0, 0);
                xs[lane][0] = a.x; xs[lane][1] = a.y; xs[lane][2] = a.z;
            }
        }
        __syncwarp();
        encodeTile<D>(N, xs, nValid, E, lane);
        __syncwarp();
        float h1[8][4], h2[8][4];
        float2 v = forwardTile(S, E, h1, h2, lane);
        if (t == 0) {
#pragma unroll
            for (int half = 0; half < 2; half++) {
                const int row = g + 8 * half;
                if (row >= nValid) continue;
                const float u = half ? v.y : v.x;
                if (MODE == 0) {
                    y[r0 + row] = u;
                } else {
                    float4 a = __ldg(rec + 2 * (r0 + row)), b = __ldg(rec + 2 * (r0 + row) + 1);
                    const int point = __float_as_int(b.y);
                    const double total = (double)(b.x + a.w * u);
                    atomicAdd(accSum + point, total);
                    atomicAdd(accSq + point, total * total);
                    atomicAdd(accN + point, 1);
                    atomicAdd(reinterpret_cast<unsigned long long*>(accLen + point),
                              (unsigned long long)__float_as_int(b.z));
                }
            }
        }
        __syncwarp();
    }
}

// ------------------------------------------------------------------ tcgen05 inference
// One CTA of 128 threads per 128-point tile, one thread per point: the thread encodes its
// point into its row of the A operand, one thread issues the layer's MMAs (M = 128, N = 64,
// K = 16 each: D = A * W^T with BF16 hi + lo operand pairs, three products per K step, FP32
// accumulation in 64 tensor-memory columns), and every thread reads its row of the
// accumulator back (tcgen05.ld), applies bias + ReLU and writes the next layer's A row.  The
// output layer (64 -> 1) is a per-thread dot product.  Weights are staged once per CTA.
constexpr int kTcRows = 128;
constexpr uint32_t kTcCols = 64;                 // tensor-memory columns (one 128 x 64 FP32 tile)
constexpr long long kTcWaitLimit = 1ll << 24;    // mbarrier polls before a wait gives up
constexpr unsigned kErrTensorWait = 32u;         // error word bit: an MMA completion wait gave up

struct TcShared {
    unsigned char E[2][kTcRows * kInputs * 2];   // encoding rows, hi / lo  (K = 32)
    unsigned char H[2][kTcRows * kHidden * 2];   // hidden-1 rows, hi / lo  (K = 64)
    unsigned char W1[2][kHidden * kInputs * 2];  // [out][in], hi / lo
    unsigned char W2[2][kHidden * kHidden * 2];
    float b1[kHidden], b2[kHidden], w3[kHidden];
    float b3;
    uint64_t mbar;
    uint32_t tmem;
};
constexpr size_t kTcSmem = sizeof(TcShared);

// 8 consecutive values of a row as BF16 hi and lo (remainder) packs of 16 bytes each
ZG_D void splitPack8(const float* v, uint4& hi, uint4& lo) {
    uint32_t h[4], l[4];
#pragma unroll
    for (int j = 0; j < 4; j++) pack2split(v[2 * j], v[2 * j + 1], h[j], l[j]);
    hi = make_uint4(h[0], h[1], h[2], h[3]);
    lo = make_uint4(l[0], l[1], l[2], l[3]);
}

template <int D, int MODE>
__global__ void __launch_bounds__(kTcRows, 1)
evalKernelTc(const Net N, const float* __restrict__ x, float* __restrict__ y, int64_t n,
             const float4* __restrict__ rec, const unsigned long long* __restrict__ recCount, double* accSum,
             double* accSq, int* accN, long long* accLen, unsigned int* errw) {
    extern __shared__ __align__(128) unsigned char smemTc[];
    TcShared& S = *reinterpret_cast<TcShared*>(smemTc);
    const int tid = threadIdx.x, warp = tid >> 5;
    for (int i = tid; i < kHidden * kInputs; i += kTcRows) {
        const uint32_t off = umma::canonicalOffset<kInputs>(i / kInputs, i % kInputs);
        *reinterpret_cast<__nv_bfloat16*>(S.W1[0] + off) = N.W1[i];
        *reinterpret_cast<__nv_bfloat16*>(S.W1[1] + off) = N.W1lo[i];
    }
    for (int i = tid; i < kHidden * kHidden; i += kTcRows) {
        const uint32_t off = umma::canonicalOffset<kHidden>(i / kHidden, i % kHidden);
        *reinterpret_cast<__nv_bfloat16*>(S.W2[0] + off) = N.W2[i];
        *reinterpret_cast<__nv_bfloat16*>(S.W2[1] + off) = N.W2lo[i];
    }
    for (int i = tid; i < kHidden; i += kTcRows) { S.b1[i] = N.b1[i]; S.b2[i] = N.b2[i]; S.w3[i] = N.w3[i]; }
    if (tid == 0) { S.b3 = *N.b3; umma::mbarInit(&S.mbar, 1); }
    if (warp == 0) umma::alloc(&S.tmem, kTcCols);
    umma::fenceProxyAsync();
    umma::fenceBeforeSync();
    __syncthreads();
    umma::fenceAfterSync();
    const uint32_t tmem = S.tmem;
    const uint32_t taddr = tmem + ((uint32_t)(32 * warp) << 16);
    const uint32_t idesc = umma::instrBf16(kTcRows, kHidden);
    const uint32_t sE0 = umma::smemAddr(S.E[0]), sE1 = umma::smemAddr(S.E[1]);
    const uint32_t sH0 = umma::smemAddr(S.H[0]), sH1 = umma::smemAddr(S.H[1]);
    const uint32_t sA0 = umma::smemAddr(S.W1[0]), sA1 = umma::smemAddr(S.W1[1]);
    const uint32_t sB0 = umma::smemAddr(S.W2[0]), sB1 = umma::smemAddr(S.W2[1]);
    const int64_t total = MODE == 1 ? (int64_t)min((unsigned long long)n, *recCount) : n;
    const int64_t tiles = (total + kTcRows - 1) / kTcRows;
    uint32_t phase = 0;
    bool ok = true;
    for (int64_t tile = blockIdx.x; tile < tiles && ok; tile += gridDim.x) {
        const int64_t r = tile * kTcRows + tid;
        const bool valid = r < total;
        float xp[3] = {0.0f, 0.0f, 0.0f};
        if (valid) {
            if (MODE == 0) {
#pragma unroll
                for (int i = 0; i < D; i++) xp[i] = __ldg(x + r * D + i);
            } else {
                const float4 a = __ldg(rec + 2 * r);
                xp[0] = a.x; xp[1] = a.y; xp[2] = a.z;
            }
        }
        // encoding row (levels beyond N.levels and rows beyond the data encode 0)
#pragma unroll 1
        for (int kg = 0; kg < kInputs / 8; kg++) {
            float v[8];
#pragma unroll
            for (int j = 0; j < 4; j++) {
                const int l = 4 * kg + j;
                float2 f = make_float2(0.0f, 0.0f);
                if (valid && l < N.levels) f = encodeLevel<D>(N, l, xp);
                v[2 * j] = f.x; v[2 * j + 1] = f.y;
            }
            uint4 hi, lo;
            splitPack8(v, hi, lo);
            const uint32_t off = umma::canonicalOffset<kInputs>(tid, 8 * kg);
            *reinterpret_cast<uint4*>(S.E[0] + off) = hi;
            *reinterpret_cast<uint4*>(S.E[1] + off) = lo;
        }
        umma::fenceProxyAsync();
        umma::fenceBeforeSync();
        __syncthreads();
        if (tid == 0) {
            umma::fenceAfterSync();
#pragma unroll
            for (int ks = 0; ks < kInputs / 16; ks++) {
                const uint32_t k = 256u * ks;      // two core matrices along K per step
                const uint64_t aHi = umma::descriptor(sE0 + k, 128, 16 * kInputs);
                const uint64_t aLo = umma::descriptor(sE1 + k, 128, 16 * kInputs);
                const uint64_t bHi = umma::descriptor(sA0 + k, 128, 16 * kInputs);
                const uint64_t bLo = umma::descriptor(sA1 + k, 128, 16 * kInputs);
                umma::mma(tmem, aHi, bHi, idesc, ks > 0);
                umma::mma(tmem, aLo, bHi, idesc, true);
                umma::mma(tmem, aHi, bLo, idesc, true);
            }
            umma::commit(&S.mbar);
        }
        ok = __syncthreads_and(umma::mbarWait(&S.mbar, phase, kTcWaitLimit));
        phase ^= 1u;
        if (!ok) break;
        umma::fenceAfterSync();
        // hidden layer 1: bias + ReLU, then this row of the layer-2 operand
#pragma unroll 1
        for (int c = 0; c < kHidden / 16; c++) {
            float v[16];
            umma::load16(taddr + 16u * c, v);
#pragma unroll
            for (int j = 0; j < 16; j++) v[j] = fmaxf(v[j] + S.b1[16 * c + j], 0.0f);
#pragma unroll
            for (int h = 0; h < 2; h++) {
                uint4 hi, lo;
                splitPack8(v + 8 * h, hi, lo);
                const uint32_t off = umma::canonicalOffset<kHidden>(tid, 16 * c + 8 * h);
                *reinterpret_cast<uint4*>(S.H[0] + off) = hi;
                *reinterpret_cast<uint4*>(S.H[1] + off) = lo;
            }
        }
        umma::fenceProxyAsync();
        umma::fenceBeforeSync();
        __syncthreads();
        if (tid == 0) {
            umma::fenceAfterSync();
#pragma unroll
            for (int ks = 0; ks < kHidden / 16; ks++) {
                const uint32_t k = 256u * ks;
                const uint64_t aHi = umma::descriptor(sH0 + k, 128, 16 * kHidden);
                const uint64_t aLo = umma::descriptor(sH1 + k, 128, 16 * kHidden);
                const uint64_t bHi = umma::descriptor(sB0 + k, 128, 16 * kHidden);
                const uint64_t bLo = umma::descriptor(sB1 + k, 128, 16 * kHidden);
                umma::mma(tmem, aHi, bHi, idesc, ks > 0);
                umma::mma(tmem, aLo, bHi, idesc, true);
                umma::mma(tmem, aHi, bLo, idesc, true);
            }
            umma::commit(&S.mbar);
        }
        ok = __syncthreads_and(umma::mbarWait(&S.mbar, phase, kTcWaitLimit));
        phase ^= 1u;
        if (!ok) break;
        umma::fenceAfterSync();
        float out = S.b3;
#pragma unroll 1
        for (int c = 0; c < kHidden / 16; c++) {
            float v[16];
            umma::load16(taddr + 16u * c, v);
#pragma unroll
            for (int j = 0; j < 16; j++) out += S.w3[16 * c + j] * fmaxf(v[j] + S.b2[16 * c + j], 0.0f);
        }
        if (valid) {
            if (MODE == 0) {
                y[r] = out;
            } else {
                const float4 a = __ldg(rec + 2 * r), b = __ldg(rec + 2 * r + 1);
                const int point = __float_as_int(b.y);
                const double v = (double)(b.x + a.w * out);
                atomicAdd(accSum + point, v);
                atomicAdd(accSq + point, v * v);
                atomicAdd(accN + point, 1);
                atomicAdd(reinterpret_cast<unsigned long long*>(accLen + point), (unsigned long long)__float_as_int(b.z));
            }
        }
        umma::fenceBeforeSync();
    }
    if (!ok && tid == 0 && errw) atomicOr(errw, kErrTensorWait);
    __syncthreads();
    if (warp == 0) umma::dealloc(tmem, kTcCols);
}

// FP32 encoding of each point (levels beyond n_levels are 0): enc [n][32]
template <int D>
__global__ void encodeKernel(const Net N, const float* __restrict__ x, float* __restrict__ enc, int64_t n) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n * kMaxLevels) return;
    const int64_t p = i / kMaxLevels;
    const int l = (int)(i % kMaxLevels);
    float xp[3] = {0.0f, 0.0f, 0.0f};
#pragma unroll
    for (int k = 0; k < D; k++) xp[k] = x[p * D + k];
    float2 f = l < N.levels ? encodeLevel<D>(N, l, xp) : make_float2(0.0f, 0.0f);
    enc[p * kInputs + 2 * l] = f.x;
    enc[p * kInputs + 2 * l + 1] = f.y;
}

// Adam over the flat parameter vector; refreshes the FP16 table and BF16 weight copies and
// clears the gradient.  Segment [0, nTable) is the table (learning rate lrGrid), the rest the
// network (lrMlp).
__global__ void adamKernel(float* __restrict__ p, float* __restrict__ gr, float* __restrict__ m, float* __restrict__ v,
                           int64_t nTotal, int64_t nTable, int64_t oW1, int64_t oW2, float lrGrid, float lrMlp,
                           float beta1, float beta2, float eps, float c1, float c2, __half* tableHalf,
                           __nv_bfloat16* W1b, __nv_bfloat16* W2b, __nv_bfloat16* W1lo, __nv_bfloat16* W2lo,
                           int apply) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < nTotal; i += (int64_t)gridDim.x * blockDim.x) {
        float w = p[i];
        if (apply) {
            float gi = gr[i];
            float mi = beta1 * m[i] + (1.0f - beta1) * gi;
            float vi = beta2 * v[i] + (1.0f - beta2) * gi * gi;
            m[i] = mi;
            v[i] = vi;
            const float lr = i < nTable ? lrGrid : lrMlp;
            w -= lr * (mi * c1) / (sqrtf(vi * c2) + eps);
            p[i] = w;
            gr[i] = 0.0f;
        }
        if (i < nTable) {
            tableHalf[i] = __float2half_rn(w);
        } else if (i >= oW1 && i < oW1 + kHidden * kInputs) {
            __nv_bfloat16 hi = __float2bfloat16_rn(w);
            W1b[i - oW1] = hi;
            W1lo[i - oW1] = __float2bfloat16_rn(w - __bfloat162float(hi));
        } else if (i >= oW2 && i < oW2 + kHidden * kHidden) {
            __nv_bfloat16 hi = __float2bfloat16_rn(w);
            W2b[i - oW2] = hi;
            W2lo[i - oW2] = __float2bfloat16_rn(w - __bfloat162float(hi));
        }
    }
}

}  // namespace

// ----------------------------------------------------------------------------- C ABI
struct zgpu_cache {
    zgpu_context* ctx = nullptr;
    zgpu_cache_config cfg;
    int device = 0;
    int numSMs = 1;
    cudaStream_t stream = nullptr;
    int64_t T = 0, oTable = 0, oW1 = 0, oB1 = 0, oW2 = 0, oB2 = 0, oW3 = 0, oB3 = 0, total = 0;
    float* master = nullptr;
    float* grad = nullptr;
    float* m = nullptr;
    float* v = nullptr;
    __half* tableHalf = nullptr;
    __nv_bfloat16* W1b = nullptr;
    __nv_bfloat16* W2b = nullptr;
    __nv_bfloat16* W1lo = nullptr;
    __nv_bfloat16* W2lo = nullptr;
    double* loss = nullptr;
    unsigned int* err = nullptr;       // device error word of the inference kernel
    float* stageX = nullptr;
    float* stageT = nullptr;
    int64_t stageCap = 0;
    long long steps = 0;
    Net net;
};

namespace {

int cfail(int status, const char* fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    setLastError(buf);
    return status;
}

#define ZC_CUDA(expr)                                                                         \
    do {                                                                                      \
        cudaError_t e_ = (expr);                                                              \
        if (e_ != cudaSuccess) return cfail(ZGPU_ERR_CUDA, "%s: %s", #expr, cudaGetErrorString(e_)); \
    } while (0)

Grads gradsOf(zgpu_cache* c) {
    Grads G;
    G.table = reinterpret_cast<float2*>(c->grad + c->oTable);
    G.W1 = c->grad + c->oW1; G.b1 = c->grad + c->oB1;
    G.W2 = c->grad + c->oW2; G.b2 = c->grad + c->oB2;
    G.w3 = c->grad + c->oW3; G.b3 = c->grad + c->oB3;
    G.loss = c->loss;
    return G;
}

int gridFor(zgpu_cache* c, int64_t rows) {
    int64_t blocks = (rows + kBlockRows - 1) / kBlockRows;
    int64_t cap = (int64_t)c->numSMs * 2;
    return (int)std::max<int64_t>(1, std::min(blocks, cap));
}

int ensureStage(zgpu_cache* c, int64_t n) {
    if (n <= c->stageCap) return ZGPU_OK;
    if (c->stageX) cudaFree(c->stageX);
    if (c->stageT) cudaFree(c->stageT);
    c->stageX = c->stageT = nullptr;
    c->stageCap = 0;
    ZC_CUDA(cudaMalloc(&c->stageX, (size_t)n * 3 * sizeof(float)));
    ZC_CUDA(cudaMalloc(&c->stageT, (size_t)n * sizeof(float)));
    c->stageCap = n;
    return ZGPU_OK;
}

int stage(zgpu_cache* c, int64_t n, const float* x, const float* t, int memory, const float** dx, const float** dt) {
    if (memory == ZGPU_MEM_DEVICE) { *dx = x; if (dt) *dt = t; return ZGPU_OK; }
    if (memory != ZGPU_MEM_HOST) return cfail(ZGPU_ERR_INVALID_ARG, "unknown memory space %d", memory);
    int st = ensureStage(c, n);
    if (st != ZGPU_OK) return st;
    const int D = c->cfg.dim;
    ZC_CUDA(cudaMemcpyAsync(c->stageX, x, (size_t)n * D * sizeof(float), cudaMemcpyHostToDevice, c->stream));
    if (t) ZC_CUDA(cudaMemcpyAsync(c->stageT, t, (size_t)n * sizeof(float), cudaMemcpyHostToDevice, c->stream));
    *dx = c->stageX;
    if (dt) *dt = c->stageT;
    return ZGPU_OK;
}

cudaError_t launchAdam(zgpu_cache* c, int apply) {
    const zgpu_cache_config& k = c->cfg;
    float c1 = 1.0f, c2 = 1.0f;
    if (apply) {
        c->steps++;
        c1 = 1.0f / (1.0f - std::pow(k.beta1, (float)c->steps));
        c2 = 1.0f / (1.0f - std::pow(k.beta2, (float)c->steps));
    }
    int blocks = c->numSMs * 8;
    adamKernel<<<blocks, 256, 0, c->stream>>>(c->master, c->grad, c->m, c->v, c->total, c->oW1, c->oW1, c->oW2,
                                               k.learning_rate_grid, k.learning_rate_mlp, k.beta1, k.beta2, k.epsilon,
                                               c1, c2, c->tableHalf, c->W1b, c->W2b, c->W1lo, c->W2lo, apply);
    return cudaGetLastError();
}

cudaError_t launchTrain(zgpu_cache* c, const float* x, const float* t, int64_t n, int64_t offset, int64_t count) {
    static bool attr2 = false, attr3 = false;
    if (!attr2) { cudaFuncSetAttribute(trainKernel<2>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kTrainSmem); attr2 = true; }
    if (!attr3) { cudaFuncSetAttribute(trainKernel<3>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kTrainSmem); attr3 = true; }
    const float invBatch = 1.0f / (float)count;
    const int blocks = gridFor(c, count);
    if (c->cfg.dim == 2)
        trainKernel<2><<<blocks, kWarps * 32, kTrainSmem, c->stream>>>(c->net, gradsOf(c), x, t, n, offset, count, invBatch);
    else
        trainKernel<3><<<blocks, kWarps * 32, kTrainSmem, c->stream>>>(c->net, gradsOf(c), x, t, n, offset, count, invBatch);
    return cudaGetLastError();
}

}  // namespace

namespace zg {
// walk-record accumulation used by zgpu_solve_cached (zgpu_api.cu)
cudaError_t launchCacheAccumulate(const zgpu_cache* c, const float4* rec, const unsigned long long* recCount,
                                  int64_t cap, double* accSum, double* accSq, int* accN, long long* accLen,
                                  unsigned int* errw, cudaStream_t s) {
    static bool a2 = false, a3 = false;
    if (!a2) { cudaFuncSetAttribute(evalKernelTc<2, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kTcSmem); a2 = true; }
    if (!a3) { cudaFuncSetAttribute(evalKernelTc<3, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kTcSmem); a3 = true; }
    const int blocks = c->numSMs * 2;
    if (c->cfg.dim == 2)
        evalKernelTc<2, 1><<<blocks, kTcRows, kTcSmem, s>>>(c->net, nullptr, nullptr, cap, rec, recCount, accSum, accSq,
                                                            accN, accLen, errw);
    else
        evalKernelTc<3, 1><<<blocks, kTcRows, kTcSmem, s>>>(c->net, nullptr, nullptr, cap, rec, recCount, accSum, accSq,
                                                            accN, accLen, errw);
    return cudaGetLastError();
}
int cacheDim(const zgpu_cache* c) { return c->cfg.dim; }
cudaStream_t cacheStream(const zgpu_cache* c) { return c->stream; }
}  // namespace zg

extern "C" {

int zgpu_cache_create(zgpu_context* ctx, const zgpu_cache_config* cfg, zgpu_cache** out) {
    if (!ctx || !cfg || !out) return cfail(ZGPU_ERR_INVALID_ARG, "NULL argument");
    *out = nullptr;
    const zgpu_cache_config& k = *cfg;
    if (k.dim != 2 && k.dim != 3) return cfail(ZGPU_ERR_INVALID_ARG, "cache dim must be 2 or 3");
    if (k.n_levels < 1 || k.n_levels > kMaxLevels) return cfail(ZGPU_ERR_INVALID_ARG, "n_levels must be in [1, 16]");
    if (k.log2_table_size < 8 || k.log2_table_size > 24) return cfail(ZGPU_ERR_INVALID_ARG, "log2_table_size must be in [8, 24]");
    if (!(k.base_resolution >= 1.0f) || !(k.max_resolution >= k.base_resolution) || k.max_resolution > 65536.0f)
        return cfail(ZGPU_ERR_INVALID_ARG, "resolutions must satisfy 1 <= base <= max <= 65536");
    for (int i = 0; i < k.dim; i++)
        if (!(k.domain_max[i] > k.domain_min[i])) return cfail(ZGPU_ERR_INVALID_ARG, "empty cache domain on axis %d", i);
    if (!(k.learning_rate_grid >= 0.0f) || !(k.learning_rate_mlp >= 0.0f) || !(k.beta1 >= 0.0f && k.beta1 < 1.0f) ||
        !(k.beta2 >= 0.0f && k.beta2 < 1.0f) || !(k.epsilon > 0.0f))
        return cfail(ZGPU_ERR_INVALID_ARG, "invalid optimiser settings");
    zgpu_cache* c = new zgpu_cache();
    c->ctx = ctx;
    c->cfg = k;
    c->stream = (cudaStream_t)zgpu_context_stream(ctx);
    c->device = contextDevice(ctx);
    if (cudaSetDevice(c->device) != cudaSuccess) { delete c; return cfail(ZGPU_ERR_CUDA, "cannot select the context's device"); }
    cudaDeviceGetAttribute(&c->numSMs, cudaDevAttrMultiProcessorCount, c->device);
    c->T = (int64_t)1 << k.log2_table_size;
    c->oTable = 0;
    c->oW1 = (int64_t)k.n_levels * c->T * 2;
    c->oB1 = c->oW1 + kHidden * kInputs;
    c->oW2 = c->oB1 + kHidden;
    c->oB2 = c->oW2 + kHidden * kHidden;
    c->oW3 = c->oB2 + kHidden;
    c->oB3 = c->oW3 + kHidden;
    c->total = c->oB3 + 1;
    // encoding constants
    Net& N = c->net;
    N.dim = k.dim; N.levels = k.n_levels; N.log2T = k.log2_table_size;
    double growth = k.n_levels > 1 ? std::exp((std::log((double)k.max_resolution) - std::log((double)k.base_resolution)) /
                                              (k.n_levels - 1))
                                   : 1.0;
    N.denseMask = 0;
    for (int l = 0; l < kMaxLevels; l++) {
        double r = l < k.n_levels ? std::floor(k.base_resolution * std::pow(growth, l) + 1e-9) : 1.0;
        N.res[l] = (float)r;
        double dense = std::pow(r + 1.0, k.dim);
        if (l < k.n_levels && dense <= (double)c->T) N.denseMask |= 1u << l;
    }
    for (int i = 0; i < 3; i++) {
        N.lo[i] = i < k.dim ? k.domain_min[i] : 0.0f;
        N.inv[i] = i < k.dim ? 1.0f / (k.domain_max[i] - k.domain_min[i]) : 0.0f;
    }
    auto cleanup = [&](int st) { zgpu_cache_destroy(c); return st; };
    size_t bytes = (size_t)c->total * sizeof(float);
    if (cudaMalloc(&c->master, bytes) != cudaSuccess || cudaMalloc(&c->grad, bytes) != cudaSuccess ||
        cudaMalloc(&c->m, bytes) != cudaSuccess || cudaMalloc(&c->v, bytes) != cudaSuccess ||
        cudaMalloc(&c->tableHalf, (size_t)c->oW1 * sizeof(__half)) != cudaSuccess ||
        cudaMalloc(&c->W1b, kHidden * kInputs * sizeof(__nv_bfloat16)) != cudaSuccess ||
        cudaMalloc(&c->W2b, kHidden * kHidden * sizeof(__nv_bfloat16)) != cudaSuccess ||
        cudaMalloc(&c->W1lo, kHidden * kInputs * sizeof(__nv_bfloat16)) != cudaSuccess ||
        cudaMalloc(&c->W2lo, kHidden * kHidden * sizeof(__nv_bfloat16)) != cudaSuccess ||
        cudaMalloc(&c->loss, sizeof(double)) != cudaSuccess || cudaMalloc(&c->err, sizeof(unsigned int)) != cudaSuccess)
        return cleanup(cfail(ZGPU_ERR_OUT_OF_MEMORY, "cannot allocate the cache parameters (%zu bytes each)", bytes));
    N.table = reinterpret_cast<const __half2*>(c->tableHalf);
    N.W1 = c->W1b; N.W2 = c->W2b; N.W1lo = c->W1lo; N.W2lo = c->W2lo;
    N.b1 = c->master + c->oB1; N.b2 = c->master + c->oB2; N.w3 = c->master + c->oW3; N.b3 = c->master + c->oB3;
    // initialisation: table U(-1e-4, 1e-4), weights Glorot-uniform, biases 0
    std::vector<float> h((size_t)c->total, 0.0f);
    std::mt19937_64 rng(k.seed);
    std::uniform_real_distribution<float> u(-1.0f, 1.0f);
    for (int64_t i = 0; i < c->oW1; i++) h[i] = 1e-4f * u(rng);
    const float a1 = std::sqrt(6.0f / (kInputs + kHidden)), a2 = std::sqrt(6.0f / (2 * kHidden)),
                a3 = std::sqrt(6.0f / (kHidden + 1));
    for (int i = 0; i < kHidden * kInputs; i++) h[c->oW1 + i] = a1 * u(rng);
    for (int i = 0; i < kHidden * kHidden; i++) h[c->oW2 + i] = a2 * u(rng);
    for (int i = 0; i < kHidden; i++) h[c->oW3 + i] = a3 * u(rng);
    if (cudaMemcpy(c->master, h.data(), bytes, cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemset(c->grad, 0, bytes) != cudaSuccess || cudaMemset(c->m, 0, bytes) != cudaSuccess ||
        cudaMemset(c->v, 0, bytes) != cudaSuccess || cudaMemset(c->loss, 0, sizeof(double)) != cudaSuccess)
        return cleanup(cfail(ZGPU_ERR_CUDA, "cannot initialise the cache parameters"));
    if (launchAdam(c, 0) != cudaSuccess || cudaStreamSynchronize(c->stream) != cudaSuccess)
        return cleanup(cfail(ZGPU_ERR_CUDA, "cannot initialise the cache copies"));
    *out = c;
    return ZGPU_OK;
}

int zgpu_cache_destroy(zgpu_cache* c) {
    if (!c) return ZGPU_OK;
    // the context's stream may already be gone: wait on the whole device instead
    cudaSetDevice(c->device);
    cudaDeviceSynchronize();
    for (void* p : {(void*)c->master, (void*)c->grad, (void*)c->m, (void*)c->v, (void*)c->tableHalf, (void*)c->W1b,
                    (void*)c->W2b, (void*)c->W1lo, (void*)c->W2lo, (void*)c->loss, (void*)c->err, (void*)c->stageX,
                    (void*)c->stageT})
        if (p) cudaFree(p);
    delete c;
    return ZGPU_OK;
}

int zgpu_cache_layout(const zgpu_cache* c, int64_t* offsets) {
    if (!c || !offsets) return cfail(ZGPU_ERR_INVALID_ARG, "NULL argument");
    const int64_t o[8] = {c->oTable, c->oW1, c->oB1, c->oW2, c->oB2, c->oW3, c->oB3, c->total};
    std::memcpy(offsets, o, sizeof(o));
    return ZGPU_OK;
}

int zgpu_cache_resolutions(const zgpu_cache* c, float* res) {
    if (!c || !res) return cfail(ZGPU_ERR_INVALID_ARG, "NULL argument");
    for (int l = 0; l < c->cfg.n_levels; l++) res[l] = c->net.res[l];
    return ZGPU_OK;
}

int zgpu_cache_set_learning_rates(zgpu_cache* c, float grid, float mlp) {
    if (!c) return cfail(ZGPU_ERR_INVALID_ARG, "NULL argument");
    if (!(grid >= 0.0f) || !(mlp >= 0.0f)) return cfail(ZGPU_ERR_INVALID_ARG, "learning rates must be >= 0");
    c->cfg.learning_rate_grid = grid;
    c->cfg.learning_rate_mlp = mlp;
    return ZGPU_OK;
}

int zgpu_cache_get_parameters(zgpu_cache* c, float* out) {
    if (!c || !out) return cfail(ZGPU_ERR_INVALID_ARG, "NULL argument");
    ZC_CUDA(cudaMemcpyAsync(out, c->master, (size_t)c->total * sizeof(float), cudaMemcpyDeviceToHost, c->stream));
    ZC_CUDA(cudaStreamSynchronize(c->stream));
    return ZGPU_OK;
}

int zgpu_cache_set_parameters(zgpu_cache* c, const float* in) {
    if (!c || !in) return cfail(ZGPU_ERR_INVALID_ARG, "NULL argument");
    ZC_CUDA(cudaMemcpyAsync(c->master, in, (size_t)c->total * sizeof(float), cudaMemcpyHostToDevice, c->stream));
    ZC_CUDA(launchAdam(c, 0));
    ZC_CUDA(cudaStreamSynchronize(c->stream));
    return ZGPU_OK;
}

int zgpu_cache_train(zgpu_cache* c, int64_t n, const float* x, const float* target, int memory, int32_t steps,
                     int32_t batch_size, float* mean_loss) {
    if (!c || (n > 0 && (!x || !target))) return cfail(ZGPU_ERR_INVALID_ARG, "NULL argument");
    if (n <= 0 || steps < 0 || batch_size <= 0) return cfail(ZGPU_ERR_INVALID_ARG, "need n > 0, steps >= 0, batch_size > 0");
    const float *dx = nullptr, *dt = nullptr;
    int st = stage(c, n, x, target, memory, &dx, &dt);
    if (st != ZGPU_OK) return st;
    ZC_CUDA(cudaMemsetAsync(c->loss, 0, sizeof(double), c->stream));
    const int64_t B = std::min<int64_t>(batch_size, n);
    int64_t offset = (c->steps * B) % n;
    for (int s = 0; s < steps; s++) {
        ZC_CUDA(launchTrain(c, dx, dt, n, offset, B));
        ZC_CUDA(launchAdam(c, 1));
        offset = (offset + B) % n;
    }
    if (mean_loss) {
        double l = 0.0;
        ZC_CUDA(cudaMemcpyAsync(&l, c->loss, sizeof(double), cudaMemcpyDeviceToHost, c->stream));
        ZC_CUDA(cudaStreamSynchronize(c->stream));
        *mean_loss = steps > 0 ? (float)(l / ((double)steps * B)) : 0.0f;
    }
    return ZGPU_OK;
}

int zgpu_cache_gradients(zgpu_cache* c, int64_t n, const float* x, const float* target, int memory, float* grads,
                         double* loss) {
    if (!c || n <= 0 || !x || !target || !grads) return cfail(ZGPU_ERR_INVALID_ARG, "NULL argument or empty batch");
    const float *dx = nullptr, *dt = nullptr;
    int st = stage(c, n, x, target, memory, &dx, &dt);
    if (st != ZGPU_OK) return st;
    ZC_CUDA(cudaMemsetAsync(c->grad, 0, (size_t)c->total * sizeof(float), c->stream));
    ZC_CUDA(cudaMemsetAsync(c->loss, 0, sizeof(double), c->stream));
    ZC_CUDA(launchTrain(c, dx, dt, n, 0, n));
    ZC_CUDA(cudaMemcpyAsync(grads, c->grad, (size_t)c->total * sizeof(float), cudaMemcpyDeviceToHost, c->stream));
    double l = 0.0;
    ZC_CUDA(cudaMemcpyAsync(&l, c->loss, sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    ZC_CUDA(cudaMemsetAsync(c->grad, 0, (size_t)c->total * sizeof(float), c->stream));
    ZC_CUDA(cudaStreamSynchronize(c->stream));
    if (loss) *loss = l / (double)n;
    return ZGPU_OK;
}

int zgpu_cache_encode(zgpu_cache* c, int64_t n, const float* x, float* enc, int memory) {
    if (!c || n < 0 || (n > 0 && (!x || !enc))) return cfail(ZGPU_ERR_INVALID_ARG, "NULL argument");
    if (n == 0) return ZGPU_OK;
    const float* dx = nullptr;
    int st = stage(c, n, x, nullptr, memory, &dx, nullptr);
    if (st != ZGPU_OK) return st;
    float* de = enc;
    if (memory == ZGPU_MEM_HOST) ZC_CUDA(cudaMalloc(&de, (size_t)n * kInputs * sizeof(float)));
    const int64_t work = n * kMaxLevels;
    const int blocks = (int)((work + 255) / 256);
    if (c->cfg.dim == 2) encodeKernel<2><<<blocks, 256, 0, c->stream>>>(c->net, dx, de, n);
    else encodeKernel<3><<<blocks, 256, 0, c->stream>>>(c->net, dx, de, n);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess && memory == ZGPU_MEM_HOST)
        e = cudaMemcpyAsync(enc, de, (size_t)n * kInputs * sizeof(float), cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    if (memory == ZGPU_MEM_HOST) cudaFree(de);
    ZC_CUDA(e);
    return ZGPU_OK;
}

int zgpu_cache_evaluate(zgpu_cache* c, int64_t n, const float* x, float* y, int memory) {
    if (!c || n < 0 || (n > 0 && (!x || !y))) return cfail(ZGPU_ERR_INVALID_ARG, "NULL argument");
    if (n == 0) return ZGPU_OK;
    const float* dx = nullptr;
    int st = stage(c, n, x, nullptr, memory, &dx, nullptr);
    if (st != ZGPU_OK) return st;
    float* dy = y;
    if (memory == ZGPU_MEM_HOST) dy = c->stageT;
    static bool a2 = false, a3 = false;
    if (!a2) { cudaFuncSetAttribute(evalKernelTc<2, 0>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kTcSmem); a2 = true; }
    if (!a3) { cudaFuncSetAttribute(evalKernelTc<3, 0>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kTcSmem); a3 = true; }
    const int blocks = (int)std::max<int64_t>(1, std::min<int64_t>((n + kTcRows - 1) / kTcRows, (int64_t)c->numSMs * 2));
    ZC_CUDA(cudaMemsetAsync(c->err, 0, sizeof(unsigned int), c->stream));
    if (c->cfg.dim == 2)
        evalKernelTc<2, 0><<<blocks, kTcRows, kTcSmem, c->stream>>>(c->net, dx, dy, n, nullptr, nullptr, nullptr,
                                                                    nullptr, nullptr, nullptr, c->err);
    else
        evalKernelTc<3, 0><<<blocks, kTcRows, kTcSmem, c->stream>>>(c->net, dx, dy, n, nullptr, nullptr, nullptr,
                                                                    nullptr, nullptr, nullptr, c->err);
    ZC_CUDA(cudaGetLastError());
    if (memory == ZGPU_MEM_HOST)
        ZC_CUDA(cudaMemcpyAsync(y, dy, (size_t)n * sizeof(float), cudaMemcpyDeviceToHost, c->stream));
    unsigned int err = 0;
    ZC_CUDA(cudaMemcpyAsync(&err, c->err, sizeof(unsigned int), cudaMemcpyDeviceToHost, c->stream));
    ZC_CUDA(cudaStreamSynchronize(c->stream));
    if (err) return cfail(ZGPU_ERR_DEVICE_STATE, "cache inference: device error word 0x%x", err);
    return ZGPU_OK;
}

}  // extern "C"
