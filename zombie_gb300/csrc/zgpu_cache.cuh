// zgpu_cache.cuh -- the neural cache on the device: multiresolution hash-grid encoding
// (FP16 table, Mueller et al. 2022) feeding a 32 -> 64 -> 64 -> 1 ReLU MLP whose two hidden
// layers run on the tensor cores (BF16 operands, FP32 accumulation, warp-level
// mma.sync.m16n8k16), with a hand-written backward pass and scatter of the table gradients.
//
// The cache has no counterpart in the reference: walks that end early query it for the
// solution at their last position.  Its definition (corner indexing, hash, blend, network) is
// restated in FP64 by the oracle; tests compare the two.
//
// Tile scheme: a warp owns 16 points (one m16 tile).  A block of 4 warps (64 points) shares
// the BF16 weights in shared memory, padded by 8 elements per row so the fragment loads of
// the 8 row groups fall in distinct banks.  The accumulator fragment of one layer is the A
// fragment of the next (two adjacent n8 tiles form one k16 tile), so activations stay in
// registers between layers; only the weight-gradient products, which contract over points,
// go through transposed shared-memory tiles.
#pragma once

#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include "zgpu_math.cuh"

namespace zg {
namespace cache {

constexpr int kHidden = 64;
constexpr int kInputs = 32;            // 16 levels x 2 features (unused levels encode 0)
constexpr int kMaxLevels = 16;
constexpr int kWarps = 4;
constexpr int kRows = 16;              // points per warp tile
constexpr int kBlockRows = kWarps * kRows;
constexpr int kS32 = kInputs + 8;      // padded row strides (BF16 elements)
constexpr int kS64 = kHidden + 8;

// device view of a cache: parameters and encoding constants
struct Net {
    int dim = 3;
    int levels = 16;
    int log2T = 19;
    uint32_t denseMask = 0;            // bit l: level l indexes its table densely
    float res[kMaxLevels];
    float lo[3], inv[3];
    const __half2* table = nullptr;            // [levels][T] (2 features per entry)
    const __nv_bfloat16* W1 = nullptr;         // [64][32] BF16 of the FP32 master
    const __nv_bfloat16* W2 = nullptr;         // [64][64]
    const __nv_bfloat16* W1lo = nullptr;       // BF16 of the rounding remainders (W = W1 + W1lo)
    const __nv_bfloat16* W2lo = nullptr;
    const float* b1 = nullptr;                 // FP32 master copies
    const float* b2 = nullptr;
    const float* w3 = nullptr;
    const float* b3 = nullptr;
};

// gradient buffers (FP32, laid out like the master parameters)
struct Grads {
    float2* table = nullptr;
    float* W1 = nullptr;
    float* b1 = nullptr;
    float* W2 = nullptr;
    float* b2 = nullptr;
    float* w3 = nullptr;
    float* b3 = nullptr;
    double* loss = nullptr;
};

// ------------------------------------------------------------------ encoding
// Corners of level l: the FP32 steps (normalise, clamp, scale, floor) are written with
// explicit round-to-nearest intrinsics so that no contraction changes the cell index.
template <int D>
ZG_D void levelCorners(const Net& N, int l, const float* x, uint32_t idx[1 << D], float w[1 << D]) {
    const float r = N.res[l];
    uint32_t cell[3];
    float frac[3];
#pragma unroll
    for (int i = 0; i < D; i++) {
        float xn = __fmul_rn(__fsub_rn(x[i], N.lo[i]), N.inv[i]);
        xn = fminf(fmaxf(xn, 0.0f), 1.0f);
        float p = __fmul_rn(xn, r);
        float c = fminf(floorf(p), r - 1.0f);
        cell[i] = (uint32_t)c;
        frac[i] = __fsub_rn(p, c);
    }
    const bool dense = (N.denseMask >> l) & 1u;
    const uint32_t stride = (uint32_t)r + 1u;
    const uint32_t mask = (1u << N.log2T) - 1u;
    const uint32_t primes[3] = {1u, 2654435761u, 805459861u};
#pragma unroll
    for (int c = 0; c < (1 << D); c++) {
        uint32_t h = 0, s = 1;
        float wt = 1.0f;
#pragma unroll
        for (int i = 0; i < D; i++) {
            uint32_t bit = (c >> i) & 1u;
            uint32_t ci = cell[i] + bit;
            if (dense) { h += ci * s; s *= stride; }
            else h ^= ci * primes[i];
            wt *= bit ? frac[i] : 1.0f - frac[i];
        }
        idx[c] = dense ? h : (h & mask);
        w[c] = wt;
    }
}

template <int D>
ZG_D float2 encodeLevel(const Net& N, int l, const float* x) {
    uint32_t idx[1 << D];
    float w[1 << D];
    levelCorners<D>(N, l, x, idx, w);
    const __half2* t = N.table + ((size_t)l << N.log2T);
    float2 f = make_float2(0.0f, 0.0f);
#pragma unroll
    for (int c = 0; c < (1 << D); c++) {
        float2 v = __half22float2(__ldg(t + idx[c]));
        f.x += w[c] * v.x;
        f.y += w[c] * v.y;
    }
    return f;
}

// Encodes the warp's 16 points into two row-major [16][kS32] BF16 tiles: E holds the
// rounded features, E + kRows * kS32 the rounding remainders (hi + lo carries ~16 mantissa
// bits into the tensor cores).  Lane j handles point j & 15 for levels (j >> 4) + 2s,
// s = 0..7; rows >= nValid and levels >= N.levels are 0.
template <int D>
ZG_D void encodeTile(const Net& N, const float (*x)[3], int nValid, __nv_bfloat16* E, int lane) {
    const int p = lane & 15;
#pragma unroll 1
    for (int s = 0; s < 8; s++) {
        int l = (lane >> 4) + 2 * s;
        float2 f = make_float2(0.0f, 0.0f);
        if (p < nValid && l < N.levels) f = encodeLevel<D>(N, l, x[p]);
        __nv_bfloat162 hi = __floats2bfloat162_rn(f.x, f.y);
        float2 h = __bfloat1622float2(hi);
        *reinterpret_cast<__nv_bfloat162*>(E + p * kS32 + 2 * l) = hi;
        *reinterpret_cast<__nv_bfloat162*>(E + kRows * kS32 + p * kS32 + 2 * l) = __floats2bfloat162_rn(f.x - h.x, f.y - h.y);
    }
}

// ------------------------------------------------------------------ tensor-core helpers
ZG_D uint32_t ld32(const __nv_bfloat16* p) { return *reinterpret_cast<const uint32_t*>(p); }
ZG_D uint32_t pack2(float lo, float hi) {
    __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
    return *reinterpret_cast<uint32_t*>(&v);
}
// BF16 pair of (a, b) and the pair of their rounding remainders
ZG_D void pack2split(float a, float b, uint32_t& hi, uint32_t& lo) {
    __nv_bfloat162 v = __floats2bfloat162_rn(a, b);
    float2 f = __bfloat1622float2(v);
    hi = *reinterpret_cast<uint32_t*>(&v);
    lo = pack2(a - f.x, b - f.y);
}
// D = A(16x16, row) * B(16x8, col) + C, BF16 in, FP32 accumulate
ZG_D void mma16816(float c[4], uint32_t a0, uint32_t a1, uint32_t a2, uint32_t a3, uint32_t b0, uint32_t b1) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};\n"
        : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
        : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b0), "r"(b1));
}

// shared-memory copy of the network weights used by a block
struct SharedWeights {
    __nv_bfloat16 W1[kHidden * kS32];    // [out][in]
    __nv_bfloat16 W2[kHidden * kS64];
    __nv_bfloat16 W1lo[kHidden * kS32];  // remainders of the BF16 rounding
    __nv_bfloat16 W2lo[kHidden * kS64];
    __nv_bfloat16 W1T[kInputs * kS64];   // [in][out] (backward)
    __nv_bfloat16 W2T[kHidden * kS64];
    float b1[kHidden], b2[kHidden], w3[kHidden];
    float b3;
};

ZG_D void loadWeights(const Net& N, SharedWeights& S, bool transposed) {
    for (int i = threadIdx.x; i < kHidden * kInputs; i += blockDim.x) {
        int o = i / kInputs, k = i % kInputs;
        __nv_bfloat16 v = N.W1[i];
        S.W1[o * kS32 + k] = v;
        S.W1lo[o * kS32 + k] = N.W1lo[i];
        if (transposed) S.W1T[k * kS64 + o] = v;
    }
    for (int i = threadIdx.x; i < kHidden * kHidden; i += blockDim.x) {
        int o = i / kHidden, k = i % kHidden;
        __nv_bfloat16 v = N.W2[i];
        S.W2[o * kS64 + k] = v;
        S.W2lo[o * kS64 + k] = N.W2lo[i];
        if (transposed) S.W2T[k * kS64 + o] = v;
    }
    for (int i = threadIdx.x; i < kHidden; i += blockDim.x) {
        S.b1[i] = N.b1[i]; S.b2[i] = N.b2[i]; S.w3[i] = N.w3[i];
    }
    if (threadIdx.x == 0) S.b3 = *N.b3;
}

// Forward pass of one warp tile.  h1/h2 hold the post-ReLU activations in accumulator layout
// (n-tile nt, element e: row g + 8 (e >> 1), column 8 nt + 2 t + (e & 1)); returns the output
// for rows g (y.x) and g + 8 (y.y), identical in the 4 lanes of a quad.  Activations and
// weights enter each layer as BF16 hi + lo pairs and every product takes three MMAs
// (hi*hi + lo*hi + hi*lo), so the output keeps FP32-class precision instead of BF16's 0.4%
// relative rounding, which would otherwise floor the cache's accuracy.
ZG_D float2 forwardTile(const SharedWeights& S, const __nv_bfloat16* E, float h1[8][4], float h2[8][4], int lane) {
    const int g = lane >> 2, t = lane & 3;
#pragma unroll
    for (int nt = 0; nt < 8; nt++) {
        float c0 = S.b1[8 * nt + 2 * t], c1 = S.b1[8 * nt + 2 * t + 1];
        h1[nt][0] = c0; h1[nt][1] = c1; h1[nt][2] = c0; h1[nt][3] = c1;
    }
#pragma unroll
    for (int kt = 0; kt < 2; kt++) {
        const __nv_bfloat16* El = E + kRows * kS32;
        const int o0 = g * kS32 + 16 * kt + 2 * t, o1 = (g + 8) * kS32 + 16 * kt + 2 * t;
        uint32_t a0 = ld32(E + o0), a1 = ld32(E + o1), a2 = ld32(E + o0 + 8), a3 = ld32(E + o1 + 8);
        uint32_t l0 = ld32(El + o0), l1 = ld32(El + o1), l2 = ld32(El + o0 + 8), l3 = ld32(El + o1 + 8);
#pragma unroll
        for (int nt = 0; nt < 8; nt++) {
            const int wo = (8 * nt + g) * kS32 + 16 * kt + 2 * t;
            const uint32_t b0 = ld32(S.W1 + wo), b1 = ld32(S.W1 + wo + 8);
            mma16816(h1[nt], a0, a1, a2, a3, b0, b1);
            mma16816(h1[nt], l0, l1, l2, l3, b0, b1);
            mma16816(h1[nt], a0, a1, a2, a3, ld32(S.W1lo + wo), ld32(S.W1lo + wo + 8));
        }
    }
#pragma unroll
    for (int nt = 0; nt < 8; nt++)
#pragma unroll
        for (int e = 0; e < 4; e++) h1[nt][e] = fmaxf(h1[nt][e], 0.0f);
#pragma unroll
    for (int nt = 0; nt < 8; nt++) {
        float c0 = S.b2[8 * nt + 2 * t], c1 = S.b2[8 * nt + 2 * t + 1];
        h2[nt][0] = c0; h2[nt][1] = c1; h2[nt][2] = c0; h2[nt][3] = c1;
    }
#pragma unroll
    for (int kt = 0; kt < 4; kt++) {
        uint32_t a0, a1, a2, a3, l0, l1, l2, l3;
        pack2split(h1[2 * kt][0], h1[2 * kt][1], a0, l0);
        pack2split(h1[2 * kt][2], h1[2 * kt][3], a1, l1);
        pack2split(h1[2 * kt + 1][0], h1[2 * kt + 1][1], a2, l2);
        pack2split(h1[2 * kt + 1][2], h1[2 * kt + 1][3], a3, l3);
#pragma unroll
        for (int nt = 0; nt < 8; nt++) {
            const int wo = (8 * nt + g) * kS64 + 16 * kt + 2 * t;
            const uint32_t b0 = ld32(S.W2 + wo), b1 = ld32(S.W2 + wo + 8);
            mma16816(h2[nt], a0, a1, a2, a3, b0, b1);
            mma16816(h2[nt], l0, l1, l2, l3, b0, b1);
            mma16816(h2[nt], a0, a1, a2, a3, ld32(S.W2lo + wo), ld32(S.W2lo + wo + 8));
        }
    }
    float y0 = 0.0f, y1 = 0.0f;
#pragma unroll
    for (int nt = 0; nt < 8; nt++) {
#pragma unroll
        for (int e = 0; e < 4; e++) h2[nt][e] = fmaxf(h2[nt][e], 0.0f);
        float wa = S.w3[8 * nt + 2 * t], wb = S.w3[8 * nt + 2 * t + 1];
        y0 += h2[nt][0] * wa + h2[nt][1] * wb;
        y1 += h2[nt][2] * wa + h2[nt][3] * wb;
    }
    y0 += __shfl_xor_sync(0xffffffffu, y0, 1);
    y0 += __shfl_xor_sync(0xffffffffu, y0, 2);
    y1 += __shfl_xor_sync(0xffffffffu, y1, 1);
    y1 += __shfl_xor_sync(0xffffffffu, y1, 2);
    return make_float2(y0 + S.b3, y1 + S.b3);
}

}  // namespace cache
}  // namespace zg
