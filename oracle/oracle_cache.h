// Oracle of the neural cache: hash-grid encoding + 2x64 MLP, forward and analytic backward
// in FP64.  TEST INFRASTRUCTURE ONLY: the GPU cache kernels (zombie_gb300/csrc/zgpu_cache.cu)
// are checked against it; nothing in the product path links or calls this file.
//
// The neural cache has no counterpart in the reference (it is an addition of this
// implementation); this file states its definition:
//   encoding (multiresolution hash grid, Mueller et al. 2022, "Instant Neural Graphics
//   Primitives"): L levels of F = 2 features; level l has resolution res[l]; a position x in
//   the domain box is normalised to [0,1]^D, scaled by res[l], and the features of the 2^D
//   cell corners are blended with multilinear weights.  A corner indexes its level's table
//   densely when (res+1)^D <= T, else by the spatial hash (c0 * 1) ^ (c1 * 2654435761) ^
//   (c2 * 805459861) modulo T (a power of two).
//   network: z1 = W1 e + b1, h1 = relu(z1), z2 = W2 h1 + b2, h2 = relu(z2), y = w3 . h2 + b3
//   with e in R^{2L}, hidden width 64.
//   loss: mean squared error (1/B) sum_i (y_i - t_i)^2.
#pragma once

#include <cmath>
#include <cstdint>
#include <vector>

namespace orc {

constexpr int kCacheHidden = 64;
constexpr int kCacheFeatures = 2;

struct CacheModel {
    int dim = 3;
    int levels = 16;
    int log2T = 19;
    std::vector<float> res;          // per level resolution (integer valued)
    double lo[3] = {0, 0, 0}, inv[3] = {1, 1, 1};   // normalisation x -> (x - lo) * inv
    // parameters (read as given; the GPU passes its rounded FP16 / BF16 copies)
    std::vector<double> table;       // levels * T * 2
    std::vector<double> W1, b1, W2, b2, w3;   // W1 [64][2L], W2 [64][64], w3 [64]
    double b3 = 0.0;

    int inputs() const { return kCacheFeatures * levels; }
    uint32_t tableSize() const { return 1u << log2T; }
};

struct CacheCorner { uint32_t index; double weight; };

// corners of level l for position x (the GPU evaluates the normalisation, the cell and the
// weights in FP32: the oracle repeats those FP32 steps so the indices are identical)
inline int cacheCorners(const CacheModel& m, int l, const float* x, CacheCorner* out) {
    const int D = m.dim;
    const uint32_t T = m.tableSize();
    const float r = m.res[l];
    int cell[3] = {0, 0, 0};
    float frac[3] = {0, 0, 0};
    for (int i = 0; i < D; i++) {
        float xn = (x[i] - (float)m.lo[i]) * (float)m.inv[i];
        xn = std::fmin(std::fmax(xn, 0.0f), 1.0f);
        float p = xn * r;
        float c = std::floor(p);
        c = std::fmin(c, r - 1.0f);
        cell[i] = (int)c;
        frac[i] = p - c;
    }
    const uint32_t stride = (uint32_t)r + 1u;
    uint64_t dense = 1;
    for (int i = 0; i < D; i++) dense *= stride;
    const bool isDense = dense <= T;
    const uint32_t primes[3] = {1u, 2654435761u, 805459861u};
    int n = 0;
    for (int c = 0; c < (1 << D); c++) {
        uint32_t idx = 0, s = 1;
        double w = 1.0;
        for (int i = 0; i < D; i++) {
            int bit = (c >> i) & 1;
            uint32_t ci = (uint32_t)(cell[i] + bit);
            if (isDense) { idx += ci * s; s *= stride; }
            else idx ^= ci * primes[i];
            w *= bit ? (double)frac[i] : 1.0 - (double)frac[i];
        }
        out[n].index = isDense ? idx : (idx & (T - 1u));
        out[n].weight = w;
        n++;
    }
    return n;
}

inline void cacheEncode(const CacheModel& m, const float* x, double* e) {
    CacheCorner cs[8];
    const uint32_t T = m.tableSize();
    for (int l = 0; l < m.levels; l++) {
        int n = cacheCorners(m, l, x, cs);
        double f0 = 0.0, f1 = 0.0;
        for (int k = 0; k < n; k++) {
            const double* t = &m.table[((size_t)l * T + cs[k].index) * 2];
            f0 += cs[k].weight * t[0];
            f1 += cs[k].weight * t[1];
        }
        e[2 * l] = f0;
        e[2 * l + 1] = f1;
    }
}

struct CacheActivations {
    double e[32], z1[kCacheHidden], h1[kCacheHidden], z2[kCacheHidden], h2[kCacheHidden], y;
};

inline double cacheForward(const CacheModel& m, const float* x, CacheActivations& a) {
    const int I = m.inputs(), H = kCacheHidden;
    cacheEncode(m, x, a.e);
    for (int o = 0; o < H; o++) {
        double s = m.b1[o];
        for (int i = 0; i < I; i++) s += m.W1[(size_t)o * I + i] * a.e[i];
        a.z1[o] = s;
        a.h1[o] = s > 0.0 ? s : 0.0;
    }
    for (int o = 0; o < H; o++) {
        double s = m.b2[o];
        for (int i = 0; i < H; i++) s += m.W2[(size_t)o * H + i] * a.h1[i];
        a.z2[o] = s;
        a.h2[o] = s > 0.0 ? s : 0.0;
    }
    double y = m.b3;
    for (int i = 0; i < H; i++) y += m.w3[i] * a.h2[i];
    a.y = y;
    return y;
}

// gradients of the mean squared error over a batch; grads laid out like the parameters
struct CacheGrads {
    std::vector<double> table, W1, b1, W2, b2, w3;
    double b3 = 0.0;
};

inline double cacheLossAndGrads(const CacheModel& m, int n, const float* x, const float* target, CacheGrads& g) {
    const int I = m.inputs(), H = kCacheHidden, D = m.dim;
    const uint32_t T = m.tableSize();
    g.table.assign(m.table.size(), 0.0);
    g.W1.assign(m.W1.size(), 0.0); g.b1.assign(H, 0.0);
    g.W2.assign(m.W2.size(), 0.0); g.b2.assign(H, 0.0);
    g.w3.assign(H, 0.0); g.b3 = 0.0;
    double loss = 0.0;
    CacheActivations a;
    double dz2[kCacheHidden], dh1[kCacheHidden], dz1[kCacheHidden], de[32];
    CacheCorner cs[8];
    for (int p = 0; p < n; p++) {
        const float* xp = x + (size_t)p * D;
        double y = cacheForward(m, xp, a);
        double r = y - (double)target[p];
        loss += r * r / n;
        double dy = 2.0 * r / n;
        g.b3 += dy;
        for (int i = 0; i < H; i++) {
            g.w3[i] += dy * a.h2[i];
            dz2[i] = a.z2[i] > 0.0 ? dy * m.w3[i] : 0.0;
        }
        for (int i = 0; i < H; i++) dh1[i] = 0.0;
        for (int o = 0; o < H; o++) {
            g.b2[o] += dz2[o];
            for (int i = 0; i < H; i++) {
                g.W2[(size_t)o * H + i] += dz2[o] * a.h1[i];
                dh1[i] += dz2[o] * m.W2[(size_t)o * H + i];
            }
        }
        for (int i = 0; i < H; i++) dz1[i] = a.z1[i] > 0.0 ? dh1[i] : 0.0;
        for (int i = 0; i < I; i++) de[i] = 0.0;
        for (int o = 0; o < H; o++) {
            g.b1[o] += dz1[o];
            for (int i = 0; i < I; i++) {
                g.W1[(size_t)o * I + i] += dz1[o] * a.e[i];
                de[i] += dz1[o] * m.W1[(size_t)o * I + i];
            }
        }
        for (int l = 0; l < m.levels; l++) {
            int nc = cacheCorners(m, l, xp, cs);
            for (int k = 0; k < nc; k++) {
                double* t = &g.table[((size_t)l * T + cs[k].index) * 2];
                t[0] += cs[k].weight * de[2 * l];
                t[1] += cs[k].weight * de[2 * l + 1];
            }
        }
    }
    return loss;
}

}  // namespace orc
