// oracle_bvc.h -- TEST INFRASTRUCTURE, NOT PRODUCT CODE (see oracle_core.h).
//
// CPU restatement of BoundaryValueCaching::splat (variance_reduction/boundary_value_caching.h:
// 380-425 for one evaluation point, :652-773 splatBoundaryData, :775-811 splatSourceData) over
// the free-space Green's functions (core/distributions.h:58-307) and their kernel
// regularisations (:13-56).  Samples are visited in cache order and every statistic is a
// running (Welford) mean, kept in FP64 here.
#pragma once

#include "oracle_core.h"

namespace orc {

template <int D>
struct FreeSpaceGreens {
    Vec<D> x;
    bool yukawa = false;
    float sqrtLambda = 0.0f;
    float evaluate(float r) const {
        if (!yukawa) return D == 2 ? -std::log(r) / (2.0f * kPi) : 1.0f / (4.0f * kPi * r);
        const float mur = r * sqrtLambda;
        if (D == 2) return (float)bessel::k0(mur) / (2.0f * kPi);
        return std::exp(-mur) / (4.0f * kPi * r);
    }
    Vec<D> gradient(float r, const Vec<D>& y) const {
        const Vec<D> xy = x - y;
        if (!yukawa) return D == 2 ? (-1.0f / (2.0f * kPi * r * r)) * xy : (-1.0f / (4.0f * kPi * r * r * r)) * xy;
        const float mur = r * sqrtLambda;
        if (D == 2) return (-sqrtLambda * (float)bessel::k1(mur) / (2.0f * kPi * r)) * xy;
        const float qr = sqrtLambda * std::exp(-mur) * (1.0f + 1.0f / mur);
        return (-qr / (4.0f * kPi * r * r)) * xy;
    }
    float poissonKernel(float r, const Vec<D>& y, const Vec<D>& n) const {
        return -dot(n, gradient(r, y));
    }
    Vec<D> poissonKernelGradient(float r, const Vec<D>& y, const Vec<D>& n) const {
        const Vec<D> xy = x - y;
        const float r2 = r * r, ndxy = dot(n, xy);
        if (!yukawa) {
            if (D == 2) return (1.0f / (2.0f * kPi * r2)) * (n - (2.0f * ndxy / r2) * xy);
            return (1.0f / (4.0f * kPi * r2 * r)) * (n - (3.0f * ndxy / r2) * xy);
        }
        const float mur = r * sqrtLambda;
        if (D == 2) {
            const float k0 = (float)bessel::k0(mur), k1 = (float)bessel::k1(mur);
            const float k2 = k0 + (2.0f / mur) * k1;
            const float q1 = sqrtLambda * k1, q2 = sqrtLambda * sqrtLambda * (k0 + k2) / 2.0f;
            return (1.0f / (2.0f * kPi * r)) * (q1 * n - (ndxy / r2) * (q1 + r * q2) * xy);
        }
        const float e = std::exp(-mur);
        const float q1 = sqrtLambda * e * (1.0f + 1.0f / mur), q2 = sqrtLambda * e / mur;
        return (1.0f / (4.0f * kPi * r2)) * (q1 * n - (ndxy / r2) * (2.0f * q1 + q2) * xy);
    }
};

inline float regGreens(int D, float r) { return D == 2 ? 1.0f : std::erf(r); }
inline float regPoisson(int D, float r) {
    if (D == 2) return 1.0f - std::exp(-r * r);
    return std::erf(r) - 2.0f * r * std::exp(-r * r) / std::sqrt(kPi);
}

// one running statistic (solution and gradient moments)
struct SplatStat {
    double mean = 0.0, m2 = 0.0, gmean[3] = {0, 0, 0}, gm2[3] = {0, 0, 0};
    int n = 0;
    void add(double v, const double* g, int D) {
        n++;
        double d = v - mean; mean += d / n; m2 += d * (v - mean);
        for (int i = 0; i < D; i++) { double e = g[i] - gmean[i]; gmean[i] += e / n; gm2[i] += e * (g[i] - gmean[i]); }
    }
};

// splats every sample onto one evaluation point: stats[5] in the order of ZGPU_BVC_*
template <int D>
void bvcSplatPoint(const zgpu_bvc_samples& s, float absorption, float radiusClamp, float reg, float robinCutoff,
                   const Vec<D>& x, int evalType, SplatStat* stats) {
    FreeSpaceGreens<D> g;
    g.x = x;
    g.yukawa = absorption > 0.0f;
    g.sqrtLambda = std::sqrt(absorption);
    const float alpha0 = (evalType == ZGPU_SAMPLE_ON_ABSORBING_BOUNDARY || evalType == ZGPU_SAMPLE_ON_REFLECTING_BOUNDARY)
                             ? 2.0f : 1.0f;
    for (int64_t j = 0; j < s.n; j++) {
        const Vec<D> y = load<D>(s.pt + j * D);
        const int type = s.type[j];
        const bool aligned = s.estimate_normal_aligned ? s.estimate_normal_aligned[j] != 0 : false;
        const float pdf = s.pdf[j];
        float r = std::max(radiusClamp, norm(y - x));
        float G = g.evaluate(r);
        const Vec<D> dG = g.gradient(r, y);
        float alpha = alpha0;
        float est;
        double grad[3] = {0, 0, 0};
        int group;
        if (type == ZGPU_SAMPLE_ON_ABSORBING_BOUNDARY || type == ZGPU_SAMPLE_ON_REFLECTING_BOUNDARY) {
            const Vec<D> n = (aligned ? -1.0f : 1.0f) * load<D>(s.normal + j * D);
            float P = g.poissonKernel(r, y, n);
            const Vec<D> dP = g.poissonKernelGradient(r, y, n);
            const float dGn = norm(dG), dPn = norm(dP);
            if (!std::isfinite(G) || !std::isfinite(P) || !std::isfinite(dGn) || !std::isfinite(dPn)) continue;
            if (reg > 0.0f) {
                const float rr = r / reg;
                G *= regGreens(D, rr);
                P *= regPoisson(D, rr);
            }
            const float u = s.solution[j], dn = s.normal_derivative[j], h = s.contribution[j];
            const float kap = s.robin_coeff ? s.robin_coeff[j] : 0.0f;
            if (std::fabs(kap) > robinCutoff) {
                est = alpha * ((G + P / kap) * dn - P * h / kap) / pdf;
                if (alpha > 1.0f) alpha = 0.0f;
                for (int i = 0; i < D; i++) grad[i] = alpha * ((dG[i] + dP[i] / kap) * dn - dP[i] * h / kap) / pdf;
            } else if (std::fabs(kap) > 0.0f) {
                est = alpha * (G * h - (P + kap * G) * u) / pdf;
                if (alpha > 1.0f) alpha = 0.0f;
                for (int i = 0; i < D; i++) grad[i] = alpha * (dG[i] * h - (dP[i] + kap * dG[i]) * u) / pdf;
            } else {
                est = alpha * (G * dn - P * u) / pdf;
                if (alpha > 1.0f) alpha = 0.0f;
                for (int i = 0; i < D; i++) grad[i] = alpha * (dG[i] * dn - dP[i] * u) / pdf;
            }
            group = type == ZGPU_SAMPLE_ON_ABSORBING_BOUNDARY ? (aligned ? ZGPU_BVC_ABSORBING_ALIGNED : ZGPU_BVC_ABSORBING)
                                                              : (aligned ? ZGPU_BVC_REFLECTING_ALIGNED : ZGPU_BVC_REFLECTING);
        } else {
            if (!std::isfinite(G) || !std::isfinite(norm(dG))) continue;
            if (reg > 0.0f) G *= regGreens(D, r / reg);
            const float f = s.contribution[j];
            est = alpha * G * f / pdf;
            if (alpha > 1.0f) alpha = 0.0f;
            for (int i = 0; i < D; i++) grad[i] = alpha * dG[i] * f / pdf;
            group = ZGPU_BVC_SOURCE;
        }
        stats[group].add((double)est, grad, D);
    }
}

}  // namespace orc
