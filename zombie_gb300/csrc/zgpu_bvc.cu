// zgpu_bvc.cu -- Boundary Value Caching splat (variance_reduction/boundary_value_caching.h)
// and device evaluation of the PDE's fields.
//
// The splat is an all-pairs kernel: every cache sample adds a free-space Green's function
// estimate of the solution and its gradient to every evaluation point.  One thread owns one
// evaluation point; the block stages the cache through shared memory in tiles of kTile
// samples, every thread reading each staged sample (a broadcast), so the cache is read from
// global memory once per block.  The five statistics of an evaluation point are filled by
// separate launches (one per statistic group present in the cache) so that a thread carries
// the moments of one group only; per-tile FP32 sums, shifted by the thread's first estimate,
// are folded into FP64 and merged with the point's moments (Chan et al.) at the end.
#include <cfloat>
#include <cmath>

#include "zgpu_internal.h"

namespace zg {
namespace {

constexpr int kSplatThreads = 128;
constexpr int kTile = 128;

// GreensFnFreeSpace (core/distributions.h:58-307) with the pole at x: harmonic, or Yukawa
// with sqrt(lambda) = sqrt(absorption coefficient)
template <int D, bool SCREENED>
struct FreeSpace {
    V<D> x;
    float mu;   // sqrt(lambda)
    ZG_D float evaluate(float r) const {
        if (!SCREENED) return D == 2 ? -logf(r) / (2.0f * kPi) : 1.0f / (4.0f * kPi * r);
        if (D == 2) return besselK0(r * mu) / (2.0f * kPi);
        return expf(-r * mu) / (4.0f * kPi * r);
    }
    // the radial factor q(r) with grad G = -xy q(r), P = n.xy q(r), xy = x - y
    ZG_D float radial(float r) const {
        if (!SCREENED) return D == 2 ? 1.0f / (2.0f * kPi * r * r) : 1.0f / (4.0f * kPi * r * r * r);
        const float mur = r * mu;
        if (D == 2) return mu * besselK1(mur) / (2.0f * kPi * r);
        return mu * expf(-mur) * (1.0f + 1.0f / mur) / (4.0f * kPi * r * r);
    }
    // gradient of the Poisson kernel at y for normal n
    ZG_D V<D> poissonGradient(float r, V<D> xy, V<D> n) const {
        const float ndxy = dot(n, xy), r2 = r * r;
        if (!SCREENED) {
            if (D == 2) return (1.0f / (2.0f * kPi * r2)) * (n - (2.0f * ndxy / r2) * xy);
            return (1.0f / (4.0f * kPi * r2 * r)) * (n - (3.0f * ndxy / r2) * xy);
        }
        const float mur = r * mu;
        if (D == 2) {
            const float k0 = besselK0(mur), k1 = besselK1(mur);
            const float k2 = k0 + (2.0f / mur) * k1;            // K2 by the recurrence
            const float q1 = mu * k1, q2 = mu * mu * (k0 + k2) / 2.0f;
            return (1.0f / (2.0f * kPi * r)) * (q1 * n - (ndxy / r2) * (q1 + r * q2) * xy);
        }
        const float e = expf(-mur);
        const float q1 = mu * e * (1.0f + 1.0f / mur), q2 = mu * e / mur;
        return (1.0f / (4.0f * kPi * r2)) * (q1 * n - (ndxy / r2) * (2.0f * q1 + q2) * xy);
    }
};


// the statistic group a sample feeds (splat / splatBoundaryData / splatSourceData)
ZG_HD int groupOf(int type, int aligned) {
    if (type == ZGPU_SAMPLE_ON_ABSORBING_BOUNDARY) return aligned ? ZGPU_BVC_ABSORBING_ALIGNED : ZGPU_BVC_ABSORBING;
    if (type == ZGPU_SAMPLE_ON_REFLECTING_BOUNDARY) return aligned ? ZGPU_BVC_REFLECTING_ALIGNED : ZGPU_BVC_REFLECTING;
    return ZGPU_BVC_SOURCE;
}

ZG_D bool finiteF(float v) { return !(isinf(v) || isnan(v)); }

template <int D, bool SCREENED>
__global__ void __launch_bounds__(kSplatThreads) splatKernel(const __grid_constant__ BvcSplatParams P) {
    __shared__ float sp[D][kTile], sn[D][kTile], spdf[kTile], ssol[kTile], sdn[kTile], scon[kTile], skap[kTile];
    __shared__ int sgrp[kTile];
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    bool active = i < P.nEval;
    V<D> x = vzero<D>();
    float alpha = 1.0f;
    if (active) {
        x = vload<D>(P.evalPt + (size_t)i * D);
        const float dA = P.evalDistA[i];
        const float dR = P.evalDistR ? P.evalDistR[i] : FLT_MAX;
        // don't evaluate closer to the boundary than the cutoffs (boundary_value_caching.h:388-390)
        if (dA < P.cutoffA || dR < P.cutoffR) active = false;
        const int t = P.evalType ? P.evalType[i] : ZGPU_SAMPLE_IN_DOMAIN;
        if (t == ZGPU_SAMPLE_ON_ABSORBING_BOUNDARY || t == ZGPU_SAMPLE_ON_REFLECTING_BOUNDARY) alpha = 2.0f;
    }
    FreeSpace<D, SCREENED> g;
    g.x = x;
    g.mu = P.sqrtLambda;
    const bool source = P.group == ZGPU_BVC_SOURCE;
    // shifted moments: K = the thread's first estimate
    bool haveK = false;
    float kS = 0.0f, kG[D];
    double accS = 0.0, accQ = 0.0, accG[D], accGQ[D];
#pragma unroll
    for (int d = 0; d < D; d++) { kG[d] = 0.0f; accG[d] = 0.0; accGQ[d] = 0.0; }
    long long count = 0;
    // this block's share of the cache (split along grid.y when the evaluation points alone
    // cannot fill the GPU)
    const int64_t begin = (int64_t)blockIdx.y * P.splitChunk;
    const int64_t end = min(P.nSamples, begin + P.splitChunk);
    for (int64_t base = begin; base < end; base += kTile) {
        const int64_t j = base + threadIdx.x;
        if (threadIdx.x < kTile) {
            int grp = -1;
            if (j < end) {
                const int al = P.aligned ? P.aligned[j] : 0;
                grp = groupOf(P.type[j], al);
                const float sgn = (grp != ZGPU_BVC_SOURCE && al) ? -1.0f : 1.0f;
#pragma unroll
                for (int d = 0; d < D; d++) {
                    sp[d][threadIdx.x] = P.pt[(size_t)j * D + d];
                    sn[d][threadIdx.x] = sgn * P.normal[(size_t)j * D + d];
                }
                spdf[threadIdx.x] = P.pdf[j];
                ssol[threadIdx.x] = P.solution[j];
                sdn[threadIdx.x] = P.normalDerivative[j];
                scon[threadIdx.x] = P.contribution[j];
                skap[threadIdx.x] = P.robinCoeff ? P.robinCoeff[j] : 0.0f;
            }
            sgrp[threadIdx.x] = grp;
        }
        __syncthreads();
        if (active) {
            const int m = end - base < kTile ? (int)(end - base) : kTile;
            float s = 0.0f, q = 0.0f, gs[D], gq[D];
#pragma unroll
            for (int d = 0; d < D; d++) { gs[d] = 0.0f; gq[d] = 0.0f; }
            int c = 0;
            for (int k = 0; k < m; k++) {
                if (sgrp[k] != P.group) continue;
                V<D> y, n, xy;
#pragma unroll
                for (int d = 0; d < D; d++) { y[d] = sp[d][k]; n[d] = sn[d][k]; xy[d] = x[d] - y[d]; }
                float r = fmaxf(P.radiusClamp, len(xy));
                float G = g.evaluate(r);
                const float qr = g.radial(r);
                const V<D> dG = -qr * xy;
                const float pdf = spdf[k];
                float est;
                V<D> grad;
                if (source) {
                    // splatSourceData (boundary_value_caching.h:775-811)
                    if (!finiteF(G) || !finiteF(len(dG))) continue;
                    if (P.regularization > 0.0f) G *= kernelRegularizationG<D>(r / P.regularization);
                    const float f = scon[k];
                    est = alpha * G * f / pdf;
                    const float a = alpha > 1.0f ? 0.0f : alpha;     // no gradient on the boundary
                    grad = (a * f / pdf) * dG;
                } else {
                    // splatBoundaryData (boundary_value_caching.h:652-773)
                    float Pk = dot(n, xy) * qr;
                    const V<D> dP = g.poissonGradient(r, xy, n);
                    if (!finiteF(G) || !finiteF(Pk) || !finiteF(len(dG)) || !finiteF(len(dP))) continue;
                    if (P.regularization > 0.0f) {
                        const float rr = r / P.regularization;
                        G *= kernelRegularizationG<D>(rr);
                        Pk *= kernelRegularizationP<D>(rr);
                    }
                    const float u = ssol[k], dn = sdn[k], h = scon[k], kap = skap[k];
                    const float a = alpha > 1.0f ? 0.0f : alpha;
                    if (fabsf(kap) > P.robinCutoff) {
                        est = alpha * ((G + Pk / kap) * dn - Pk * h / kap) / pdf;
                        // a ((dG + dP / kappa) dn - dP h / kappa) / pdf
                        grad = (a / pdf) * (((dn - h) / kap) * dP + dn * dG);
                    } else if (fabsf(kap) > 0.0f) {
                        est = alpha * (G * h - (Pk + kap * G) * u) / pdf;
                        grad = (a / pdf) * (h * dG - u * (dP + kap * dG));
                    } else {
                        est = alpha * (G * dn - Pk * u) / pdf;
                        grad = (a / pdf) * (dn * dG - u * dP);
                    }
                }
                if (!haveK) {
                    haveK = true;
                    kS = est;
#pragma unroll
                    for (int d = 0; d < D; d++) kG[d] = grad[d];
                }
                const float ds = est - kS;
                s += ds; q += ds * ds;
#pragma unroll
                for (int d = 0; d < D; d++) { const float e = grad[d] - kG[d]; gs[d] += e; gq[d] += e * e; }
                c++;
            }
            accS += s; accQ += q;
#pragma unroll
            for (int d = 0; d < D; d++) { accG[d] += gs[d]; accGQ[d] += gq[d]; }
            count += c;
        }
        __syncthreads();
    }
    if (i >= P.nEval) return;
    const double n2 = (double)count;
    const double mean2 = count ? kS + accS / n2 : 0.0;
    const double m22 = count ? fmax(0.0, accQ - accS * accS / n2) : 0.0;
    if (P.partial) {
        // split cache: this block's moments for the merge kernel (count 0 included)
        double* out = P.partial + ((size_t)blockIdx.y * P.nEval + i) * (3 + 2 * D);
        out[0] = n2; out[1] = mean2; out[2] = m22;
#pragma unroll
        for (int d = 0; d < D; d++) {
            out[3 + d] = count ? kG[d] + accG[d] / n2 : 0.0;
            out[3 + D + d] = count ? fmax(0.0, accGQ[d] - accG[d] * accG[d] / n2) : 0.0;
        }
        return;
    }
    if (!active || count == 0) return;
    // moments of this launch, merged with the point's (SampleStatistics::merge, common.h:268-310)
    const size_t slot = (size_t)i * ZGPU_BVC_GROUPS + P.group;
    const int n1 = P.count[slot];
    const double nt = (double)n1 + n2;
    if (n1 == 0) {
        P.mean[slot] = mean2;
        P.m2[slot] = m22;
    } else {
        const double m1 = P.mean[slot], delta = mean2 - m1;
        P.mean[slot] = m1 + delta * (n2 / nt);
        P.m2[slot] = P.m2[slot] + m22 + delta * delta * ((double)n1 * n2 / nt);
    }
#pragma unroll
    for (int d = 0; d < D; d++) {
        const size_t gslot = slot * D + d;
        const double gm2 = kG[d] + accG[d] / n2;
        const double gv2 = fmax(0.0, accGQ[d] - accG[d] * accG[d] / n2);
        if (n1 == 0) {
            P.gradMean[gslot] = gm2;
            if (P.gradM2) P.gradM2[gslot] = gv2;
        } else {
            const double m1 = P.gradMean[gslot], delta = gm2 - m1;
            P.gradMean[gslot] = m1 + delta * (n2 / nt);
            if (P.gradM2) P.gradM2[gslot] = P.gradM2[gslot] + gv2 + delta * delta * ((double)n1 * n2 / nt);
        }
    }
    P.count[slot] = (int)(n1 + count);
}

// merges the split moments of every evaluation point, then into its statistics
template <int D>
__global__ void splatMergeKernel(const __grid_constant__ BvcSplatParams P, int splits) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= P.nEval) return;
    double n = 0.0, mean = 0.0, m2 = 0.0, gm[D], gv[D];
#pragma unroll
    for (int d = 0; d < D; d++) { gm[d] = 0.0; gv[d] = 0.0; }
    for (int sp = 0; sp < splits; sp++) {
        const double* in = P.partial + ((size_t)sp * P.nEval + i) * (3 + 2 * D);
        const double nb = in[0];
        if (nb == 0.0) continue;
        const double nt = n + nb, delta = in[1] - mean;
        mean += delta * (nb / nt);
        m2 += in[2] + delta * delta * (n * nb / nt);
#pragma unroll
        for (int d = 0; d < D; d++) {
            const double e = in[3 + d] - gm[d];
            gm[d] += e * (nb / nt);
            gv[d] += in[3 + D + d] + e * e * (n * nb / nt);
        }
        n = nt;
    }
    if (n == 0.0) return;
    const size_t slot = (size_t)i * ZGPU_BVC_GROUPS + P.group;
    const int n1 = P.count[slot];
    const double nt = (double)n1 + n;
    const double delta = mean - P.mean[slot];
    if (n1 == 0) {
        P.mean[slot] = mean;
        P.m2[slot] = m2;
    } else {
        P.mean[slot] += delta * (n / nt);
        P.m2[slot] += m2 + delta * delta * ((double)n1 * n / nt);
    }
#pragma unroll
    for (int d = 0; d < D; d++) {
        const size_t gslot = slot * D + d;
        if (n1 == 0) {
            P.gradMean[gslot] = gm[d];
            if (P.gradM2) P.gradM2[gslot] = gv[d];
        } else {
            const double e = gm[d] - P.gradMean[gslot];
            P.gradMean[gslot] += e * (n / nt);
            if (P.gradM2) P.gradM2[gslot] += gv[d] + e * e * ((double)n1 * n / nt);
        }
    }
    P.count[slot] = n1 + (int)n;
}

// PDE fields at points (zgpu_pde_evaluate)
template <int D>
__global__ void pdeKernel(const zgpu_pde pde, int64_t n, const float* __restrict__ x, const float* __restrict__ nrm,
                          const int* __restrict__ aligned, float* src, float* dir, float* rob, float* kap) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    DevicePde<D> p;
    p.p = &pde;
    const V<D> xi = vload<D>(x + (size_t)i * D);
    const V<D> ni = nrm ? vload<D>(nrm + (size_t)i * D) : vzero<D>();
    const bool al = aligned ? aligned[i] != 0 : false;
    if (src) src[i] = p.source(xi);
    if (dir) dir[i] = p.dirichlet(xi, al);
    if (rob) rob[i] = p.robin(xi, ni, al);
    if (kap) kap[i] = p.robinCoeff(xi, al);
}

}  // namespace

int bvcSplitCount(int64_t nEval, int64_t nSamples, int numSMs) {
    // enough blocks for ~8 resident per SM, each split at least 8 tiles of the cache
    const int64_t evalBlocks = (nEval + kSplatThreads - 1) / kSplatThreads;
    const int64_t want = ((int64_t)numSMs * 8 + evalBlocks - 1) / evalBlocks;
    const int64_t maxSplits = (nSamples + 8 * kTile - 1) / (8 * kTile);
    int64_t s = want < maxSplits ? want : maxSplits;
    if (s > 64) s = 64;
    return s < 1 ? 1 : (int)s;
}

cudaError_t launchBvcSplat(int D, bool screened, const BvcSplatParams& p0, int splits, cudaStream_t s) {
    if (p0.nEval == 0 || p0.nSamples == 0) return cudaSuccess;
    BvcSplatParams p = p0;
    if (splits <= 1) { p.partial = nullptr; splits = 1; }
    const int64_t tiles = (p.nSamples + kTile - 1) / kTile;
    p.splitChunk = ((tiles + splits - 1) / splits) * kTile;
    const dim3 grid((unsigned)((p.nEval + kSplatThreads - 1) / kSplatThreads), (unsigned)splits);
    if (D == 2) {
        if (screened) splatKernel<2, true><<<grid, kSplatThreads, 0, s>>>(p);
        else splatKernel<2, false><<<grid, kSplatThreads, 0, s>>>(p);
    } else {
        if (screened) splatKernel<3, true><<<grid, kSplatThreads, 0, s>>>(p);
        else splatKernel<3, false><<<grid, kSplatThreads, 0, s>>>(p);
    }
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess || !p.partial) return e;
    const unsigned mg = (unsigned)((p.nEval + 127) / 128);
    if (D == 2) splatMergeKernel<2><<<mg, 128, 0, s>>>(p, splits);
    else splatMergeKernel<3><<<mg, 128, 0, s>>>(p, splits);
    return cudaGetLastError();
}

cudaError_t launchPdeEvaluate(int D, const zgpu_pde& pde, int64_t n, const float* x, const float* nrm, const int* aligned,
                              float* src, float* dir, float* rob, float* kap, cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    const unsigned grid = (unsigned)((n + 255) / 256);
    if (D == 2) pdeKernel<2><<<grid, 256, 0, s>>>(pde, n, x, nrm, aligned, src, dir, rob, kap);
    else pdeKernel<3><<<grid, 256, 0, s>>>(pde, n, x, nrm, aligned, src, dir, rob, kap);
    return cudaGetLastError();
}

}  // namespace zg
