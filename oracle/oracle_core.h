// oracle_core.h -- TEST INFRASTRUCTURE, NOT PRODUCT CODE.
//
// CPU restatement of rohan-sawhney/zombie's walk hot path, used only as the checker
// by tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg.  Nothing in the
// zombie_gb300 package may include, link or call it.
//
// Parity status: the reference itself cannot be built (its FCPW, pcg32, Eigen and TBB
// dependencies are absent and it ships no tests or golden vectors), so this oracle is
// "parity unpinned" against the reference binary.  It is pinned instead by
//  (1) FP64 analytic solutions of the manufactured problems (tests/test_oracle_*.py),
//  (2) brute-force geometric queries vs. its own BVH traversals,
//  (3) Green's-function identities and A&S Bessel tables.
//
// Each function cites the reference file:line it restates (paths inside the zombie project).
#pragma once

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <functional>
#include <limits>
#include <memory>
#include <queue>
#include <thread>
#include <vector>

#include "../include/zgpu.h"

namespace orc {

static constexpr float kPi = 3.14159265358979323846f;
static constexpr float kMaxFloat = std::numeric_limits<float>::max();
static constexpr float kFcpwEpsilon = 1e-6f;  // tolerance used by the reflectance primitives

// ---------------------------------------------------------------------------------------
// small fixed-size vector (stands in for Eigen::Matrix<float,DIM,1>, core/pde.h:14-17)
template <int D>
struct Vec {
    float v[D];
    Vec() { for (int i = 0; i < D; i++) v[i] = 0.0f; }
    float& operator[](int i) { return v[i]; }
    float operator[](int i) const { return v[i]; }
    static Vec zero() { return Vec(); }
    static Vec constant(float c) { Vec r; for (int i = 0; i < D; i++) r.v[i] = c; return r; }
};
template <int D> inline Vec<D> operator+(const Vec<D>& a, const Vec<D>& b) { Vec<D> r; for (int i = 0; i < D; i++) r.v[i] = a.v[i] + b.v[i]; return r; }
template <int D> inline Vec<D> operator-(const Vec<D>& a, const Vec<D>& b) { Vec<D> r; for (int i = 0; i < D; i++) r.v[i] = a.v[i] - b.v[i]; return r; }
template <int D> inline Vec<D> operator-(const Vec<D>& a) { Vec<D> r; for (int i = 0; i < D; i++) r.v[i] = -a.v[i]; return r; }
template <int D> inline Vec<D> operator*(float s, const Vec<D>& a) { Vec<D> r; for (int i = 0; i < D; i++) r.v[i] = s * a.v[i]; return r; }
template <int D> inline Vec<D> operator*(const Vec<D>& a, float s) { return s * a; }
template <int D> inline Vec<D> operator/(const Vec<D>& a, float s) { Vec<D> r; for (int i = 0; i < D; i++) r.v[i] = a.v[i] / s; return r; }
template <int D> inline float dot(const Vec<D>& a, const Vec<D>& b) { float s = 0.0f; for (int i = 0; i < D; i++) s += a.v[i] * b.v[i]; return s; }
template <int D> inline float norm2(const Vec<D>& a) { return dot(a, a); }
template <int D> inline float norm(const Vec<D>& a) { return std::sqrt(norm2(a)); }
template <int D> inline Vec<D> normalized(const Vec<D>& a) { float n = norm(a); return n > 0.0f ? a / n : a; }
inline float cross2(const Vec<2>& a, const Vec<2>& b) { return a[0] * b[1] - a[1] * b[0]; }
inline Vec<3> cross3(const Vec<3>& a, const Vec<3>& b) {
    Vec<3> r; r[0] = a[1] * b[2] - a[2] * b[1]; r[1] = a[2] * b[0] - a[0] * b[2]; r[2] = a[0] * b[1] - a[1] * b[0]; return r;
}
template <int D> inline Vec<D> load(const float* p) { Vec<D> r; for (int i = 0; i < D; i++) r.v[i] = p[i]; return r; }
template <int D> inline void store(const Vec<D>& a, float* p) { for (int i = 0; i < D; i++) p[i] = a.v[i]; }

// ---------------------------------------------------------------------------------------
// PCG32 (O'Neill, "PCG: A Family of Simple Fast Space-Efficient Statistically Good
// Algorithms for Random Number Generation", 2014): 64-bit LCG state, XSH-RR output.
// The reference stores one such generator per SamplePoint (point_estimation/common.h:182).
struct Pcg32 {
    uint64_t state = 0x853c49e6748fea9bULL;
    uint64_t inc = 0xda3e39cb94b95bdbULL;
    Pcg32() {}
    Pcg32(uint64_t initstate, uint64_t initseq) { seed(initstate, initseq); }
    void seed(uint64_t initstate, uint64_t initseq) {
        state = 0u;
        inc = (initseq << 1u) | 1u;
        nextUInt();
        state += initstate;
        nextUInt();
    }
    uint32_t nextUInt() {
        uint64_t old = state;
        state = old * 6364136223846793005ULL + inc;
        uint32_t xorshifted = (uint32_t)(((old >> 18u) ^ old) >> 27u);
        uint32_t rot = (uint32_t)(old >> 59u);
        return (xorshifted >> rot) | (xorshifted << ((~rot + 1u) & 31));
    }
    // uniform float in [0,1) built from the top 23 bits
    float nextFloat() {
        uint32_t bits = (nextUInt() >> 9) | 0x3f800000u;
        float f;
        std::memcpy(&f, &bits, 4);
        return f - 1.0f;
    }
};

// ---------------------------------------------------------------------------------------
// sphere sampling (core/sampling.h:104-111 for 2D, :164-174 for 3D)
template <int D> Vec<D> sampleUnitSphereUniform(Pcg32& rng);
template <> inline Vec<2> sampleUnitSphereUniform<2>(Pcg32& rng) {
    float u = rng.nextFloat();
    float phi = 2.0f * kPi * u;
    Vec<2> r; r[0] = std::cos(phi); r[1] = std::sin(phi); return r;
}
template <> inline Vec<3> sampleUnitSphereUniform<3>(Pcg32& rng) {
    float u0 = rng.nextFloat();
    float u1 = rng.nextFloat();
    float z = 1.0f - 2.0f * u0;
    float r = std::sqrt(std::max(0.0f, 1.0f - z * z));
    float phi = 2.0f * kPi * u1;
    Vec<3> v; v[0] = r * std::cos(phi); v[1] = r * std::sin(phi); v[2] = z; return v;
}
template <int D> inline float pdfSampleSphereUniform(float r) {
    return D == 2 ? 1.0f / (2.0f * kPi * r) : 1.0f / (4.0f * kPi * r * r);
}

// ---------------------------------------------------------------------------------------
// Modified Bessel functions I0, I1, K0, K1 by the polynomial approximations of
// Abramowitz & Stegun, Handbook of Mathematical Functions, 9.8.1-9.8.8; evaluated in
// FP64 and returned as float, as core/bessel.h:219-368 does.
namespace bessel {
inline double i0(double x) {
    double ax = std::fabs(x);
    if (ax < 3.75) {
        double t = (x / 3.75) * (x / 3.75);
        return 1.0 + t * (3.5156229 + t * (3.0899424 + t * (1.2067492 + t * (0.2659732 + t * (0.0360768 + t * 0.0045813)))));
    }
    double t = 3.75 / ax;
    return (std::exp(ax) / std::sqrt(ax)) *
           (0.39894228 + t * (0.01328592 + t * (0.00225319 + t * (-0.00157565 + t * (0.00916281 +
            t * (-0.02057706 + t * (0.02635537 + t * (-0.01647633 + t * 0.00392377))))))));
}
inline double i1(double x) {
    double ax = std::fabs(x), r;
    if (ax < 3.75) {
        double t = (x / 3.75) * (x / 3.75);
        r = ax * (0.5 + t * (0.87890594 + t * (0.51498869 + t * (0.15084934 + t * (0.02658733 + t * (0.00301532 + t * 0.00032411))))));
    } else {
        double t = 3.75 / ax;
        r = 0.39894228 + t * (-0.03988024 + t * (-0.00362018 + t * (0.00163801 + t * (-0.01031555 +
            t * (0.02282967 + t * (-0.02895312 + t * (0.01787654 - t * 0.00420059)))))));
        r *= std::exp(ax) / std::sqrt(ax);
    }
    return x < 0.0 ? -r : r;
}
inline double k0(double x) {
    if (x <= 2.0) {
        double t = x * x / 4.0;
        return -std::log(x / 2.0) * i0(x) +
               (-0.57721566 + t * (0.42278420 + t * (0.23069756 + t * (0.03488590 + t * (0.00262698 + t * (0.00010750 + t * 0.0000074))))));
    }
    double t = 2.0 / x;
    return (std::exp(-x) / std::sqrt(x)) *
           (1.25331414 + t * (-0.07832358 + t * (0.02189568 + t * (-0.01062446 + t * (0.00587872 + t * (-0.00251540 + t * 0.00053208))))));
}
inline double k1(double x) {
    if (x <= 2.0) {
        double t = x * x / 4.0;
        return std::log(x / 2.0) * i1(x) +
               (1.0 / x) * (1.0 + t * (0.15443144 + t * (-0.67278579 + t * (-0.18156897 + t * (-0.01919402 + t * (-0.00110404 - t * 0.00004686))))));
    }
    double t = 2.0 / x;
    return (std::exp(-x) / std::sqrt(x)) *
           (1.25331414 + t * (0.23498619 + t * (-0.03655620 + t * (0.01504268 + t * (-0.00780353 + t * (0.00325614 - t * 0.00068245))))));
}
}  // namespace bessel

// ---------------------------------------------------------------------------------------
// Green's functions on a ball (core/distributions.h:323-1005)
template <int D>
struct GreensFnBall {
    Vec<D> c;
    float R = 0.0f;
    float rClamp = 1e-4f;
    virtual ~GreensFnBall() {}
    virtual void updateBall(const Vec<D>& c_, float R_) { c = c_; R = R_; rClamp = 1e-4f; }
    virtual Vec<D> sampleVolume(const Vec<D>& dir, Pcg32& rng, float& r, float& pdf) = 0;
    Vec<D> sampleVolume(Pcg32& rng, float& r, float& pdf) {
        Vec<D> dir = sampleUnitSphereUniform<D>(rng);
        return sampleVolume(dir, rng, r, pdf);
    }
    virtual float evaluate(float r) const = 0;
    virtual float norm() const = 0;
    virtual float directionSampledPoissonKernel(const Vec<D>& y) const = 0;
    virtual float reflectance(float r, const Vec<D>& dir, const Vec<D>& n, float robinCoeff) const = 0;
    // the gradient estimator's first step: |grad G| / r, the Poisson kernel at the centre and
    // its gradient at a point of the sphere (distributions.h:493-550, :600-659, :744-822, :905-994)
    virtual float gradientNorm(float r) const = 0;
    virtual float poissonKernelCentre() const = 0;
    virtual Vec<D> poissonKernelGradient(const Vec<D>& y) const = 0;
    Vec<D> gradient(float r, const Vec<D>& y) const { return gradientNorm(r) * (y - c); }

    // distributions.h:419-440
    Vec<D> rejectionSampleGreensFn(const Vec<D>& dir, float bound, Pcg32& rng, float& r, float& pdf) {
        int iter = 0;
        float fnNorm = norm();
        do {
            float u = rng.nextFloat();
            r = rng.nextFloat() * R;
            pdf = evaluate(r) / fnNorm;
            float pdfRadius = pdf / pdfSampleSphereUniform<D>(r);
            iter++;
            if (u < pdfRadius / bound) break;
        } while (iter < 1000);
        r = std::max(rClamp, r);
        if (r > R) r = R / 2.0f;
        return c + r * dir;
    }
};

template <int D> struct HarmonicGreensFnBall;
// distributions.h:453-556
template <> struct HarmonicGreensFnBall<2> : GreensFnBall<2> {
    Vec<2> sampleVolume(const Vec<2>& dir, Pcg32& rng, float& r, float& pdf) override {
        float u1 = rng.nextFloat();
        float u2 = rng.nextFloat();
        r = R * std::sqrt(u1 * u2);
        r = std::max(rClamp, r);
        if (r > R) r = R / 2.0f;
        pdf = evaluate(r) / norm();
        return c + r * dir;
    }
    float evaluate(float r) const override { return std::log(R / r) / (2.0f * kPi); }
    float norm() const override { return R * R / 4.0f; }
    float gradientNorm(float r) const override { return (1.0f / (r * r) - 1.0f / (R * R)) / (2.0f * kPi); }
    float poissonKernelCentre() const override { return 1.0f / (2.0f * kPi); }
    Vec<2> poissonKernelGradient(const Vec<2>& y) const override { return (2.0f / (2.0f * kPi * R * R)) * (y - c); }
    float directionSampledPoissonKernel(const Vec<2>&) const override { return 1.0f; }
    float reflectance(float r, const Vec<2>& dir, const Vec<2>& n, float robinCoeff) const override {
        if (std::fabs(robinCoeff) > 0.0f) {
            float P = dot(n, dir) / r;
            float G = std::log(R / r);
            return 1.0f - robinCoeff * G / P;
        }
        return 1.0f;
    }
};
// distributions.h:558-665
template <> struct HarmonicGreensFnBall<3> : GreensFnBall<3> {
    Vec<3> sampleVolume(const Vec<3>& dir, Pcg32& rng, float& r, float& pdf) override {
        float u1 = rng.nextFloat();
        float u2 = rng.nextFloat();
        float u3 = rng.nextFloat();
        float uMedian = std::max(std::min(u1, u2), std::min(std::max(u1, u2), u3));
        r = R * uMedian;
        r = std::max(rClamp, r);
        if (r > R) r = R / 2.0f;
        pdf = evaluate(r) / norm();
        return c + r * dir;
    }
    float evaluate(float r) const override { return (1.0f / r - 1.0f / R) / (4.0f * kPi); }
    float norm() const override { return R * R / 6.0f; }
    float gradientNorm(float r) const override { return (1.0f / (r * r * r) - 1.0f / (R * R * R)) / (4.0f * kPi); }
    float poissonKernelCentre() const override { return 1.0f / (4.0f * kPi); }
    Vec<3> poissonKernelGradient(const Vec<3>& y) const override { return (3.0f / (4.0f * kPi * R * R)) * (y - c); }
    float directionSampledPoissonKernel(const Vec<3>&) const override { return 1.0f; }
    float reflectance(float r, const Vec<3>& dir, const Vec<3>& n, float robinCoeff) const override {
        if (std::fabs(robinCoeff) > 0.0f) {
            float P = dot(n, dir) / (r * r);
            float G = 1.0f / r - 1.0f / R;
            return 1.0f - robinCoeff * G / P;
        }
        return 1.0f;
    }
};

template <int D> struct YukawaGreensFnBall;
// distributions.h:677-833
template <> struct YukawaGreensFnBall<2> : GreensFnBall<2> {
    float sqrtLambda, muR = 0, K0muR = 0, I0muR = 0, K1muR = 0, I1muR = 0;
    explicit YukawaGreensFnBall(float lambda) : sqrtLambda(std::sqrt(lambda)) {}
    void updateBall(const Vec<2>& c_, float R_) override {
        GreensFnBall<2>::updateBall(c_, R_);
        muR = R * sqrtLambda;
        K0muR = (float)bessel::k0(muR);
        I0muR = (float)bessel::i0(muR);
        K1muR = (float)bessel::k1(muR);
        I1muR = (float)bessel::i1(muR);
    }
    Vec<2> sampleVolume(const Vec<2>& dir, Pcg32& rng, float& r, float& pdf) override {
        float lambda = sqrtLambda * sqrtLambda;
        float bound = R <= lambda ?
                      std::max(std::max(2.2f / R, 2.2f / lambda), std::max(0.6f * std::sqrt(R), 0.6f * sqrtLambda)) :
                      std::max(std::min(2.2f / R, 2.2f / lambda), std::min(0.6f * std::sqrt(R), 0.6f * sqrtLambda));
        return rejectionSampleGreensFn(dir, bound, rng, r, pdf);
    }
    float evaluate(float r) const override {
        float mur = r * sqrtLambda;
        float K0mur = (float)bessel::k0(mur);
        float I0mur = (float)bessel::i0(mur);
        return (K0mur - I0mur * K0muR / I0muR) / (2.0f * kPi);
    }
    float poissonKernel() const { return 1.0f / (2.0f * kPi * I0muR); }
    float poissonKernelCentre() const override { return poissonKernel(); }
    float gradientNorm(float r) const override {
        float mur = r * sqrtLambda;
        float Qr = sqrtLambda * ((float)bessel::k1(mur) - (float)bessel::i1(mur) * K1muR / I1muR);
        return Qr / (2.0f * kPi * r);
    }
    Vec<2> poissonKernelGradient(const Vec<2>& y) const override {
        return (sqrtLambda / (R * I1muR) / (2.0f * kPi)) * (y - c);
    }
    float norm() const override { return (1.0f - 2.0f * kPi * poissonKernel()) / (sqrtLambda * sqrtLambda); }
    float dampening(float r) const {
        float mur = r * sqrtLambda;
        float K1mur = (float)bessel::k1(mur);
        float I1mur = (float)bessel::i1(mur);
        float Q = K1mur + I1mur * K0muR / I0muR;
        return mur * Q;
    }
    float directionSampledPoissonKernel(const Vec<2>& y) const override {
        float r = std::max(rClamp, orc::norm(y - c));
        return dampening(r);
    }
    float reflectance(float r, const Vec<2>& dir, const Vec<2>& n, float robinCoeff) const override {
        float Q = dampening(r);
        if (std::fabs(robinCoeff) > 0.0f) {
            float P = dot(n, dir) / r;
            float mur = r * sqrtLambda;
            float K0mur = (float)bessel::k0(mur);
            float I0mur = (float)bessel::i0(mur);
            float G = K0mur - I0mur * K0muR / I0muR;
            return Q - robinCoeff * G / P;
        }
        return Q;
    }
};
// distributions.h:835-1005
template <> struct YukawaGreensFnBall<3> : GreensFnBall<3> {
    float sqrtLambda, muR = 0, expmuR = 0, sinhmuR = 0, K32muR = 0, I32muR = 0;
    explicit YukawaGreensFnBall(float lambda) : sqrtLambda(std::sqrt(lambda)) {}
    void updateBall(const Vec<3>& c_, float R_) override {
        GreensFnBall<3>::updateBall(c_, R_);
        muR = R * sqrtLambda;
        expmuR = std::exp(-muR);
        float exp2muR = expmuR * expmuR;
        float coshmuR = (1.0f + exp2muR) / (2.0f * expmuR);
        sinhmuR = (1.0f - exp2muR) / (2.0f * expmuR);
        K32muR = expmuR * (1.0f + 1.0f / muR);
        I32muR = coshmuR - sinhmuR / muR;
    }
    Vec<3> sampleVolume(const Vec<3>& dir, Pcg32& rng, float& r, float& pdf) override {
        float lambda = sqrtLambda * sqrtLambda;
        float bound = R <= lambda ?
                      std::max(std::max(2.0f / R, 2.0f / lambda), std::max(0.5f * std::sqrt(R), 0.5f * sqrtLambda)) :
                      std::max(std::min(2.0f / R, 2.0f / lambda), std::min(0.5f * std::sqrt(R), 0.5f * sqrtLambda));
        return rejectionSampleGreensFn(dir, bound, rng, r, pdf);
    }
    float evaluate(float r) const override {
        float mur = r * sqrtLambda;
        float expmur = std::exp(-mur);
        float sinhmur = (1.0f - expmur * expmur) / (2.0f * expmur);
        return (expmur - expmuR * sinhmur / sinhmuR) / (4.0f * kPi * r);
    }
    float poissonKernel() const { return muR / (4.0f * kPi * sinhmuR); }
    float poissonKernelCentre() const override { return poissonKernel(); }
    float gradientNorm(float r) const override {
        float mur = r * sqrtLambda;
        float expmur = std::exp(-mur);
        float exp2mur = expmur * expmur;
        float coshmur = (1.0f + exp2mur) / (2.0f * expmur);
        float sinhmur = (1.0f - exp2mur) / (2.0f * expmur);
        float K32mur = expmur * (1.0f + 1.0f / mur);
        float I32mur = coshmur - sinhmur / mur;
        float Qr = sqrtLambda * (K32mur - I32mur * K32muR / I32muR);
        return Qr / (4.0f * kPi * r * r);
    }
    Vec<3> poissonKernelGradient(const Vec<3>& y) const override {
        return (sqrtLambda * sqrtLambda / I32muR / (4.0f * kPi)) * (y - c);
    }
    float norm() const override { return (1.0f - 4.0f * kPi * poissonKernel()) / (sqrtLambda * sqrtLambda); }
    float dampening(float r) const {
        float mur = r * sqrtLambda;
        float expmur = std::exp(-mur);
        float exp2mur = expmur * expmur;
        float coshmur = (1.0f + exp2mur) / (2.0f * expmur);
        float sinhmur = (1.0f - exp2mur) / (2.0f * expmur);
        float K32mur = expmur * (1.0f + 1.0f / mur);
        float I32mur = coshmur - sinhmur / mur;
        float Q = K32mur + I32mur * expmuR / sinhmuR;
        return mur * Q;
    }
    float directionSampledPoissonKernel(const Vec<3>& y) const override {
        float r = std::max(rClamp, orc::norm(y - c));
        return dampening(r);
    }
    float reflectance(float r, const Vec<3>& dir, const Vec<3>& n, float robinCoeff) const override {
        float Q = dampening(r);
        if (std::fabs(robinCoeff) > 0.0f) {
            float P = dot(n, dir) / (r * r);
            float mur = r * sqrtLambda;
            float expmur = std::exp(-mur);
            float sinhmur = (1.0f - expmur * expmur) / (2.0f * expmur);
            float G = (expmur - expmuR * sinhmur / sinhmuR) / r;
            return Q - robinCoeff * G / P;
        }
        return Q;
    }
};

}  // namespace orc
