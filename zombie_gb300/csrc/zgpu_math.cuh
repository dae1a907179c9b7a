// zgpu_math.cuh -- device math for the walk engine: small vectors, PCG32, direction
// sampling, modified Bessel functions, ball Green's functions and the device-evaluable
// PDE fields.  Everything is FP32 (the reference computes in float, with Bessel
// functions in double; here the A&S polynomials are evaluated in float, ~1e-7 relative).
#pragma once

#include <cstdint>
#include <cuda_runtime.h>
#include "../../include/zgpu.h"

#define ZG_HD __host__ __device__ __forceinline__
#define ZG_D __device__ __forceinline__

namespace zg {

constexpr float kPi = 3.14159265358979323846f;
constexpr float kFltMax = 3.402823466e+38f;
constexpr float kFltEps = 1.192092896e-07f;     // std::numeric_limits<float>::epsilon()
constexpr float kRayOffsetOrigin = 1.0f / 32.0f;
constexpr float kRayOffsetFloatScale = 1.0f / 65536.0f;
constexpr float kRayOffsetIntScale = 256.0f;
constexpr float kRadiusShrink = 0.99f;           // ZOMBIE_RADIUS_SHRINK_PERCENTAGE (point_estimation/common.h:15)
constexpr float kRClamp = 1e-4f;                 // GreensFnBall rClamp default (core/distributions.h:335)
constexpr float kReflEps = 1e-6f;                // tolerance of the reflectance primitives

template <int D>
struct V {
    float v[D];
    ZG_HD float& operator[](int i) { return v[i]; }
    ZG_HD float operator[](int i) const { return v[i]; }
};
template <int D> ZG_HD V<D> vzero() { V<D> r; _Pragma("unroll") for (int i = 0; i < D; i++) r.v[i] = 0.0f; return r; }
template <int D> ZG_HD V<D> operator+(V<D> a, V<D> b) { _Pragma("unroll") for (int i = 0; i < D; i++) a.v[i] += b.v[i]; return a; }
template <int D> ZG_HD V<D> operator-(V<D> a, V<D> b) { _Pragma("unroll") for (int i = 0; i < D; i++) a.v[i] -= b.v[i]; return a; }
template <int D> ZG_HD V<D> operator-(V<D> a) { _Pragma("unroll") for (int i = 0; i < D; i++) a.v[i] = -a.v[i]; return a; }
template <int D> ZG_HD V<D> operator*(float s, V<D> a) { _Pragma("unroll") for (int i = 0; i < D; i++) a.v[i] *= s; return a; }
template <int D> ZG_HD V<D> operator*(V<D> a, float s) { return s * a; }
template <int D> ZG_HD float dot(V<D> a, V<D> b) { float s = 0.0f; _Pragma("unroll") for (int i = 0; i < D; i++) s += a.v[i] * b.v[i]; return s; }
template <int D> ZG_HD float len2(V<D> a) { return dot(a, a); }
template <int D> ZG_HD float len(V<D> a) { return sqrtf(dot(a, a)); }
ZG_HD float cross2(V<2> a, V<2> b) { return a[0] * b[1] - a[1] * b[0]; }
ZG_HD V<3> cross3(V<3> a, V<3> b) {
    V<3> r; r[0] = a[1] * b[2] - a[2] * b[1]; r[1] = a[2] * b[0] - a[0] * b[2]; r[2] = a[0] * b[1] - a[1] * b[0]; return r;
}
template <int D> ZG_HD V<D> vload(const float* p) { V<D> r; _Pragma("unroll") for (int i = 0; i < D; i++) r.v[i] = p[i]; return r; }
template <int D> ZG_HD void vstore(V<D> a, float* p) { _Pragma("unroll") for (int i = 0; i < D; i++) p[i] = a.v[i]; }

// -----------------------------------------------------------------------------------
// PCG32 (O'Neill 2014): 64-bit LCG state with the XSH-RR output permutation.
struct Pcg32 {
    uint64_t state, inc;
    ZG_HD uint32_t next() {
        uint64_t old = state;
        state = old * 6364136223846793005ULL + inc;
        uint32_t xs = (uint32_t)(((old >> 18u) ^ old) >> 27u);
        uint32_t rot = (uint32_t)(old >> 59u);
        return (xs >> rot) | (xs << ((~rot + 1u) & 31u));
    }
    ZG_HD void seed(uint64_t initstate, uint64_t initseq) {
        state = 0u;
        inc = (initseq << 1u) | 1u;
        next();
        state += initstate;
        next();
    }
    ZG_HD float uniform() {   // [0,1) from the top 23 bits
        union { uint32_t u; float f; } x;
        x.u = (next() >> 9) | 0x3f800000u;
        return x.f - 1.0f;
    }
};

// uniform direction on the unit sphere
ZG_D V<2> sampleSphere(Pcg32& rng, V<2>) {
    float u = rng.uniform();
    float s, c;
    sincospif(2.0f * u, &s, &c);
    V<2> r; r[0] = c; r[1] = s; return r;
}
ZG_D V<3> sampleSphere(Pcg32& rng, V<3>) {
    float u0 = rng.uniform(), u1 = rng.uniform();
    float z = 1.0f - 2.0f * u0;
    float r = sqrtf(fmaxf(0.0f, 1.0f - z * z));
    float s, c;
    sincospif(2.0f * u1, &s, &c);
    V<3> v; v[0] = r * c; v[1] = r * s; v[2] = z; return v;
}
template <int D> ZG_D V<D> sampleSphere(Pcg32& rng) { return sampleSphere(rng, V<D>()); }
// the same maps from given uniforms (stratified first steps of the gradient estimator)
ZG_D V<2> sphereFromUniform(const float* u, V<2>) {
    float s, c;
    sincospif(2.0f * u[0], &s, &c);
    V<2> r; r[0] = c; r[1] = s; return r;
}
ZG_D V<3> sphereFromUniform(const float* u, V<3>) {
    float z = 1.0f - 2.0f * u[0];
    float r = sqrtf(fmaxf(0.0f, 1.0f - z * z));
    float s, c;
    sincospif(2.0f * u[1], &s, &c);
    V<3> v; v[0] = r * c; v[1] = r * s; v[2] = z; return v;
}
template <int D> ZG_D V<D> sphereFromUniform(const float* u) { return sphereFromUniform(u, V<D>()); }

// Cosine-weighted direction on the unit hemisphere about the last axis from uniforms u
// (SphereSampler::sampleUnitHemisphereCosine, core/sampling.h:124-129, :211-216).  2D: the
// abscissa x = 2u - 1 is uniform, so the angle from the axis has density cos / 2.  3D:
// Shirley and Chiu's concentric map of the square onto the disk (JGT 1997), lifted to the
// hemisphere (Malley's method), density cos / pi.
ZG_D V<2> hemisphereCosine(const float* u, V<2>) {
    const float x = 2.0f * u[0] - 1.0f;
    V<2> r; r[0] = x; r[1] = sqrtf(fmaxf(0.0f, 1.0f - x * x)); return r;
}
ZG_D V<3> hemisphereCosine(const float* u, V<3>) {
    const float a = 2.0f * u[0] - 1.0f, b = 2.0f * u[1] - 1.0f;
    float rad = 0.0f, ang = 0.0f;                   // angle in units of pi
    if (a != 0.0f || b != 0.0f) {
        if (fabsf(a) > fabsf(b)) { rad = a; ang = 0.25f * (b / a); }
        else { rad = b; ang = 0.5f - 0.25f * (a / b); }
    }
    float s, c;
    sincospif(ang, &s, &c);
    V<3> v; v[0] = rad * c; v[1] = rad * s; v[2] = sqrtf(fmaxf(0.0f, 1.0f - rad * rad)); return v;
}
template <int D> ZG_D V<D> hemisphereCosine(const float* u) { return hemisphereCosine(u, V<D>()); }
// density of hemisphereCosine over directions at angle acos(cosTheta) from the axis
template <int D> ZG_D float hemisphereCosinePdf(float cosTheta) {
    return D == 2 ? 0.5f * cosTheta : cosTheta * (1.0f / kPi);
}

// d given in a frame whose last axis is the unit vector n, expressed in world coordinates
// (SphereSampler::transformCoordinates, core/sampling.h:151-157, :236-246).  2D: tangent
// (n1, -n0).  3D: the branchless orthonormal basis of Duff et al., "Building an Orthonormal
// Basis, Revisited" (JCGT 2017).
ZG_D V<2> toFrame(const V<2>& n, const V<2>& d) {
    V<2> r; r[0] = d[0] * n[1] + d[1] * n[0]; r[1] = -d[0] * n[0] + d[1] * n[1]; return r;
}
ZG_D V<3> toFrame(const V<3>& n, const V<3>& d) {
    const float sg = copysignf(1.0f, n[2]);
    const float a = -1.0f / (sg + n[2]);
    const float b = n[0] * n[1] * a;
    V<3> t1, t2;
    t1[0] = 1.0f + sg * n[0] * n[0] * a; t1[1] = sg * b; t1[2] = -sg * n[0];
    t2[0] = b; t2[1] = sg + n[1] * n[1] * a; t2[2] = -n[1];
    V<3> r;
#pragma unroll
    for (int i = 0; i < 3; i++) r[i] = d[0] * t1[i] + d[1] * t2[i] + d[2] * n[i];
    return r;
}

// KernelRegularization (core/distributions.h:13-56): factors that smooth the singularity of
// the Green's function and the Poisson kernel at r (in units of the regularisation radius)
template <int D> ZG_D float kernelRegularizationG(float r) { return D == 2 ? 1.0f : erff(r); }
template <int D> ZG_D float kernelRegularizationP(float r) {
    if (D == 2) return 1.0f - expf(-r * r);
    return erff(r) - 2.0f * r * expf(-r * r) * 0.56418958354775628f;   // 1 / sqrt(pi)
}

// Latin-hypercube stratum of sample k among m for dimension j of point `key`: an affine
// permutation k -> (a k + b) mod m with a coprime to m, a and b hashed from (key, j)
ZG_D uint32_t lhsStratum(uint64_t key, int j, uint32_t k, uint32_t m) {
    if (m <= 1) return 0;
    uint64_t h = key ^ (0x9E3779B97F4A7C15ull * (uint64_t)(j + 1));
    h = (h ^ (h >> 30)) * 0xBF58476D1CE4E5B9ull;
    h = (h ^ (h >> 27)) * 0x94D049BB133111EBull;
    h ^= h >> 31;
    uint32_t a = 1u + (uint32_t)(h % (uint64_t)(m - 1));
    for (int guard = 0; guard < 64; guard++) {          // next a coprime to m
        uint32_t x = a, y = m;
        while (y) { uint32_t t = x % y; x = y; y = t; }
        if (x == 1u) break;
        a = a + 1u < m ? a + 1u : 1u;
    }
    const uint32_t b = (uint32_t)((h >> 32) % m);
    return (uint32_t)(((uint64_t)a * k + b) % m);
}
template <int D> ZG_D float pdfSphere(float r) { return D == 2 ? 1.0f / (2.0f * kPi * r) : 1.0f / (4.0f * kPi * r * r); }

// -----------------------------------------------------------------------------------
// Modified Bessel functions of order 0 and 1, Abramowitz & Stegun 9.8.1-9.8.8.
ZG_D float besselI0(float x) {
    float ax = fabsf(x);
    if (ax < 3.75f) {
        float t = (x / 3.75f) * (x / 3.75f);
        return 1.0f + t * (3.5156229f + t * (3.0899424f + t * (1.2067492f + t * (0.2659732f + t * (0.0360768f + t * 0.0045813f)))));
    }
    float t = 3.75f / ax;
    return (expf(ax) * rsqrtf(ax)) *
           (0.39894228f + t * (0.01328592f + t * (0.00225319f + t * (-0.00157565f + t * (0.00916281f +
            t * (-0.02057706f + t * (0.02635537f + t * (-0.01647633f + t * 0.00392377f))))))));
}
ZG_D float besselI1(float x) {
    float ax = fabsf(x), r;
    if (ax < 3.75f) {
        float t = (x / 3.75f) * (x / 3.75f);
        r = ax * (0.5f + t * (0.87890594f + t * (0.51498869f + t * (0.15084934f + t * (0.02658733f + t * (0.00301532f + t * 0.00032411f))))));
    } else {
        float t = 3.75f / ax;
        r = 0.39894228f + t * (-0.03988024f + t * (-0.00362018f + t * (0.00163801f + t * (-0.01031555f +
            t * (0.02282967f + t * (-0.02895312f + t * (0.01787654f - t * 0.00420059f)))))));
        r *= expf(ax) * rsqrtf(ax);
    }
    return x < 0.0f ? -r : r;
}
ZG_D float besselK0(float x) {
    if (x <= 2.0f) {
        float t = x * x * 0.25f;
        return -logf(0.5f * x) * besselI0(x) +
               (-0.57721566f + t * (0.42278420f + t * (0.23069756f + t * (0.03488590f + t * (0.00262698f + t * (0.00010750f + t * 0.0000074f))))));
    }
    float t = 2.0f / x;
    return (expf(-x) * rsqrtf(x)) *
           (1.25331414f + t * (-0.07832358f + t * (0.02189568f + t * (-0.01062446f + t * (0.00587872f + t * (-0.00251540f + t * 0.00053208f))))));
}
ZG_D float besselK1(float x) {
    if (x <= 2.0f) {
        float t = x * x * 0.25f;
        return logf(0.5f * x) * besselI1(x) +
               (1.0f / x) * (1.0f + t * (0.15443144f + t * (-0.67278579f + t * (-0.18156897f + t * (-0.01919402f + t * (-0.00110404f - t * 0.00004686f))))));
    }
    float t = 2.0f / x;
    return (expf(-x) * rsqrtf(x)) *
           (1.25331414f + t * (0.23498619f + t * (-0.03655620f + t * (0.01504268f + t * (-0.00780353f + t * (0.00325614f - t * 0.00068245f))))));
}

// -----------------------------------------------------------------------------------
// Green's function of -Lap + lambda on the ball B(c, R) centred at the walk position
// (core/distributions.h:443-1005).  One POD for both kernels: `yukawa` selects the
// screened variant; the ball-dependent constants are cached by update().
template <int D, bool SCREENED = true>
struct Greens {
    V<D> c;
    float R;
    float sqrtLambda;
    bool yukawa;   // only honoured when SCREENED (harmonic-only kernels compile no Bessel code)
    // cached per ball: 2D Yukawa K0(muR), I0(muR); 3D Yukawa exp(-muR), sinh(muR)
    float k0R, i0R;

    ZG_D void update(V<D> c_, float R_) {
        c = c_; R = R_;
        if (SCREENED && yukawa) {
            float muR = R * sqrtLambda;
            if (D == 2) { k0R = besselK0(muR); i0R = besselI0(muR); }
            else { float e = expf(-muR); k0R = e; i0R = (1.0f - e * e) / (2.0f * e); }
        }
    }
    // G(r) (distributions.h:478-480, :585-587, :712-718, :872-878)
    ZG_D float evaluate(float r) const {
        if (!SCREENED || !yukawa) {
            if (D == 2) return logf(R / r) / (2.0f * kPi);
            return (1.0f / r - 1.0f / R) / (4.0f * kPi);
        }
        float mur = r * sqrtLambda;
        if (D == 2) return (besselK0(mur) - besselI0(mur) * k0R / i0R) / (2.0f * kPi);
        float e = expf(-mur);
        float sinhmur = (1.0f - e * e) / (2.0f * e);
        return (e - k0R * sinhmur / i0R) / (4.0f * kPi * r);
    }
    // |G| integrated over the ball (distributions.h:489-491, :596-598, :739-742, :899-902)
    ZG_D float norm() const {
        if (!SCREENED || !yukawa) return D == 2 ? R * R * 0.25f : R * R / 6.0f;
        float lambda = sqrtLambda * sqrtLambda;
        if (D == 2) return (1.0f - 1.0f / i0R) / lambda;     // 1 - 2 pi P, P = 1/(2 pi I0(muR))
        float muR = R * sqrtLambda;
        return (1.0f - muR / i0R) / lambda;                  // 1 - 4 pi P, P = muR/(4 pi sinh(muR))
    }
    // radial damping of the Poisson kernel (distributions.h:774-781, :939-950)
    ZG_D float dampening(float r) const {
        float mur = r * sqrtLambda;
        if (D == 2) return mur * (besselK1(mur) + besselI1(mur) * k0R / i0R);
        float e = expf(-mur);
        float e2 = e * e;
        float coshmur = (1.0f + e2) / (2.0f * e);
        float sinhmur = (1.0f - e2) / (2.0f * e);
        float K32 = e * (1.0f + 1.0f / mur);
        float I32 = coshmur - sinhmur / mur;
        return mur * (K32 + I32 * k0R / i0R);
    }
    ZG_D float directionSampledPoissonKernel(V<D> y) const {
        if (!SCREENED || !yukawa) return 1.0f;
        float r = fmaxf(kRClamp, len(y - c));
        return dampening(r);
    }
    // Robin reflectance (distributions.h:535-543, :643-652, :801-814, :971-985)
    ZG_D float reflectance(float r, V<D> dir, V<D> n, float kappa) const {
        float Q = (SCREENED && yukawa) ? dampening(r) : 1.0f;
        if (fabsf(kappa) > 0.0f) {
            float P = D == 2 ? dot(n, dir) / r : dot(n, dir) / (r * r);
            float G;
            if (!SCREENED || !yukawa) {
                G = D == 2 ? logf(R / r) : 1.0f / r - 1.0f / R;
            } else {
                float mur = r * sqrtLambda;
                if (D == 2) G = besselK0(mur) - besselI0(mur) * k0R / i0R;
                else { float e = expf(-mur); float sh = (1.0f - e * e) / (2.0f * e); G = (e - k0R * sh / i0R) / r; }
            }
            return Q - kappa * G / P;
        }
        return Q;
    }
    // rejection sampling of the radius for the screened kernel (distributions.h:419-440)
    ZG_D float rejectionRadius(Pcg32& rng, float bound) const {
        float fnNorm = norm();
        float r = 0.0f;
        for (int iter = 0; iter < 1000; iter++) {
            float u = rng.uniform();
            r = rng.uniform() * R;
            float pdf = evaluate(r) / fnNorm;
            float pdfRadius = pdf / pdfSphere<D>(r);
            if (u < pdfRadius / bound) break;
        }
        r = fmaxf(kRClamp, r);
        if (r > R) r = R * 0.5f;
        return r;
    }
    // radius of GreensFnBall::sampleVolume(dir, ...) (distributions.h:460-470, :565-577, :695-704, :855-864)
    ZG_D float sampleRadius(Pcg32& rng) const {
        float r;
        if (!SCREENED || !yukawa) {
            if (D == 2) {
                float u1 = rng.uniform(), u2 = rng.uniform();
                r = R * sqrtf(u1 * u2);
            } else {
                float u1 = rng.uniform(), u2 = rng.uniform(), u3 = rng.uniform();
                r = R * fmaxf(fminf(u1, u2), fminf(fmaxf(u1, u2), u3));
            }
            r = fmaxf(kRClamp, r);
            if (r > R) r = R * 0.5f;
            return r;
        }
        float lambda = sqrtLambda * sqrtLambda;
        float bound;
        if (D == 2) {
            bound = R <= lambda ? fmaxf(fmaxf(2.2f / R, 2.2f / lambda), fmaxf(0.6f * sqrtf(R), 0.6f * sqrtLambda))
                                : fmaxf(fminf(2.2f / R, 2.2f / lambda), fminf(0.6f * sqrtf(R), 0.6f * sqrtLambda));
        } else {
            bound = R <= lambda ? fmaxf(fmaxf(2.0f / R, 2.0f / lambda), fmaxf(0.5f * sqrtf(R), 0.5f * sqrtLambda))
                                : fmaxf(fminf(2.0f / R, 2.0f / lambda), fminf(0.5f * sqrtf(R), 0.5f * sqrtLambda));
        }
        return rejectionRadius(rng, bound);
    }

    // ---- the gradient estimator's first step (estimateSolutionAndGradient)
    // Poisson kernel of the ball centre (distributions.h:514-516, :621-623, :769-771, :934-936)
    ZG_D float poissonKernelCentre() const {
        const float s = D == 2 ? 1.0f / (2.0f * kPi) : 1.0f / (4.0f * kPi);
        if (!SCREENED || !yukawa) return s;
        if (D == 2) return s / i0R;
        return s * R * sqrtLambda / i0R;                     // muR / (4 pi sinh(muR))
    }
    // 2D: K1(muR), I1(muR); 3D: K_{3/2}, I_{3/2} of muR up to the factors the formulas share
    ZG_D void outerTerms(float& kR, float& iR) const {
        const float muR = R * sqrtLambda;
        if (D == 2) { kR = besselK1(muR); iR = besselI1(muR); return; }
        const float e = expf(-muR), e2 = e * e;
        const float coshmuR = (1.0f + e2) / (2.0f * e), sinhmuR = (1.0f - e2) / (2.0f * e);
        kR = e * (1.0f + 1.0f / muR);
        iR = coshmuR - sinhmuR / muR;
    }
    // |grad G| / r at distance r (distributions.h:493-497, :600-604, :744-752, :905-918)
    ZG_D float gradientNorm(float r) const {
        if (!SCREENED || !yukawa) {
            if (D == 2) return (1.0f / (r * r) - 1.0f / (R * R)) / (2.0f * kPi);
            return (1.0f / (r * r * r) - 1.0f / (R * R * R)) / (4.0f * kPi);
        }
        float kR, iR;
        outerTerms(kR, iR);
        const float mur = r * sqrtLambda;
        if (D == 2) return sqrtLambda * (besselK1(mur) - besselI1(mur) * kR / iR) / (2.0f * kPi * r);
        const float e = expf(-mur), e2 = e * e;
        const float coshmur = (1.0f + e2) / (2.0f * e), sinhmur = (1.0f - e2) / (2.0f * e);
        const float K32 = e * (1.0f + 1.0f / mur), I32 = coshmur - sinhmur / mur;
        return sqrtLambda * (K32 - I32 * kR / iR) / (4.0f * kPi * r * r);
    }
    ZG_D V<D> gradient(float r, V<D> y) const { return gradientNorm(r) * (y - c); }
    // gradient of the Poisson kernel at a point y of the sphere (distributions.h:546-550,
    // :655-659, :817-822, :988-994)
    ZG_D V<D> poissonKernelGradient(V<D> y) const {
        const V<D> d = y - c;
        if (!SCREENED || !yukawa) return (D == 2 ? 2.0f / (2.0f * kPi * R * R) : 3.0f / (4.0f * kPi * R * R)) * d;
        float kR, iR;
        outerTerms(kR, iR);
        if (D == 2) return (sqrtLambda / (R * iR) / (2.0f * kPi)) * d;
        return (sqrtLambda * sqrtLambda / iR / (4.0f * kPi)) * d;
    }
};

// -----------------------------------------------------------------------------------
// ray-origin offset (core/geometric_queries.h:175-207; Wachter & Binder, Ray Tracing Gems ch. 6)
template <int D>
ZG_D V<D> offsetPoint(V<D> p, V<D> n) {
    V<D> r;
#pragma unroll
    for (int i = 0; i < D; i++) {
        int off = (int)(n[i] * kRayOffsetIntScale);
        float po = __int_as_float(__float_as_int(p[i]) + (p[i] < 0.0f ? -off : off));
        r[i] = fabsf(p[i]) < kRayOffsetOrigin ? p[i] + kRayOffsetFloatScale * n[i] : po;
    }
    return r;
}

// -----------------------------------------------------------------------------------
// device PDE (zgpu_pde): closed-form fields
template <int D>
struct FieldEval { float u, lap; V<D> grad; };

// sin and cos of a moderate argument: reduce by 2 pi with a two-term split of 2 pi
// (Cody & Waite), then the hardware approximation on [-pi, pi] (abs. error ~2^-21).
ZG_D void sincosReduced(float x, float* s, float* c) {
    const float inv2pi = 0.15915494309189535f;
    const float twoPiHi = 6.28318548202514648f;      // float nearest 2 pi
    const float twoPiLo = -1.7484555314695172e-07f;  // 2 pi - twoPiHi
    float k = rintf(x * inv2pi);
    float r = fmaf(-k, twoPiHi, x);
    r = fmaf(-k, twoPiLo, r);
    __sincosf(r, s, c);
}

template <int D>
__device__ __noinline__ FieldEval<D> evalAnalytic(const zgpu_analytic& a, V<D> x) {
    FieldEval<D> r;
    r.u = a.d; r.lap = 0.0f;
#pragma unroll
    for (int i = 0; i < D; i++) {
        r.u += a.q[i] * x[i] * x[i] + a.l[i] * x[i];
        r.grad[i] = 2.0f * a.q[i] * x[i] + a.l[i];
        r.lap += 2.0f * a.q[i];
    }
    for (int k = 0; k < a.n_terms; k++) {
        float ax = 0.0f, bx = a.phi[k], aa = 0.0f, bb = 0.0f, ab = 0.0f;
#pragma unroll
        for (int i = 0; i < D; i++) {
            ax += a.a[k][i] * x[i]; bx += a.b[k][i] * x[i];
            aa += a.a[k][i] * a.a[k][i]; bb += a.b[k][i] * a.b[k][i]; ab += a.a[k][i] * a.b[k][i];
        }
        float E = expf(ax), S, C;
        sincosReduced(bx, &S, &C);
        r.u += a.c[k] * E * C;
#pragma unroll
        for (int i = 0; i < D; i++) r.grad[i] += a.c[k] * E * (a.a[k][i] * C - a.b[k][i] * S);
        r.lap += a.c[k] * E * ((aa - bb) * C - 2.0f * ab * S);
    }
    return r;
}

// DenseGrid<float, 1, D>::operator() (utils/dense_grid.h:264-355) over a zgpu_grid: local
// coordinates t = (x - min) / (max - min); nearest: cell floor(t * shape) clamped to the
// grid; interpolated: between the cell centres around t * shape - 1/2, indices clamped to
// the grid and blend fractions to [0, 1].  Row-major, last axis fastest.
template <int D>
ZG_D float gridValue(const zgpu_grid& g, V<D> x, bool aligned) {
    const float* __restrict__ v = (aligned && g.values_aligned) ? g.values_aligned : g.values;
    int lo[D], hi[D];
    float w[D];
#pragma unroll
    for (int i = 0; i < D; i++) {
        const int n = g.shape[i];
        const float t = (x[i] - g.grid_min[i]) / (g.grid_max[i] - g.grid_min[i]);
        if (g.enable_interpolation) {
            const float u = n == 1 ? 0.0f : t * (float)n - 0.5f;
            const int i0 = min(max((int)floorf(u), 0), n - 1);
            lo[i] = i0;
            hi[i] = min(i0 + 1, n - 1);
            w[i] = fminf(fmaxf(u - (float)i0, 0.0f), 1.0f);
        } else {
            lo[i] = hi[i] = min(max((int)floorf(t * (float)n), 0), n - 1);
            w[i] = 0.0f;
        }
    }
    if (!g.enable_interpolation) {
        long long k = lo[0];
#pragma unroll
        for (int i = 1; i < D; i++) k = k * g.shape[i] + lo[i];
        return __ldg(v + k);
    }
    float acc = 0.0f;
#pragma unroll
    for (int c = 0; c < (1 << D); c++) {
        long long k = 0;
        float wt = 1.0f;
#pragma unroll
        for (int i = 0; i < D; i++) {
            const bool up = (c >> (D - 1 - i)) & 1;
            k = k * g.shape[i] + (up ? hi[i] : lo[i]);
            wt *= up ? w[i] : 1.0f - w[i];
        }
        acc += wt * __ldg(v + k);
    }
    return acc;
}

// Analytic and grid field values.  Out of line: they are read once per walk end, boundary
// sample or source sample, and inlining them into the walk kernel costs it registers on
// every step (measured: 2.5% of the mixed 2D Walk on Stars throughput).
template <int D>
__device__ __noinline__ float fieldSource(const zgpu_pde* p, V<D> x) {
    if (p->source_kind == ZGPU_FIELD_ANALYTIC) {
        FieldEval<D> e = evalAnalytic<D>(p->solution, x);
        return -e.lap + p->absorption_coeff * e.u;
    }
    return gridValue<D>(p->source_grid, x, false);
}
template <int D>
__device__ __noinline__ float fieldDirichlet(const zgpu_pde* p, V<D> x, bool aligned) {
    if (p->dirichlet_kind == ZGPU_FIELD_ANALYTIC) return evalAnalytic<D>(p->solution, x).u;
    return gridValue<D>(p->dirichlet_grid, x, aligned);
}
template <int D>
ZG_D float fieldRobinCoeff(const zgpu_pde* p, V<D> x, bool aligned) {
    if (p->robin_coeff_kind == ZGPU_FIELD_ZERO) return 0.0f;
    if (p->robin_coeff_kind == ZGPU_FIELD_GRID) return gridValue<D>(p->robin_coeff_grid, x, aligned);
    return aligned ? p->robin_coeff_value_aligned : p->robin_coeff_value;
}
template <int D>
__device__ __noinline__ float fieldRobin(const zgpu_pde* p, V<D> x, V<D> n, bool aligned) {
    if (p->robin_kind == ZGPU_FIELD_ANALYTIC) {
        FieldEval<D> e = evalAnalytic<D>(p->solution, x);
        float s = aligned ? -1.0f : 1.0f;
        return s * dot(e.grad, n) + fieldRobinCoeff<D>(p, x, aligned) * e.u;
    }
    return gridValue<D>(p->robin_grid, x, aligned);
}

// PDE<T,DIM> (core/pde.h:19-45) over a device-evaluable descriptor; ZERO and CONSTANT
// fields inline, the rest through the functions above
template <int D>
struct DevicePde {
    const zgpu_pde* p;   // in constant or global memory
    // the Robin coefficient; grids depend on the position only (getDenseGridCallback3/4
    // ignore the normal)
    ZG_D float robinCoeff(V<D> x, bool aligned) const { return fieldRobinCoeff<D>(p, x, aligned); }
    ZG_D float source(V<D> x) const {
        if (p->source_kind == ZGPU_FIELD_CONSTANT) return p->source_value;
        if (p->source_kind == ZGPU_FIELD_ZERO) return 0.0f;
        return fieldSource<D>(p, x);
    }
    ZG_D float dirichlet(V<D> x, bool aligned) const {
        if (p->dirichlet_kind == ZGPU_FIELD_CONSTANT) return aligned ? p->dirichlet_value_aligned : p->dirichlet_value;
        if (p->dirichlet_kind == ZGPU_FIELD_ZERO) return 0.0f;
        return fieldDirichlet<D>(p, x, aligned);
    }
    // Robin data h = du/dn + kappa u, n outward (the aligned side sees -n)
    ZG_D float robin(V<D> x, V<D> n, bool aligned) const {
        if (p->robin_kind == ZGPU_FIELD_CONSTANT) return aligned ? p->robin_value_aligned : p->robin_value;
        if (p->robin_kind == ZGPU_FIELD_ZERO) return 0.0f;
        return fieldRobin<D>(p, x, n, aligned);
    }
    // PDE::hasNonZeroRobinCoeff (core/pde.h:62-78)
    ZG_D bool hasNonZeroRobinCoeff(V<D> x) const {
        if (p->are_robin_conditions_pure_neumann) return false;
        return fabsf(robinCoeff(x, true)) > 0.0f || fabsf(robinCoeff(x, false)) > 0.0f;
    }
};

}  // namespace zg
