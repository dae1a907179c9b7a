/*
 * zombie_gb300_variance_reduction.hpp -- C++17 host interface for boundary value caching and
 * reverse Walk on Stars over the C ABI (zgpu_solve, zgpu_bvc_splat, zgpu_rws_solve,
 * zgpu_pde_evaluate), with the class names and signatures of rohan-sawhney/zombie's
 * include/zombie/variance_reduction/{boundary_samplers,domain_samplers,
 * boundary_value_caching,reverse_walk_solver}.h.
 *
 * Sample generation (CDF tables over the boundary mesh, stratified candidates in the domain)
 * is host bookkeeping, as in the reference; the walks, the all-pairs splat and the reverse
 * walks with their splats run on the GPU.  Differences from the reference:
 *   - samplers draw from std::mt19937_64 (seeded by an optional constructor argument, else by
 *     seedRng()) instead of pcg32, and give every sample its own 64-bit walk seed;
 *   - evaluation points accumulate in FP64;
 *   - ReverseWalkOnStarsSolver's NearestNeighborFinder parameter is accepted and ignored: the
 *     radius searches run on a device tree over the evaluation points.
 */
#ifndef ZOMBIE_GB300_VARIANCE_REDUCTION_HPP
#define ZOMBIE_GB300_VARIANCE_REDUCTION_HPP

#include <algorithm>
#include <array>
#include <cmath>
#include <functional>
#include <memory>
#include <numeric>
#include <random>
#include <vector>

#include "zombie_gb300.hpp"

namespace zombie_gb300 {

namespace detail {
// moments of a SampleStatistics in and out of the structure-of-arrays C ABI
struct StatsAccess {
    template <typename S> static double& mean(S& s) { return s.solutionMean; }
    template <typename S> static double& m2(S& s) { return s.solutionM2; }
    template <typename S> static int& count(S& s) { return s.nSolutionEstimates; }
    template <typename S> static double* gradientMean(S& s) { return s.gradientMean; }
    template <typename S> static double* gradientM2(S& s) { return s.gradientM2; }
    template <typename S> static int& gradientCount(S& s) { return s.nGradientEstimates; }
};

template <size_t DIM>
inline std::vector<float> flatten(const std::vector<Vector<DIM>>& v) {
    std::vector<float> f(v.size() * DIM);
    for (size_t i = 0; i < v.size(); i++)
        for (size_t k = 0; k < DIM; k++) f[i * DIM + k] = v[i][k];
    return f;
}

// generateStratifiedSamples (core/sampling.h): n jittered strata per dimension, in random order
inline std::vector<double> stratified(int n, int dim, std::mt19937_64& rng) {
    std::vector<double> u((size_t)std::max(n, 0) * dim);
    std::uniform_real_distribution<double> U(0.0, 1.0);
    std::vector<int> perm((size_t)std::max(n, 0));
    for (int j = 0; j < dim; j++) {
        std::iota(perm.begin(), perm.end(), 0);
        std::shuffle(perm.begin(), perm.end(), rng);
        for (int i = 0; i < n; i++) u[(size_t)i * dim + j] = std::min((perm[i] + U(rng)) / n, 1.0 - 1e-7);
    }
    return u;
}

// pde.source / dirichlet / robin / robinCoeff at many points, as the walks read them
template <typename T, size_t DIM>
struct FieldValues {
    std::vector<float> source, dirichlet, robin, robinCoeff;
};
template <typename T, size_t DIM>
FieldValues<T, DIM> evaluatePde(Context& ctx, const PDE<T, DIM>& pde, const std::vector<Vector<DIM>>& x,
                                const std::vector<std::enable_if_t<true, Vector<DIM>>>* normals,   // not deduced
                                const std::vector<int32_t>* aligned) {
    FieldValues<T, DIM> f;
    const size_t n = x.size();
    f.source.resize(n); f.dirichlet.resize(n); f.robin.resize(n); f.robinCoeff.resize(n);
    if (n == 0) return f;
    std::vector<float> px = flatten<DIM>(x), pn;
    if (normals) pn = flatten<DIM>(*normals);
    const zgpu_pde p = pde.toC();
    check(zgpu_pde_evaluate(ctx.handle(), (int)DIM, &p, (int64_t)n, px.data(), normals ? pn.data() : nullptr,
                            aligned ? aligned->data() : nullptr, ZGPU_MEM_HOST, f.source.data(), f.dirichlet.data(),
                            f.robin.data(), f.robinCoeff.data()));
    return f;
}

inline uint64_t drawSeed(std::mt19937_64& rng) { return rng() & 0x7FFFFFFFFFFFFFFFull; }
}  // namespace detail

// --------------------------------------------------------------------------- samplers
// BoundarySampler (variance_reduction/boundary_samplers.h:16-34)
template <typename T, size_t DIM>
class BoundarySampler {
public:
    virtual ~BoundarySampler() = default;
    virtual void initialize(float normalOffsetForBoundary, bool solveDoubleSided) = 0;
    virtual int getSampleCount(int nTotalSamples, bool boundaryNormalAlignedSamples = false) const = 0;
    virtual void generateSamples(int nSamples, SampleType sampleType, float normalOffsetForBoundary,
                                 const GeometricQueries<DIM>& queries, std::vector<SamplePoint<T, DIM>>& samplePts,
                                 bool generateBoundaryNormalAlignedSamples = false) = 0;
};

// UniformLineSegmentBoundarySampler / UniformTriangleBoundarySampler (boundary_samplers.h:36-186):
// uniform samples over the mesh displaced along its vertex normals, in proportion to area x
// primitive weight, restricted to primitives whose displaced midpoint lies in the solve region
template <typename T, size_t DIM>
class UniformMeshBoundarySampler : public BoundarySampler<T, DIM> {
public:
    UniformMeshBoundarySampler(const std::vector<Vector<DIM>>& positions_, const std::vector<Vectori<DIM>>& indices_,
                               const std::vector<float>& primitiveWeights_,
                               const std::vector<float>& primitiveWeightsNormalAligned_,
                               std::function<bool(const Vector<DIM>&)> insideSolveRegion_,
                               bool computeWeightedNormals = false, uint64_t seed = seedRng())
        : positions(positions_), indices(indices_), insideSolveRegion(std::move(insideSolveRegion_)), rng(seed) {
        const size_t n = indices.size();
        weights.assign(primitiveWeights_.begin(), primitiveWeights_.end());
        weightsAligned.assign(primitiveWeightsNormalAligned_.begin(), primitiveWeightsNormalAligned_.end());
        if (weights.empty()) weights.assign(n, 1.0);
        if (weightsAligned.empty()) weightsAligned = weights;
        if (weights.size() != n || weightsAligned.size() != n)
            throw Error(ZGPU_ERR_INVALID_ARG, "one primitive weight per primitive is required");
        for (size_t i = 0; i < n; i++)
            if (!(weights[i] >= 0.0 && std::isfinite(weights[i]) && weightsAligned[i] >= 0.0 &&
                  std::isfinite(weightsAligned[i])))
                throw Error(ZGPU_ERR_INVALID_ARG, "primitive weights must be non-negative and finite");
        for (const auto& f : indices)
            for (size_t k = 0; k < DIM; k++)
                if (f[k] < 0 || (size_t)f[k] >= positions.size())
                    throw Error(ZGPU_ERR_INVALID_ARG, "primitive index outside the vertex list");
        faceNormalsUnit.resize(n);
        std::vector<std::array<double, DIM>> vn(positions.size());
        for (auto& v : vn) v.fill(0.0);
        for (size_t i = 0; i < n; i++) {
            std::array<double, DIM> fn = faceNormal(corners(i, 0.0));
            const double l = std::max(norm(fn), 1e-30);
            std::array<double, DIM> fu;
            for (size_t k = 0; k < DIM; k++) fu[k] = fn[k] / l;
            faceNormalsUnit[i] = fu;
            for (size_t j = 0; j < DIM; j++)
                for (size_t k = 0; k < DIM; k++) vn[indices[i][j]][k] += computeWeightedNormals ? fn[k] : fu[k];
        }
        vertexNormals.resize(positions.size());
        for (size_t v = 0; v < vn.size(); v++) {
            const double l = std::max(norm(vn[v]), 1e-30);
            for (size_t k = 0; k < DIM; k++) vertexNormals[v][k] = vn[v][k] / l;
        }
    }

    void initialize(float normalOffsetForBoundary, bool solveDoubleSided) override {
        mass = buildTable(-normalOffsetForBoundary, weights, cdf);
        massAligned = 0.0;
        cdfAligned.clear();
        if (solveDoubleSided) massAligned = buildTable(normalOffsetForBoundary, weightsAligned, cdfAligned);
    }

    int getSampleCount(int nTotalSamples, bool boundaryNormalAlignedSamples = false) const override {
        const double total = mass + massAligned;
        if (!(total > 0.0)) return 0;
        const double m = boundaryNormalAlignedSamples ? massAligned : mass;
        return (int)std::ceil(nTotalSamples * m / total);
    }

    void generateSamples(int nSamples, SampleType sampleType, float normalOffsetForBoundary,
                         const GeometricQueries<DIM>& queries, std::vector<SamplePoint<T, DIM>>& samplePts,
                         bool generateBoundaryNormalAlignedSamples = false) override {
        samplePts.clear();
        const bool aligned = generateBoundaryNormalAlignedSamples;
        const std::vector<double>& table = aligned ? cdfAligned : cdf;
        const double m = aligned ? massAligned : mass;
        const std::vector<double>& w = aligned ? weightsAligned : weights;
        const double offset = aligned ? normalOffsetForBoundary : -normalOffsetForBoundary;
        if (table.empty() || !(m > 0.0) || nSamples <= 0) return;
        std::uniform_real_distribution<double> U(0.0, 1.0);
        const std::vector<double> u = detail::stratified(nSamples, 1, rng);
        std::vector<Vector<DIM>> pts(nSamples), normals(nSamples);
        std::vector<float> pdfs(nSamples);
        for (int s = 0; s < nSamples; s++) {
            const size_t face = std::min((size_t)(std::upper_bound(table.begin(), table.end(), u[s]) - table.begin()),
                                         table.size() - 1);
            const std::array<std::array<double, DIM>, DIM> p = corners(face, offset);
            std::array<double, DIM> x;
            if (DIM == 2) {
                const double t = U(rng);
                for (size_t k = 0; k < DIM; k++) x[k] = p[0][k] + t * (p[1][k] - p[0][k]);
            } else {
                const double r1 = U(rng), r2 = U(rng), sq = std::sqrt(r1);
                const double b0 = 1.0 - sq, b1 = r2 * sq;
                for (size_t k = 0; k < DIM; k++) x[k] = b0 * p[0][k] + b1 * p[1][k] + (1.0 - b0 - b1) * p[DIM - 1][k];
            }
            const std::array<double, DIM> fn = faceNormal(p);
            const double l = std::max(norm(fn), 1e-30);
            for (size_t k = 0; k < DIM; k++) {
                pts[s][k] = (float)x[k];
                normals[s][k] = (float)(fn[k] / l);
            }
            pdfs[s] = (float)(w[face] / m);
        }
        const std::vector<float> dA = queries.computeDistToAbsorbingBoundary(pts, false);
        const std::vector<float> dR = queries.computeDistToReflectingBoundary(pts, false);
        samplePts.reserve(nSamples);
        for (int s = 0; s < nSamples; s++) {
            samplePts.emplace_back(pts[s], normals[s], sampleType, EstimationQuantity::Solution, pdfs[s], dA[s], dR[s]);
            samplePts.back().estimateBoundaryNormalAligned = aligned;
            samplePts.back().seed = detail::drawSeed(rng);
        }
    }

    const std::vector<Vector<DIM>>& getPositions() const { return positions; }
    const std::vector<Vectori<DIM>>& getIndices() const { return indices; }

private:
    static double norm(const std::array<double, DIM>& v) {
        double s = 0.0;
        for (size_t k = 0; k < DIM; k++) s += v[k] * v[k];
        return std::sqrt(s);
    }
    // corners of primitive i displaced by `offset` along the vertex normals
    std::array<std::array<double, DIM>, DIM> corners(size_t i, double offset) const {
        std::array<std::array<double, DIM>, DIM> p;
        for (size_t j = 0; j < DIM; j++)
            for (size_t k = 0; k < DIM; k++) {
                const int v = indices[i][j];
                p[j][k] = (double)positions[v][k] + (offset != 0.0 ? offset * vertexNormals[v][k] : 0.0);
            }
        return p;
    }
    static std::array<double, DIM> faceNormal(const std::array<std::array<double, DIM>, DIM>& p) {
        std::array<double, DIM> n;
        if (DIM == 2) {
            n[0] = p[1][1] - p[0][1];
            n[1] = -(p[1][0] - p[0][0]);
        } else {
            const double a[3] = {p[1][0] - p[0][0], p[1][1] - p[0][1], p[1][DIM - 1] - p[0][DIM - 1]};
            const double b[3] = {p[DIM - 1][0] - p[0][0], p[DIM - 1][1] - p[0][1], p[DIM - 1][DIM - 1] - p[0][DIM - 1]};
            const double c[3] = {a[1] * b[2] - a[2] * b[1], a[2] * b[0] - a[0] * b[2], a[0] * b[1] - a[1] * b[0]};
            for (size_t k = 0; k < DIM; k++) n[k] = c[k];
        }
        return n;
    }
    static double area(const std::array<std::array<double, DIM>, DIM>& p) {
        if (DIM == 2) {
            const double dx = p[1][0] - p[0][0], dy = p[1][1] - p[0][1];
            return std::sqrt(dx * dx + dy * dy);
        }
        return 0.5 * norm(faceNormal(p));
    }
    // buildCDFTable: area x weight of the primitives whose displaced midpoint is in the solve region
    double buildTable(double offset, const std::vector<double>& w, std::vector<double>& table) const {
        const size_t n = indices.size();
        table.assign(n, 0.0);
        double total = 0.0;
        for (size_t i = 0; i < n; i++) {
            const auto p0 = corners(i, 0.0);
            Vector<DIM> mid;
            for (size_t k = 0; k < DIM; k++) {
                double c = 0.0;
                for (size_t j = 0; j < DIM; j++) c += p0[j][k];
                mid[k] = (float)(c / DIM + offset * faceNormalsUnit[i][k]);
            }
            if (insideSolveRegion(mid)) total += area(corners(i, offset)) * w[i];
            table[i] = total;
        }
        if (!(total > 0.0)) {
            table.clear();
            return 0.0;
        }
        for (double& t : table) t /= total;
        return total;
    }

    std::vector<Vector<DIM>> positions;
    std::vector<Vectori<DIM>> indices;
    std::vector<double> weights, weightsAligned;
    std::function<bool(const Vector<DIM>&)> insideSolveRegion;
    std::vector<std::array<double, DIM>> faceNormalsUnit;
    std::vector<std::array<double, DIM>> vertexNormals;
    std::vector<double> cdf, cdfAligned;
    double mass = 0.0, massAligned = 0.0;
    std::mt19937_64 rng;
};

template <typename T>
class UniformLineSegmentBoundarySampler : public UniformMeshBoundarySampler<T, 2> {
public:
    using UniformMeshBoundarySampler<T, 2>::UniformMeshBoundarySampler;
};
template <typename T>
class UniformTriangleBoundarySampler : public UniformMeshBoundarySampler<T, 3> {
public:
    using UniformMeshBoundarySampler<T, 3>::UniformMeshBoundarySampler;
};

// createUniformLineSegmentBoundarySampler / createUniformTriangleBoundarySampler
// (boundary_samplers.h:102-122, :190-210): unit weights, one weight array, or one per side
template <typename T>
std::shared_ptr<BoundarySampler<T, 2>> createUniformLineSegmentBoundarySampler(
    const std::vector<Vector2>& positions, const std::vector<Vectori<2>>& indices,
    std::function<bool(const Vector2&)> insideSolveRegion, bool computeWeightedNormals = false) {
    return std::make_shared<UniformLineSegmentBoundarySampler<T>>(positions, indices, std::vector<float>{},
                                                                  std::vector<float>{}, insideSolveRegion,
                                                                  computeWeightedNormals);
}
template <typename T>
std::shared_ptr<BoundarySampler<T, 2>> createUniformLineSegmentBoundarySampler(
    const std::vector<Vector2>& positions, const std::vector<Vectori<2>>& indices,
    const std::vector<float>& primitiveWeights, std::function<bool(const Vector2&)> insideSolveRegion,
    bool computeWeightedNormals = false) {
    return std::make_shared<UniformLineSegmentBoundarySampler<T>>(positions, indices, primitiveWeights,
                                                                  primitiveWeights, insideSolveRegion,
                                                                  computeWeightedNormals);
}
template <typename T>
std::shared_ptr<BoundarySampler<T, 2>> createUniformLineSegmentBoundarySampler(
    const std::vector<Vector2>& positions, const std::vector<Vectori<2>>& indices,
    const std::vector<float>& primitiveWeights, const std::vector<float>& primitiveWeightsNormalAligned,
    std::function<bool(const Vector2&)> insideSolveRegion, bool computeWeightedNormals = false) {
    return std::make_shared<UniformLineSegmentBoundarySampler<T>>(positions, indices, primitiveWeights,
                                                                  primitiveWeightsNormalAligned, insideSolveRegion,
                                                                  computeWeightedNormals);
}
template <typename T>
std::shared_ptr<BoundarySampler<T, 3>> createUniformTriangleBoundarySampler(
    const std::vector<Vector3>& positions, const std::vector<Vectori<3>>& indices,
    std::function<bool(const Vector3&)> insideSolveRegion, bool computeWeightedNormals = false) {
    return std::make_shared<UniformTriangleBoundarySampler<T>>(positions, indices, std::vector<float>{},
                                                               std::vector<float>{}, insideSolveRegion,
                                                               computeWeightedNormals);
}
template <typename T>
std::shared_ptr<BoundarySampler<T, 3>> createUniformTriangleBoundarySampler(
    const std::vector<Vector3>& positions, const std::vector<Vectori<3>>& indices,
    const std::vector<float>& primitiveWeights, std::function<bool(const Vector3&)> insideSolveRegion,
    bool computeWeightedNormals = false) {
    return std::make_shared<UniformTriangleBoundarySampler<T>>(positions, indices, primitiveWeights, primitiveWeights,
                                                               insideSolveRegion, computeWeightedNormals);
}
template <typename T>
std::shared_ptr<BoundarySampler<T, 3>> createUniformTriangleBoundarySampler(
    const std::vector<Vector3>& positions, const std::vector<Vectori<3>>& indices,
    const std::vector<float>& primitiveWeights, const std::vector<float>& primitiveWeightsNormalAligned,
    std::function<bool(const Vector3&)> insideSolveRegion, bool computeWeightedNormals = false) {
    return std::make_shared<UniformTriangleBoundarySampler<T>>(positions, indices, primitiveWeights,
                                                               primitiveWeightsNormalAligned, insideSolveRegion,
                                                               computeWeightedNormals);
}

// DomainSampler / UniformDomainSampler (variance_reduction/domain_samplers.h:14-110)
template <typename T, size_t DIM>
class DomainSampler {
public:
    virtual ~DomainSampler() = default;
    virtual void generateSamples(int nSamples, const GeometricQueries<DIM>& queries,
                                 std::vector<SamplePoint<T, DIM>>& samplePts) = 0;
};

template <typename T, size_t DIM>
class UniformDomainSampler : public DomainSampler<T, DIM> {
public:
    UniformDomainSampler(std::function<bool(const Vector<DIM>&)> insideSolveRegion_, const Vector<DIM>& solveRegionMin_,
                         const Vector<DIM>& solveRegionMax_, float solveRegionVolume_, uint64_t seed = seedRng())
        : insideSolveRegion(std::move(insideSolveRegion_)), solveRegionMin(solveRegionMin_),
          solveRegionMax(solveRegionMax_), solveRegionVolume(solveRegionVolume_), rng(seed) {}

    // stratified candidates over the region's box, oversampled by box volume / region volume
    // and kept inside the region (may return a count other than nSamples, as the reference's)
    void generateSamples(int nSamples, const GeometricQueries<DIM>& queries,
                         std::vector<SamplePoint<T, DIM>>& samplePts) override {
        samplePts.clear();
        double boxVolume = 1.0;
        for (size_t k = 0; k < DIM; k++) boxVolume *= (double)solveRegionMax[k] - solveRegionMin[k];
        const double pdf = solveRegionVolume > 0.0f ? 1.0 / solveRegionVolume : 0.0;
        int n = nSamples;
        if (solveRegionVolume > 0.0f) n = (int)std::min((double)nSamples * boxVolume * pdf, 1e8);
        const std::vector<double> u = detail::stratified(n, (int)DIM, rng);
        std::vector<Vector<DIM>> pts;
        pts.reserve(n);
        for (int i = 0; i < n; i++) {
            Vector<DIM> x;
            for (size_t k = 0; k < DIM; k++)
                x[k] = (float)(solveRegionMin[k] + ((double)solveRegionMax[k] - solveRegionMin[k]) * u[(size_t)i * DIM + k]);
            if (insideSolveRegion(x)) pts.push_back(x);
        }
        const std::vector<float> dA = queries.computeDistToAbsorbingBoundary(pts, false);
        const std::vector<float> dR = queries.computeDistToReflectingBoundary(pts, false);
        samplePts.reserve(pts.size());
        for (size_t i = 0; i < pts.size(); i++) {
            samplePts.emplace_back(pts[i], Vector<DIM>(), SampleType::InDomain, EstimationQuantity::Solution,
                                   (float)pdf, dA[i], dR[i]);
            samplePts.back().seed = detail::drawSeed(rng);
        }
    }

private:
    std::function<bool(const Vector<DIM>&)> insideSolveRegion;
    Vector<DIM> solveRegionMin, solveRegionMax;
    float solveRegionVolume;
    std::mt19937_64 rng;
};

template <typename T, size_t DIM>
std::shared_ptr<DomainSampler<T, DIM>> createUniformDomainSampler(std::function<bool(const Vector<DIM>&)> inside,
                                                                 const Vector<DIM>& solveRegionMin,
                                                                 const Vector<DIM>& solveRegionMax,
                                                                 float solveRegionVolume) {
    return std::make_shared<UniformDomainSampler<T, DIM>>(inside, solveRegionMin, solveRegionMax, solveRegionVolume);
}

// ------------------------------------------------------------- boundary value caching
namespace bvc {

// EvaluationPoint (boundary_value_caching.h:19-56): five statistics, one per kind of sample
template <typename T, size_t DIM>
struct EvaluationPoint {
    EvaluationPoint(const Vector<DIM>& pt_, const Vector<DIM>& normal_, SampleType type_,
                    float distToAbsorbingBoundary_, float distToReflectingBoundary_)
        : pt(pt_), normal(normal_), type(type_), distToAbsorbingBoundary(distToAbsorbingBoundary_),
          distToReflectingBoundary(distToReflectingBoundary_) {}

    T getEstimatedSolution() const {
        T u = 0;
        for (const auto* s : groups()) u += s->getEstimatedSolution();
        return u;
    }
    void getEstimatedGradient(std::vector<T>& gradient) const {
        gradient.assign(DIM, T(0));
        for (size_t k = 0; k < DIM; k++) gradient[k] = getEstimatedGradient((int)k);
    }
    T getEstimatedGradient(int channel) const {
        T g = 0;
        for (const auto* s : groups()) g += s->getEstimatedGradient(channel);
        return g;
    }
    void reset() {
        for (auto* s : groups()) s->reset();
    }

    Vector<DIM> pt;
    Vector<DIM> normal;
    SampleType type;
    float distToAbsorbingBoundary;
    float distToReflectingBoundary;

protected:
    SampleStatistics<T, DIM> absorbingBoundaryStatistics;
    SampleStatistics<T, DIM> absorbingBoundaryNormalAlignedStatistics;
    SampleStatistics<T, DIM> reflectingBoundaryStatistics;
    SampleStatistics<T, DIM> reflectingBoundaryNormalAlignedStatistics;
    SampleStatistics<T, DIM> sourceStatistics;

    // in ZGPU_BVC_* order
    std::array<SampleStatistics<T, DIM>*, ZGPU_BVC_GROUPS> groups() {
        return {&absorbingBoundaryStatistics, &absorbingBoundaryNormalAlignedStatistics, &reflectingBoundaryStatistics,
                &reflectingBoundaryNormalAlignedStatistics, &sourceStatistics};
    }
    std::array<const SampleStatistics<T, DIM>*, ZGPU_BVC_GROUPS> groups() const {
        return {&absorbingBoundaryStatistics, &absorbingBoundaryNormalAlignedStatistics, &reflectingBoundaryStatistics,
                &reflectingBoundaryNormalAlignedStatistics, &sourceStatistics};
    }
    template <typename A, size_t B> friend class BoundaryValueCaching;
};

// BoundaryValueCaching (boundary_value_caching.h:59-176)
template <typename T, size_t DIM>
class BoundaryValueCaching {
public:
    BoundaryValueCaching(const GeometricQueries<DIM>& queries_, const WalkOnStars<T, DIM>& walkOnStars_,
                         std::shared_ptr<Context> ctx_ = defaultContext())
        : queries(queries_), walkOnStars(walkOnStars_), ctx(std::move(ctx_)) {}

    // computeBoundaryEstimates (:319-343): solution (and normal derivative through the
    // gradient estimator along the sample's normal) at every boundary sample
    void computeBoundaryEstimates(const PDE<T, DIM>& pde, const WalkSettings& walkSettings,
                                  int nWalksForSolutionEstimates, int nWalksForGradientEstimates,
                                  float robinCoeffCutoffForNormalDerivative,
                                  std::vector<SamplePoint<T, DIM>>& samplePts, bool useFiniteDifferences = false,
                                  bool /*runSingleThreaded*/ = false,
                                  std::function<void(int, int)> reportProgress = {}) const {
        const size_t n = samplePts.size();
        if (n == 0) return;
        std::vector<int> nWalks = setEstimationData(pde, walkSettings, nWalksForSolutionEstimates,
                                                    nWalksForGradientEstimates, robinCoeffCutoffForNormalDerivative,
                                                    useFiniteDifferences, samplePts);
        std::vector<SampleStatistics<T, DIM>> stats(n);
        walkOnStars.solve(pde, walkSettings, nWalks, samplePts, stats);
        setEstimatedBoundaryData(pde, walkSettings, robinCoeffCutoffForNormalDerivative, useFiniteDifferences,
                                 samplePts, stats);
        if (reportProgress) reportProgress((int)n, 0);
    }

    // setSourceValues (:345-370)
    void setSourceValues(const PDE<T, DIM>& pde, std::vector<SamplePoint<T, DIM>>& samplePts,
                         bool /*runSingleThreaded*/ = false) const {
        if (samplePts.empty()) return;
        std::vector<Vector<DIM>> x;
        for (const auto& s : samplePts) x.push_back(s.pt);
        const auto f = detail::evaluatePde(*ctx, pde, x, nullptr, nullptr);
        for (size_t i = 0; i < samplePts.size(); i++) {
            samplePts[i].contribution = f.source[i];
            samplePts[i].estimationQuantity = EstimationQuantity::Skip;
        }
    }

    // splat (:408-459): every sample onto every evaluation point, on the GPU
    void splat(const PDE<T, DIM>& pde, const std::vector<SamplePoint<T, DIM>>& samplePts, float radiusClamp,
               float kernelRegularization, float robinCoeffCutoffForNormalDerivative,
               float cutoffDistToAbsorbingBoundary, float cutoffDistToReflectingBoundary,
               std::vector<EvaluationPoint<T, DIM>>& evalPts, std::function<void(int, int)> reportProgress = {}) const {
        const size_t ns = samplePts.size(), ne = evalPts.size();
        if (ns > 0 && ne > 0) {
            std::vector<float> pt(ns * DIM), nrm(ns * DIM), pdf(ns), sol(ns), dn(ns), contrib(ns), kappa(ns);
            std::vector<int32_t> type(ns), aligned(ns);
            for (size_t i = 0; i < ns; i++) {
                const auto& s = samplePts[i];
                for (size_t k = 0; k < DIM; k++) { pt[i * DIM + k] = s.pt[k]; nrm[i * DIM + k] = s.normal[k]; }
                pdf[i] = s.pdf; sol[i] = s.solution; dn[i] = s.normalDerivative; contrib[i] = s.contribution;
                kappa[i] = s.robinCoeff; type[i] = (int32_t)s.type; aligned[i] = s.estimateBoundaryNormalAligned;
            }
            zgpu_bvc_samples smp{};
            smp.n = (int64_t)ns;
            smp.pt = pt.data(); smp.normal = nrm.data(); smp.pdf = pdf.data(); smp.type = type.data();
            smp.estimate_normal_aligned = aligned.data(); smp.solution = sol.data(); smp.normal_derivative = dn.data();
            smp.contribution = contrib.data(); smp.robin_coeff = kappa.data();
            std::vector<float> ept(ne * DIM), eda(ne), edr(ne);
            std::vector<int32_t> etype(ne);
            std::vector<double> mean(ne * ZGPU_BVC_GROUPS), m2(ne * ZGPU_BVC_GROUPS),
                gmean(ne * ZGPU_BVC_GROUPS * DIM), gm2(ne * ZGPU_BVC_GROUPS * DIM);
            std::vector<int32_t> count(ne * ZGPU_BVC_GROUPS);
            using SA = detail::StatsAccess;
            for (size_t i = 0; i < ne; i++) {
                auto& e = evalPts[i];
                for (size_t k = 0; k < DIM; k++) ept[i * DIM + k] = e.pt[k];
                eda[i] = e.distToAbsorbingBoundary; edr[i] = e.distToReflectingBoundary; etype[i] = (int32_t)e.type;
                auto g = e.groups();
                for (int j = 0; j < ZGPU_BVC_GROUPS; j++) {
                    const size_t o = i * ZGPU_BVC_GROUPS + j;
                    mean[o] = SA::mean(*g[j]); m2[o] = SA::m2(*g[j]); count[o] = SA::count(*g[j]);
                    for (size_t k = 0; k < DIM; k++) {
                        gmean[o * DIM + k] = SA::gradientMean(*g[j])[k];
                        gm2[o * DIM + k] = SA::gradientM2(*g[j])[k];
                    }
                }
            }
            zgpu_bvc_eval_points ev{};
            ev.n = (int64_t)ne;
            ev.pt = ept.data(); ev.type = etype.data(); ev.dist_to_absorbing = eda.data();
            ev.dist_to_reflecting = edr.data(); ev.mean = mean.data(); ev.m2 = m2.data(); ev.count = count.data();
            ev.gradient_mean = gmean.data(); ev.gradient_m2 = gm2.data();
            const zgpu_pde p = pde.toC();
            check(zgpu_bvc_splat(ctx->handle(), (int)DIM, &p, &smp, radiusClamp, kernelRegularization,
                                 robinCoeffCutoffForNormalDerivative, cutoffDistToAbsorbingBoundary,
                                 cutoffDistToReflectingBoundary, &ev, ZGPU_MEM_HOST));
            for (size_t i = 0; i < ne; i++) {
                auto g = evalPts[i].groups();
                for (int j = 0; j < ZGPU_BVC_GROUPS; j++) {
                    const size_t o = i * ZGPU_BVC_GROUPS + j;
                    SA::mean(*g[j]) = mean[o]; SA::m2(*g[j]) = m2[o]; SA::count(*g[j]) = count[o];
                    SA::gradientCount(*g[j]) = count[o];
                    for (size_t k = 0; k < DIM; k++) {
                        SA::gradientMean(*g[j])[k] = gmean[o * DIM + k];
                        SA::gradientM2(*g[j])[k] = gm2[o * DIM + k];
                    }
                }
            }
        }
        if (reportProgress) reportProgress((int)ns, 0);
    }

    void splat(const PDE<T, DIM>& pde, const std::vector<SamplePoint<T, DIM>>& samplePts, float radiusClamp,
               float kernelRegularization, float robinCoeffCutoffForNormalDerivative,
               float cutoffDistToAbsorbingBoundary, float cutoffDistToReflectingBoundary,
               EvaluationPoint<T, DIM>& evalPt) const {
        std::vector<EvaluationPoint<T, DIM>> one{evalPt};
        splat(pde, samplePts, radiusClamp, kernelRegularization, robinCoeffCutoffForNormalDerivative,
              cutoffDistToAbsorbingBoundary, cutoffDistToReflectingBoundary, one);
        evalPt = one[0];
    }

    // estimateSolutionNearBoundary (:461-563): points nearer the boundary than the cutoff get a
    // plain Walk on Stars estimate in place of their splats
    void estimateSolutionNearBoundary(const PDE<T, DIM>& pde, const WalkSettings& walkSettings,
                                      bool useDistanceToAbsorbingBoundary, float cutoffDistToBoundary, int nWalks,
                                      std::vector<EvaluationPoint<T, DIM>>& evalPts,
                                      bool /*runSingleThreaded*/ = false) const {
        std::vector<size_t> near;
        for (size_t i = 0; i < evalPts.size(); i++) {
            const float d = useDistanceToAbsorbingBoundary ? evalPts[i].distToAbsorbingBoundary
                                                           : evalPts[i].distToReflectingBoundary;
            if (d < cutoffDistToBoundary) near.push_back(i);
        }
        if (near.empty()) return;
        std::vector<SamplePoint<T, DIM>> pts;
        for (size_t i : near) {
            const auto& e = evalPts[i];
            pts.emplace_back(e.pt, e.normal, e.type, EstimationQuantity::Solution, 1.0f, e.distToAbsorbingBoundary,
                             e.distToReflectingBoundary);
        }
        std::vector<SampleStatistics<T, DIM>> stats(pts.size());
        walkOnStars.solve(pde, walkSettings, std::vector<int>(pts.size(), nWalks), pts, stats);
        using SA = detail::StatsAccess;
        for (size_t j = 0; j < near.size(); j++) {
            auto& e = evalPts[near[j]];
            e.reset();
            SampleStatistics<T, DIM>& g = e.type == SampleType::OnAbsorbingBoundary  ? e.absorbingBoundaryStatistics
                                          : e.type == SampleType::OnReflectingBoundary ? e.reflectingBoundaryStatistics
                                                                                       : e.sourceStatistics;
            SA::mean(g) = SA::mean(stats[j]);
            SA::count(g) = 1;
        }
    }

protected:
    // setEstimationData (:565-621)
    std::vector<int> setEstimationData(const PDE<T, DIM>& pde, const WalkSettings& ws, int nSol, int nGrad,
                                       float robinCutoff, bool useFd,
                                       std::vector<SamplePoint<T, DIM>>& samplePts) const {
        const size_t n = samplePts.size();
        std::vector<int> nWalks(n, 0);
        std::vector<Vector<DIM>> rx, rn;
        std::vector<int32_t> ra;
        std::vector<size_t> ri;
        for (size_t i = 0; i < n; i++) {
            auto& s = samplePts[i];
            const float flip = ws.solveDoubleSided && s.estimateBoundaryNormalAligned ? -1.0f : 1.0f;
            if (s.type == SampleType::OnAbsorbingBoundary) {
                if (useFd) {
                    s.type = SampleType::InDomain;
                    s.estimationQuantity = EstimationQuantity::Solution;
                } else {
                    for (size_t k = 0; k < DIM; k++) s.directionForDerivative[k] = flip * s.normal[k];
                    s.estimationQuantity = EstimationQuantity::SolutionAndGradient;
                }
                nWalks[i] = nGrad;
            } else if (s.type == SampleType::OnReflectingBoundary) {
                ri.push_back(i);
                rx.push_back(s.pt);
                rn.push_back(s.normal);
                ra.push_back(ws.solveDoubleSided && s.estimateBoundaryNormalAligned);
            } else {
                throw Error(ZGPU_ERR_INVALID_ARG, "boundary value caching estimates boundary samples only");
            }
        }
        if (!ri.empty()) {
            std::vector<float> kappa(ri.size(), 0.0f);
            if (!pde.areRobinConditionsPureNeumann) kappa = detail::evaluatePde(*ctx, pde, rx, &rn, &ra).robinCoeff;
            for (size_t j = 0; j < ri.size(); j++) {
                auto& s = samplePts[ri[j]];
                s.robinCoeff = kappa[j];
                if (std::fabs(s.robinCoeff) > robinCutoff) {
                    const float flip = ws.solveDoubleSided && s.estimateBoundaryNormalAligned ? -1.0f : 1.0f;
                    for (size_t k = 0; k < DIM; k++) s.directionForDerivative[k] = flip * s.normal[k];
                    s.estimationQuantity = EstimationQuantity::SolutionAndGradient;
                    nWalks[ri[j]] = nGrad;
                } else {
                    s.estimationQuantity = EstimationQuantity::Solution;
                    nWalks[ri[j]] = nSol;
                }
            }
        }
        return nWalks;
    }

    // setEstimatedBoundaryData (:623-650)
    void setEstimatedBoundaryData(const PDE<T, DIM>& pde, const WalkSettings& ws, float robinCutoff, bool useFd,
                                  std::vector<SamplePoint<T, DIM>>& samplePts,
                                  const std::vector<SampleStatistics<T, DIM>>& stats) const {
        const size_t n = samplePts.size();
        std::vector<Vector<DIM>> rx, rn, ox, on;
        std::vector<int32_t> ra;
        std::vector<size_t> ri, oi;
        for (size_t i = 0; i < n; i++) {
            auto& s = samplePts[i];
            s.solution = stats[i].getEstimatedSolution();
            if (s.type == SampleType::OnReflectingBoundary) {
                if (ws.ignoreReflectingBoundaryContribution) continue;
                ri.push_back(i);
                rx.push_back(s.pt);
                rn.push_back(s.normal);
                ra.push_back(ws.solveDoubleSided && s.estimateBoundaryNormalAligned);
            } else {
                oi.push_back(i);
                ox.push_back(s.pt);
                on.push_back(s.normal);
            }
        }
        if (!ri.empty()) {
            const auto f = detail::evaluatePde(*ctx, pde, rx, &rn, &ra);
            for (size_t j = 0; j < ri.size(); j++) {
                auto& s = samplePts[ri[j]];
                if (pde.areRobinConditionsPureNeumann) {
                    s.normalDerivative = f.robin[j];
                } else {
                    s.contribution = f.robin[j];
                    if (std::fabs(s.robinCoeff) > robinCutoff) s.normalDerivative = stats[ri[j]].getEstimatedDerivative();
                }
            }
        }
        if (oi.empty()) return;
        if (useFd) {
            // biased finite-difference normal derivatives from the projection onto the boundary
            const std::vector<float> sd = queries.computeDistToAbsorbingBoundary(ox, true);
            std::vector<Vector<DIM>> proj(ox.size());
            std::vector<int32_t> al(ox.size());
            for (size_t j = 0; j < ox.size(); j++) {
                for (size_t k = 0; k < DIM; k++) proj[j][k] = ox[j][k] - sd[j] * on[j][k];
                al[j] = ws.solveDoubleSided && sd[j] > 0.0f;
            }
            std::vector<float> g(ox.size(), 0.0f);
            if (!ws.ignoreAbsorbingBoundaryContribution) g = detail::evaluatePde(*ctx, pde, proj, nullptr, &al).dirichlet;
            for (size_t j = 0; j < oi.size(); j++) {
                auto& s = samplePts[oi[j]];
                s.normalDerivative = (g[j] - s.solution) / std::fabs(sd[j]);
                s.type = SampleType::OnAbsorbingBoundary;
            }
        } else {
            for (size_t j = 0; j < oi.size(); j++)
                samplePts[oi[j]].normalDerivative = stats[oi[j]].getEstimatedDerivative();
        }
    }

    const GeometricQueries<DIM>& queries;
    const WalkOnStars<T, DIM>& walkOnStars;
    std::shared_ptr<Context> ctx;
};

// BoundaryValueCachingSolver (boundary_value_caching.h:178-247, :813-945)
template <typename T, size_t DIM>
class BoundaryValueCachingSolver {
public:
    BoundaryValueCachingSolver(const GeometricQueries<DIM>& queries_,
                               std::shared_ptr<BoundarySampler<T, DIM>> absorbingBoundarySampler_,
                               std::shared_ptr<BoundarySampler<T, DIM>> reflectingBoundarySampler_,
                               std::shared_ptr<DomainSampler<T, DIM>> domainSampler_,
                               std::shared_ptr<Context> ctx = defaultContext())
        : queries(queries_), absorbingBoundarySampler(std::move(absorbingBoundarySampler_)),
          reflectingBoundarySampler(std::move(reflectingBoundarySampler_)), domainSampler(std::move(domainSampler_)),
          walkOnStars(queries_, ctx), boundaryValueCaching(queries_, walkOnStars, ctx) {}
    // boundaryValueCaching refers to this object's walkOnStars
    BoundaryValueCachingSolver(const BoundaryValueCachingSolver&) = delete;
    BoundaryValueCachingSolver& operator=(const BoundaryValueCachingSolver&) = delete;

    void generateSamples(int absorbingBoundaryCacheSize, int reflectingBoundaryCacheSize, int domainCacheSize,
                         float normalOffsetForAbsorbingBoundary, float normalOffsetForReflectingBoundary,
                         bool solveDoubleSided) {
        auto gen = [&](BoundarySampler<T, DIM>* s, int size, SampleType type, float offset, bool aligned,
                       std::vector<SamplePoint<T, DIM>>& out) {
            out.clear();
            if (s) s->generateSamples(s->getSampleCount(size, aligned), type, offset, queries, out, aligned);
        };
        gen(absorbingBoundarySampler.get(), absorbingBoundaryCacheSize, SampleType::OnAbsorbingBoundary,
            normalOffsetForAbsorbingBoundary, false, absorbingBoundaryCache);
        absorbingBoundaryCacheNormalAligned.clear();
        if (solveDoubleSided)
            gen(absorbingBoundarySampler.get(), absorbingBoundaryCacheSize, SampleType::OnAbsorbingBoundary,
                normalOffsetForAbsorbingBoundary, true, absorbingBoundaryCacheNormalAligned);
        gen(reflectingBoundarySampler.get(), reflectingBoundaryCacheSize, SampleType::OnReflectingBoundary,
            normalOffsetForReflectingBoundary, false, reflectingBoundaryCache);
        reflectingBoundaryCacheNormalAligned.clear();
        if (solveDoubleSided)
            gen(reflectingBoundarySampler.get(), reflectingBoundaryCacheSize, SampleType::OnReflectingBoundary,
                normalOffsetForReflectingBoundary, true, reflectingBoundaryCacheNormalAligned);
        domainCache.clear();
        if (domainSampler) domainSampler->generateSamples(domainCacheSize, queries, domainCache);
    }

    void computeSampleEstimates(const PDE<T, DIM>& pde, const WalkSettings& walkSettings,
                                int nWalksForSolutionEstimates, int nWalksForGradientEstimates,
                                float robinCoeffCutoffForNormalDerivative, bool useFiniteDifferences = false,
                                bool runSingleThreaded = false, std::function<void(int, int)> reportProgress = {}) {
        for (auto* c : boundaryCaches())
            boundaryValueCaching.computeBoundaryEstimates(pde, walkSettings, nWalksForSolutionEstimates,
                                                          nWalksForGradientEstimates,
                                                          robinCoeffCutoffForNormalDerivative, *c,
                                                          useFiniteDifferences, runSingleThreaded, reportProgress);
        boundaryValueCaching.setSourceValues(pde, domainCache, runSingleThreaded);
    }

    void splat(const PDE<T, DIM>& pde, float radiusClamp, float kernelRegularization,
               float robinCoeffCutoffForNormalDerivative, float cutoffDistToAbsorbingBoundary,
               float cutoffDistToReflectingBoundary, std::vector<EvaluationPoint<T, DIM>>& evalPts,
               std::function<void(int, int)> reportProgress = {}) const {
        auto caches = boundaryCaches();
        for (const auto* c : caches)
            boundaryValueCaching.splat(pde, *c, radiusClamp, kernelRegularization, robinCoeffCutoffForNormalDerivative,
                                       cutoffDistToAbsorbingBoundary, cutoffDistToReflectingBoundary, evalPts,
                                       reportProgress);
        boundaryValueCaching.splat(pde, domainCache, radiusClamp, kernelRegularization,
                                   robinCoeffCutoffForNormalDerivative, cutoffDistToAbsorbingBoundary,
                                   cutoffDistToReflectingBoundary, evalPts, reportProgress);
    }

    void estimateSolutionNearBoundary(const PDE<T, DIM>& pde, const WalkSettings& walkSettings,
                                      float cutoffDistToAbsorbingBoundary, float cutoffDistToReflectingBoundary,
                                      int nWalksForSolutionEstimates, std::vector<EvaluationPoint<T, DIM>>& evalPts,
                                      bool runSingleThreaded = false) const {
        boundaryValueCaching.estimateSolutionNearBoundary(pde, walkSettings, true, cutoffDistToAbsorbingBoundary,
                                                          nWalksForSolutionEstimates, evalPts, runSingleThreaded);
        boundaryValueCaching.estimateSolutionNearBoundary(pde, walkSettings, false, cutoffDistToReflectingBoundary,
                                                          nWalksForSolutionEstimates, evalPts, runSingleThreaded);
    }

    const std::vector<SamplePoint<T, DIM>>& getAbsorbingBoundaryCache(bool returnBoundaryNormalAligned = false) const {
        return returnBoundaryNormalAligned ? absorbingBoundaryCacheNormalAligned : absorbingBoundaryCache;
    }
    const std::vector<SamplePoint<T, DIM>>& getReflectingBoundaryCache(bool returnBoundaryNormalAligned = false) const {
        return returnBoundaryNormalAligned ? reflectingBoundaryCacheNormalAligned : reflectingBoundaryCache;
    }
    const std::vector<SamplePoint<T, DIM>>& getDomainCache() const { return domainCache; }

protected:
    std::array<std::vector<SamplePoint<T, DIM>>*, 4> boundaryCaches() {
        return {&absorbingBoundaryCache, &absorbingBoundaryCacheNormalAligned, &reflectingBoundaryCache,
                &reflectingBoundaryCacheNormalAligned};
    }
    std::array<const std::vector<SamplePoint<T, DIM>>*, 4> boundaryCaches() const {
        return {&absorbingBoundaryCache, &absorbingBoundaryCacheNormalAligned, &reflectingBoundaryCache,
                &reflectingBoundaryCacheNormalAligned};
    }

    const GeometricQueries<DIM>& queries;
    std::shared_ptr<BoundarySampler<T, DIM>> absorbingBoundarySampler;
    std::shared_ptr<BoundarySampler<T, DIM>> reflectingBoundarySampler;
    std::shared_ptr<DomainSampler<T, DIM>> domainSampler;
    WalkOnStars<T, DIM> walkOnStars;
    BoundaryValueCaching<T, DIM> boundaryValueCaching;
    std::vector<SamplePoint<T, DIM>> absorbingBoundaryCache, absorbingBoundaryCacheNormalAligned;
    std::vector<SamplePoint<T, DIM>> reflectingBoundaryCache, reflectingBoundaryCacheNormalAligned;
    std::vector<SamplePoint<T, DIM>> domainCache;
};

}  // namespace bvc

// --------------------------------------------------------------- reverse Walk on Stars
namespace rws {

// EvaluationPoint (reverse_walk_solver.h:19-45): running sums of the splatted contributions
template <typename T, size_t DIM>
struct EvaluationPoint {
    EvaluationPoint(const Vector<DIM>& pt_, const Vector<DIM>& normal_, SampleType type_,
                    float distToAbsorbingBoundary_, float distToReflectingBoundary_)
        : pt(pt_), normal(normal_), type(type_), distToAbsorbingBoundary(distToAbsorbingBoundary_),
          distToReflectingBoundary(distToReflectingBoundary_) {
        reset();
    }

    // getEstimatedSolution (:129-166): the absorbing part self-normalised by the Poisson-kernel
    // sum when one was kept, the other parts divided by their sample counts
    T getEstimatedSolution(int nAbsorbingBoundarySamples, int nAbsorbingBoundaryNormalAlignedSamples,
                           int nReflectingBoundarySamples, int nReflectingBoundaryNormalAlignedSamples,
                           int nSourceSamples) const {
        if (type == SampleType::OnAbsorbingBoundary) return (T)totalAbsorbingBoundaryContribution;
        double u = 0.0;
        if (nAbsorbingBoundarySamples > 0)
            u += totalPoissonKernelContribution > 0.0 ? totalAbsorbingBoundaryContribution / totalPoissonKernelContribution
                                                      : totalAbsorbingBoundaryContribution / nAbsorbingBoundarySamples;
        if (nAbsorbingBoundaryNormalAlignedSamples > 0)
            u += totalAbsorbingBoundaryNormalAlignedContribution / nAbsorbingBoundaryNormalAlignedSamples;
        if (nReflectingBoundarySamples > 0) u += totalReflectingBoundaryContribution / nReflectingBoundarySamples;
        if (nReflectingBoundaryNormalAlignedSamples > 0)
            u += totalReflectingBoundaryNormalAlignedContribution / nReflectingBoundaryNormalAlignedSamples;
        if (nSourceSamples > 0) u += totalSourceContribution / nSourceSamples;
        return (T)u;
    }

    void reset() {
        totalPoissonKernelContribution = 0.0;
        totalAbsorbingBoundaryContribution = totalAbsorbingBoundaryNormalAlignedContribution = 0.0;
        totalReflectingBoundaryContribution = totalReflectingBoundaryNormalAlignedContribution = 0.0;
        totalSourceContribution = 0.0;
    }

    Vector<DIM> pt;
    Vector<DIM> normal;
    SampleType type;
    float distToAbsorbingBoundary;
    float distToReflectingBoundary;
    double totalPoissonKernelContribution;
    double totalAbsorbingBoundaryContribution;
    double totalAbsorbingBoundaryNormalAlignedContribution;
    double totalReflectingBoundaryContribution;
    double totalReflectingBoundaryNormalAlignedContribution;
    double totalSourceContribution;
};

// ReverseWalkOnStarsSolver (reverse_walk_solver.h:47-118, :168-372)
template <typename T, size_t DIM, typename NearestNeighborFinder = void>
class ReverseWalkOnStarsSolver {
public:
    ReverseWalkOnStarsSolver(const GeometricQueries<DIM>& queries_,
                             std::shared_ptr<BoundarySampler<T, DIM>> absorbingBoundarySampler_,
                             std::shared_ptr<BoundarySampler<T, DIM>> reflectingBoundarySampler_,
                             std::shared_ptr<DomainSampler<T, DIM>> domainSampler_,
                             std::shared_ptr<Context> ctx_ = defaultContext())
        : queries(queries_), absorbingBoundarySampler(std::move(absorbingBoundarySampler_)),
          reflectingBoundarySampler(std::move(reflectingBoundarySampler_)), domainSampler(std::move(domainSampler_)),
          ctx(std::move(ctx_)) {}

    // generateSamples (:188-213): absorbing samples offset into the domain, reflecting samples
    // on the boundary
    void generateSamples(int absorbingBoundarySampleCount, int reflectingBoundarySampleCount, int domainSampleCount,
                         float normalOffsetForAbsorbingBoundary, bool solveDoubleSided) {
        auto gen = [&](BoundarySampler<T, DIM>* s, int count, SampleType type, float offset, bool aligned,
                       std::vector<SamplePoint<T, DIM>>& out) {
            out.clear();
            if (s && count > 0) s->generateSamples(s->getSampleCount(count, aligned), type, offset, queries, out, aligned);
        };
        gen(absorbingBoundarySampler.get(), absorbingBoundarySampleCount, SampleType::OnAbsorbingBoundary,
            normalOffsetForAbsorbingBoundary, false, absorbingBoundarySamplePts);
        absorbingBoundaryNormalAlignedSamplePts.clear();
        if (solveDoubleSided)
            gen(absorbingBoundarySampler.get(), absorbingBoundarySampleCount, SampleType::OnAbsorbingBoundary,
                normalOffsetForAbsorbingBoundary, true, absorbingBoundaryNormalAlignedSamplePts);
        gen(reflectingBoundarySampler.get(), reflectingBoundarySampleCount, SampleType::OnReflectingBoundary, 0.0f,
            false, reflectingBoundarySamplePts);
        reflectingBoundaryNormalAlignedSamplePts.clear();
        if (solveDoubleSided)
            gen(reflectingBoundarySampler.get(), reflectingBoundarySampleCount, SampleType::OnReflectingBoundary, 0.0f,
                true, reflectingBoundaryNormalAlignedSamplePts);
        domainSamplePts.clear();
        if (domainSampler && domainSampleCount > 0) domainSampler->generateSamples(domainSampleCount, queries, domainSamplePts);
    }

    // solve (:304-338): one reverse walk per sample, walks of call k on pcg32 stream k
    void solve(const PDE<T, DIM>& pde, const WalkSettings& walkSettings, float normalOffsetForAbsorbingBoundary,
               float radiusClamp, float kernelRegularization, std::vector<EvaluationPoint<T, DIM>>& evalPts,
               bool /*updatedEvalPtLocations*/ = true, bool /*runSingleThreaded*/ = false,
               std::function<void(int, int)> reportProgress = {}) {
        const size_t ne = evalPts.size();
        std::vector<float> ept(ne * DIM), enrm(ne * DIM);
        std::vector<int32_t> etype(ne);
        std::vector<double> totals(ne * ZGPU_RWS_TOTALS);
        for (size_t i = 0; i < ne; i++) {
            const auto& e = evalPts[i];
            for (size_t k = 0; k < DIM; k++) { ept[i * DIM + k] = e.pt[k]; enrm[i * DIM + k] = e.normal[k]; }
            etype[i] = (int32_t)e.type;
            double* t = &totals[i * ZGPU_RWS_TOTALS];
            t[ZGPU_RWS_ABSORBING] = e.totalAbsorbingBoundaryContribution;
            t[ZGPU_RWS_ABSORBING_ALIGNED] = e.totalAbsorbingBoundaryNormalAlignedContribution;
            t[ZGPU_RWS_REFLECTING] = e.totalReflectingBoundaryContribution;
            t[ZGPU_RWS_REFLECTING_ALIGNED] = e.totalReflectingBoundaryNormalAlignedContribution;
            t[ZGPU_RWS_SOURCE] = e.totalSourceContribution;
            t[ZGPU_RWS_POISSON_KERNEL] = e.totalPoissonKernelContribution;
        }
        const zgpu_geometric_queries q = queries.toC();
        const zgpu_pde p = pde.toC();
        const zgpu_walk_settings ws = walkSettings.toC();
        lastReports.clear();
        for (auto* c : {&absorbingBoundarySamplePts, &absorbingBoundaryNormalAlignedSamplePts,
                        &reflectingBoundarySamplePts, &reflectingBoundaryNormalAlignedSamplePts, &domainSamplePts}) {
            std::vector<size_t> idx = setContributions(pde, walkSettings, *c);
            if (idx.empty() || ne == 0) continue;
            const size_t n = idx.size();
            std::vector<float> pt(n * DIM), nrm(n * DIM), pdf(n), contrib(n), dA(n);
            std::vector<int32_t> type(n), aligned(n);
            std::vector<uint64_t> seed(n);
            for (size_t j = 0; j < n; j++) {
                const auto& s = (*c)[idx[j]];
                for (size_t k = 0; k < DIM; k++) { pt[j * DIM + k] = s.pt[k]; nrm[j * DIM + k] = s.normal[k]; }
                type[j] = (int32_t)s.type; aligned[j] = s.estimateBoundaryNormalAligned; pdf[j] = s.pdf;
                contrib[j] = s.contribution; dA[j] = s.distToAbsorbingBoundary; seed[j] = s.seed;
            }
            zgpu_rws_samples smp{};
            smp.n = (int64_t)n;
            smp.pt = pt.data(); smp.normal = nrm.data(); smp.type = type.data(); smp.estimate_normal_aligned = aligned.data();
            smp.pdf = pdf.data(); smp.contribution = contrib.data(); smp.dist_to_absorbing = dA.data();
            smp.seed = seed.data();
            zgpu_rws_eval_points ev{};
            ev.n = (int64_t)ne;
            ev.pt = ept.data(); ev.normal = enrm.data(); ev.type = etype.data(); ev.totals = totals.data();
            zgpu_solve_report rep{};
            check(zgpu_rws_solve(ctx->handle(), &q, &p, &ws, &smp, normalOffsetForAbsorbingBoundary, radiusClamp,
                                 kernelRegularization, calls, &ev, ZGPU_MEM_HOST, &rep));
            lastReports.push_back(rep);
            if (reportProgress) reportProgress((int)n, 0);
        }
        calls++;
        // evaluation points on the absorbing boundary take the boundary value
        std::vector<size_t> onAbs;
        std::vector<Vector<DIM>> ax;
        for (size_t i = 0; i < ne; i++)
            if (evalPts[i].type == SampleType::OnAbsorbingBoundary) { onAbs.push_back(i); ax.push_back(evalPts[i].pt); }
        std::vector<float> g(onAbs.size(), 0.0f);
        if (!onAbs.empty() && !walkSettings.ignoreAbsorbingBoundaryContribution)
            g = detail::evaluatePde(*ctx, pde, ax, nullptr, nullptr).dirichlet;
        for (size_t j = 0; j < onAbs.size(); j++) totals[onAbs[j] * ZGPU_RWS_TOTALS + ZGPU_RWS_ABSORBING] = g[j];
        for (size_t i = 0; i < ne; i++) {
            auto& e = evalPts[i];
            const double* t = &totals[i * ZGPU_RWS_TOTALS];
            e.totalAbsorbingBoundaryContribution = t[ZGPU_RWS_ABSORBING];
            e.totalAbsorbingBoundaryNormalAlignedContribution = t[ZGPU_RWS_ABSORBING_ALIGNED];
            e.totalReflectingBoundaryContribution = t[ZGPU_RWS_REFLECTING];
            e.totalReflectingBoundaryNormalAlignedContribution = t[ZGPU_RWS_REFLECTING_ALIGNED];
            e.totalSourceContribution = t[ZGPU_RWS_SOURCE];
            e.totalPoissonKernelContribution = t[ZGPU_RWS_POISSON_KERNEL];
        }
    }

    const std::vector<SamplePoint<T, DIM>>& getAbsorbingBoundarySamplePts(bool returnBoundaryNormalAligned = false) const {
        return returnBoundaryNormalAligned ? absorbingBoundaryNormalAlignedSamplePts : absorbingBoundarySamplePts;
    }
    const std::vector<SamplePoint<T, DIM>>& getReflectingBoundarySamplePts(bool returnBoundaryNormalAligned = false) const {
        return returnBoundaryNormalAligned ? reflectingBoundaryNormalAlignedSamplePts : reflectingBoundarySamplePts;
    }
    const std::vector<SamplePoint<T, DIM>>& getDomainSamplePts() const { return domainSamplePts; }
    int getAbsorbingBoundarySampleCount(bool returnBoundaryNormalAligned = false) const {
        return (int)getAbsorbingBoundarySamplePts(returnBoundaryNormalAligned).size();
    }
    int getReflectingBoundarySampleCount(bool returnBoundaryNormalAligned = false) const {
        return (int)getReflectingBoundarySamplePts(returnBoundaryNormalAligned).size();
    }
    int getDomainSampleCount() const { return (int)domainSamplePts.size(); }

    // the evaluation points' solution with this solver's sample counts times the number of solve
    // calls the points accumulated
    T getEstimatedSolution(const EvaluationPoint<T, DIM>& e) const {
        const int k = std::max(calls, 1);
        return e.getEstimatedSolution(k * getAbsorbingBoundarySampleCount(), k * getAbsorbingBoundarySampleCount(true),
                                      k * getReflectingBoundarySampleCount(), k * getReflectingBoundarySampleCount(true),
                                      k * getDomainSampleCount());
    }
    const std::vector<zgpu_solve_report>& lastSolveReports() const { return lastReports; }

protected:
    // ReverseWalkOnStars::solve's contribution of each sample (reverse_walk_on_stars.h:95-120):
    // returns the samples that walk
    std::vector<size_t> setContributions(const PDE<T, DIM>& pde, const WalkSettings& ws,
                                         std::vector<SamplePoint<T, DIM>>& c) const {
        std::vector<size_t> walk, src, ab, rf;
        for (size_t i = 0; i < c.size(); i++) {
            if (c[i].type == SampleType::InDomain && !ws.ignoreSourceContribution) src.push_back(i);
            if (c[i].type == SampleType::OnAbsorbingBoundary && !ws.ignoreAbsorbingBoundaryContribution) ab.push_back(i);
            if (c[i].type == SampleType::OnReflectingBoundary && !ws.ignoreReflectingBoundaryContribution) rf.push_back(i);
        }
        if (!src.empty()) {
            std::vector<Vector<DIM>> x;
            for (size_t i : src) x.push_back(c[i].pt);
            const auto f = detail::evaluatePde(*ctx, pde, x, nullptr, nullptr);
            for (size_t j = 0; j < src.size(); j++) c[src[j]].contribution = f.source[j];
        }
        if (!ab.empty()) {
            std::vector<Vector<DIM>> x, proj;
            for (size_t i : ab) x.push_back(c[i].pt);
            const std::vector<float> sd = queries.computeDistToAbsorbingBoundary(x, true);
            std::vector<int32_t> al(ab.size());
            proj.resize(ab.size());
            for (size_t j = 0; j < ab.size(); j++) {
                for (size_t k = 0; k < DIM; k++) proj[j][k] = x[j][k] - sd[j] * c[ab[j]].normal[k];
                al[j] = ws.solveDoubleSided && sd[j] > 0.0f;
            }
            const auto f = detail::evaluatePde(*ctx, pde, proj, nullptr, &al);
            for (size_t j = 0; j < ab.size(); j++) c[ab[j]].contribution = f.dirichlet[j];
        }
        if (!rf.empty()) {
            std::vector<Vector<DIM>> x, n;
            std::vector<int32_t> al;
            for (size_t i : rf) {
                x.push_back(c[i].pt);
                n.push_back(c[i].normal);
                al.push_back(ws.solveDoubleSided && c[i].estimateBoundaryNormalAligned);
            }
            const auto f = detail::evaluatePde(*ctx, pde, x, &n, &al);
            for (size_t j = 0; j < rf.size(); j++) c[rf[j]].contribution = f.robin[j];
        }
        walk.insert(walk.end(), src.begin(), src.end());
        walk.insert(walk.end(), ab.begin(), ab.end());
        walk.insert(walk.end(), rf.begin(), rf.end());
        std::sort(walk.begin(), walk.end());
        return walk;
    }

    const GeometricQueries<DIM>& queries;
    std::shared_ptr<BoundarySampler<T, DIM>> absorbingBoundarySampler;
    std::shared_ptr<BoundarySampler<T, DIM>> reflectingBoundarySampler;
    std::shared_ptr<DomainSampler<T, DIM>> domainSampler;
    std::shared_ptr<Context> ctx;
    std::vector<SamplePoint<T, DIM>> absorbingBoundarySamplePts, absorbingBoundaryNormalAlignedSamplePts;
    std::vector<SamplePoint<T, DIM>> reflectingBoundarySamplePts, reflectingBoundaryNormalAlignedSamplePts;
    std::vector<SamplePoint<T, DIM>> domainSamplePts;
    int calls = 0;
    std::vector<zgpu_solve_report> lastReports;
};

}  // namespace rws
}  // namespace zombie_gb300

#endif  // ZOMBIE_GB300_VARIANCE_REDUCTION_HPP
