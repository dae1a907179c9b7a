/*
 * zombie_gb300.hpp -- header-only C++17 host interface over the C ABI of zgpu.h, with the
 * class names, constructors and solve() signatures of rohan-sawhney/zombie's walk path
 * (include/zombie/...), so that C++ callers of WalkOnSpheres / WalkOnStars change their
 * include and namespace and keep their call shapes.
 *
 * Differences forced by running the walks on the GPU (each is an error at compile time or an
 * exception at run time, never a silent change):
 *   - PDE fields are device-evaluable descriptors (Field: zero, constant, closed form, dense
 *     grid) instead of std::function members; a host lambda does not convert to a Field.
 *   - ignoreCandidateSilhouette / branchTraversalWeight are the value objects that
 *     getIgnoreCandidateSilhouetteCallback / getBranchTraversalWeightCallback return; the
 *     device sampler has min radial distance 1e-2 compiled in (other values throw).
 *   - walkStateCallback / terminalContributionCallback cannot run on the device: a solver
 *     constructed with a non-empty one throws Error(ZGPU_ERR_UNSUPPORTED_CALLBACK).
 *   - SamplePoint::rng is a 64-bit seed: walk w of a point draws from
 *     pcg32(seed, w + number of estimates the point already holds), so repeated solves extend
 *     the same sequence of walks.
 *   - Vector<DIM> is a small POD (operator[] and operator()), not an Eigen matrix.
 * T must be float (the configurations the engine is built for).
 */
#ifndef ZOMBIE_GB300_HPP
#define ZOMBIE_GB300_HPP

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstddef>
#include <cstdint>
#include <functional>
#include <limits>
#include <memory>
#include <stdexcept>
#include <string>
#include <type_traits>
#include <vector>

#include "zgpu.h"

namespace zombie_gb300 {

// ------------------------------------------------------------------------------ basics
template <size_t DIM, typename S = float>
struct VectorN {
    static_assert(DIM == 2 || DIM == 3, "DIM must be 2 or 3");
    S v[DIM] = {};
    VectorN() = default;
    template <typename... A, typename = std::enable_if_t<sizeof...(A) == DIM>>
    VectorN(A... a) : v{static_cast<S>(a)...} {}
    S& operator[](size_t i) { return v[i]; }
    const S& operator[](size_t i) const { return v[i]; }
    S& operator()(size_t i) { return v[i]; }
    const S& operator()(size_t i) const { return v[i]; }
    static VectorN Zero() { return VectorN(); }
    static constexpr size_t size() { return DIM; }
};
// Vector<DIM> / Vectori<DIM> (core/pde.h:14-17, utils/fcpw_geometric_queries.h)
template <size_t DIM> using Vector = VectorN<DIM, float>;
template <size_t DIM> using Vectori = VectorN<DIM, int>;
using Vector2 = Vector<2>;
using Vector3 = Vector<3>;

class Error : public std::runtime_error {
public:
    Error(int status, const std::string& what) : std::runtime_error(what), status_(status) {}
    int status() const { return status_; }
private:
    int status_;
};

inline void check(int status) {
    if (status != ZGPU_OK) {
        const char* m = zgpu_last_error();
        throw Error(status, m ? m : "zgpu error");
    }
}

// One CUDA device context (stream, scratch buffers); shared by handlers and solvers.
class Context {
public:
    explicit Context(int device = 0) {
        if (zgpu_abi_version() != ZGPU_ABI_VERSION)
            throw Error(ZGPU_ERR_UNSUPPORTED, "libzgpu was built for another zgpu.h (ABI version mismatch)");
        check(zgpu_context_create(device, &h_));
    }
    ~Context() { if (h_) zgpu_context_destroy(h_); }
    Context(const Context&) = delete;
    Context& operator=(const Context&) = delete;
    zgpu_context* handle() const { return h_; }
    void synchronize() const { check(zgpu_context_synchronize(h_)); }
private:
    zgpu_context* h_ = nullptr;
};

inline std::shared_ptr<Context> defaultContext() {
    static std::shared_ptr<Context> ctx = std::make_shared<Context>(0);
    return ctx;
}

// seedRng (core/sampling.h:36-41): clock-derived seed, distinct per call through a counter
inline uint64_t seedRng() {
    static std::atomic<uint64_t> counter{0};
    uint64_t t = (uint64_t)std::chrono::duration_cast<std::chrono::nanoseconds>(
        std::chrono::high_resolution_clock::now().time_since_epoch()).count();
    uint64_t z = t + 0x9E3779B97F4A7C15ull * (counter.fetch_add(1, std::memory_order_relaxed) + 1);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

// --------------------------------------------------------------------- walk settings
// WalkSettings (point_estimation/common.h:19-91): same constructors, fields and defaults
struct WalkSettings {
    WalkSettings(float epsilonShellForAbsorbingBoundary_, float epsilonShellForReflectingBoundary_,
                 int maxWalkLength_, bool solveDoubleSided_)
        : epsilonShellForAbsorbingBoundary(epsilonShellForAbsorbingBoundary_),
          epsilonShellForReflectingBoundary(epsilonShellForReflectingBoundary_),
          silhouettePrecision(1e-3f), russianRouletteThreshold(0.0f),
          splittingThreshold(std::numeric_limits<float>::max()), maxWalkLength(maxWalkLength_),
          stepsBeforeApplyingTikhonov(0), stepsBeforeUsingMaximalSpheres(maxWalkLength_),
          solveDoubleSided(solveDoubleSided_), useGradientControlVariates(true),
          useGradientAntitheticVariates(true), useCosineSamplingForDerivatives(false),
          ignoreAbsorbingBoundaryContribution(false), ignoreReflectingBoundaryContribution(false),
          ignoreSourceContribution(false), printLogs(false) {}
    WalkSettings(float epsilonShellForAbsorbingBoundary_, float epsilonShellForReflectingBoundary_,
                 float silhouettePrecision_, float russianRouletteThreshold_, float splittingThreshold_,
                 int maxWalkLength_, int stepsBeforeApplyingTikhonov_, int stepsBeforeUsingMaximalSpheres_,
                 bool solveDoubleSided_, bool useGradientControlVariates_, bool useGradientAntitheticVariates_,
                 bool useCosineSamplingForDerivatives_, bool ignoreAbsorbingBoundaryContribution_,
                 bool ignoreReflectingBoundaryContribution_, bool ignoreSourceContribution_, bool printLogs_)
        : epsilonShellForAbsorbingBoundary(epsilonShellForAbsorbingBoundary_),
          epsilonShellForReflectingBoundary(epsilonShellForReflectingBoundary_),
          silhouettePrecision(silhouettePrecision_), russianRouletteThreshold(russianRouletteThreshold_),
          splittingThreshold(splittingThreshold_), maxWalkLength(maxWalkLength_),
          stepsBeforeApplyingTikhonov(stepsBeforeApplyingTikhonov_),
          stepsBeforeUsingMaximalSpheres(stepsBeforeUsingMaximalSpheres_), solveDoubleSided(solveDoubleSided_),
          useGradientControlVariates(useGradientControlVariates_),
          useGradientAntitheticVariates(useGradientAntitheticVariates_),
          useCosineSamplingForDerivatives(useCosineSamplingForDerivatives_),
          ignoreAbsorbingBoundaryContribution(ignoreAbsorbingBoundaryContribution_),
          ignoreReflectingBoundaryContribution(ignoreReflectingBoundaryContribution_),
          ignoreSourceContribution(ignoreSourceContribution_), printLogs(printLogs_) {}

    zgpu_walk_settings toC() const {
        zgpu_walk_settings s;
        s.epsilon_shell_for_absorbing_boundary = epsilonShellForAbsorbingBoundary;
        s.epsilon_shell_for_reflecting_boundary = epsilonShellForReflectingBoundary;
        s.silhouette_precision = silhouettePrecision;
        s.russian_roulette_threshold = russianRouletteThreshold;
        s.splitting_threshold = splittingThreshold;
        s.max_walk_length = maxWalkLength;
        s.steps_before_applying_tikhonov = stepsBeforeApplyingTikhonov;
        s.steps_before_using_maximal_spheres = stepsBeforeUsingMaximalSpheres;
        s.solve_double_sided = solveDoubleSided;
        s.use_gradient_control_variates = useGradientControlVariates;
        s.use_gradient_antithetic_variates = useGradientAntitheticVariates;
        s.use_cosine_sampling_for_derivatives = useCosineSamplingForDerivatives;
        s.ignore_absorbing_boundary_contribution = ignoreAbsorbingBoundaryContribution;
        s.ignore_reflecting_boundary_contribution = ignoreReflectingBoundaryContribution;
        s.ignore_source_contribution = ignoreSourceContribution;
        s.print_logs = printLogs;
        return s;
    }

    float epsilonShellForAbsorbingBoundary;
    float epsilonShellForReflectingBoundary;
    float silhouettePrecision;
    float russianRouletteThreshold;
    float splittingThreshold;
    int maxWalkLength;
    int stepsBeforeApplyingTikhonov;
    int stepsBeforeUsingMaximalSpheres;
    bool solveDoubleSided;
    bool useGradientControlVariates;
    bool useGradientAntitheticVariates;
    bool useCosineSamplingForDerivatives;
    bool ignoreAbsorbingBoundaryContribution;
    bool ignoreReflectingBoundaryContribution;
    bool ignoreSourceContribution;
    bool printLogs;
};

// --------------------------------------------------------------- points and statistics
// SampleType / EstimationQuantity (point_estimation/common.h:139-149)
enum class SampleType { InDomain = ZGPU_SAMPLE_IN_DOMAIN, OnAbsorbingBoundary = ZGPU_SAMPLE_ON_ABSORBING_BOUNDARY,
                        OnReflectingBoundary = ZGPU_SAMPLE_ON_REFLECTING_BOUNDARY };
enum class EstimationQuantity { Solution = ZGPU_ESTIMATE_SOLUTION,
                                SolutionAndGradient = ZGPU_ESTIMATE_SOLUTION_AND_GRADIENT,
                                Skip = ZGPU_ESTIMATE_SKIP };

// SamplePoint (point_estimation/common.h:151-195); `seed` replaces the pcg32 member
template <typename T, size_t DIM>
struct SamplePoint {
    static_assert(std::is_same<T, float>::value, "the GPU engine solves for T = float");
    SamplePoint(const Vector<DIM>& pt_, const Vector<DIM>& normal_, SampleType type_,
                EstimationQuantity estimationQuantity_, float pdf_, float distToAbsorbingBoundary_,
                float distToReflectingBoundary_)
        : pt(pt_), normal(normal_), type(type_), estimationQuantity(estimationQuantity_), pdf(pdf_),
          distToAbsorbingBoundary(distToAbsorbingBoundary_), distToReflectingBoundary(distToReflectingBoundary_),
          estimateBoundaryNormalAligned(false) {
        directionForDerivative = Vector<DIM>::Zero();
        directionForDerivative(0) = 1.0f;
        reset();
    }
    void reset() {
        seed = seedRng();
        firstSphereRadius = 0.0f;
        robinCoeff = 0.0f;
        solution = T(0.0f);
        normalDerivative = T(0.0f);
        contribution = T(0.0f);
    }

    uint64_t seed;
    Vector<DIM> pt;
    Vector<DIM> normal;
    Vector<DIM> directionForDerivative;
    SampleType type;
    EstimationQuantity estimationQuantity;
    float pdf;
    float distToAbsorbingBoundary;
    float distToReflectingBoundary;
    float firstSphereRadius;
    float robinCoeff;
    T solution, normalDerivative, contribution;
    bool estimateBoundaryNormalAligned;
};

template <typename T, size_t DIM> class WalkSolverBase;
namespace detail { struct StatsAccess; }   // marshals moments for the variance reduction layer

// SampleStatistics (point_estimation/common.h:199-390): the same running moments and getters.
// The device accumulates in FP64; the getters return T.
template <typename T, size_t DIM>
class SampleStatistics {
public:
    SampleStatistics() { reset(); }
    void reset() {
        solutionMean = solutionM2 = 0.0;
        for (size_t i = 0; i < DIM; i++) gradientMean[i] = gradientM2[i] = 0.0;
        totalFirstSourceContribution = totalDerivativeContribution = 0.0;
        nSolutionEstimates = nGradientEstimates = 0;
        totalWalkLength = totalSplits = 0;
    }
    void addSolutionEstimate(const T& estimate) {
        nSolutionEstimates += 1;
        update(estimate, solutionMean, solutionM2, nSolutionEstimates);
    }
    void addGradientEstimate(const T* boundaryEstimate, const T* sourceEstimate) {
        nGradientEstimates += 1;
        for (size_t i = 0; i < DIM; i++)
            update(boundaryEstimate[i] + sourceEstimate[i], gradientMean[i], gradientM2[i], nGradientEstimates);
    }
    void addGradientEstimate(const T* estimate) {
        nGradientEstimates += 1;
        for (size_t i = 0; i < DIM; i++) update(estimate[i], gradientMean[i], gradientM2[i], nGradientEstimates);
    }
    void addFirstSourceContribution(const T& c) { totalFirstSourceContribution += c; }
    void addDerivativeContribution(const T& c) { totalDerivativeContribution += c; }
    void addWalkLength(int length) { totalWalkLength += length; }
    void addSplits(int nSplits) { totalSplits += nSplits; }
    // merge (common.h:268-310): Chan et al.'s parallel combination of the moments
    void merge(const SampleStatistics& other) {
        mergeMoments(solutionMean, solutionM2, nSolutionEstimates, &other.solutionMean, &other.solutionM2,
                     other.nSolutionEstimates, 1);
        int nG = nGradientEstimates;
        mergeMoments(gradientMean[0], gradientM2[0], nG, other.gradientMean, other.gradientM2,
                     other.nGradientEstimates, DIM);
        nGradientEstimates = nG;
        totalFirstSourceContribution += other.totalFirstSourceContribution;
        totalDerivativeContribution += other.totalDerivativeContribution;
        totalWalkLength += other.totalWalkLength;
        totalSplits += other.totalSplits;
    }
    T getEstimatedSolution() const { return (T)solutionMean; }
    T getEstimatedSolutionVariance() const { return (T)(solutionM2 / std::max(1, nSolutionEstimates - 1)); }
    T getEstimatedGradient(int channel) const { return (T)gradientMean[channel]; }
    std::vector<T> getEstimatedGradient() const {
        std::vector<T> g(DIM);
        for (size_t i = 0; i < DIM; i++) g[i] = (T)gradientMean[i];
        return g;
    }
    std::vector<T> getEstimatedGradientVariance() const {
        std::vector<T> v(DIM);
        for (size_t i = 0; i < DIM; i++) v[i] = (T)(gradientM2[i] / std::max(1, nGradientEstimates - 1));
        return v;
    }
    T getMeanFirstSourceContribution() const {
        return (T)(totalFirstSourceContribution / std::max(1, nSolutionEstimates));
    }
    T getEstimatedDerivative() const { return (T)(totalDerivativeContribution / std::max(1, nSolutionEstimates)); }
    int getSolutionEstimateCount() const { return nSolutionEstimates; }
    int getGradientEstimateCount() const { return nGradientEstimates; }
    float getMeanWalkLength() const { return (float)totalWalkLength / std::max(1, nSolutionEstimates); }
    float getMeanSplits() const { return (float)totalSplits / std::max(1, nSolutionEstimates); }

protected:
    friend class WalkSolverBase<T, DIM>;
    friend struct detail::StatsAccess;
    static void update(double estimate, double& mean, double& M2, int N) {
        double delta = estimate - mean;
        mean += delta / N;
        M2 += delta * (estimate - mean);
    }
    // mean/M2 point at `k` consecutive channels (gradientMean and gradientM2 are arrays)
    static void mergeMoments(double& mean0, double& m20, int& n, const double* omean, const double* om2, int on,
                             size_t k) {
        if (on <= 0) return;
        double* mean = &mean0;
        double* m2 = &m20;
        const int N = n + on;
        for (size_t i = 0; i < k; i++) {
            if (n == 0) { mean[i] = omean[i]; m2[i] = om2[i]; continue; }
            const double delta = omean[i] - mean[i];
            mean[i] += delta * ((double)on / N);
            m2[i] += om2[i] + delta * delta * ((double)n * on / N);
        }
        n = N;
    }
    double solutionMean, solutionM2;
    double gradientMean[DIM], gradientM2[DIM];
    double totalFirstSourceContribution, totalDerivativeContribution;
    int nSolutionEstimates, nGradientEstimates;
    long long totalWalkLength, totalSplits;
};

// -------------------------------------------------------------------------- PDE data
// DenseGrid<float, 1, DIM> (utils/dense_grid.h): cell-centred values over [gridMin, gridMax],
// row-major with the last axis fastest
template <size_t DIM>
struct DenseGrid {
    DenseGrid(std::vector<float> data_, const Vectori<DIM>& shape_, const Vector<DIM>& gridMin_,
              const Vector<DIM>& gridMax_, bool enableInterpolation_ = false)
        : data(std::make_shared<std::vector<float>>(std::move(data_))), shape(shape_), gridMin(gridMin_),
          gridMax(gridMax_), enableInterpolation(enableInterpolation_) {
        size_t n = 1;
        for (size_t i = 0; i < DIM; i++) {
            if (shape[i] <= 0) throw Error(ZGPU_ERR_INVALID_ARG, "DenseGrid: shape must be positive");
            n *= (size_t)shape[i];
        }
        if (data->size() != n) throw Error(ZGPU_ERR_INVALID_ARG, "DenseGrid: data size does not match the shape");
    }
    std::shared_ptr<std::vector<float>> data;
    Vectori<DIM> shape;
    Vector<DIM> gridMin, gridMax;
    bool enableInterpolation;
};

// A device-evaluable PDE field (replaces the std::function members of PDE, core/pde.h:31-45)
struct Field {
    int kind = ZGPU_FIELD_ZERO;
    float value = 0.0f, valueAligned = 0.0f;
    zgpu_grid grid{};
    std::shared_ptr<const void> keepAlive;

    static Field zero() { return Field(); }
    static Field constant(float v) { return constant(v, v); }
    static Field constant(float v, float vAligned) {
        Field f;
        f.kind = ZGPU_FIELD_CONSTANT; f.value = v; f.valueAligned = vAligned;
        return f;
    }
    // the closed form of PDE::solution (its value, normal derivative + kappa u, or -Lap u + sigma u)
    static Field analytic() { Field f; f.kind = ZGPU_FIELD_ANALYTIC; return f; }
    template <size_t DIM>
    static Field fromGrid(const DenseGrid<DIM>& g) { return fromGrids<DIM>(g, nullptr); }
    template <size_t DIM>
    static Field fromGrids(const DenseGrid<DIM>& g, const DenseGrid<DIM>* aligned) {
        Field f;
        f.kind = ZGPU_FIELD_GRID;
        f.grid.values = g.data->data();
        f.grid.values_aligned = aligned ? aligned->data->data() : nullptr;
        for (size_t i = 0; i < DIM; i++) {
            f.grid.shape[i] = g.shape[i];
            f.grid.grid_min[i] = g.gridMin[i];
            f.grid.grid_max[i] = g.gridMax[i];
            if (aligned && aligned->shape[i] != g.shape[i])
                throw Error(ZGPU_ERR_INVALID_ARG, "DenseGrid: the normal-aligned grid has another shape");
        }
        f.grid.enable_interpolation = g.enableInterpolation;
        auto keep = std::make_shared<std::vector<std::shared_ptr<std::vector<float>>>>();
        keep->push_back(g.data);
        if (aligned) keep->push_back(aligned->data);
        f.keepAlive = keep;
        return f;
    }
};

// getDenseGridCallback0..4 (utils/dense_grid.h): source (x), Dirichlet (x, aligned), Robin
// (x, n, aligned), with one grid or a grid per side of the boundary
template <size_t DIM> Field getDenseGridCallback0(const DenseGrid<DIM>& g) { return Field::fromGrid(g); }
template <size_t DIM> Field getDenseGridCallback1(const DenseGrid<DIM>& g) { return Field::fromGrid(g); }
template <size_t DIM> Field getDenseGridCallback2(const DenseGrid<DIM>& g, const DenseGrid<DIM>& gAligned) {
    return Field::fromGrids(g, &gAligned);
}
template <size_t DIM> Field getDenseGridCallback3(const DenseGrid<DIM>& g) { return Field::fromGrid(g); }
template <size_t DIM> Field getDenseGridCallback4(const DenseGrid<DIM>& g, const DenseGrid<DIM>& gAligned) {
    return Field::fromGrids(g, &gAligned);
}

// PDE (core/pde.h:19-60): the flags of the reference and device-evaluable fields
template <typename T, size_t DIM>
struct PDE {
    static_assert(std::is_same<T, float>::value, "the GPU engine solves for T = float");
    float absorptionCoeff = 0.0f;
    bool isSourceConstant = false;
    bool areRobinConditionsPureNeumann = true;
    bool areRobinCoeffsNonnegative = true;
    Field source, dirichlet, robin, robinCoeff;
    zgpu_analytic solution{};   // read by Field::analytic() fields

    zgpu_pde toC() const {
        zgpu_pde p{};
        p.absorption_coeff = absorptionCoeff;
        p.is_source_constant = isSourceConstant;
        p.are_robin_conditions_pure_neumann = areRobinConditionsPureNeumann;
        p.are_robin_coeffs_nonnegative = areRobinCoeffsNonnegative;
        p.solution = solution;
        p.source_kind = source.kind; p.source_value = source.value;
        p.dirichlet_kind = dirichlet.kind; p.dirichlet_value = dirichlet.value;
        p.dirichlet_value_aligned = dirichlet.valueAligned;
        p.robin_kind = robin.kind; p.robin_value = robin.value; p.robin_value_aligned = robin.valueAligned;
        p.robin_coeff_kind = robinCoeff.kind; p.robin_coeff_value = robinCoeff.value;
        p.robin_coeff_value_aligned = robinCoeff.valueAligned;
        p.source_grid = source.grid; p.dirichlet_grid = dirichlet.grid;
        p.robin_grid = robin.grid; p.robin_coeff_grid = robinCoeff.grid;
        p.memory = ZGPU_MEM_HOST;
        return p;
    }
};

// ------------------------------------------------------------------------- boundaries
// getIgnoreCandidateSilhouetteCallback (utils/fcpw_geometric_queries.h:1029-1038) as a value
struct IgnoreCandidateSilhouette {
    bool solveDoubleSided = false;
    float silhouettePrecision = 1e-3f;
    bool operator()(float dihedralAngle, int /*index*/) const {
        return solveDoubleSided ? false : dihedralAngle < silhouettePrecision;
    }
};
inline IgnoreCandidateSilhouette getIgnoreCandidateSilhouetteCallback(bool solveDoubleSided = false,
                                                                      float silhouettePrecision = 1e-3f) {
    return IgnoreCandidateSilhouette{solveDoubleSided, silhouettePrecision};
}

// getBranchTraversalWeightCallback (utils/fcpw_geometric_queries.h:1391-1398) as a value:
// |G_3D(max(sqrt(r2), minRadialDist))|
struct BranchTraversalWeight {
    float minRadialDist = 1e-2f;
    float operator()(float r2) const {
        const float r = std::max(std::sqrt(r2), minRadialDist);
        return 1.0f / (4.0f * 3.14159265358979f * r);
    }
};
inline BranchTraversalWeight getBranchTraversalWeightCallback(float minRadialDist = 1e-2f) {
    return BranchTraversalWeight{minRadialDist};
}

template <size_t DIM>
class BoundaryHandler {
public:
    explicit BoundaryHandler(std::shared_ptr<Context> ctx = defaultContext()) : ctx_(std::move(ctx)) {}
    virtual ~BoundaryHandler() { release(); }
    BoundaryHandler(const BoundaryHandler&) = delete;
    BoundaryHandler& operator=(const BoundaryHandler&) = delete;
    zgpu_boundary* handle() const { return b_; }
    Context& context() const { return *ctx_; }
    // builds the tree on the GPU instead of the host (zgpu_boundary_create_on_device)
    bool buildOnDevice = false;

protected:
    void release() {
        if (b_) { zgpu_boundary_destroy(b_); b_ = nullptr; }
    }
    void build(const std::vector<Vector<DIM>>& positions, const std::vector<Vectori<DIM>>& indices, int kind,
               const float* minRobin, const float* maxRobin, bool solveDoubleSided, float silhouettePrecision) {
        release();
        std::vector<float> pos(positions.size() * DIM);
        std::vector<int> idx(indices.size() * DIM);
        for (size_t i = 0; i < positions.size(); i++)
            for (size_t k = 0; k < DIM; k++) pos[i * DIM + k] = positions[i][k];
        for (size_t i = 0; i < indices.size(); i++)
            for (size_t k = 0; k < DIM; k++) idx[i * DIM + k] = indices[i][k];
        if (buildOnDevice)
            check(zgpu_boundary_create_on_device(ctx_->handle(), (int)DIM, pos.data(), (int)positions.size(),
                                                 idx.data(), (int)indices.size(), kind, minRobin, maxRobin,
                                                 solveDoubleSided, silhouettePrecision, ZGPU_MEM_HOST, &b_));
        else
            check(zgpu_boundary_create(ctx_->handle(), (int)DIM, pos.data(), (int)positions.size(), idx.data(),
                                       (int)indices.size(), kind, minRobin, maxRobin, solveDoubleSided,
                                       silhouettePrecision, 4, &b_));
    }
    std::shared_ptr<Context> ctx_;
    zgpu_boundary* b_ = nullptr;
};

// FcpwDirichletBoundaryHandler (utils/fcpw_geometric_queries.h:79-89)
template <size_t DIM>
class FcpwDirichletBoundaryHandler : public BoundaryHandler<DIM> {
public:
    using BoundaryHandler<DIM>::BoundaryHandler;
    void buildAccelerationStructure(const std::vector<Vector<DIM>>& positions,
                                    const std::vector<Vectori<DIM>>& indices, bool /*buildBvh*/ = true,
                                    bool /*enableBvhVectorization*/ = false, bool /*printStats*/ = true) {
        this->build(positions, indices, ZGPU_BOUNDARY_ABSORBING, nullptr, nullptr, false, 0.0f);
    }
};

// FcpwNeumannBoundaryHandler (utils/fcpw_geometric_queries.h:94-106)
template <size_t DIM>
class FcpwNeumannBoundaryHandler : public BoundaryHandler<DIM> {
public:
    using BoundaryHandler<DIM>::BoundaryHandler;
    void buildAccelerationStructure(const std::vector<Vector<DIM>>& positions,
                                    const std::vector<Vectori<DIM>>& indices,
                                    IgnoreCandidateSilhouette ignoreCandidateSilhouette, bool /*buildBvh*/ = true,
                                    bool /*enableBvhVectorization*/ = false, bool /*printStats*/ = true) {
        this->build(positions, indices, ZGPU_BOUNDARY_NEUMANN, nullptr, nullptr,
                    ignoreCandidateSilhouette.solveDoubleSided, ignoreCandidateSilhouette.silhouettePrecision);
    }
};

// FcpwRobinBoundaryHandler (utils/fcpw_geometric_queries.h:111-129)
template <size_t DIM>
class FcpwRobinBoundaryHandler : public BoundaryHandler<DIM> {
public:
    using BoundaryHandler<DIM>::BoundaryHandler;
    void buildAccelerationStructure(const std::vector<Vector<DIM>>& positions,
                                    const std::vector<Vectori<DIM>>& indices,
                                    IgnoreCandidateSilhouette ignoreCandidateSilhouette,
                                    const std::vector<float>& minRobinCoeffValues,
                                    const std::vector<float>& maxRobinCoeffValues, bool /*buildBvh*/ = true,
                                    bool /*enableBvhVectorization*/ = false, bool /*printStats*/ = true) {
        if (minRobinCoeffValues.size() != indices.size() || maxRobinCoeffValues.size() != indices.size())
            throw Error(ZGPU_ERR_INVALID_ARG, "one Robin coefficient range per primitive is required");
        this->build(positions, indices, ZGPU_BOUNDARY_ROBIN, minRobinCoeffValues.data(), maxRobinCoeffValues.data(),
                    ignoreCandidateSilhouette.solveDoubleSided, ignoreCandidateSilhouette.silhouettePrecision);
    }
    void updateCoefficientValues(const std::vector<float>& minRobinCoeffValues,
                                 const std::vector<float>& maxRobinCoeffValues) {
        if (!this->b_) throw Error(ZGPU_ERR_INVALID_ARG, "updateCoefficientValues before buildAccelerationStructure");
        if (minRobinCoeffValues.size() != maxRobinCoeffValues.size())
            throw Error(ZGPU_ERR_INVALID_ARG, "Robin coefficient arrays differ in length");
        check(zgpu_boundary_update_robin_coefficients(this->b_, minRobinCoeffValues.data(),
                                                      maxRobinCoeffValues.data()));
    }
};

// ------------------------------------------------------------------ geometric queries
// GeometricQueries (core/geometric_queries.h:58-124): the domain box and the boundaries whose
// queries the walks issue; the host-side query members run one batched device query each.
template <size_t DIM>
struct GeometricQueries {
    GeometricQueries() : domainIsWatertight(true) {
        for (size_t i = 0; i < DIM; i++) {
            domainMin[i] = -std::numeric_limits<float>::max();
            domainMax[i] = std::numeric_limits<float>::max();
        }
    }
    GeometricQueries(bool domainIsWatertight_, const Vector<DIM>& domainMin_, const Vector<DIM>& domainMax_)
        : domainIsWatertight(domainIsWatertight_), domainMin(domainMin_), domainMax(domainMax_) {}

    zgpu_geometric_queries toC() const {
        zgpu_geometric_queries q{};
        q.dim = (int32_t)DIM;
        q.domain_is_watertight = domainIsWatertight;
        for (size_t i = 0; i < DIM; i++) { q.domain_min[i] = domainMin[i]; q.domain_max[i] = domainMax[i]; }
        q.absorbing = absorbing;
        q.reflecting = reflecting;
        return q;
    }

    // computeDistToAbsorbingBoundary / computeDistToReflectingBoundary (geometric_queries.h:233-254)
    std::vector<float> computeDistToAbsorbingBoundary(const std::vector<Vector<DIM>>& x,
                                                      bool computeSignedDistance) const {
        return distances(absorbing, x, computeSignedDistance);
    }
    std::vector<float> computeDistToReflectingBoundary(const std::vector<Vector<DIM>>& x,
                                                       bool computeSignedDistance) const {
        return distances(reflecting, x, computeSignedDistance);
    }
    float computeDistToAbsorbingBoundary(const Vector<DIM>& x, bool computeSignedDistance) const {
        return computeDistToAbsorbingBoundary(std::vector<Vector<DIM>>{x}, computeSignedDistance)[0];
    }
    float computeDistToReflectingBoundary(const Vector<DIM>& x, bool computeSignedDistance) const {
        return computeDistToReflectingBoundary(std::vector<Vector<DIM>>{x}, computeSignedDistance)[0];
    }
    // computeDistToBoundary (geometric_queries.h:256-270)
    float computeDistToBoundary(const Vector<DIM>& x, bool computeSignedDistance, bool& closerToAbsorbing) const {
        const float dA = computeDistToAbsorbingBoundary(x, computeSignedDistance);
        const float dR = computeDistToReflectingBoundary(x, computeSignedDistance);
        closerToAbsorbing = std::fabs(dA) < std::fabs(dR);
        return closerToAbsorbing ? dA : dR;
    }
    // projectToAbsorbingBoundary / projectToReflectingBoundary (geometric_queries.h:272-300)
    bool projectToAbsorbingBoundary(Vector<DIM>& x, Vector<DIM>& normal, float& distance,
                                    bool computeSignedDistance) const {
        return project(absorbing, x, normal, distance, computeSignedDistance);
    }
    bool projectToReflectingBoundary(Vector<DIM>& x, Vector<DIM>& normal, float& distance,
                                     bool computeSignedDistance) const {
        return project(reflecting, x, normal, distance, computeSignedDistance);
    }
    // insideDomain (geometric_queries.h:357-371): odd hit parity along every axis
    std::vector<bool> insideDomain(const std::vector<Vector<DIM>>& x) const {
        const int64_t n = (int64_t)x.size();
        std::vector<bool> inside(x.size(), true);
        if (!domainIsWatertight || n == 0) return inside;
        std::vector<float> o = flat(x), d(x.size() * DIM), tmax(x.size(), std::numeric_limits<float>::max());
        std::vector<int32_t> total(x.size()), count(x.size());
        for (size_t axis = 0; axis < DIM; axis++) {
            std::fill(d.begin(), d.end(), 0.0f);
            for (size_t i = 0; i < x.size(); i++) d[i * DIM + axis] = 1.0f;
            std::fill(total.begin(), total.end(), 0);
            for (zgpu_boundary* b : {absorbing, reflecting}) {
                if (!b) continue;
                check(zgpu_query_count_hits(b, n, o.data(), d.data(), tmax.data(), count.data(), ZGPU_MEM_HOST));
                for (size_t i = 0; i < x.size(); i++) total[i] += count[i];
            }
            for (size_t i = 0; i < x.size(); i++) inside[i] = inside[i] && (total[i] % 2 == 1);
        }
        return inside;
    }
    bool insideDomain(const Vector<DIM>& x) const { return insideDomain(std::vector<Vector<DIM>>{x})[0]; }
    // outsideBoundingDomain (geometric_queries.h:376-379)
    bool outsideBoundingDomain(const Vector<DIM>& x) const {
        for (size_t i = 0; i < DIM; i++)
            if (x[i] < domainMin[i] || x[i] > domainMax[i]) return true;
        return false;
    }

    bool domainIsWatertight;
    Vector<DIM> domainMin, domainMax;
    zgpu_boundary* absorbing = nullptr;
    zgpu_boundary* reflecting = nullptr;

private:
    static std::vector<float> flat(const std::vector<Vector<DIM>>& x) {
        std::vector<float> f(x.size() * DIM);
        for (size_t i = 0; i < x.size(); i++)
            for (size_t k = 0; k < DIM; k++) f[i * DIM + k] = x[i][k];
        return f;
    }
    static std::vector<float> distances(zgpu_boundary* b, const std::vector<Vector<DIM>>& x, bool signedDist) {
        std::vector<float> d(x.size(), std::numeric_limits<float>::max());
        if (!b || x.empty()) return d;
        std::vector<float> f = flat(x);
        check(zgpu_query_closest_point(b, (int64_t)x.size(), f.data(), signedDist, nullptr, nullptr, d.data(),
                                       nullptr, ZGPU_MEM_HOST));
        return d;
    }
    static bool project(zgpu_boundary* b, Vector<DIM>& x, Vector<DIM>& normal, float& distance, bool signedDist) {
        if (!b) { distance = 0.0f; return false; }
        float pt[DIM], nrm[DIM];
        check(zgpu_query_closest_point(b, 1, x.v, signedDist, pt, nrm, &distance, nullptr, ZGPU_MEM_HOST));
        for (size_t k = 0; k < DIM; k++) { x[k] = pt[k]; normal[k] = nrm[k]; }
        return true;
    }
};

// populateGeometricQueriesFor{Dirichlet,Neumann,Robin}Boundary (utils/fcpw_geometric_queries.h:139-152)
template <size_t DIM>
void populateGeometricQueriesForDirichletBoundary(FcpwDirichletBoundaryHandler<DIM>& handler,
                                                  GeometricQueries<DIM>& geometricQueries) {
    geometricQueries.absorbing = handler.handle();
}
inline void checkBranchTraversalWeight(const BranchTraversalWeight& w) {
    if (w.minRadialDist != 1e-2f)
        throw Error(ZGPU_ERR_UNSUPPORTED, "the device boundary sampler is built for a min radial distance of 1e-2");
}
template <size_t DIM>
void populateGeometricQueriesForNeumannBoundary(FcpwNeumannBoundaryHandler<DIM>& handler,
                                                BranchTraversalWeight branchTraversalWeight,
                                                GeometricQueries<DIM>& geometricQueries) {
    checkBranchTraversalWeight(branchTraversalWeight);
    geometricQueries.reflecting = handler.handle();
}
template <size_t DIM>
void populateGeometricQueriesForRobinBoundary(FcpwRobinBoundaryHandler<DIM>& handler,
                                              BranchTraversalWeight branchTraversalWeight,
                                              GeometricQueries<DIM>& geometricQueries) {
    checkBranchTraversalWeight(branchTraversalWeight);
    geometricQueries.reflecting = handler.handle();
}

// ---------------------------------------------------------------------------- solvers
// the walk state and completion code the reference hands its callbacks (common.h:93-137);
// here only their types, for the constructor signatures
enum class WalkCompletionCode { ReachedAbsorbingBoundary, TerminatedWithRussianRoulette, ExceededMaxWalkLength,
                                EscapedDomain };
template <typename T, size_t DIM> struct WalkState;

template <typename T, size_t DIM>
class WalkSolverBase {
public:
    using WalkStateCallback = std::function<void(const WalkState<T, DIM>&)>;
    using TerminalContributionCallback = std::function<T(WalkCompletionCode, const WalkState<T, DIM>&)>;

    WalkSolverBase(int solverId, const GeometricQueries<DIM>& queries, std::shared_ptr<Context> ctx,
                   const WalkStateCallback& walkStateCallback = {},
                   const TerminalContributionCallback& terminalContributionCallback = {})
        : solverId_(solverId), queries_(queries), ctx_(std::move(ctx)) {
        if (walkStateCallback || terminalContributionCallback)
            throw Error(ZGPU_ERR_UNSUPPORTED_CALLBACK,
                        "walk state and terminal contribution callbacks run on the host and cannot be called "
                        "from the device walks");
    }

    // solve for one point (walk_on_spheres.h:115-129, walk_on_stars.h:131-148)
    void solve(const PDE<T, DIM>& pde, const WalkSettings& walkSettings, int nWalks, SamplePoint<T, DIM>& samplePt,
               SampleStatistics<T, DIM>& statistics) const {
        std::vector<SamplePoint<T, DIM>> pts{samplePt};
        std::vector<SampleStatistics<T, DIM>> stats{statistics};
        solve(pde, walkSettings, std::vector<int>{nWalks}, pts, stats);
        samplePt = pts[0];
        statistics = stats[0];
    }

    // solve for many points (walk_on_spheres.h:132-168, walk_on_stars.h:151-187): every walk
    // of every point in one device solve; the estimates are merged into `statistics`
    void solve(const PDE<T, DIM>& pde, const WalkSettings& walkSettings, const std::vector<int>& nWalks,
               std::vector<SamplePoint<T, DIM>>& samplePts, std::vector<SampleStatistics<T, DIM>>& statistics,
               bool /*runSingleThreaded*/ = false, std::function<void(int, int)> reportProgress = {}) const {
        const size_t n = samplePts.size();
        if (nWalks.size() != n) throw Error(ZGPU_ERR_INVALID_ARG, "nWalks must hold one count per sample point");
        if (statistics.size() != n) {
            statistics.clear();
            statistics.resize(n);
        }
        if (n == 0) return;
        bool gradients = false;
        for (const auto& p : samplePts) gradients |= p.estimationQuantity == EstimationQuantity::SolutionAndGradient;

        std::vector<float> pt(n * DIM), nrm(n * DIM), dA(n), dR(n), fsr(n), dir(gradients ? n * DIM : 0);
        std::vector<int32_t> type(n), eq(n), walks(nWalks.begin(), nWalks.end()), aligned(n);
        std::vector<uint64_t> seed(n);
        std::vector<double> mean(n), m2(n), gmean(gradients ? n * DIM : 0), gm2(gradients ? n * DIM : 0),
            fsrc(gradients ? n : 0), deriv(gradients ? n : 0);
        std::vector<int32_t> count(n), gcount(gradients ? n : 0);
        std::vector<int64_t> len(n), splits(n);
        for (size_t i = 0; i < n; i++) {
            const auto& p = samplePts[i];
            const auto& s = statistics[i];
            for (size_t k = 0; k < DIM; k++) {
                pt[i * DIM + k] = p.pt[k];
                nrm[i * DIM + k] = p.normal[k];
                if (gradients) {
                    dir[i * DIM + k] = p.directionForDerivative[k];
                    gmean[i * DIM + k] = s.gradientMean[k];
                    gm2[i * DIM + k] = s.gradientM2[k];
                }
            }
            dA[i] = p.distToAbsorbingBoundary;
            dR[i] = p.distToReflectingBoundary;
            fsr[i] = p.firstSphereRadius;
            type[i] = (int32_t)p.type;
            eq[i] = (int32_t)p.estimationQuantity;
            aligned[i] = p.estimateBoundaryNormalAligned;
            seed[i] = p.seed;
            mean[i] = s.solutionMean;
            m2[i] = s.solutionM2;
            count[i] = s.nSolutionEstimates;
            len[i] = s.totalWalkLength;
            splits[i] = s.totalSplits;
            if (gradients) {
                gcount[i] = s.nGradientEstimates;
                fsrc[i] = s.totalFirstSourceContribution;
                deriv[i] = s.totalDerivativeContribution;
            }
        }
        zgpu_sample_points sp{};
        sp.n = (int64_t)n;
        sp.memory = ZGPU_MEM_HOST;
        sp.pt = pt.data(); sp.normal = nrm.data(); sp.type = type.data(); sp.estimation_quantity = eq.data();
        sp.dist_to_absorbing = dA.data(); sp.dist_to_reflecting = dR.data(); sp.n_walks = walks.data();
        sp.seed = seed.data(); sp.first_sphere_radius = fsr.data(); sp.estimate_normal_aligned = aligned.data();
        sp.scene_id = nullptr;
        sp.direction_for_derivative = gradients ? dir.data() : nullptr;
        zgpu_sample_statistics st{};
        st.memory = ZGPU_MEM_HOST;
        st.solution_mean = mean.data(); st.solution_m2 = m2.data(); st.n_solution_estimates = count.data();
        st.total_walk_length = len.data(); st.total_splits = splits.data();
        if (gradients) {
            st.gradient_mean = gmean.data(); st.gradient_m2 = gm2.data(); st.n_gradient_estimates = gcount.data();
            st.total_first_source_contribution = fsrc.data(); st.total_derivative_contribution = deriv.data();
        }
        const zgpu_geometric_queries q = queries_.toC();
        const zgpu_pde p = pde.toC();
        const zgpu_walk_settings ws = walkSettings.toC();
        check(zgpu_solve(ctx_->handle(), solverId_, &q, &p, &ws, &sp, &st, hasOptions_ ? &options_ : nullptr,
                         &report_));
        for (size_t i = 0; i < n; i++) {
            auto& s = statistics[i];
            samplePts[i].firstSphereRadius = fsr[i];
            s.solutionMean = mean[i];
            s.solutionM2 = m2[i];
            s.nSolutionEstimates = count[i];
            s.totalWalkLength = len[i];
            s.totalSplits = splits[i];
            if (gradients) {
                for (size_t k = 0; k < DIM; k++) {
                    s.gradientMean[k] = gmean[i * DIM + k];
                    s.gradientM2[k] = gm2[i * DIM + k];
                }
                s.nGradientEstimates = gcount[i];
                s.totalFirstSourceContribution = fsrc[i];
                s.totalDerivativeContribution = deriv[i];
            }
        }
        if (reportProgress) reportProgress((int)n, 0);
    }

    // launch options of the device solve (block size, query mode, CUDA graph replay)
    void setSolveOptions(const zgpu_solve_options& options) { options_ = options; hasOptions_ = true; }
    // counters of the most recent solve (steps, walks, kernel time)
    const zgpu_solve_report& lastReport() const { return report_; }

private:
    int solverId_;
    const GeometricQueries<DIM>& queries_;   // held by reference, as the reference's solvers do
    std::shared_ptr<Context> ctx_;
    zgpu_solve_options options_{};
    bool hasOptions_ = false;
    mutable zgpu_solve_report report_{};
};

// WalkOnSpheres (point_estimation/walk_on_spheres.h:20-92)
template <typename T, size_t DIM>
class WalkOnSpheres : public WalkSolverBase<T, DIM> {
public:
    using Base = WalkSolverBase<T, DIM>;
    explicit WalkOnSpheres(const GeometricQueries<DIM>& queries, std::shared_ptr<Context> ctx = defaultContext())
        : Base(ZGPU_SOLVER_WALK_ON_SPHERES, queries, std::move(ctx)) {}
    WalkOnSpheres(const GeometricQueries<DIM>& queries, typename Base::WalkStateCallback walkStateCallback,
                  typename Base::TerminalContributionCallback terminalContributionCallback,
                  std::shared_ptr<Context> ctx = defaultContext())
        : Base(ZGPU_SOLVER_WALK_ON_SPHERES, queries, std::move(ctx), walkStateCallback,
               terminalContributionCallback) {}
};

// WalkOnStars (point_estimation/walk_on_stars.h:22-118)
template <typename T, size_t DIM>
class WalkOnStars : public WalkSolverBase<T, DIM> {
public:
    using Base = WalkSolverBase<T, DIM>;
    explicit WalkOnStars(const GeometricQueries<DIM>& queries, std::shared_ptr<Context> ctx = defaultContext())
        : Base(ZGPU_SOLVER_WALK_ON_STARS, queries, std::move(ctx)) {}
    WalkOnStars(const GeometricQueries<DIM>& queries, typename Base::WalkStateCallback walkStateCallback,
                typename Base::TerminalContributionCallback terminalContributionCallback,
                std::shared_ptr<Context> ctx = defaultContext())
        : Base(ZGPU_SOLVER_WALK_ON_STARS, queries, std::move(ctx), walkStateCallback, terminalContributionCallback) {}
};

}  // namespace zombie_gb300

#endif  // ZOMBIE_GB300_HPP
