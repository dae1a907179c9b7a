// Drives the C++ facade (include/zombie_gb300.hpp) the way a zombie C++ caller drives
// WalkOnSpheres / WalkOnStars: a star-shaped polygon (r = 1 + 0.3 sin 5 theta, 1,024
// counter-clockwise segments), u = e^x cos y (harmonic), Dirichlet data from the closed form
// and, for the mixed problem, Neumann data du/dn on theta in [pi, 2 pi).
//
// Checks (exit status 1 on the first failure):
//   1. Walk on Spheres, all Dirichlet: per-point z-scores against the exact solution.
//   2. Walk on Stars, mixed Dirichlet / Neumann: the same.
//   3. Two solves of 128 walks extend one sequence of walks: they equal one solve of 256.
//   4. Solution and gradient estimates (WoSt) against the exact gradient.
//   5. Dirichlet data read from a DenseGrid (bilinear) matches the closed-form solve.
//   6. A solver constructed with a walk-state callback throws ZGPU_ERR_UNSUPPORTED_CALLBACK.
//   7. Host queries: insideDomain, distances, projection.
// Writes the mixed problem's inputs and estimates to the directory argv[1] (raw little-endian
// arrays) so that the same solve can be replayed through the Python interface.
#include <cmath>
#include <cstdio>
#include <fstream>
#include <string>
#include <vector>

#include "zombie_gb300.hpp"

namespace zg = zombie_gb300;
using Vec = zg::Vector<2>;
using Veci = zg::Vectori<2>;

static int failures = 0;
#define EXPECT(cond, ...)                                          \
    do {                                                           \
        if (!(cond)) {                                             \
            std::fprintf(stderr, "FAILED %s: ", #cond);            \
            std::fprintf(stderr, __VA_ARGS__);                     \
            std::fprintf(stderr, "\n");                            \
            failures++;                                            \
        }                                                          \
    } while (0)

static double exactU(const Vec& x) { return std::exp((double)x[0]) * std::cos((double)x[1]); }
static void exactGrad(const Vec& x, double g[2]) {
    g[0] = std::exp((double)x[0]) * std::cos((double)x[1]);
    g[1] = -std::exp((double)x[0]) * std::sin((double)x[1]);
}

template <typename V>
static void writeRaw(const std::string& dir, const std::string& name, const std::vector<V>& v) {
    std::ofstream f(dir + "/" + name, std::ios::binary);
    f.write(reinterpret_cast<const char*>(v.data()), (std::streamsize)(v.size() * sizeof(V)));
}

struct Polyline {
    std::vector<Vec> pos;
    std::vector<Veci> idx;
};

// segments k -> k+1 of the star polygon whose midpoint angle lies in [a0, a1)
static Polyline starPart(int n, double a0, double a1) {
    const double kPi = 3.14159265358979323846;
    std::vector<Vec> all(n);
    for (int k = 0; k < n; k++) {
        const float t = (float)(2.0 * kPi * k / n);
        const float r = 1.0f * (1.0f + 0.3f * std::sin(5.0f * t));
        all[k] = Vec(r * std::cos(t), r * std::sin(t));
    }
    Polyline p;
    std::vector<int> remap(n, -1);
    for (int k = 0; k < n; k++) {
        const int k1 = (k + 1) % n;
        double mid = std::atan2(0.5 * (all[k][1] + all[k1][1]), 0.5 * (all[k][0] + all[k1][0]));
        if (mid < 0) mid += 2.0 * kPi;
        if (mid < a0 || mid >= a1) continue;
        int ids[2] = {k, k1};
        Veci seg;
        for (int j = 0; j < 2; j++) {
            if (remap[ids[j]] < 0) {
                remap[ids[j]] = (int)p.pos.size();
                p.pos.push_back(all[ids[j]]);
            }
            seg[j] = remap[ids[j]];
        }
        p.idx.push_back(seg);
    }
    return p;
}

// fraction of points whose estimate lies within `k` standard errors of the exact value
template <typename Stats>
static double withinSE(const std::vector<Vec>& pts, const std::vector<Stats>& stats, double k, double& meanAbsErr) {
    int ok = 0;
    meanAbsErr = 0.0;
    for (size_t i = 0; i < pts.size(); i++) {
        const double est = stats[i].getEstimatedSolution();
        const double se = std::sqrt(stats[i].getEstimatedSolutionVariance() / stats[i].getSolutionEstimateCount());
        const double err = std::fabs(est - exactU(pts[i]));
        meanAbsErr += err;
        ok += err <= k * se + 1e-4;
    }
    meanAbsErr /= (double)pts.size();
    return (double)ok / (double)pts.size();
}

int main(int argc, char** argv) {
    const std::string out = argc > 1 ? argv[1] : ".";
    const double kPi = 3.14159265358979323846;
    const int nSeg = 1024;

    // ------------------------------------------------------------------ problem setup
    Polyline whole = starPart(nSeg, 0.0, 2.0 * kPi);
    Polyline absorbingPart = starPart(nSeg, 0.0, kPi);
    Polyline reflectingPart = starPart(nSeg, kPi, 2.0 * kPi);
    Vec lo(-1.3f, -1.3f), hi(1.3f, 1.3f);

    zg::PDE<float, 2> pde;
    pde.solution.n_terms = 1;
    pde.solution.c[0] = 1.0f;
    pde.solution.a[0][0] = 1.0f;
    pde.solution.b[0][1] = 1.0f;
    pde.dirichlet = zg::Field::analytic();
    pde.robin = zg::Field::analytic();       // du/dn + 0 u on the Neumann part
    pde.source = zg::Field::zero();
    pde.isSourceConstant = true;

    zg::FcpwDirichletBoundaryHandler<2> wholeHandler;
    wholeHandler.buildAccelerationStructure(whole.pos, whole.idx);
    zg::GeometricQueries<2> dirichletQueries(true, lo, hi);
    zg::populateGeometricQueriesForDirichletBoundary(wholeHandler, dirichletQueries);

    zg::FcpwDirichletBoundaryHandler<2> absorbingHandler;
    absorbingHandler.buildAccelerationStructure(absorbingPart.pos, absorbingPart.idx);
    zg::FcpwNeumannBoundaryHandler<2> neumannHandler;
    neumannHandler.buildAccelerationStructure(reflectingPart.pos, reflectingPart.idx,
                                              zg::getIgnoreCandidateSilhouetteCallback(false, 0.0f));
    zg::GeometricQueries<2> mixedQueries(true, lo, hi);
    zg::populateGeometricQueriesForDirichletBoundary(absorbingHandler, mixedQueries);
    zg::populateGeometricQueriesForNeumannBoundary(neumannHandler, zg::getBranchTraversalWeightCallback(),
                                                   mixedQueries);

    // interior grid points kept 0.05 away from the boundary
    std::vector<Vec> grid;
    const int G = 24;
    for (int i = 0; i < G; i++)
        for (int j = 0; j < G; j++)
            grid.push_back(Vec(-1.3f + 2.6f * (i + 0.5f) / G, -1.3f + 2.6f * (j + 0.5f) / G));
    std::vector<bool> inside = mixedQueries.insideDomain(grid);
    std::vector<float> dA = mixedQueries.computeDistToAbsorbingBoundary(grid, false);
    std::vector<float> dR = mixedQueries.computeDistToReflectingBoundary(grid, false);
    std::vector<float> dW = dirichletQueries.computeDistToAbsorbingBoundary(grid, false);
    std::vector<Vec> pts;
    std::vector<float> ptsDA, ptsDR, ptsDW;
    for (size_t i = 0; i < grid.size(); i++) {
        if (!inside[i] || dA[i] < 0.05f || dR[i] < 0.05f) continue;
        pts.push_back(grid[i]);
        ptsDA.push_back(dA[i]);
        ptsDR.push_back(dR[i]);
        ptsDW.push_back(dW[i]);
    }
    const size_t n = pts.size();
    EXPECT(n > 150 && n < G * G, "%zu interior points", n);

    auto makePoints = [&](bool mixed, uint64_t seedBase, zg::EstimationQuantity q) {
        std::vector<zg::SamplePoint<float, 2>> sp;
        sp.reserve(n);
        for (size_t i = 0; i < n; i++) {
            sp.emplace_back(pts[i], Vec(), zg::SampleType::InDomain, q, 1.0f, mixed ? ptsDA[i] : ptsDW[i],
                            mixed ? ptsDR[i] : std::numeric_limits<float>::max());
            sp.back().seed = seedBase + 7919ull * i;
        }
        return sp;
    };
    zg::WalkSettings settings(1e-3f, 1e-3f, 1024, false);
    settings.silhouettePrecision = 0.0f;

    // ---------------------------------------------------- 1. Walk on Spheres, Dirichlet
    {
        zg::WalkOnSpheres<float, 2> wos(dirichletQueries);
        auto sp = makePoints(false, 1000, zg::EstimationQuantity::Solution);
        std::vector<zg::SampleStatistics<float, 2>> stats;
        int reported = 0;
        wos.solve(pde, settings, std::vector<int>(n, 256), sp, stats, false,
                  [&](int done, int) { reported += done; });
        double mae;
        const double frac = withinSE(pts, stats, 4.0, mae);
        std::printf("wos_dirichlet points=%zu within4se=%.4f mae=%.5f steps=%llu\n", n, frac, mae,
                    (unsigned long long)wos.lastReport().total_steps);
        EXPECT(frac > 0.98, "WoS within 4 SE: %.4f", frac);
        EXPECT(mae < 0.06, "WoS mean abs error %.5f", mae);   // standard error ~0.03 at 256 walks
        EXPECT(reported == (int)n, "reportProgress saw %d points", reported);
        EXPECT(stats[0].getSolutionEstimateCount() == 256, "count %d", stats[0].getSolutionEstimateCount());
        EXPECT(stats[0].getMeanWalkLength() > 1.0f, "mean walk length %f", stats[0].getMeanWalkLength());
    }

    // ---------------------------------------- 2. Walk on Stars, mixed Dirichlet / Neumann
    std::vector<zg::SampleStatistics<float, 2>> mixedStats;
    auto mixedPts = makePoints(true, 5000, zg::EstimationQuantity::Solution);
    {
        zg::WalkOnStars<float, 2> wost(mixedQueries);
        wost.solve(pde, settings, std::vector<int>(n, 512), mixedPts, mixedStats);
        double mae;
        const double frac = withinSE(pts, mixedStats, 4.0, mae);
        std::printf("wost_mixed points=%zu within4se=%.4f mae=%.5f steps=%llu\n", n, frac, mae,
                    (unsigned long long)wost.lastReport().total_steps);
        EXPECT(frac > 0.98, "WoSt within 4 SE: %.4f", frac);
        EXPECT(mae < 0.1, "WoSt mean abs error %.5f", mae);   // longer walks, standard error ~0.05
        EXPECT(mixedPts[0].firstSphereRadius > 0.0f, "first sphere radius %f", mixedPts[0].firstSphereRadius);
    }

    // ------------------------------------------ 3. progressive solves extend the walks
    {
        zg::WalkOnStars<float, 2> wost(mixedQueries);
        auto a = makePoints(true, 9000, zg::EstimationQuantity::Solution);
        auto b = a;
        std::vector<zg::SampleStatistics<float, 2>> sa, sb;
        wost.solve(pde, settings, std::vector<int>(n, 128), a, sa);
        wost.solve(pde, settings, std::vector<int>(n, 128), a, sa);
        wost.solve(pde, settings, std::vector<int>(n, 256), b, sb);
        double worst = 0.0;
        int countMismatch = 0;
        for (size_t i = 0; i < n; i++) {
            const double d = std::fabs((double)sa[i].getEstimatedSolution() - (double)sb[i].getEstimatedSolution());
            worst = std::max(worst, d / std::max(1.0, std::fabs((double)sb[i].getEstimatedSolution())));
            countMismatch += sa[i].getSolutionEstimateCount() != sb[i].getSolutionEstimateCount();
        }
        std::printf("progressive worst_rel_diff=%.3g count_mismatch=%d\n", worst, countMismatch);
        EXPECT(countMismatch == 0, "%d points with other counts", countMismatch);
        EXPECT(worst < 1e-6, "128 + 128 walks differ from 256 by %.3g", worst);
    }

    // ----------------------------------------------------- 4. solution and gradient
    {
        zg::WalkOnStars<float, 2> wost(mixedQueries);
        auto sp = makePoints(true, 13000, zg::EstimationQuantity::SolutionAndGradient);
        std::vector<zg::SampleStatistics<float, 2>> stats;
        wost.solve(pde, settings, std::vector<int>(n, 512), sp, stats);
        int ok = 0;
        double err = 0.0;
        for (size_t i = 0; i < n; i++) {
            double g[2];
            exactGrad(pts[i], g);
            auto var = stats[i].getEstimatedGradientVariance();
            bool good = true;
            for (int k = 0; k < 2; k++) {
                const double se = std::sqrt(var[k] / std::max(1, stats[i].getGradientEstimateCount()));
                const double e = std::fabs(stats[i].getEstimatedGradient(k) - g[k]);
                err += e;
                good = good && e <= 5.0 * se + 1e-3;
            }
            ok += good;
        }
        const double frac = (double)ok / n;
        std::printf("gradient within5se=%.4f mean_abs_err=%.5f\n", frac, err / (2.0 * n));
        EXPECT(frac > 0.97, "gradient within 5 SE: %.4f", frac);
        EXPECT(stats[0].getGradientEstimateCount() > 0, "no gradient estimates");
    }

    // ------------------------------------------------ 5. Dirichlet data from a dense grid
    {
        const int R = 512;
        std::vector<float> values((size_t)R * R);
        for (int i = 0; i < R; i++)
            for (int j = 0; j < R; j++) {
                const Vec c(-1.3f + 2.6f * (i + 0.5f) / R, -1.3f + 2.6f * (j + 0.5f) / R);
                values[(size_t)i * R + j] = (float)exactU(c);
            }
        zg::DenseGrid<2> g(values, Veci(R, R), lo, hi, true);
        zg::PDE<float, 2> gridPde = pde;
        gridPde.dirichlet = zg::getDenseGridCallback1(g);
        zg::WalkOnSpheres<float, 2> wos(dirichletQueries);
        auto a = makePoints(false, 17000, zg::EstimationQuantity::Solution);
        auto b = a;
        std::vector<zg::SampleStatistics<float, 2>> sa, sb;
        wos.solve(gridPde, settings, std::vector<int>(n, 64), a, sa);
        wos.solve(pde, settings, std::vector<int>(n, 64), b, sb);
        double worst = 0.0;
        for (size_t i = 0; i < n; i++)
            worst = std::max(worst, std::fabs((double)sa[i].getEstimatedSolution() - sb[i].getEstimatedSolution()));
        std::printf("dense_grid worst_abs_diff=%.3g\n", worst);
        EXPECT(worst < 2e-3, "grid Dirichlet data differ from the closed form by %.3g", worst);
    }

    // ------------------------------------------------------------- 6. host callbacks
    {
        bool threw = false;
        try {
            zg::WalkOnStars<float, 2> bad(mixedQueries, [](const zg::WalkState<float, 2>&) {}, {});
        } catch (const zg::Error& e) {
            threw = e.status() == ZGPU_ERR_UNSUPPORTED_CALLBACK;
        }
        EXPECT(threw, "walk state callback accepted");
        bool threwWeight = false;
        try {
            zg::GeometricQueries<2> q(true, lo, hi);
            zg::populateGeometricQueriesForNeumannBoundary(neumannHandler, zg::getBranchTraversalWeightCallback(0.5f),
                                                           q);
        } catch (const zg::Error& e) {
            threwWeight = e.status() == ZGPU_ERR_UNSUPPORTED;
        }
        EXPECT(threwWeight, "branch traversal weight with another min radial distance accepted");
    }

    // ------------------------------------------------------------------ 7. host queries
    {
        Vec x(0.2f, 0.1f), nrm;
        float d = 0.0f;
        const float before = dirichletQueries.computeDistToAbsorbingBoundary(x, true);
        const bool projected = dirichletQueries.projectToAbsorbingBoundary(x, nrm, d, true);
        const double r = std::sqrt((double)x[0] * x[0] + (double)x[1] * x[1]);
        const double theta = std::atan2((double)x[1], (double)x[0]);
        const double rStar = 1.0 + 0.3 * std::sin(5.0 * theta);
        std::printf("queries signed_dist=%.5f projected_radius=%.5f star_radius=%.5f\n", before, r, rStar);
        EXPECT(projected && std::fabs(d - before) < 1e-6f, "projection distance %f vs %f", d, before);
        EXPECT(before < 0.0f, "signed distance inside should be negative: %f", before);
        EXPECT(std::fabs(r - rStar) < 5e-3, "projected point off the curve: %f vs %f", r, rStar);
        EXPECT(dirichletQueries.insideDomain(Vec(0.0f, 0.0f)) && !dirichletQueries.insideDomain(Vec(1.35f, 0.0f)),
               "insideDomain");
        EXPECT(dirichletQueries.outsideBoundingDomain(Vec(2.0f, 0.0f)), "outsideBoundingDomain");
    }

    // ----------------------------------------------------------- replay data for Python
    {
        std::vector<float> absPos, reflPos, p;
        std::vector<int32_t> absIdx, reflIdx;
        for (auto& v : absorbingPart.pos) { absPos.push_back(v[0]); absPos.push_back(v[1]); }
        for (auto& v : reflectingPart.pos) { reflPos.push_back(v[0]); reflPos.push_back(v[1]); }
        for (auto& s : absorbingPart.idx) { absIdx.push_back(s[0]); absIdx.push_back(s[1]); }
        for (auto& s : reflectingPart.idx) { reflIdx.push_back(s[0]); reflIdx.push_back(s[1]); }
        std::vector<uint64_t> seeds;
        std::vector<double> mean, var;
        std::vector<int32_t> count;
        for (size_t i = 0; i < n; i++) {
            p.push_back(pts[i][0]);
            p.push_back(pts[i][1]);
            seeds.push_back(mixedPts[i].seed);
            mean.push_back(mixedStats[i].getEstimatedSolution());
            var.push_back(mixedStats[i].getEstimatedSolutionVariance());
            count.push_back(mixedStats[i].getSolutionEstimateCount());
        }
        writeRaw(out, "abs_pos.f32", absPos);
        writeRaw(out, "abs_idx.i32", absIdx);
        writeRaw(out, "refl_pos.f32", reflPos);
        writeRaw(out, "refl_idx.i32", reflIdx);
        writeRaw(out, "pts.f32", p);
        writeRaw(out, "dist_abs.f32", ptsDA);
        writeRaw(out, "dist_refl.f32", ptsDR);
        writeRaw(out, "seeds.u64", seeds);
        writeRaw(out, "mean.f64", mean);
        writeRaw(out, "var.f64", var);
        writeRaw(out, "count.i32", count);
    }

    if (failures) {
        std::fprintf(stderr, "%d check(s) failed\n", failures);
        return 1;
    }
    std::printf("facade ok\n");
    return 0;
}
