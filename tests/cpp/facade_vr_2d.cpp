// Drives the C++ variance reduction layer (include/zombie_gb300_variance_reduction.hpp) the way
// a zombie C++ caller drives bvc::BoundaryValueCachingSolver and rws::ReverseWalkOnStarsSolver,
// on the star-shaped polygon r = 1 + 0.3 sin 5 theta (1,024 counter-clockwise segments,
// all absorbing):
//   1. samplers: counts, pdfs (1 / perimeter for unit weights), offsets into the domain;
//   2. boundary value caching for u = e^x cos y: cached u and du/dn against the exact values,
//      splatted estimates at interior grid points, walk estimates near the boundary;
//   3. reverse Walk on Stars for the same u (self-normalised absorbing samples, two calls);
//   4. reverse Walk on Stars for u = e^x cos y + (x^2 + y^2) / 4 with f = -1 (domain samples).
// Exit status 1 on any failed check.
#include <cmath>
#include <cstdio>
#include <vector>

#include "zombie_gb300_variance_reduction.hpp"

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

static double exactU(const Vec& x, double quad) {
    return std::exp((double)x[0]) * std::cos((double)x[1]) + quad * ((double)x[0] * x[0] + (double)x[1] * x[1]);
}

struct Stats {
    double rmse = 0, bias = 0, stdev = 0, corr = 0;
};
static Stats compare(const std::vector<double>& est, const std::vector<double>& ex) {
    Stats s;
    const double n = (double)est.size();
    double me = 0, mx = 0;
    for (size_t i = 0; i < est.size(); i++) { me += est[i]; mx += ex[i]; }
    me /= n; mx /= n;
    double se = 0, sx = 0, sxy = 0;
    for (size_t i = 0; i < est.size(); i++) {
        const double d = est[i] - ex[i];
        s.rmse += d * d;
        s.bias += d;
        se += (est[i] - me) * (est[i] - me);
        sx += (ex[i] - mx) * (ex[i] - mx);
        sxy += (est[i] - me) * (ex[i] - mx);
    }
    s.rmse = std::sqrt(s.rmse / n);
    s.bias /= n;
    s.stdev = std::sqrt(sx / n);
    s.corr = sxy / std::sqrt(se * sx);
    return s;
}

int main() {
    const double kPi = 3.14159265358979323846;
    const int nSeg = 1024;
    std::vector<Vec> pos(nSeg);
    std::vector<Veci> idx(nSeg);
    for (int k = 0; k < nSeg; k++) {
        const float t = (float)(2.0 * kPi * k / nSeg);
        const float r = 1.0f + 0.3f * std::sin(5.0f * t);
        pos[k] = Vec(r * std::cos(t), r * std::sin(t));
        idx[k] = Veci(k, (k + 1) % nSeg);
    }
    double perimeter = 0.0, area = 0.0;
    for (int k = 0; k < nSeg; k++) {
        const Vec& a = pos[k];
        const Vec& b = pos[(k + 1) % nSeg];
        perimeter += std::hypot((double)b[0] - a[0], (double)b[1] - a[1]);
        area += 0.5 * ((double)a[0] * b[1] - (double)b[0] * a[1]);
    }
    // crossing-number point-in-polygon test (the solve region)
    auto inside = [&](const Vec& x) {
        bool in = false;
        for (int k = 0; k < nSeg; k++) {
            const Vec& a = pos[k];
            const Vec& b = pos[(k + 1) % nSeg];
            if ((a[1] > x[1]) != (b[1] > x[1])) {
                const float xc = a[0] + (x[1] - a[1]) * (b[0] - a[0]) / (b[1] - a[1]);
                if (x[0] < xc) in = !in;
            }
        }
        return in;
    };
    Vec lo(-1.3f, -1.3f), hi(1.3f, 1.3f);
    zg::FcpwDirichletBoundaryHandler<2> handler;
    handler.buildAccelerationStructure(pos, idx);
    zg::GeometricQueries<2> queries(true, lo, hi);
    zg::populateGeometricQueriesForDirichletBoundary(handler, queries);

    auto makePde = [&](double quad) {
        zg::PDE<float, 2> pde;
        pde.solution.n_terms = 1;
        pde.solution.c[0] = 1.0f;
        pde.solution.a[0][0] = 1.0f;
        pde.solution.b[0][1] = 1.0f;
        pde.solution.q[0] = pde.solution.q[1] = (float)quad;
        pde.dirichlet = zg::Field::analytic();
        pde.source = quad != 0.0 ? zg::Field::constant(-1.0f) : zg::Field::zero();
        pde.isSourceConstant = true;
        return pde;
    };
    const zg::PDE<float, 2> laplace = makePde(0.0), poisson = makePde(0.25);
    zg::WalkSettings settings(1e-3f, 1e-3f, 1024, false);

    // interior grid points and their distances
    std::vector<Vec> grid;
    const int G = 24;
    for (int i = 0; i < G; i++)
        for (int j = 0; j < G; j++) {
            Vec x(-1.3f + 2.6f * (i + 0.5f) / G, -1.3f + 2.6f * (j + 0.5f) / G);
            if (inside(x)) grid.push_back(x);
        }
    const std::vector<float> dist = queries.computeDistToAbsorbingBoundary(grid, false);
    const size_t m = grid.size();

    // ----------------------------------------------------------------------- 1. samplers
    auto sampler = std::make_shared<zg::UniformLineSegmentBoundarySampler<float>>(
        pos, idx, std::vector<float>{}, std::vector<float>{}, inside, false, 11);
    sampler->initialize(1e-3f, false);
    EXPECT(sampler->getSampleCount(8192) == 8192 && sampler->getSampleCount(8192, true) == 0, "sample counts");
    {
        std::vector<zg::SamplePoint<float, 2>> s;
        sampler->generateSamples(2000, zg::SampleType::OnAbsorbingBoundary, 1e-3f, queries, s);
        int offsetOk = 0;
        double pdfErr = 0.0;
        for (const auto& p : s) {
            offsetOk += inside(p.pt) && std::fabs(p.distToAbsorbingBoundary - 1e-3f) < 2e-4f;
            pdfErr = std::max(pdfErr, std::fabs(p.pdf * perimeter - 1.0));
        }
        std::printf("samplers n=%zu offset_ok=%d pdf_rel_err=%.2e perimeter=%.4f\n", s.size(), offsetOk, pdfErr,
                    perimeter);
        EXPECT(s.size() == 2000 && offsetOk >= 1990, "boundary samples: %zu, %d offset into the domain", s.size(),
               offsetOk);
        EXPECT(pdfErr < 1e-2, "boundary pdf x perimeter off by %.3g", pdfErr);
    }

    // ---------------------------------------------------- 2. boundary value caching
    {
        zg::bvc::BoundaryValueCachingSolver<float, 2> solver(queries, sampler, nullptr, nullptr);
        solver.generateSamples(8192, 0, 0, 1e-3f, 1e-3f, false);
        solver.computeSampleEstimates(laplace, settings, 256, 256, std::numeric_limits<float>::infinity());
        const auto& cache = solver.getAbsorbingBoundaryCache();
        double dnBias = 0.0, dnSq = 0.0, uSq = 0.0;
        for (const auto& s : cache) {
            const double gx = std::exp((double)s.pt[0]) * std::cos((double)s.pt[1]);
            const double gy = -std::exp((double)s.pt[0]) * std::sin((double)s.pt[1]);
            const double e = s.normalDerivative - (gx * s.normal[0] + gy * s.normal[1]);
            dnBias += e;
            dnSq += e * e;
            const double du = s.solution - exactU(s.pt, 0.0);
            uSq += du * du;
        }
        const double nC = (double)cache.size();
        dnBias /= nC;
        const double dnSe = std::sqrt(std::max(dnSq / nC - dnBias * dnBias, 0.0) / nC);
        const double uRms = std::sqrt(uSq / nC);
        std::vector<zg::bvc::EvaluationPoint<float, 2>> evalPts;
        for (size_t i = 0; i < m; i++) evalPts.emplace_back(grid[i], Vec(), zg::SampleType::InDomain, dist[i],
                                                            std::numeric_limits<float>::max());
        solver.splat(laplace, 1e-3f, 0.0f, std::numeric_limits<float>::infinity(), 0.05f, 0.0f, evalPts);
        std::vector<double> est, ex, estNear, exNear;
        int nearZero = 0;
        for (size_t i = 0; i < m; i++) {
            if (dist[i] >= 0.05f) {
                est.push_back(evalPts[i].getEstimatedSolution());
                ex.push_back(exactU(grid[i], 0.0));
            } else {
                nearZero += evalPts[i].getEstimatedSolution() == 0.0f;
            }
        }
        const Stats st = compare(est, ex);
        // splatted gradients at the far points against grad u
        std::vector<double> gEst, gEx;
        for (size_t i = 0; i < m; i++) {
            if (dist[i] < 0.05f) continue;
            std::vector<float> g;
            evalPts[i].getEstimatedGradient(g);
            gEst.push_back(g[0]);
            gEst.push_back(g[1]);
            gEx.push_back(std::exp((double)grid[i][0]) * std::cos((double)grid[i][1]));
            gEx.push_back(-std::exp((double)grid[i][0]) * std::sin((double)grid[i][1]));
        }
        const Stats sg = compare(gEst, gEx);
        solver.estimateSolutionNearBoundary(laplace, settings, 0.05f, 0.0f, 256, evalPts);
        for (size_t i = 0; i < m; i++)
            if (dist[i] < 0.05f) {
                estNear.push_back(evalPts[i].getEstimatedSolution());
                exNear.push_back(exactU(grid[i], 0.0));
            }
        const Stats stNear = compare(estNear, exNear);
        std::printf("bvc cache=%zu dn_bias=%.4f (se %.4f) u_rms=%.4f splat_rmse=%.4f corr=%.4f std=%.3f near=%zu "
                    "near_rmse=%.4f gradient_rmse=%.4f gradient_corr=%.4f\n", cache.size(), dnBias, dnSe, uRms, st.rmse,
                    st.corr, st.stdev, estNear.size(), stNear.rmse, sg.rmse, sg.corr);
        EXPECT(cache.size() == 8192, "cache size %zu", cache.size());
        EXPECT(std::fabs(dnBias) < 4.0 * dnSe + 1e-3, "normal derivative bias %.4f (se %.4f)", dnBias, dnSe);
        EXPECT(uRms < 0.05, "cached solution rms error %.4f", uRms);
        EXPECT(st.rmse < 0.1 * st.stdev + 0.02 && st.corr > 0.99, "splat rmse %.4f corr %.4f", st.rmse, st.corr);
        EXPECT(nearZero == (int)estNear.size(), "%d of %zu near points held no splat", nearZero, estNear.size());
        EXPECT(sg.corr > 0.95 && sg.rmse < 0.25 * sg.stdev + 0.05, "splatted gradients rmse %.4f corr %.4f", sg.rmse,
               sg.corr);
        EXPECT(!estNear.empty() && stNear.rmse < 0.05, "near-boundary walk estimates rmse %.4f", stNear.rmse);
    }

    // ---------------------------------------------- 3. reverse Walk on Stars, Laplace
    {
        auto sa = std::make_shared<zg::UniformLineSegmentBoundarySampler<float>>(
            pos, idx, std::vector<float>{}, std::vector<float>{}, inside, false, 3);
        sa->initialize(5e-3f, false);
        zg::rws::ReverseWalkOnStarsSolver<float, 2> solver(queries, sa, nullptr, nullptr);
        solver.generateSamples(40000, 0, 0, 5e-3f, false);
        std::vector<zg::rws::EvaluationPoint<float, 2>> evalPts;
        for (size_t i = 0; i < m; i++)
            evalPts.emplace_back(grid[i], Vec(), zg::SampleType::InDomain, dist[i], std::numeric_limits<float>::max());
        for (int call = 0; call < 2; call++) solver.solve(laplace, settings, 5e-3f, 1e-3f, 0.0f, evalPts);
        std::vector<double> est, ex;
        int pk = 0;
        for (size_t i = 0; i < m; i++) {
            if (dist[i] <= 0.05f) continue;
            est.push_back(solver.getEstimatedSolution(evalPts[i]));
            ex.push_back(exactU(grid[i], 0.0));
            pk += evalPts[i].totalPoissonKernelContribution > 0.0;
        }
        const Stats st = compare(est, ex);
        unsigned long long steps = 0;
        for (const auto& r : solver.lastSolveReports()) steps += r.total_steps;
        std::printf("rws_laplace samples=%d rmse=%.4f corr=%.4f std=%.3f self_normalised=%d/%zu steps=%llu\n",
                    solver.getAbsorbingBoundarySampleCount(), st.rmse, st.corr, st.stdev, pk, est.size(), steps);
        EXPECT(solver.getAbsorbingBoundarySampleCount() == 40000, "samples %d", solver.getAbsorbingBoundarySampleCount());
        EXPECT(st.rmse < 0.15 * st.stdev + 0.02 && st.corr > 0.97, "rmse %.4f corr %.4f", st.rmse, st.corr);
        EXPECT(pk == (int)est.size(), "Poisson-kernel sums at %d of %zu points", pk, est.size());
    }

    // ------------------------------------------ 4. reverse Walk on Stars with a source
    {
        auto sa = std::make_shared<zg::UniformLineSegmentBoundarySampler<float>>(
            pos, idx, std::vector<float>{}, std::vector<float>{}, inside, false, 5);
        sa->initialize(5e-3f, false);
        auto sd = std::make_shared<zg::UniformDomainSampler<float, 2>>(inside, lo, hi, (float)area, 7);
        zg::rws::ReverseWalkOnStarsSolver<float, 2> solver(queries, sa, nullptr, sd);
        solver.generateSamples(30000, 0, 60000, 5e-3f, false);
        std::vector<zg::rws::EvaluationPoint<float, 2>> evalPts;
        for (size_t i = 0; i < m; i++)
            evalPts.emplace_back(grid[i], Vec(), zg::SampleType::InDomain, dist[i], std::numeric_limits<float>::max());
        solver.solve(poisson, settings, 5e-3f, 1e-3f, 0.0f, evalPts);
        std::vector<double> est, ex;
        for (size_t i = 0; i < m; i++) {
            if (dist[i] <= 0.05f) continue;
            est.push_back(solver.getEstimatedSolution(evalPts[i]));
            ex.push_back(exactU(grid[i], 0.25));
        }
        const Stats st = compare(est, ex);
        const int nd = solver.getDomainSampleCount();
        std::printf("rws_poisson absorbing=%d domain=%d rmse=%.4f bias=%.4f corr=%.4f std=%.3f\n",
                    solver.getAbsorbingBoundarySampleCount(), nd, st.rmse, st.bias, st.corr, st.stdev);
        EXPECT(std::abs(nd - 60000) < 1500, "domain samples %d", nd);
        EXPECT(st.rmse < 0.2 * st.stdev + 0.03 && std::fabs(st.bias) < 0.05, "rmse %.4f bias %.4f", st.rmse, st.bias);
    }

    if (failures) {
        std::fprintf(stderr, "%d check(s) failed\n", failures);
        return 1;
    }
    std::printf("variance reduction facade ok\n");
    return 0;
}
