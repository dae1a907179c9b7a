"""The C++ host interfaces (include/zombie_gb300.hpp, include/zombie_gb300_variance_reduction.hpp):
compile for 2D and 3D instantiations of the reference's class names on any machine; on the GPU
the variance reduction driver (tests/cpp/facade_vr_2d.cpp: samplers, boundary value caching,
reverse Walk on Stars with and without a source) runs, and so does the facade driver
(tests/cpp/facade_solve_2d.cpp: WoS and WoSt solves, progressive solves, gradients, dense
grids, callback rejection, host queries) and replays its mixed Dirichlet / Neumann solve
through the Python interface with the same seeds: both host sides reach the same estimates."""
import os
import shutil
import subprocess

import numpy as np
import pytest

from zombie_gb300 import _abi as A
from zombie_gb300 import problems as P

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
INCLUDE = os.path.join(ROOT, "include")
DRIVER = os.path.join(HERE, "cpp", "facade_solve_2d.cpp")
DRIVER_VR = os.path.join(HERE, "cpp", "facade_vr_2d.cpp")

INSTANTIATIONS_3D = r"""
#include "zombie_gb300_variance_reduction.hpp"
namespace zg = zombie_gb300;
template class zg::UniformTriangleBoundarySampler<float>;
template class zg::UniformDomainSampler<float, 3>;
template class zg::bvc::BoundaryValueCaching<float, 3>;
template class zg::bvc::BoundaryValueCachingSolver<float, 3>;
template struct zg::bvc::EvaluationPoint<float, 3>;
template class zg::rws::ReverseWalkOnStarsSolver<float, 3>;
template struct zg::rws::EvaluationPoint<float, 3>;
template class zg::WalkOnSpheres<float, 3>;
template class zg::WalkOnStars<float, 3>;
template struct zg::GeometricQueries<3>;
template class zg::FcpwDirichletBoundaryHandler<3>;
template class zg::FcpwNeumannBoundaryHandler<3>;
template class zg::FcpwRobinBoundaryHandler<3>;
template class zg::SampleStatistics<float, 3>;
template struct zg::SamplePoint<float, 3>;
int main() {
    zg::SampleStatistics<float, 3> a, b;
    a.addSolutionEstimate(1.0f); b.addSolutionEstimate(3.0f); b.addSolutionEstimate(5.0f);
    a.merge(b);
    zg::DenseGrid<3> g(std::vector<float>(8, 1.0f), zg::Vectori<3>(2, 2, 2), zg::Vector3(0, 0, 0), zg::Vector3(1, 1, 1));
    zg::PDE<float, 3> pde;
    pde.source = zg::getDenseGridCallback0(g);
    zg::WalkSettings ws(1e-3f, 1e-3f, 1024, false);
    int bad = !(a.getSolutionEstimateCount() == 3 && a.getEstimatedSolution() == 3.0f &&
                a.getEstimatedSolutionVariance() == 4.0f && pde.toC().source_kind == ZGPU_FIELD_GRID &&
                ws.toC().max_walk_length == 1024 && ws.toC().steps_before_using_maximal_spheres == 1024);
    // a unit cube's 12 triangles: sample counts split by side, validation of the inputs
    std::vector<zg::Vector3> v;
    for (int i = 0; i < 8; i++) v.push_back(zg::Vector3(i & 1, (i >> 1) & 1, (i >> 2) & 1));
    const int f[12][3] = {{0,2,1},{1,2,3},{4,5,6},{5,7,6},{0,1,4},{1,5,4},{2,6,3},{3,6,7},{0,4,2},{2,4,6},{1,3,5},{3,7,5}};
    std::vector<zg::Vectori<3>> t;
    for (auto& q : f) t.push_back(zg::Vectori<3>(q[0], q[1], q[2]));
    auto all = [](const zg::Vector3&) { return true; };
    zg::UniformTriangleBoundarySampler<float> s(v, t, {}, {}, all, false, 5);
    s.initialize(0.0f, false);
    bad += !(s.getSampleCount(100) == 100 && s.getSampleCount(100, true) == 0);
    s.initialize(0.0f, true);
    bad += !(s.getSampleCount(100) == 50 && s.getSampleCount(100, true) == 50);
    auto none = [](const zg::Vector3&) { return false; };
    zg::UniformTriangleBoundarySampler<float> empty(v, t, {}, {}, none, false, 5);
    empty.initialize(0.0f, false);
    bad += empty.getSampleCount(100) != 0;
    auto throwsInvalid = [](auto fn) {
        try { fn(); } catch (const zg::Error& e) { return e.status() == ZGPU_ERR_INVALID_ARG; }
        return false;
    };
    bad += !throwsInvalid([&] { zg::UniformTriangleBoundarySampler<float>(v, t, std::vector<float>(12, -1.0f), {}, all); });
    bad += !throwsInvalid([&] { zg::UniformTriangleBoundarySampler<float>(v, t, std::vector<float>(3, 1.0f), {}, all); });
    bad += !throwsInvalid([&] { zg::DenseGrid<3>(std::vector<float>(7), zg::Vectori<3>(2, 2, 2), zg::Vector3(), zg::Vector3(1, 1, 1)); });
    // reverse-walk evaluation point: self-normalised absorbing part + per-count other parts
    zg::rws::EvaluationPoint<float, 3> e(zg::Vector3(), zg::Vector3(), zg::SampleType::InDomain, 1.0f, 1.0f);
    e.totalAbsorbingBoundaryContribution = 6.0; e.totalPoissonKernelContribution = 3.0; e.totalSourceContribution = 4.0;
    bad += e.getEstimatedSolution(10, 0, 0, 0, 8) != 2.5f;
    e.totalPoissonKernelContribution = 0.0;
    bad += e.getEstimatedSolution(10, 0, 0, 0, 8) != 1.1f;
    // sample generation against queries without boundaries (host-only distances: FLT_MAX)
    zg::GeometricQueries<3> noBoundary(true, zg::Vector3(0, 0, 0), zg::Vector3(1, 1, 1));
    std::vector<zg::SamplePoint<float, 3>> sp;
    s.initialize(0.0f, false);
    s.generateSamples(1200, zg::SampleType::OnAbsorbingBoundary, 0.0f, noBoundary, sp);
    int onFace = 0, unitNormal = 0, pdfOk = 0;
    for (const auto& q : sp) {
        int faces = 0;
        for (int k = 0; k < 3; k++) faces += std::fabs(q.pt[k]) < 1e-6f || std::fabs(q.pt[k] - 1.0f) < 1e-6f;
        onFace += faces >= 1;
        const float nn = q.normal[0] * q.normal[0] + q.normal[1] * q.normal[1] + q.normal[2] * q.normal[2];
        const float nmax = std::max(std::fabs(q.normal[0]), std::max(std::fabs(q.normal[1]), std::fabs(q.normal[2])));
        unitNormal += std::fabs(nn - 1.0f) < 1e-5f && std::fabs(nmax - 1.0f) < 1e-5f;
        pdfOk += std::fabs(q.pdf - 1.0f / 6.0f) < 1e-6f && q.type == zg::SampleType::OnAbsorbingBoundary &&
                 q.distToAbsorbingBoundary == std::numeric_limits<float>::max();
    }
    bad += !(sp.size() == 1200 && onFace == 1200 && unitNormal == 1200 && pdfOk == 1200);
    zg::UniformDomainSampler<float, 3> ds([](const zg::Vector3& x) { return x[0] < 0.5f; }, zg::Vector3(0, 0, 0),
                                          zg::Vector3(1, 1, 1), 0.5f, 9);
    ds.generateSamples(2000, noBoundary, sp);
    int inRegion = 0;
    for (const auto& q : sp) inRegion += q.pt[0] < 0.5f && q.pdf == 2.0f && q.type == zg::SampleType::InDomain;
    bad += !(sp.size() > 1900 && sp.size() < 2100 && inRegion == (int)sp.size());
    zg::bvc::EvaluationPoint<float, 3> ep(zg::Vector3(), zg::Vector3(), zg::SampleType::InDomain, 1.0f, 1.0f);
    std::vector<float> grad;
    ep.getEstimatedGradient(grad);
    bad += !(ep.getEstimatedSolution() == 0.0f && grad.size() == 3 && grad[2] == 0.0f);
    return bad ? 1 : 0;
}
"""


def _gxx():
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("g++ not available")
    return gxx


def test_facade_compiles_for_2d_and_3d(tmp_path):
    """Syntax and template instantiation of every facade class for DIM = 2 (the driver) and 3."""
    gxx = _gxx()
    src = tmp_path / "inst3d.cpp"
    src.write_text(INSTANTIATIONS_3D)
    for f in (DRIVER, DRIVER_VR, str(src)):
        r = subprocess.run([gxx, "-std=c++17", "-fsyntax-only", "-Wall", "-Wextra", "-Werror", "-I", INCLUDE, f],
                           capture_output=True, text=True)
        assert r.returncode == 0, r.stderr


def _compile(gxx, src, out, lib_dir):
    r = subprocess.run([gxx, "-std=c++17", "-O2", "-I", INCLUDE, src, "-L", lib_dir, "-lzgpu",
                        f"-Wl,-rpath,{lib_dir}", "-o", out], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


def test_facade_host_classes_run_without_a_gpu(tmp_path):
    """Linked against the library, the 3D instantiations run their host-only parts (no
    context is created): SampleStatistics::merge (Chan et al.) gives the pooled mean 3 and
    variance 4 of {1, 3, 5}; a DenseGrid becomes a grid field; settings carry over; a cube's
    triangle sampler splits sample counts by side and keeps none outside the solve region;
    negative or missing primitive weights and mis-sized grids throw INVALID_ARG; cube-surface
    samples lie on its faces with pdf 1 / area and unit axis-aligned normals, domain samples
    stay in the solve region with pdf 1 / volume (queries without boundaries answer on the
    host); the reverse-walk evaluation point self-normalises its absorbing part."""
    from zombie_gb300 import build
    build.build()
    LIBDIR = build.LIBDIR
    gxx = _gxx()
    src = tmp_path / "inst3d.cpp"
    src.write_text(INSTANTIATIONS_3D)
    exe = str(tmp_path / "inst3d")
    _compile(gxx, str(src), exe, LIBDIR)
    assert subprocess.run([exe]).returncode == 0


@pytest.mark.gpu
def test_facade_driver_and_python_replay(zgpu, tmp_path):
    import zombie_gb300 as Z
    from zombie_gb300.build import LIBDIR
    gxx = _gxx()
    exe = str(tmp_path / "facade_solve_2d")
    _compile(gxx, DRIVER, exe, LIBDIR)
    out = tmp_path / "out"
    out.mkdir()
    r = subprocess.run([exe, str(out)], capture_output=True, text=True, timeout=600)
    print(r.stdout)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "facade ok" in r.stdout

    def load(name, dtype, cols=None):
        a = np.fromfile(out / name, dtype=dtype)
        return a.reshape(-1, cols) if cols else a

    abs_pos, abs_idx = load("abs_pos.f32", np.float32, 2), load("abs_idx.i32", np.int32, 2)
    refl_pos, refl_idx = load("refl_pos.f32", np.float32, 2), load("refl_idx.i32", np.int32, 2)
    pts, seeds = load("pts.f32", np.float32, 2), load("seeds.u64", np.uint64)
    d_abs, d_refl = load("dist_abs.f32", np.float32), load("dist_refl.f32", np.float32)
    mean_cpp, count_cpp = load("mean.f64", np.float64), load("count.i32", np.int32)

    q = Z.Core.GeometricQueries(True, [-1.3, -1.3], [1.3, 1.3], dim=2)
    ab = Z.Utils.FcpwDirichletBoundaryHandler(dim=2)
    ab.build_acceleration_structure(abs_pos, abs_idx)
    Z.Utils.populate_geometric_queries_for_dirichlet_boundary(ab, q, dim=2)
    rf = Z.Utils.FcpwNeumannBoundaryHandler(dim=2)
    rf.build_acceleration_structure(refl_pos, refl_idx, Z.Utils.get_ignore_candidate_silhouette_callback(False, 0.0))
    Z.Utils.populate_geometric_queries_for_neumann_boundary(rf, Z.Utils.get_branch_traversal_weight_callback(), q,
                                                            dim=2)
    pde = Z.api.PDE.from_c(2, P.make_pde(P.solution_expcos(0.0), robin=True, source=False))
    ws = Z.Solvers.WalkSettings(1e-3, 1e-3, 0.0, 0.0, A.FLT_MAX, 1024, 0, 1024, False, True, True, False, False,
                                False, False, False)
    sp = [Z.Solvers.SamplePoint(p, np.zeros(2), Z.Solvers.SampleType.InDomain, Z.Solvers.EstimationQuantity.Solution,
                                1.0, float(da), float(dr), seed=int(s), dim=2)
          for p, da, dr, s in zip(pts, d_abs, d_refl, seeds)]
    stats = Z.Solvers.create_sample_statistics_list(len(sp), dim=2)
    Z.Solvers.WalkOnStars(q, dim=2).solve(pde, ws, [512] * len(sp), sp, stats)
    mean_py = np.array([s.get_estimated_solution() for s in stats])
    count_py = np.array([s.get_solution_estimate_count() for s in stats])
    assert np.array_equal(count_py, count_cpp)
    # the C++ getters return float; the walks themselves are the same
    assert np.allclose(mean_py, mean_cpp, rtol=1e-6, atol=1e-6), np.abs(mean_py - mean_cpp).max()


@pytest.mark.gpu
def test_variance_reduction_facade_driver(zgpu, tmp_path):
    from zombie_gb300.build import LIBDIR
    gxx = _gxx()
    exe = str(tmp_path / "facade_vr_2d")
    _compile(gxx, DRIVER_VR, exe, LIBDIR)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=900)
    print(r.stdout)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "variance reduction facade ok" in r.stdout
