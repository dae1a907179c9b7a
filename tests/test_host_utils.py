"""Host-side utilities of the Python interface that mirror the reference's python/zombie module
(python/zombie_bindings.h, utils/fcpw_geometric_queries.h, core/geometric_queries.h): mesh
helpers with the reference's output-list calling convention, indicator callbacks, list types,
and the per-point reverse-walk evaluation point.  No GPU needed."""
import numpy as np
import pytest

import zombie_gb300 as Z
from zombie_gb300 import io
from zombie_gb300 import problems as P


def test_every_reference_python_name_outside_the_declared_scope_exists():
    """Names the reference's Python package attaches to Core / Solvers / Samplers / Utils, less
    the Kelvin transform and SDF grids (outside the walk path this engine replaces)."""
    names = {
        "Core": ["PDE", "GeometricQueries", "IntersectionPoint", "get_constant_source_callback",
                 "get_constant_dirichlet_callback", "get_constant_robin_callback",
                 "get_constant_indicator_callback", "get_constant_robin_coefficient_callback"],
        "Solvers": ["WalkSettings", "SamplePoint", "SampleStatistics", "SamplePointList", "SampleStatisticsList",
                    "create_sample_statistics_list", "WalkOnSpheres", "WalkOnStars", "BVCEvaluationPoint",
                    "BVCEvaluationPointList", "RWSEvaluationPoint", "RWSEvaluationPointList",
                    "get_empty_walk_state_callback", "get_empty_terminal_contribution_callback"],
        "Samplers": ["BoundarySampler", "DomainSampler", "create_uniform_line_segment_boundary_sampler",
                     "create_uniform_triangle_boundary_sampler", "create_uniform_domain_sampler"],
        "Utils": ["FloatDenseGrid", "BoolDenseGrid", "load_boundary_mesh", "load_textured_boundary_mesh",
                  "normalize", "apply_shift", "flip_orientation", "compute_bounding_box", "build_bounding_box_mesh",
                  "add_bounding_box_to_boundary_mesh", "compute_signed_volume", "compute_dist_to_boundary",
                  "partition_boundary_mesh", "get_spatially_sorted_point_indices", "FcpwDirichletBoundaryHandler",
                  "FcpwNeumannBoundaryHandler", "FcpwRobinBoundaryHandler",
                  "populate_geometric_queries_for_dirichlet_boundary",
                  "populate_geometric_queries_for_neumann_boundary", "populate_geometric_queries_for_robin_boundary",
                  "get_ignore_candidate_silhouette_callback", "get_branch_traversal_weight_callback",
                  "get_dense_grid_source_callback", "get_dense_grid_dirichlet_callback", "get_dense_grid_robin_callback",
                  "get_dense_grid_indicator_callback", "get_dense_grid_robin_coefficient_callback"],
    }
    missing = [f"{m}.{n}" for m, ns in names.items() for n in ns if not hasattr(getattr(Z, m), n)]
    assert not missing, missing


@pytest.mark.parametrize("dim", [2, 3])
def test_bounding_box_mesh_is_outward_and_fills_lists(dim):
    lo, hi = np.zeros(dim), np.arange(1, dim + 1, dtype=float)
    pos, idx = [], []
    P_, I_ = Z.Utils.build_bounding_box_mesh(lo, hi, pos, idx, dim=dim)
    assert len(pos) == 2 ** dim and len(idx) == (4 if dim == 2 else 12)
    assert np.allclose(np.array(pos), P_) and np.array_equal(np.array(idx), I_)
    # outward orientation: positive signed volume equal to the box volume
    assert Z.Utils.compute_signed_volume(P_, I_, dim=dim) == pytest.approx(float(np.prod(hi - lo)))
    assert io.compute_signed_volume(P_, io.flip_orientation(I_.copy())) == pytest.approx(-float(np.prod(hi - lo)))


def test_add_bounding_box_appends_with_offset_indices():
    pos, idx = P.star_polygon(64)
    area = io.compute_signed_volume(pos, idx)
    shoelace = 0.5 * np.sum(pos[idx[:, 0], 0] * pos[idx[:, 1], 1] - pos[idx[:, 1], 0] * pos[idx[:, 0], 1])
    assert area == pytest.approx(float(shoelace), rel=1e-6)
    P2, I2 = Z.Utils.add_bounding_box_to_boundary_mesh([-2, -2], [2, 2], pos, idx)
    assert P2.shape == (68, 2) and I2.shape == (68, 2) and I2[64:].min() == 64
    assert io.compute_signed_volume(P2, I2) == pytest.approx(area + 16.0, rel=1e-6)
    lp, li = [p for p in pos], [i for i in idx]
    Z.Utils.add_bounding_box_to_boundary_mesh([-2, -2], [2, 2], lp, li)
    assert len(lp) == 68 and np.array_equal(np.array(li), I2)


def test_partition_boundary_mesh_fills_output_lists_and_takes_point_callbacks():
    pos, idx = P.star_polygon(64)
    ap, ai, rp, ri = [], [], [], []
    (a_p, a_i), (r_p, r_i) = Z.Utils.partition_boundary_mesh(lambda m: bool(m[1] < 0), pos, idx, ap, ai, rp, ri,
                                                              dim=2)
    assert len(ai) + len(ri) == 64 and len(ap) == a_p.shape[0] and len(rp) == r_p.shape[0]
    assert np.all(r_p[r_i].mean(1)[:, 1] < 0) and np.all(a_p[a_i].mean(1)[:, 1] >= 0)
    ind = Z.Core.get_constant_indicator_callback(True, dim=2)
    (_, none_i), (_, all_i) = Z.Utils.partition_boundary_mesh(ind, pos, idx)
    assert none_i.shape[0] == 0 and all_i.shape[0] == 64


def test_spatially_sorted_indices_are_a_local_permutation():
    x = np.random.default_rng(0).random((4096, 3)).astype(np.float32)
    out = []
    order = Z.Utils.get_spatially_sorted_point_indices(x, out, dim=3)
    assert sorted(order.tolist()) == list(range(4096)) and out == order.tolist()
    step = np.linalg.norm(np.diff(x[order], axis=0), axis=1).mean()
    assert step < 0.25 * np.linalg.norm(np.diff(x, axis=0), axis=1).mean()


def test_textured_mesh_and_list_style_mesh_loading(tmp_path):
    f = tmp_path / "quad.obj"
    f.write_text("v 0 0 0\nv 1 0 0\nv 1 1 0\nv 0 1 0\nvt 0 0\nvt 1 0\nvt 1 1\nvt 0 1\nf 1/1 2/2 3/3 4/4\n")
    pos, uv, idx, tidx = [], [], [], []
    Z.Utils.load_textured_boundary_mesh(str(f), pos, uv, idx, tidx, dim=3)
    assert len(pos) == 4 and len(uv) == 4
    assert np.array_equal(np.array(idx), [[0, 1, 2], [0, 2, 3]]) and np.array_equal(np.array(tidx), [[0, 1, 2], [0, 2, 3]])
    with pytest.raises(ValueError):
        Z.Utils.load_textured_boundary_mesh(str(f), dim=2)
    p2, i2 = [], []
    Z.Utils.load_boundary_mesh(str(f), p2, i2, dim=3)
    assert len(p2) == 4 and len(i2) == 2
    arr_p, arr_i = Z.Utils.load_boundary_mesh(str(f), 3)
    assert arr_p.shape == (4, 3) and arr_i.shape == (2, 3)


def test_indicator_callbacks_and_intersection_point():
    g = Z.Utils.BoolDenseGrid(np.array([[1, 0], [0, 1]]), [2, 2], [0, 0], [1, 1], dim=2)
    f = Z.Utils.get_dense_grid_indicator_callback(g, dim=2)
    assert f([0.1, 0.1]) is True and f([0.1, 0.9]) is False
    assert list(f(np.array([[0.9, 0.9], [0.9, 0.1]]))) == [True, False]
    f2 = Z.Utils.get_dense_grid_indicator_callback(np.array([[1, 0], [0, 1]]), [2, 2], [0, 0], [1, 1], dim=2)
    assert f2([0.9, 0.9]) is True
    ip = Z.Core.IntersectionPoint(dim=3)
    assert ip.pt.shape == (3,) and ip.dist == pytest.approx(np.finfo(np.float32).max)
    pde = Z.Core.PDE(dim=2)
    assert pde.has_reflecting_boundary_conditions is None


def test_compute_dist_to_boundary_fills_lists():
    class Q:
        dim = 2

        def compute_dist_to_absorbing_boundary(self, x):
            return np.linalg.norm(x, axis=1)

        def compute_dist_to_reflecting_boundary(self, x):
            return np.full(len(x), 2.0)
    da, dr = [], []
    a, r = Z.Utils.compute_dist_to_boundary(Q(), [[3.0, 4.0], [0.0, 1.0]], da, dr, dim=2)
    assert da == [5.0, 1.0] and dr == [2.0, 2.0] and a.dtype == np.float32


def test_list_types_empty_callbacks_and_rws_point_sums():
    assert Z.Solvers.SamplePointList(dim=2) == [] and Z.Solvers.RWSEvaluationPointList([1], dim=3) == [1]
    assert Z.Solvers.get_empty_walk_state_callback(dim=2) is None
    assert Z.Solvers.get_empty_terminal_contribution_callback(dim=3) is None
    p = Z.Solvers.RWSEvaluationPoint([0.1, 0.2], [0.0, 0.0], Z.Solvers.SampleType.InDomain, 1.0, 1.0)
    from zombie_gb300 import _abi as A
    p._pts.totals[0, A.ZGPU_RWS_ABSORBING] = 6.0
    p._pts.totals[0, A.ZGPU_RWS_POISSON_KERNEL] = 3.0
    p._pts.totals[0, A.ZGPU_RWS_SOURCE] = 4.0
    assert p.total_absorbing_boundary_contribution == 6.0
    assert p.get_estimated_solution(10, 0, 0, 0, 8) == pytest.approx(2.0 + 0.5)
    p._pts.totals[0, A.ZGPU_RWS_POISSON_KERNEL] = 0.0
    assert p.get_estimated_solution(10, 0, 0, 0, 8) == pytest.approx(0.6 + 0.5)
    p.reset()
    assert p.total_source_contribution == 0.0


def test_host_utilities_accept_empty_inputs():
    out = [1, 2]
    assert Z.Utils.get_spatially_sorted_point_indices(np.zeros((0, 3)), out).size == 0 and out == []
    assert io.compute_signed_volume(np.zeros((0, 2)), np.zeros((0, 2), np.int32)) == 0.0
    assert io.compute_signed_volume(np.zeros((0, 3)), np.zeros((0, 3), np.int32)) == 0.0
    (ap, ai), (rp, ri) = io.partition_boundary_mesh(lambda m: m[:, 0] > 0, np.zeros((0, 2)), np.zeros((0, 2), np.int32))
    assert ap.shape == (0, 2) and ri.shape == (0, 2)
