"""zombie_gb300: GB300-native Walk on Spheres / Walk on Stars engine.

The Python surface mirrors rohan-sawhney/zombie's module layout (python/zombie/__init__.py):
`Core`, `Solvers` and `Utils` namespaces whose factories take `dim=` (and `channels=`).
Compute runs in the CUDA library zombie_gb300/lib/libzgpu.so through the C ABI of
include/zgpu.h; there is no CPU fallback.
"""
import types as _types

from . import _abi
from .api import (BranchTraversalWeight, Context, DenseGrid, EstimationQuantity, Field, GeometricQueries,
                  GpuDirichletBoundaryHandler, GpuNeumannBoundaryHandler, GpuRobinBoundaryHandler,
                  IgnoreCandidateSilhouette, NeuralCache, PDE, SampleArrays, SamplePoint, SampleStatistics, SampleType,
                  WalkCompletionCode, WalkOnSpheres, WalkOnStars, WalkSettings, create_sample_statistics_list,
                  default_context, get_dense_grid_dirichlet_callback, get_dense_grid_robin_callback,
                  get_dense_grid_robin_coefficient_callback, get_dense_grid_source_callback,
                  populate_geometric_queries_for_dirichlet_boundary,
                  populate_geometric_queries_for_neumann_boundary, populate_geometric_queries_for_robin_boundary)
from ._lib import ZgpuError
from . import bvc as _bvc
from . import api as _api
from . import io as _io
from . import rws as _rws

__all__ = ["Core", "Solvers", "Samplers", "Utils", "ZgpuError", "Context", "default_context"]


def _dim_factory(cls):
    def factory(*args, dim, channels=1, **kw):
        if channels != 1:
            raise ValueError("channels must be 1 in this build")
        return cls(*args, dim=dim, **kw) if "dim" in cls.__init__.__code__.co_varnames else cls(*args, **kw)
    factory.__name__ = cls.__name__
    factory.__doc__ = cls.__doc__
    return factory


def _solver_factory(cls):
    def factory(geometric_queries, *args, dim, channels=1, **kw):
        return cls(geometric_queries, *args, dim=dim, channels=channels, **kw)
    factory.__name__ = cls.__name__
    factory.__doc__ = cls.__doc__
    return factory


def _list_factory(*args, dim=None, channels=1):
    return list(*args)


def _load_boundary_mesh(obj_file, positions=None, indices=None, dim=None):
    """load_boundary_mesh(obj_file, positions, indices, dim=...) filling the two lists as the
    reference does, or load_boundary_mesh(obj_file, dim) returning arrays."""
    if isinstance(positions, int) and dim is None:
        dim, positions = positions, None
    p, i = _io.load_boundary_mesh(obj_file, dim)
    return _io._fill(positions, p), _io._fill(indices, i)


def _load_textured_boundary_mesh(obj_file, positions=None, texture_coordinates=None, indices=None,
                                 texture_indices=None, dim=3):
    if dim != 3:
        raise ValueError("load_textured_boundary_mesh is only supported for dim=3")
    return _io.load_textured_boundary_mesh(obj_file, positions, texture_coordinates, indices, texture_indices)


Core = _types.SimpleNamespace(
    PDE=_dim_factory(PDE),
    GeometricQueries=_dim_factory(GeometricQueries),
    Field=Field,
    get_constant_source_callback=lambda value, dim=None, channels=1: Field.constant(value),
    get_constant_dirichlet_callback=lambda value, value_aligned=None, dim=None, channels=1: Field.constant(value, value_aligned),
    get_constant_robin_callback=lambda value, value_aligned=None, dim=None, channels=1: Field.constant(value, value_aligned),
    get_constant_robin_coefficient_callback=lambda value, value_aligned=None, dim=None: Field.constant(value, value_aligned),
    get_analytic_callback=lambda dim=None, channels=1: Field.analytic(),
    get_constant_indicator_callback=_api.get_constant_indicator_callback,
    IntersectionPoint=_dim_factory(_api.IntersectionPoint),
)

Solvers = _types.SimpleNamespace(
    WalkSettings=WalkSettings,
    SampleType=SampleType,
    EstimationQuantity=EstimationQuantity,
    WalkCompletionCode=WalkCompletionCode,
    SamplePoint=_dim_factory(SamplePoint),
    SampleStatistics=_dim_factory(SampleStatistics),
    SampleArrays=SampleArrays,
    create_sample_statistics_list=lambda size, dim=None, channels=1: create_sample_statistics_list(size),
    WalkOnSpheres=_solver_factory(WalkOnSpheres),
    WalkOnStars=_solver_factory(WalkOnStars),
    NeuralCache=NeuralCache,
    BVCEvaluationPoint=_bvc.EvaluationPoint,
    BVCEvaluationPoints=_bvc.EvaluationPoints,
    BoundaryValueCaching=_bvc.BoundaryValueCachingSolver,
    RWSEvaluationPoints=_rws.EvaluationPoints,
    RWSEvaluationPoint=_rws.EvaluationPoint,
    ReverseWalkOnStars=_rws.ReverseWalkOnStarsSolver,
    # the reference's bound std::vector types are Python lists here
    SamplePointList=_list_factory,
    SampleStatisticsList=_list_factory,
    BVCEvaluationPointList=_list_factory,
    RWSEvaluationPointList=_list_factory,
    # empty host callbacks (the solvers accept None and reject any non-empty callback)
    get_empty_walk_state_callback=lambda dim=None, channels=1: None,
    get_empty_terminal_contribution_callback=lambda dim=None, channels=1: None,
)

Samplers = _types.SimpleNamespace(
    BoundarySampler=_bvc._MeshBoundarySampler,
    DomainSampler=_bvc.UniformDomainSampler,
    create_uniform_line_segment_boundary_sampler=_bvc.create_uniform_line_segment_boundary_sampler,
    create_uniform_triangle_boundary_sampler=_bvc.create_uniform_triangle_boundary_sampler,
    create_uniform_domain_sampler=_bvc.create_uniform_domain_sampler,
)

Utils = _types.SimpleNamespace(
    DenseGrid=_dim_factory(DenseGrid),
    FloatDenseGrid=_dim_factory(DenseGrid),
    BoolDenseGrid=_api.bool_dense_grid,
    get_dense_grid_indicator_callback=_api.get_dense_grid_indicator_callback,
    load_boundary_mesh=_load_boundary_mesh,
    load_textured_boundary_mesh=_load_textured_boundary_mesh,
    build_bounding_box_mesh=lambda bounding_box_min, bounding_box_max, positions=None, indices=None, dim=None:
        _io.build_bounding_box_mesh(bounding_box_min, bounding_box_max, positions, indices),
    add_bounding_box_to_boundary_mesh=lambda bounding_box_min, bounding_box_max, positions, indices, dim=None:
        _io.add_bounding_box_to_boundary_mesh(bounding_box_min, bounding_box_max, positions, indices),
    compute_signed_volume=lambda boundary_positions, boundary_indices, dim=None:
        _io.compute_signed_volume(boundary_positions, boundary_indices),
    compute_dist_to_boundary=_api.compute_dist_to_boundary,
    partition_boundary_mesh=lambda on_reflecting_boundary, positions, indices, *out, dim=None:
        _io.partition_boundary_mesh(on_reflecting_boundary, positions, indices, *out),
    get_spatially_sorted_point_indices=lambda points, out_indices=None, dim=None:
        _io.get_spatially_sorted_point_indices(points, out_indices),
    write_boundary_mesh=_io.write_boundary_mesh,
    normalize=_io.normalize,
    apply_shift=_io.apply_shift,
    flip_orientation=_io.flip_orientation,
    compute_bounding_box=_io.compute_bounding_box,
    read_pfm=_io.read_pfm,
    write_pfm=_io.write_pfm,
    image_to_grid=_io.image_to_grid,
    get_dense_grid_source_callback=get_dense_grid_source_callback,
    get_dense_grid_dirichlet_callback=get_dense_grid_dirichlet_callback,
    get_dense_grid_robin_callback=get_dense_grid_robin_callback,
    get_dense_grid_robin_coefficient_callback=get_dense_grid_robin_coefficient_callback,
    FcpwDirichletBoundaryHandler=_dim_factory(GpuDirichletBoundaryHandler),
    FcpwNeumannBoundaryHandler=_dim_factory(GpuNeumannBoundaryHandler),
    FcpwRobinBoundaryHandler=_dim_factory(GpuRobinBoundaryHandler),
    GpuDirichletBoundaryHandler=_dim_factory(GpuDirichletBoundaryHandler),
    GpuNeumannBoundaryHandler=_dim_factory(GpuNeumannBoundaryHandler),
    GpuRobinBoundaryHandler=_dim_factory(GpuRobinBoundaryHandler),
    populate_geometric_queries_for_dirichlet_boundary=populate_geometric_queries_for_dirichlet_boundary,
    populate_geometric_queries_for_neumann_boundary=populate_geometric_queries_for_neumann_boundary,
    populate_geometric_queries_for_robin_boundary=populate_geometric_queries_for_robin_boundary,
    get_ignore_candidate_silhouette_callback=lambda solve_double_sided=False, silhouette_precision=1e-3:
        IgnoreCandidateSilhouette(solve_double_sided, silhouette_precision),
    get_branch_traversal_weight_callback=lambda min_radial_distance=1e-2: BranchTraversalWeight(min_radial_distance),
)
