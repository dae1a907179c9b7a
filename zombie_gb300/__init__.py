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


Core = _types.SimpleNamespace(
    PDE=_dim_factory(PDE),
    GeometricQueries=_dim_factory(GeometricQueries),
    Field=Field,
    get_constant_source_callback=lambda value, dim=None, channels=1: Field.constant(value),
    get_constant_dirichlet_callback=lambda value, value_aligned=None, dim=None, channels=1: Field.constant(value, value_aligned),
    get_constant_robin_callback=lambda value, value_aligned=None, dim=None, channels=1: Field.constant(value, value_aligned),
    get_constant_robin_coefficient_callback=lambda value, value_aligned=None, dim=None: Field.constant(value, value_aligned),
    get_analytic_callback=lambda dim=None, channels=1: Field.analytic(),
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
    ReverseWalkOnStars=_rws.ReverseWalkOnStarsSolver,
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
    load_boundary_mesh=_io.load_boundary_mesh,
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
