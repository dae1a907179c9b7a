"""ctypes mirrors of the POD structs and constants declared in include/zgpu.h.

Layouts must match the C header field for field; tests/test_abi.py checks sizes and
offsets against the compiled library.
"""
import ctypes as C

ZGPU_ABI_VERSION = 3

ZGPU_OK = 0
ZGPU_ERR_INVALID_ARG = 1
ZGPU_ERR_OUT_OF_MEMORY = 2
ZGPU_ERR_CUDA = 3
ZGPU_ERR_TIMEOUT_BUDGET = 4
ZGPU_ERR_UNSUPPORTED_CALLBACK = 5
ZGPU_ERR_UNSUPPORTED = 6
ZGPU_ERR_DEVICE_STATE = 7

STATUS_NAMES = {
    0: "ZGPU_OK", 1: "ZGPU_ERR_INVALID_ARG", 2: "ZGPU_ERR_OUT_OF_MEMORY", 3: "ZGPU_ERR_CUDA",
    4: "ZGPU_ERR_TIMEOUT_BUDGET", 5: "ZGPU_ERR_UNSUPPORTED_CALLBACK", 6: "ZGPU_ERR_UNSUPPORTED",
    7: "ZGPU_ERR_DEVICE_STATE",
}

ZGPU_MEM_HOST = 0
ZGPU_MEM_DEVICE = 1

ZGPU_BOUNDARY_ABSORBING = 0
ZGPU_BOUNDARY_NEUMANN = 1
ZGPU_BOUNDARY_ROBIN = 2

ZGPU_SAMPLE_IN_DOMAIN = 0
ZGPU_SAMPLE_ON_ABSORBING_BOUNDARY = 1
ZGPU_SAMPLE_ON_REFLECTING_BOUNDARY = 2

ZGPU_ESTIMATE_SOLUTION = 0
ZGPU_ESTIMATE_SOLUTION_AND_GRADIENT = 1
ZGPU_ESTIMATE_SKIP = 2

ZGPU_FIELD_ZERO = 0
ZGPU_FIELD_CONSTANT = 1
ZGPU_FIELD_ANALYTIC = 2
ZGPU_FIELD_GRID = 3

ZGPU_SOLVER_WALK_ON_SPHERES = 0
ZGPU_SOLVER_WALK_ON_STARS = 1

ZGPU_MAX_TERMS = 8
ZGPU_STATIC_MAX_POINTS = 65536
ZGPU_STATIC_SCRATCH_BYTES = 4 << 20
FLT_MAX = 3.4028234663852886e38
ZGPU_QUERY_MODE_AUTO, ZGPU_QUERY_MODE_LANE, ZGPU_QUERY_MODE_WARP = 0, 1, 2
ZGPU_SCHEDULE_AUTO, ZGPU_SCHEDULE_PERSISTENT, ZGPU_SCHEDULE_WAVEFRONT = 0, 1, 2


class Analytic(C.Structure):
    _fields_ = [
        ("n_terms", C.c_int32),
        ("c", C.c_float * ZGPU_MAX_TERMS),
        ("a", (C.c_float * 3) * ZGPU_MAX_TERMS),
        ("b", (C.c_float * 3) * ZGPU_MAX_TERMS),
        ("phi", C.c_float * ZGPU_MAX_TERMS),
        ("q", C.c_float * 3),
        ("l", C.c_float * 3),
        ("d", C.c_float),
    ]


class Grid(C.Structure):
    _fields_ = [
        ("values", C.c_void_p),
        ("values_aligned", C.c_void_p),
        ("shape", C.c_int32 * 3),
        ("grid_min", C.c_float * 3),
        ("grid_max", C.c_float * 3),
        ("enable_interpolation", C.c_int32),
    ]


class Pde(C.Structure):
    _fields_ = [
        ("absorption_coeff", C.c_float),
        ("is_source_constant", C.c_int32),
        ("are_robin_conditions_pure_neumann", C.c_int32),
        ("are_robin_coeffs_nonnegative", C.c_int32),
        ("solution", Analytic),
        ("source_kind", C.c_int32), ("source_value", C.c_float),
        ("dirichlet_kind", C.c_int32), ("dirichlet_value", C.c_float), ("dirichlet_value_aligned", C.c_float),
        ("robin_kind", C.c_int32), ("robin_value", C.c_float), ("robin_value_aligned", C.c_float),
        ("robin_coeff_kind", C.c_int32), ("robin_coeff_value", C.c_float), ("robin_coeff_value_aligned", C.c_float),
        ("source_grid", Grid),
        ("dirichlet_grid", Grid),
        ("robin_grid", Grid),
        ("robin_coeff_grid", Grid),
        ("memory", C.c_int32),
    ]


class WalkSettingsC(C.Structure):
    _fields_ = [
        ("epsilon_shell_for_absorbing_boundary", C.c_float),
        ("epsilon_shell_for_reflecting_boundary", C.c_float),
        ("silhouette_precision", C.c_float),
        ("russian_roulette_threshold", C.c_float),
        ("splitting_threshold", C.c_float),
        ("max_walk_length", C.c_int32),
        ("steps_before_applying_tikhonov", C.c_int32),
        ("steps_before_using_maximal_spheres", C.c_int32),
        ("solve_double_sided", C.c_int32),
        ("use_gradient_control_variates", C.c_int32),
        ("use_gradient_antithetic_variates", C.c_int32),
        ("use_cosine_sampling_for_derivatives", C.c_int32),
        ("ignore_absorbing_boundary_contribution", C.c_int32),
        ("ignore_reflecting_boundary_contribution", C.c_int32),
        ("ignore_source_contribution", C.c_int32),
        ("print_logs", C.c_int32),
    ]


class SamplePointsC(C.Structure):
    _fields_ = [
        ("n", C.c_int64),
        ("memory", C.c_int32),
        ("pt", C.c_void_p),
        ("normal", C.c_void_p),
        ("type", C.c_void_p),
        ("estimation_quantity", C.c_void_p),
        ("dist_to_absorbing", C.c_void_p),
        ("dist_to_reflecting", C.c_void_p),
        ("n_walks", C.c_void_p),
        ("seed", C.c_void_p),
        ("first_sphere_radius", C.c_void_p),
        ("estimate_normal_aligned", C.c_void_p),
        ("scene_id", C.c_void_p),
        ("direction_for_derivative", C.c_void_p),
    ]


class SampleStatisticsC(C.Structure):
    _fields_ = [
        ("memory", C.c_int32),
        ("solution_mean", C.c_void_p),
        ("solution_m2", C.c_void_p),
        ("n_solution_estimates", C.c_void_p),
        ("total_walk_length", C.c_void_p),
        ("total_splits", C.c_void_p),
        ("gradient_mean", C.c_void_p),
        ("gradient_m2", C.c_void_p),
        ("n_gradient_estimates", C.c_void_p),
        ("total_first_source_contribution", C.c_void_p),
        ("total_derivative_contribution", C.c_void_p),
    ]


class SolveOptions(C.Structure):
    _fields_ = [
        ("block_size", C.c_int32),
        ("blocks_per_sm", C.c_int32),
        ("use_graph", C.c_int32),
        ("query_mode", C.c_int32),
        ("step_budget", C.c_int64),
        ("bvh_width", C.c_int32),
        ("schedule", C.c_int32),
    ]


class SolveReport(C.Structure):
    _fields_ = [
        ("total_steps", C.c_uint64),
        ("total_walks", C.c_uint64),
        ("escaped_walks", C.c_uint64),
        ("exceeded_walks", C.c_uint64),
        ("rr_terminated", C.c_uint64),
        ("kernel_ms", C.c_float),
        ("total_ms", C.c_float),
        ("error_word", C.c_uint32),
        ("cache_terminated", C.c_uint64),
    ]


class GeometricQueriesC(C.Structure):
    _fields_ = [
        ("dim", C.c_int32),
        ("domain_is_watertight", C.c_int32),
        ("domain_min", C.c_float * 3),
        ("domain_max", C.c_float * 3),
        ("absorbing", C.c_void_p),
        ("reflecting", C.c_void_p),
    ]


def ptr(a):
    """Address of a numpy array / torch tensor (or None -> NULL)."""
    if a is None:
        return None
    if hasattr(a, "data_ptr"):
        return a.data_ptr()
    return a.ctypes.data


class CacheConfig(C.Structure):
    _fields_ = [
        ("dim", C.c_int32),
        ("n_levels", C.c_int32),
        ("log2_table_size", C.c_int32),
        ("base_resolution", C.c_float),
        ("max_resolution", C.c_float),
        ("domain_min", C.c_float * 3),
        ("domain_max", C.c_float * 3),
        ("learning_rate_grid", C.c_float),
        ("learning_rate_mlp", C.c_float),
        ("beta1", C.c_float),
        ("beta2", C.c_float),
        ("epsilon", C.c_float),
        ("seed", C.c_uint64),
    ]


ZGPU_BVC_ABSORBING, ZGPU_BVC_ABSORBING_ALIGNED, ZGPU_BVC_REFLECTING, ZGPU_BVC_REFLECTING_ALIGNED, ZGPU_BVC_SOURCE = range(5)
ZGPU_BVC_GROUPS = 5


class BvcSamplesC(C.Structure):
    _fields_ = [
        ("n", C.c_int64),
        ("pt", C.c_void_p),
        ("normal", C.c_void_p),
        ("pdf", C.c_void_p),
        ("type", C.c_void_p),
        ("estimate_normal_aligned", C.c_void_p),
        ("solution", C.c_void_p),
        ("normal_derivative", C.c_void_p),
        ("contribution", C.c_void_p),
        ("robin_coeff", C.c_void_p),
    ]


class BvcEvalPointsC(C.Structure):
    _fields_ = [
        ("n", C.c_int64),
        ("pt", C.c_void_p),
        ("type", C.c_void_p),
        ("dist_to_absorbing", C.c_void_p),
        ("dist_to_reflecting", C.c_void_p),
        ("mean", C.c_void_p),
        ("m2", C.c_void_p),
        ("count", C.c_void_p),
        ("gradient_mean", C.c_void_p),
        ("gradient_m2", C.c_void_p),
    ]


ZGPU_RWS_ABSORBING, ZGPU_RWS_ABSORBING_ALIGNED, ZGPU_RWS_REFLECTING, ZGPU_RWS_REFLECTING_ALIGNED, ZGPU_RWS_SOURCE, \
    ZGPU_RWS_POISSON_KERNEL = range(6)
ZGPU_RWS_TOTALS = 6


class RwsSamplesC(C.Structure):
    _fields_ = [
        ("n", C.c_int64),
        ("pt", C.c_void_p),
        ("normal", C.c_void_p),
        ("type", C.c_void_p),
        ("estimate_normal_aligned", C.c_void_p),
        ("pdf", C.c_void_p),
        ("contribution", C.c_void_p),
        ("dist_to_absorbing", C.c_void_p),
        ("seed", C.c_void_p),
    ]


class RwsEvalPointsC(C.Structure):
    _fields_ = [
        ("n", C.c_int64),
        ("pt", C.c_void_p),
        ("normal", C.c_void_p),
        ("type", C.c_void_p),
        ("totals", C.c_void_p),
    ]
