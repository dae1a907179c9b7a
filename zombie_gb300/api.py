"""Python mirror of rohan-sawhney/zombie's Python API (python/zombie/__init__.py and the
nanobind module of python/zombie_bindings.h) for the walk hot path, backed by the GB300
C ABI (include/zgpu.h).

Names, argument meanings and defaults follow the reference: Core.PDE / GeometricQueries,
Solvers.WalkSettings / SamplePoint / SampleStatistics / WalkOnSpheres / WalkOnStars,
Utils.*BoundaryHandler / populate_geometric_queries_for_*_boundary, all with the same
`dim=` / `channels=` factory keywords.  Documented deviations:
  * PDE fields are device-evaluable descriptors (constant or closed-form analytic) instead
    of C++ std::functions;
  * walk_state_callback / terminal_contribution_callback (host callbacks per step) are
    rejected with ZGPU_ERR_UNSUPPORTED_CALLBACK;
  * walk w of a point draws from pcg32(seed, w + previous estimate count).
"""
import ctypes as C
import atexit
import enum
import weakref

import numpy as np

from . import _abi as A
from ._lib import ZgpuError, check, lib

_VALID_DIMS = {2, 3}
_VALID_CHANNELS = {1}


def _validate(dim, channels=1):
    if dim not in _VALID_DIMS:
        raise ValueError(f"dim must be one of {sorted(_VALID_DIMS)}, got {dim}")
    if channels not in _VALID_CHANNELS:
        raise ValueError(f"channels must be 1 in this build, got {channels}")


# --------------------------------------------------------------------------- context
class Context:
    """One CUDA stream plus cached device scratch on one GPU."""

    def __init__(self, device=0):
        h = C.c_void_p()
        check(lib().zgpu_context_create(device, C.byref(h)))
        self.h = h
        self.device = device

    def synchronize(self):
        check(lib().zgpu_context_synchronize(self.h))

    @property
    def stream(self):
        return lib().zgpu_context_stream(self.h)

    def close(self):
        if getattr(self, "h", None):
            lib().zgpu_context_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


_default_ctx = None
_live_caches = weakref.WeakSet()


def default_context():
    global _default_ctx
    if _default_ctx is None:
        _default_ctx = Context(0)
    return _default_ctx


@atexit.register
def _shutdown():
    """Release caches before the contexts whose streams they run on, while the CUDA runtime
    is still up (interpreter teardown would finalise them in arbitrary order)."""
    global _default_ctx
    for c in list(_live_caches):
        c.close()
    if _default_ctx is not None:
        _default_ctx.close()
        _default_ctx = None


# ----------------------------------------------------------------------------- enums
class SampleType(enum.IntEnum):
    InDomain = A.ZGPU_SAMPLE_IN_DOMAIN
    OnAbsorbingBoundary = A.ZGPU_SAMPLE_ON_ABSORBING_BOUNDARY
    OnReflectingBoundary = A.ZGPU_SAMPLE_ON_REFLECTING_BOUNDARY


class EstimationQuantity(enum.IntEnum):
    Solution = A.ZGPU_ESTIMATE_SOLUTION
    SolutionAndGradient = A.ZGPU_ESTIMATE_SOLUTION_AND_GRADIENT
    Skip = A.ZGPU_ESTIMATE_SKIP


class WalkCompletionCode(enum.IntEnum):
    ReachedAbsorbingBoundary = 0
    TerminatedWithRussianRoulette = 1
    ExceededMaxWalkLength = 2
    EscapedDomain = 3


# ----------------------------------------------------------------------- PDE fields
class DenseGrid:
    """DenseGrid<float, 1, DIM> (utils/dense_grid.h:29-72): cell-centred samples over the box
    [grid_min, grid_max], row-major with the last axis fastest.  The walk kernels read the
    values on the device; __call__ is the same lookup on the host for inspection.

    DenseGrid(grid_min, grid_max, enable_interpolation=False) or
    DenseGrid(grid_data, grid_shape, grid_min, grid_max, enable_interpolation=False)."""

    def __init__(self, *args, enable_interpolation=False, dim=None):
        if len(args) in (2, 3):
            grid_min, grid_max = args[0], args[1]
            data, shape = None, None
            if len(args) == 3:
                enable_interpolation = args[2]
        elif len(args) in (4, 5):
            data, shape, grid_min, grid_max = args[:4]
            if len(args) == 5:
                enable_interpolation = args[4]
        else:
            raise TypeError("DenseGrid(grid_min, grid_max[, interp]) or DenseGrid(data, shape, grid_min, grid_max[, interp])")
        self.origin = np.asarray(grid_min, np.float32).ravel()
        self.extent = (np.asarray(grid_max, np.float32).ravel() - self.origin).astype(np.float32)
        self.dim = int(self.origin.size if dim is None else dim)
        if self.dim not in (2, 3) or self.extent.size != self.dim:
            raise ValueError("grid_min / grid_max must have 2 or 3 entries")
        self.interpolation_enabled = bool(enable_interpolation)
        self.data = np.zeros(0, np.float32)
        self.shape = np.zeros(self.dim, np.int32)
        if data is not None:
            self.set(data, shape)

    def set(self, grid_data, grid_shape=None):
        """set(grid_data, grid_shape), or set(callback, grid_shape) with callback(x) -> value
        evaluated at every cell centre (dense_grid.h:157-190)."""
        shape = np.asarray(grid_shape, np.int64).ravel()
        if shape.size != self.dim or np.any(shape < 1):
            raise ValueError("grid_shape must hold dim positive entries")
        if callable(grid_data):
            centres = self.get(np.arange(int(np.prod(shape))), shape)
            grid_data = np.array([grid_data(c) for c in centres], np.float32)
        data = np.ascontiguousarray(np.asarray(grid_data, np.float32).ravel())
        if data.size != int(np.prod(shape)):
            raise ValueError(f"grid data has {data.size} values, the shape holds {int(np.prod(shape))}")
        self.data = data
        self.shape = shape.astype(np.int32)

    def get(self, index, shape=None):
        """Cell centre(s) of flat index(es) (dense_grid.h:224-240)."""
        shape = self.shape if shape is None else np.asarray(shape)
        idx = np.asarray(index, np.int64)
        out = np.zeros(idx.shape + (self.dim,), np.float32)
        rem = idx.copy()
        for i in range(self.dim - 1, -1, -1):
            out[..., i] = self.origin[i] + (rem % shape[i] + 0.5) * (self.extent[i] / shape[i])
            rem //= shape[i]
        return out

    def __call__(self, x):
        x = np.asarray(x, np.float32)
        one = x.ndim == 1
        x = x.reshape(-1, self.dim)
        t = (x - self.origin) / self.extent
        n = self.shape.astype(np.int64)
        if not self.interpolation_enabled:
            idx = np.clip(np.floor(t * n).astype(np.int64), 0, n - 1)
            flat = np.zeros(len(x), np.int64)
            for i in range(self.dim):
                flat = flat * n[i] + idx[:, i]
            r = self.data[flat]
        else:
            u = np.where(n == 1, 0.0, t * n - 0.5).astype(np.float32)
            i0 = np.clip(np.floor(u).astype(np.int64), 0, n - 1)
            i1 = np.clip(i0 + 1, 0, n - 1)
            f = np.clip(u - i0, 0.0, 1.0)
            r = np.zeros(len(x), np.float32)
            for corner in range(1 << self.dim):
                flat = np.zeros(len(x), np.int64)
                w = np.ones(len(x), np.float32)
                for i in range(self.dim):
                    hi = (corner >> i) & 1
                    flat = flat * n[i] + (i1[:, i] if hi else i0[:, i])
                    w = w * (f[:, i] if hi else 1.0 - f[:, i])
                r = r + w * self.data[flat]
        return float(r[0]) if one else r

    def min(self):
        return float(self.data.min())

    def max(self):
        return float(self.data.max())

    def to_c(self, aligned=None):
        g = A.Grid()
        g.values = A.ptr(self.data)
        g.values_aligned = A.ptr(aligned.data) if aligned is not None else None
        for i in range(self.dim):
            g.shape[i] = int(self.shape[i])
            g.grid_min[i] = float(self.origin[i])
            g.grid_max[i] = float(self.origin[i] + self.extent[i])
        g.enable_interpolation = int(self.interpolation_enabled)
        return g


class Field:
    """Device-evaluable replacement for one PDE std::function member."""

    def __init__(self, kind, value=0.0, value_aligned=None, grid=None, grid_aligned=None, raw_grid=None):
        self.kind = kind
        self.value = float(value)
        self.value_aligned = float(value if value_aligned is None else value_aligned)
        self.grid = grid                  # DenseGrid (kind GRID)
        self.grid_aligned = grid_aligned  # DenseGrid for returnBoundaryNormalAlignedValue = true
        self.raw_grid = raw_grid          # a zgpu_grid given directly (its arrays owned by the caller)

    @staticmethod
    def dense_grid(grid, grid_aligned=None):
        """A DenseGrid field (getDenseGridCallback0-4, utils/dense_grid.h:374-560)."""
        if grid_aligned is not None and (grid_aligned.data.size != grid.data.size or
                                         np.any(grid_aligned.shape != grid.shape)):
            raise ValueError("the normal-aligned grid must have the grid's shape")
        return Field(A.ZGPU_FIELD_GRID, grid=grid, grid_aligned=grid_aligned)

    def grid_to_c(self):
        if self.raw_grid is not None:
            return self.raw_grid
        if self.grid is None:
            return A.Grid()
        return self.grid.to_c(self.grid_aligned)

    @staticmethod
    def zero():
        return Field(A.ZGPU_FIELD_ZERO)

    @staticmethod
    def constant(value, value_aligned=None):
        return Field(A.ZGPU_FIELD_CONSTANT, value, value_aligned)

    @staticmethod
    def analytic():
        """Derived from PDE.solution: g = u, h = du/dn + kappa u, f = -Lap u + sigma u."""
        return Field(A.ZGPU_FIELD_ANALYTIC)


def _dense_grid_field(args, kw, aligned):
    """The get_dense_grid_*_callback overloads (python/zombie_bindings.h:852-1125): a DenseGrid
    (plus its normal-aligned twin), or raw data (plus aligned data), shape, min, max and the
    interpolation flag."""
    interp = kw.pop("enable_interpolation", False)
    kw.pop("dim", None)
    kw.pop("channels", None)
    if args and isinstance(args[0], DenseGrid):
        g = args[0]
        ga = args[1] if len(args) > 1 else kw.pop("grid_boundary_normal_aligned", None)
        if ga is not None and not aligned:
            raise TypeError("this field has no normal-aligned variant")
        return Field.dense_grid(g, ga)
    args = list(args)
    data = args.pop(0) if args else kw.pop("grid_data")
    da = None
    if aligned and (len(args) >= 4 and not isinstance(args[3], (bool, np.bool_)) or
                    "grid_data_boundary_normal_aligned" in kw):
        da = args.pop(0) if "grid_data_boundary_normal_aligned" not in kw else kw.pop("grid_data_boundary_normal_aligned")
    shape = args.pop(0) if args else kw.pop("grid_shape")
    gmin = args.pop(0) if args else kw.pop("grid_min")
    gmax = args.pop(0) if args else kw.pop("grid_max")
    if args:
        interp = args.pop(0)
    g = DenseGrid(data, shape, gmin, gmax, bool(interp))
    ga = DenseGrid(da, shape, gmin, gmax, bool(interp)) if da is not None else None
    return Field.dense_grid(g, ga)


def get_dense_grid_source_callback(*args, **kw):
    return _dense_grid_field(args, kw, aligned=False)


def get_dense_grid_dirichlet_callback(*args, **kw):
    return _dense_grid_field(args, kw, aligned=True)


def get_dense_grid_robin_callback(*args, **kw):
    return _dense_grid_field(args, kw, aligned=True)


def get_dense_grid_robin_coefficient_callback(*args, **kw):
    return _dense_grid_field(args, kw, aligned=True)


class _Indicator:
    """A host-side boolean field of points (the reference's FloatNToTypeFunc<bool, DIM>):
    called with one point it returns a bool, with an [N, dim] array a bool array.  Used
    where the reference takes an indicator on the host, e.g. PDE.has_reflecting_boundary_conditions
    or the on_reflecting_boundary argument of partition_boundary_mesh."""

    def __init__(self, fn):
        self._fn = fn

    def __call__(self, x):
        x = np.asarray(x, np.float32)
        if x.ndim == 1:
            return bool(self._fn(x[None])[0])
        return np.asarray(self._fn(x), bool)


def get_constant_indicator_callback(value, dim=None):
    """get_constant_indicator_callback (python/zombie_bindings.h:843-849)."""
    v = bool(value)
    return _Indicator(lambda x: np.full(x.shape[0], v, bool))


def get_dense_grid_indicator_callback(*args, **kw):
    """get_dense_grid_indicator_callback (python/zombie_bindings.h:852-862): nearest-cell lookup
    of a boolean DenseGrid, or of raw boolean data with its shape, min and max."""
    kw.pop("dim", None)
    if args and isinstance(args[0], DenseGrid):
        g = args[0]
    else:
        args = list(args)
        data = args.pop(0) if args else kw.pop("grid_data")
        shape = args.pop(0) if args else kw.pop("grid_shape")
        gmin = args.pop(0) if args else kw.pop("grid_min")
        gmax = args.pop(0) if args else kw.pop("grid_max")
        g = DenseGrid(np.asarray(data, bool).astype(np.float32), shape, gmin, gmax, False)
    return _Indicator(lambda x: np.asarray(g(x)) > 0.5)


def bool_dense_grid(*args, dim=None, **kw):
    """DenseGrid<bool, 1, DIM> (utils/dense_grid.h): a DenseGrid holding 0 / 1, looked up by
    nearest cell (no interpolation)."""
    if len(args) >= 4:
        args = (np.asarray(args[0], bool).astype(np.float32),) + tuple(args[1:4])
    kw.pop("enable_interpolation", None)
    return DenseGrid(*args[:4] if len(args) >= 4 else args[:2], enable_interpolation=False, dim=dim)


class IntersectionPoint:
    """IntersectionPoint<DIM> (core/geometric_queries.h:29-41): a boundary point, its normal
    and its distance along the query (FLT_MAX when nothing was hit)."""

    def __init__(self, pt=None, normal=None, dist=None, dim=2):
        self.pt = np.zeros(dim, np.float32) if pt is None else np.asarray(pt, np.float32)
        self.normal = np.zeros(dim, np.float32) if normal is None else np.asarray(normal, np.float32)
        self.dist = float(np.finfo(np.float32).max if dist is None else dist)

    def __repr__(self):
        return f"IntersectionPoint(pt={self.pt.tolist()}, normal={self.normal.tolist()}, dist={self.dist})"


class PDE:
    """PDE<T,DIM> (core/pde.h:19-45)."""

    def __init__(self, dim=2, channels=1):
        _validate(dim, channels)
        self.dim = dim
        self.absorption_coeff = 0.0
        self.is_source_constant = False
        self.are_robin_conditions_pure_neumann = True
        self.are_robin_coeffs_nonnegative = True
        self.solution = A.Analytic()
        self.source = Field.zero()
        self.dirichlet = Field.zero()
        self.robin = Field.zero()
        self.robin_coeff = Field.zero()
        self.grid_memory = A.ZGPU_MEM_HOST   # where raw zgpu_grid values live (DenseGrid data is host)
        # host-side indicator of points with reflecting conditions (PDE::hasReflectingBoundaryConditions,
        # core/pde.h:44); the walks take the reflecting boundary from the geometric queries
        self.has_reflecting_boundary_conditions = None

    def has_non_zero_robin_coeff(self, x=None):
        """PDE::hasNonZeroRobinCoeff (core/pde.h:62-78) at x (grids need x)."""
        if self.are_robin_conditions_pure_neumann:
            return False
        rc = self.robin_coeff
        if rc.kind == A.ZGPU_FIELD_GRID and rc.grid is not None and x is not None:
            g = rc.grid_aligned or rc.grid
            return abs(rc.grid(x)) > 0 or abs(g(x)) > 0
        if rc.kind == A.ZGPU_FIELD_GRID:
            return True
        return rc.kind != A.ZGPU_FIELD_ZERO and (rc.value != 0 or rc.value_aligned != 0)

    def to_c(self):
        p = A.Pde()
        p.absorption_coeff = self.absorption_coeff
        p.is_source_constant = int(self.is_source_constant)
        p.are_robin_conditions_pure_neumann = int(self.are_robin_conditions_pure_neumann)
        p.are_robin_coeffs_nonnegative = int(self.are_robin_coeffs_nonnegative)
        p.solution = self.solution
        p.source_kind, p.source_value = self.source.kind, self.source.value
        p.dirichlet_kind, p.dirichlet_value, p.dirichlet_value_aligned = \
            self.dirichlet.kind, self.dirichlet.value, self.dirichlet.value_aligned
        p.robin_kind, p.robin_value, p.robin_value_aligned = self.robin.kind, self.robin.value, self.robin.value_aligned
        p.robin_coeff_kind, p.robin_coeff_value, p.robin_coeff_value_aligned = \
            self.robin_coeff.kind, self.robin_coeff.value, self.robin_coeff.value_aligned
        p.source_grid = self.source.grid_to_c()
        p.dirichlet_grid = self.dirichlet.grid_to_c()
        p.robin_grid = self.robin.grid_to_c()
        p.robin_coeff_grid = self.robin_coeff.grid_to_c()
        p.memory = self.grid_memory
        return p

    @staticmethod
    def from_c(dim, p):
        pde = PDE(dim)
        pde.absorption_coeff = p.absorption_coeff
        pde.is_source_constant = bool(p.is_source_constant)
        pde.are_robin_conditions_pure_neumann = bool(p.are_robin_conditions_pure_neumann)
        pde.are_robin_coeffs_nonnegative = bool(p.are_robin_coeffs_nonnegative)
        pde.solution = p.solution
        def raw(kind, g):
            return g if kind == A.ZGPU_FIELD_GRID else None
        pde.source = Field(p.source_kind, p.source_value, raw_grid=raw(p.source_kind, p.source_grid))
        pde.dirichlet = Field(p.dirichlet_kind, p.dirichlet_value, p.dirichlet_value_aligned,
                              raw_grid=raw(p.dirichlet_kind, p.dirichlet_grid))
        pde.robin = Field(p.robin_kind, p.robin_value, p.robin_value_aligned, raw_grid=raw(p.robin_kind, p.robin_grid))
        pde.robin_coeff = Field(p.robin_coeff_kind, p.robin_coeff_value, p.robin_coeff_value_aligned,
                                raw_grid=raw(p.robin_coeff_kind, p.robin_coeff_grid))
        pde.grid_memory = p.memory
        return pde


def pde_evaluate(pde, x, normals=None, aligned=None, dim=None, context=None):
    """The PDE's fields at points x as the walk kernels read them (zgpu_pde_evaluate):
    returns (source, dirichlet, robin, robin_coeff) as float32 arrays."""
    ctx = context or default_context()
    p = pde.to_c() if isinstance(pde, PDE) else pde
    dim = dim or (pde.dim if isinstance(pde, PDE) else None)
    x = np.ascontiguousarray(x, np.float32)
    dim = dim or x.shape[-1]
    x = x.reshape(-1, dim)
    n = x.shape[0]
    nrm = None if normals is None else np.ascontiguousarray(normals, np.float32).reshape(-1, dim)
    al = None if aligned is None else np.ascontiguousarray(np.broadcast_to(np.asarray(aligned, np.int32), (n,)))
    out = [np.zeros(n, np.float32) for _ in range(4)]
    check(lib().zgpu_pde_evaluate(ctx.h, dim, C.byref(p), n, A.ptr(x), A.ptr(nrm), A.ptr(al), A.ZGPU_MEM_HOST,
                                  *[A.ptr(o) for o in out]))
    return tuple(out)


# ---------------------------------------------------------------------- settings
class WalkSettings:
    """WalkSettings (point_estimation/common.h:19-91): both constructors, same defaults."""

    _FIELDS = ["epsilon_shell_for_absorbing_boundary", "epsilon_shell_for_reflecting_boundary",
               "silhouette_precision", "russian_roulette_threshold", "splitting_threshold", "max_walk_length",
               "steps_before_applying_tikhonov", "steps_before_using_maximal_spheres", "solve_double_sided",
               "use_gradient_control_variates", "use_gradient_antithetic_variates",
               "use_cosine_sampling_for_derivatives", "ignore_absorbing_boundary_contribution",
               "ignore_reflecting_boundary_contribution", "ignore_source_contribution", "print_logs"]

    def __init__(self, *args, **kw):
        vals = dict(zip(self._FIELDS if len(args) + len(kw) > 4 else
                        ["epsilon_shell_for_absorbing_boundary", "epsilon_shell_for_reflecting_boundary",
                         "max_walk_length", "solve_double_sided"], args))
        vals.update(kw)
        if len(vals) <= 4:
            mwl = int(vals["max_walk_length"])
            full = dict(silhouette_precision=1e-3, russian_roulette_threshold=0.0, splitting_threshold=A.FLT_MAX,
                        steps_before_applying_tikhonov=0, steps_before_using_maximal_spheres=mwl,
                        use_gradient_control_variates=True, use_gradient_antithetic_variates=True,
                        use_cosine_sampling_for_derivatives=False, ignore_absorbing_boundary_contribution=False,
                        ignore_reflecting_boundary_contribution=False, ignore_source_contribution=False,
                        print_logs=False)
            full.update(vals)
            vals = full
        missing = [f for f in self._FIELDS if f not in vals]
        if missing:
            raise TypeError(f"WalkSettings missing arguments: {missing}")
        for f in self._FIELDS:
            setattr(self, f, vals[f])

    def to_c(self):
        s = A.WalkSettingsC()
        for f in self._FIELDS:
            v = getattr(self, f)
            setattr(s, f, float(v) if isinstance(getattr(s, f), float) else int(v))
        return s


# ------------------------------------------------------------------ sample points
class SamplePoint:
    """SamplePoint (point_estimation/common.h:151-195); `seed` replaces the pcg32 member."""

    _counter = 0

    def __init__(self, pt, normal, type, estimation_quantity, pdf, dist_to_absorbing_boundary,
                 dist_to_reflecting_boundary, seed=None):
        self.pt = np.asarray(pt, np.float32)
        self.normal = np.asarray(normal, np.float32)
        self.type = SampleType(type)
        self.estimation_quantity = EstimationQuantity(estimation_quantity)
        self.pdf = float(pdf)
        self.dist_to_absorbing_boundary = float(dist_to_absorbing_boundary)
        self.dist_to_reflecting_boundary = float(dist_to_reflecting_boundary)
        self.direction_for_derivative = np.zeros_like(self.pt)
        self.direction_for_derivative[0] = 1.0
        self.estimate_boundary_normal_aligned = False
        if seed is None:
            SamplePoint._counter += 1
            seed = int(np.random.SeedSequence().entropy & 0xFFFFFFFFFFFFFFFF) ^ SamplePoint._counter
        self.seed = int(seed) & 0xFFFFFFFFFFFFFFFF
        self.reset()

    def reset(self):
        self.first_sphere_radius = 0.0
        self.robin_coeff = 0.0
        self.solution = 0.0
        self.normal_derivative = 0.0
        self.contribution = 0.0


class SampleStatistics:
    """SampleStatistics (point_estimation/common.h:200-395) with FP64 moments."""

    def __init__(self):
        self.reset()

    def reset(self):
        self.solution_mean = 0.0
        self.solution_m2 = 0.0
        self.n_solution_estimates = 0
        self.total_walk_length = 0
        self.total_splits = 0
        self.gradient_mean = None        # per-dimension lists once gradients are estimated
        self.gradient_m2 = None
        self.n_gradient_estimates = 0
        self.total_first_source_contribution = 0.0
        self.total_derivative_contribution = 0.0

    def get_estimated_solution(self):
        return self.solution_mean

    def get_estimated_gradient(self):
        return list(self.gradient_mean) if self.gradient_mean is not None else []

    def get_estimated_gradient_variance(self):
        if self.gradient_m2 is None:
            return []
        return [m / max(1, self.n_gradient_estimates - 1) for m in self.gradient_m2]

    def get_gradient_estimate_count(self):
        return self.n_gradient_estimates

    def get_mean_first_source_contribution(self):
        return self.total_first_source_contribution / max(1, self.n_solution_estimates)

    def get_estimated_derivative(self):
        return self.total_derivative_contribution / max(1, self.n_solution_estimates)

    def get_estimated_solution_variance(self):
        return self.solution_m2 / max(1, self.n_solution_estimates - 1)

    def get_solution_estimate_count(self):
        return self.n_solution_estimates

    def get_mean_walk_length(self):
        return self.total_walk_length / max(1, self.n_solution_estimates)

    def get_mean_splits(self):
        return self.total_splits / max(1, self.n_solution_estimates)


def create_sample_statistics_list(size):
    return [SampleStatistics() for _ in range(size)]


class SampleArrays:
    """Structure-of-arrays points + statistics for the fast path (numpy host arrays or
    torch CUDA tensors).  Field names follow zgpu_sample_points / zgpu_sample_statistics."""

    POINT_FIELDS = ("pt", "normal", "type", "estimation_quantity", "dist_to_absorbing", "dist_to_reflecting",
                    "n_walks", "seed", "first_sphere_radius", "estimate_normal_aligned", "scene_id",
                    "direction_for_derivative")
    STAT_FIELDS = ("solution_mean", "solution_m2", "n_solution_estimates", "total_walk_length", "total_splits",
                   "gradient_mean", "gradient_m2", "n_gradient_estimates", "total_first_source_contribution",
                   "total_derivative_contribution")

    def __init__(self, **arrays):
        self.arrays = arrays
        self.n = int(arrays["pt"].shape[0])
        first = arrays["pt"]
        self.memory = A.ZGPU_MEM_DEVICE if hasattr(first, "is_cuda") and first.is_cuda else A.ZGPU_MEM_HOST

    @staticmethod
    def host(points, dist, n_walks, seeds, normals=None, types=None, first_sphere_radius=True, gradients=False):
        n = points.shape[0]
        arr = dict(pt=np.ascontiguousarray(points, np.float32),
                   dist_to_absorbing=np.ascontiguousarray(dist, np.float32),
                   n_walks=np.ascontiguousarray(n_walks, np.int32),
                   seed=np.ascontiguousarray(seeds, np.uint64),
                   solution_mean=np.zeros(n), solution_m2=np.zeros(n),
                   n_solution_estimates=np.zeros(n, np.int32), total_walk_length=np.zeros(n, np.int64),
                   total_splits=np.zeros(n, np.int64))
        if gradients:
            d = points.shape[1]
            arr["estimation_quantity"] = np.full(n, int(EstimationQuantity.SolutionAndGradient), np.int32)
            arr["gradient_mean"] = np.zeros((n, d))
            arr["gradient_m2"] = np.zeros((n, d))
            arr["n_gradient_estimates"] = np.zeros(n, np.int32)
            arr["total_first_source_contribution"] = np.zeros(n)
            arr["total_derivative_contribution"] = np.zeros(n)
        if first_sphere_radius:
            arr["first_sphere_radius"] = np.zeros(n, np.float32)
        if normals is not None:
            arr["normal"] = np.ascontiguousarray(normals, np.float32)
        if types is not None:
            arr["type"] = np.ascontiguousarray(types, np.int32)
        return SampleArrays(**arr)

    def to_c(self):
        sp = A.SamplePointsC()
        sp.n = self.n
        sp.memory = self.memory
        for f in self.POINT_FIELDS:
            setattr(sp, f, A.ptr(self.arrays.get(f)))
        st = A.SampleStatisticsC()
        st.memory = self.memory
        for f in self.STAT_FIELDS:
            setattr(st, f, A.ptr(self.arrays.get(f)))
        return sp, st

    def __getitem__(self, k):
        return self.arrays[k]


# ----------------------------------------------------------------- boundaries / queries
class _BoundaryHandler:
    kind = A.ZGPU_BOUNDARY_ABSORBING

    def __init__(self, dim=2, context=None):
        _validate(dim)
        self.dim = dim
        self.ctx = context or default_context()
        self.h = None
        self.n_prims = 0

    def _build(self, positions, indices, kmin=None, kmax=None, solve_double_sided=False,
               silhouette_precision=1e-3, bvh_width=4, build_on_device=False):
        """Builds on the host (binned SAH), or with build_on_device on the GPU
        (zgpu_boundary_create_on_device: linear BVH, cones and silhouette trees built there);
        the arrays may then be CUDA tensors."""
        dev = build_on_device and hasattr(positions, "is_cuda") and positions.is_cuda
        if dev:
            import torch
            pos = positions.contiguous().to(torch.float32).reshape(-1, self.dim)
            idx = indices.contiguous().to(torch.int32).reshape(-1, self.dim)
            kmn = None if kmin is None else torch.as_tensor(kmin, dtype=torch.float32, device=pos.device).contiguous()
            kmx = None if kmax is None else torch.as_tensor(kmax, dtype=torch.float32, device=pos.device).contiguous()
        else:
            pos = np.ascontiguousarray(positions, np.float32).reshape(-1, self.dim)
            idx = np.ascontiguousarray(indices, np.int32).reshape(-1, self.dim)
            kmn = None if kmin is None else np.ascontiguousarray(kmin, np.float32)
            kmx = None if kmax is None else np.ascontiguousarray(kmax, np.float32)
        self.close()
        h = C.c_void_p()
        if build_on_device:
            check(lib().zgpu_boundary_create_on_device(self.ctx.h, self.dim, A.ptr(pos), int(pos.shape[0]), A.ptr(idx),
                                                       int(idx.shape[0]), self.kind, A.ptr(kmn), A.ptr(kmx),
                                                       int(solve_double_sided), float(silhouette_precision),
                                                       A.ZGPU_MEM_DEVICE if dev else A.ZGPU_MEM_HOST, C.byref(h)))
        else:
            check(lib().zgpu_boundary_create(self.ctx.h, self.dim, A.ptr(pos), pos.shape[0], A.ptr(idx), idx.shape[0],
                                             self.kind, A.ptr(kmn), A.ptr(kmx), int(solve_double_sided),
                                             float(silhouette_precision), int(bvh_width), C.byref(h)))
        self.h = h
        self.n_prims = int(idx.shape[0])
        self.positions, self.indices = pos, idx

    def info(self):
        n, d, nb, pb = C.c_int64(), C.c_int32(), C.c_int64(), C.c_int64()
        check(lib().zgpu_boundary_info(self.h, C.byref(n), C.byref(d), C.byref(nb), C.byref(pb)))
        return dict(n_nodes=n.value, depth=d.value, node_bytes=nb.value, prim_bytes=pb.value)

    def signed_volume(self):
        v = C.c_float()
        check(lib().zgpu_boundary_signed_volume(self.h, C.byref(v)))
        return v.value

    def close(self):
        if getattr(self, "h", None):
            lib().zgpu_boundary_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_query_mode(self, mode):
        """ZGPU_QUERY_MODE_LANE (one GPU lane per query, the default) or ZGPU_QUERY_MODE_WARP
        (a warp per closest-point query and per Robin star-radius query) for the batched
        queries below."""
        check(lib().zgpu_boundary_set_query_mode(self.h, int(mode)))

    # batched geometric queries on host arrays (device tensors: pass memory=1 arrays)
    def closest_point(self, x, compute_signed=False):
        x = np.ascontiguousarray(x, np.float32).reshape(-1, self.dim)
        n = x.shape[0]
        pt = np.zeros_like(x); nrm = np.zeros_like(x)
        d = np.zeros(n, np.float32); prim = np.zeros(n, np.int32)
        check(lib().zgpu_query_closest_point(self.h, n, A.ptr(x), int(compute_signed), A.ptr(pt), A.ptr(nrm),
                                             A.ptr(d), A.ptr(prim), A.ZGPU_MEM_HOST))
        return pt, nrm, d, prim

    def intersect(self, origin, normal, direction, t_max, on_boundary):
        o = np.ascontiguousarray(origin, np.float32).reshape(-1, self.dim)
        nn = np.ascontiguousarray(normal, np.float32).reshape(-1, self.dim)
        dr = np.ascontiguousarray(direction, np.float32).reshape(-1, self.dim)
        tm = np.ascontiguousarray(t_max, np.float32)
        ob = np.ascontiguousarray(on_boundary, np.int32)
        n = o.shape[0]
        hit = np.zeros(n, np.int32); pt = np.zeros_like(o); nrm = np.zeros_like(o)
        dist = np.zeros(n, np.float32); prim = np.zeros(n, np.int32)
        check(lib().zgpu_query_intersect(self.h, n, A.ptr(o), A.ptr(nn), A.ptr(dr), A.ptr(tm), A.ptr(ob),
                                         A.ptr(hit), A.ptr(pt), A.ptr(nrm), A.ptr(dist), A.ptr(prim),
                                         A.ZGPU_MEM_HOST))
        return hit, pt, nrm, dist, prim

    def count_hits(self, origin, direction, t_max):
        o = np.ascontiguousarray(origin, np.float32).reshape(-1, self.dim)
        dr = np.ascontiguousarray(direction, np.float32).reshape(-1, self.dim)
        tm = np.ascontiguousarray(t_max, np.float32)
        out = np.zeros(o.shape[0], np.int32)
        check(lib().zgpu_query_count_hits(self.h, o.shape[0], A.ptr(o), A.ptr(dr), A.ptr(tm), A.ptr(out),
                                          A.ZGPU_MEM_HOST))
        return out

    def star_radius(self, x, min_r, max_r, precision, flip):
        x = np.ascontiguousarray(x, np.float32).reshape(-1, self.dim)
        out = np.zeros(x.shape[0], np.float32)
        mn = np.ascontiguousarray(min_r, np.float32); mx = np.ascontiguousarray(max_r, np.float32)
        fl = np.ascontiguousarray(flip, np.int32)
        check(lib().zgpu_query_star_radius(self.h, x.shape[0], A.ptr(x), A.ptr(mn), A.ptr(mx), float(precision),
                                           A.ptr(fl), A.ptr(out), A.ZGPU_MEM_HOST))
        return out

    def occluded(self, xi, xj, ni, nj, oi, oj):
        xi = np.ascontiguousarray(xi, np.float32).reshape(-1, self.dim)
        arrs = [np.ascontiguousarray(a, np.float32).reshape(-1, self.dim) for a in (xj, ni, nj)]
        o1 = np.ascontiguousarray(oi, np.int32); o2 = np.ascontiguousarray(oj, np.int32)
        out = np.zeros(xi.shape[0], np.int32)
        check(lib().zgpu_query_occluded(self.h, xi.shape[0], A.ptr(xi), A.ptr(arrs[0]), A.ptr(arrs[1]),
                                        A.ptr(arrs[2]), A.ptr(o1), A.ptr(o2), A.ptr(out), A.ZGPU_MEM_HOST))
        return out

    def sample(self, x, radius, u):
        x = np.ascontiguousarray(x, np.float32).reshape(-1, self.dim)
        r = np.ascontiguousarray(radius, np.float32)
        uu = np.ascontiguousarray(u, np.float32).reshape(-1, self.dim)
        n = x.shape[0]
        found = np.zeros(n, np.int32); pt = np.zeros_like(x); nrm = np.zeros_like(x); pdf = np.zeros(n, np.float32)
        check(lib().zgpu_query_sample_boundary(self.h, n, A.ptr(x), A.ptr(r), A.ptr(uu), A.ptr(found), A.ptr(pt),
                                               A.ptr(nrm), A.ptr(pdf), A.ZGPU_MEM_HOST))
        return found, pt, nrm, pdf


class IgnoreCandidateSilhouette:
    """getIgnoreCandidateSilhouetteCallback (utils/fcpw_geometric_queries.h:1029-1038): ignore
    features with dihedral angle < silhouette_precision unless solving double-sided."""

    def __init__(self, solve_double_sided=False, silhouette_precision=1e-3):
        self.solve_double_sided = bool(solve_double_sided)
        self.silhouette_precision = float(silhouette_precision)

    def __call__(self, dihedral_angle, index):
        return False if self.solve_double_sided else dihedral_angle < self.silhouette_precision


class BranchTraversalWeight:
    """getBranchTraversalWeightCallback (utils/fcpw_geometric_queries.h:1391-1398)."""

    def __init__(self, min_radial_distance=1e-2):
        self.min_radial_distance = float(min_radial_distance)

    def __call__(self, r2):
        r = max(np.sqrt(r2), self.min_radial_distance)
        return abs(1.0 / (4.0 * np.pi * r))


class GpuDirichletBoundaryHandler(_BoundaryHandler):
    """FcpwDirichletBoundaryHandler (utils/fcpw_geometric_queries.h:75-89)."""
    kind = A.ZGPU_BOUNDARY_ABSORBING

    def build_acceleration_structure(self, positions, indices, build_bvh=True, enable_bvh_vectorization=False,
                                     print_stats=False, build_on_device=False, bvh_width=4):
        """bvh_width = 8 builds 8-wide nodes (3D, host build) for closest-point and ray queries."""
        self._build(positions, indices, bvh_width=bvh_width, build_on_device=build_on_device)


class GpuNeumannBoundaryHandler(_BoundaryHandler):
    """FcpwNeumannBoundaryHandler (utils/fcpw_geometric_queries.h:91-106)."""
    kind = A.ZGPU_BOUNDARY_NEUMANN

    def build_acceleration_structure(self, positions, indices, ignore_candidate_silhouette=None, build_bvh=True,
                                     enable_bvh_vectorization=False, print_stats=False, build_on_device=False):
        ic = ignore_candidate_silhouette or IgnoreCandidateSilhouette()
        self._build(positions, indices, solve_double_sided=ic.solve_double_sided,
                    silhouette_precision=ic.silhouette_precision, build_on_device=build_on_device)


class GpuRobinBoundaryHandler(_BoundaryHandler):
    """FcpwRobinBoundaryHandler (utils/fcpw_geometric_queries.h:108-129)."""
    kind = A.ZGPU_BOUNDARY_ROBIN

    def build_acceleration_structure(self, positions, indices, ignore_candidate_silhouette=None,
                                     min_robin_coeff_values=None, max_robin_coeff_values=None, build_bvh=True,
                                     enable_bvh_vectorization=False, print_stats=False, build_on_device=False):
        ic = ignore_candidate_silhouette or IgnoreCandidateSilhouette()
        n = int(indices.shape[0]) if hasattr(indices, "is_cuda") else np.asarray(indices).reshape(-1, self.dim).shape[0]
        kmin = np.zeros(n, np.float32) if min_robin_coeff_values is None else min_robin_coeff_values
        kmax = np.zeros(n, np.float32) if max_robin_coeff_values is None else max_robin_coeff_values
        self._build(positions, indices, kmin, kmax, solve_double_sided=ic.solve_double_sided,
                    silhouette_precision=ic.silhouette_precision, build_on_device=build_on_device)

    def update_coefficient_values(self, min_robin_coeff_values, max_robin_coeff_values):
        kmin = np.ascontiguousarray(min_robin_coeff_values, np.float32)
        kmax = np.ascontiguousarray(max_robin_coeff_values, np.float32)
        check(lib().zgpu_boundary_update_robin_coefficients(self.h, A.ptr(kmin), A.ptr(kmax)))


class GeometricQueries:
    """GeometricQueries<DIM> (core/geometric_queries.h:58-124)."""

    def __init__(self, domain_is_watertight=True, domain_min=None, domain_max=None, dim=2):
        _validate(dim)
        self.dim = dim
        self.domain_is_watertight = bool(domain_is_watertight)
        lo = np.full(dim, np.finfo(np.float32).min) if domain_min is None else np.asarray(domain_min, np.float32)
        hi = np.full(dim, np.finfo(np.float32).max) if domain_max is None else np.asarray(domain_max, np.float32)
        self.domain_min = lo
        self.domain_max = hi
        self.absorbing = None
        self.reflecting = None

    @property
    def has_non_empty_absorbing_boundary(self):
        return self.absorbing is not None and self.absorbing.n_prims > 0

    @property
    def has_non_empty_reflecting_boundary(self):
        return self.reflecting is not None and self.reflecting.n_prims > 0

    def to_c(self):
        q = A.GeometricQueriesC()
        q.dim = self.dim
        q.domain_is_watertight = int(self.domain_is_watertight)
        for i in range(self.dim):
            q.domain_min[i] = float(self.domain_min[i])
            q.domain_max[i] = float(self.domain_max[i])
        q.absorbing = self.absorbing.h if self.absorbing is not None else None
        q.reflecting = self.reflecting.h if self.reflecting is not None else None
        return q

    # host-callable queries (the std::function members), batched over rows of x
    def compute_dist_to_absorbing_boundary(self, x, compute_signed_distance=False):
        x = np.asarray(x, np.float32).reshape(-1, self.dim)
        if self.has_non_empty_absorbing_boundary:
            return self.absorbing.closest_point(x, compute_signed_distance)[2]
        m = np.minimum(self.domain_min - x, x - self.domain_max)
        return np.linalg.norm(m, axis=1).astype(np.float32)

    def compute_dist_to_reflecting_boundary(self, x, compute_signed_distance=False):
        x = np.asarray(x, np.float32).reshape(-1, self.dim)
        if self.has_non_empty_reflecting_boundary:
            return self.reflecting.closest_point(x, compute_signed_distance)[2]
        return np.full(x.shape[0], np.finfo(np.float32).max, np.float32)

    def inside_domain(self, x):
        """insideDomain (core/geometric_queries.h:357-371): odd hit parity along every axis."""
        x = np.asarray(x, np.float32).reshape(-1, self.dim)
        if not self.domain_is_watertight:
            return np.ones(x.shape[0], bool)
        inside = np.ones(x.shape[0], bool)
        for i in range(self.dim):
            d = np.zeros_like(x); d[:, i] = 1.0
            hits = np.zeros(x.shape[0], np.int64)
            tm = np.full(x.shape[0], np.finfo(np.float32).max, np.float32)
            for b in (self.absorbing, self.reflecting):
                if b is not None and b.n_prims > 0:
                    hits += b.count_hits(x, d, tm)
            inside &= hits % 2 == 1
        return inside

    def outside_bounding_domain(self, x):
        x = np.asarray(x).reshape(-1, self.dim)
        return np.any((x < self.domain_min) | (x > self.domain_max), axis=1)


def compute_dist_to_boundary(geometric_queries, solve_locations, dist_to_absorbing_boundary=None,
                             dist_to_reflecting_boundary=None, dim=None):
    """compute_dist_to_boundary (python/zombie_bindings.h:732-749): unsigned distances of the
    solve locations to the absorbing and the reflecting boundary (batched on the device).
    Fills the output lists when given; returns both as arrays."""
    x = np.asarray(solve_locations, np.float32).reshape(-1, geometric_queries.dim)
    da = np.asarray(geometric_queries.compute_dist_to_absorbing_boundary(x), np.float32)
    dr = np.asarray(geometric_queries.compute_dist_to_reflecting_boundary(x), np.float32)
    for out, v in ((dist_to_absorbing_boundary, da), (dist_to_reflecting_boundary, dr)):
        if out is not None:
            out.clear()
            out.extend(float(t) for t in v)
    return da, dr


def populate_geometric_queries_for_dirichlet_boundary(handler, geometric_queries, dim=None):
    geometric_queries.absorbing = handler


def populate_geometric_queries_for_neumann_boundary(handler, branch_traversal_weight, geometric_queries, dim=None):
    _check_branch_weight(branch_traversal_weight)
    geometric_queries.reflecting = handler


def populate_geometric_queries_for_robin_boundary(handler, branch_traversal_weight, geometric_queries, dim=None):
    _check_branch_weight(branch_traversal_weight)
    geometric_queries.reflecting = handler


def _check_branch_weight(w):
    if w is not None and not isinstance(w, BranchTraversalWeight):
        raise ZgpuError(A.ZGPU_ERR_UNSUPPORTED_CALLBACK, "branch traversal weight must come from "
                                                         "get_branch_traversal_weight_callback")
    if isinstance(w, BranchTraversalWeight) and w.min_radial_distance != 1e-2:
        raise ZgpuError(A.ZGPU_ERR_UNSUPPORTED, "only min_radial_distance = 1e-2 is compiled into the device sampler")


# ------------------------------------------------------------------------- solvers
class SolveReport:
    def __init__(self, r, kernel_launches=None):
        self.kernel_launches = kernel_launches   # kernels the solve launched (zgpu_last_solve_launches)
        self.total_steps = r.total_steps
        self.total_walks = r.total_walks
        self.escaped_walks = r.escaped_walks
        self.exceeded_walks = r.exceeded_walks
        self.rr_terminated = r.rr_terminated
        self.kernel_ms = r.kernel_ms
        self.total_ms = r.total_ms
        self.error_word = r.error_word
        self.cache_terminated = r.cache_terminated


class _Solver:
    solver_id = A.ZGPU_SOLVER_WALK_ON_SPHERES

    def __init__(self, geometric_queries, walk_state_callback=None, terminal_contribution_callback=None,
                 dim=None, channels=1, context=None, options=None):
        if walk_state_callback is not None or terminal_contribution_callback is not None:
            raise ZgpuError(A.ZGPU_ERR_UNSUPPORTED_CALLBACK,
                            "per-step host callbacks cannot run inside the device walk kernel")
        self.queries = geometric_queries
        self.dim = geometric_queries.dim if dim is None else dim
        _validate(self.dim, channels)
        self.ctx = context or default_context()
        self.options = options
        self.last_report = None

    def solve_arrays(self, pde, walk_settings, arrays, options=None, cache=None, cache_min_distance=0.05):
        """Fast path: structure-of-arrays points/statistics (host numpy or CUDA tensors).
        With `cache` (a NeuralCache) walks end early through it (zgpu_solve_cached)."""
        q = self.queries.to_c()
        p = pde.to_c() if isinstance(pde, PDE) else pde
        ws = walk_settings.to_c() if isinstance(walk_settings, WalkSettings) else walk_settings
        sp, st = arrays.to_c()
        opt = options or self.options
        rep = A.SolveReport()
        optp = C.byref(opt) if opt is not None else None
        if cache is None:
            check(lib().zgpu_solve(self.ctx.h, self.solver_id, C.byref(q), C.byref(p), C.byref(ws), C.byref(sp),
                                   C.byref(st), optp, C.byref(rep)))
        else:
            check(lib().zgpu_solve_cached(self.ctx.h, self.solver_id, C.byref(q), C.byref(p), C.byref(ws),
                                          C.byref(sp), C.byref(st), optp, cache.h, float(cache_min_distance),
                                          C.byref(rep)))
        launches = C.c_int64()
        check(lib().zgpu_last_solve_launches(self.ctx.h, C.byref(launches)))
        self.last_report = SolveReport(rep, launches.value)
        return self.last_report

    def autotune(self, pde, walk_settings, arrays, sample_points=4096, sample_walks=16):
        """Fastest launch configuration for this problem (zgpu_autotune); also becomes this
        solver's default options."""
        q = self.queries.to_c()
        p = pde.to_c() if isinstance(pde, PDE) else pde
        ws = walk_settings.to_c() if isinstance(walk_settings, WalkSettings) else walk_settings
        sp, _ = arrays.to_c()
        opt = A.SolveOptions()
        rate = C.c_float()
        check(lib().zgpu_autotune(self.ctx.h, self.solver_id, C.byref(q), C.byref(p), C.byref(ws), C.byref(sp),
                                  int(sample_points), int(sample_walks), C.byref(opt), C.byref(rate)))
        self.options = opt
        return opt, rate.value

    def solve(self, pde, walk_settings, n_walks, sample_pts, statistics, run_single_threaded=False,
              report_progress=None):
        """solve(pde, walk_settings, n_walks, sample_pts, statistics[, run_single_threaded, report_progress])
        for a list of points (walk_on_spheres.h:132-168) or a single point (:115-129)."""
        single = isinstance(sample_pts, SamplePoint)
        pts = [sample_pts] if single else list(sample_pts)
        if single:
            stats = [statistics]
            nw = [int(n_walks)]
        else:
            if len(statistics) != len(pts):
                statistics.clear()
                statistics.extend(SampleStatistics() for _ in pts)
            stats = statistics
            nw = list(n_walks)
        n = len(pts)
        D = self.dim
        arr = dict(
            pt=np.array([p.pt for p in pts], np.float32).reshape(n, D),
            normal=np.array([p.normal for p in pts], np.float32).reshape(n, D),
            type=np.array([int(p.type) for p in pts], np.int32),
            estimation_quantity=np.array([int(p.estimation_quantity) for p in pts], np.int32),
            dist_to_absorbing=np.array([p.dist_to_absorbing_boundary for p in pts], np.float32),
            dist_to_reflecting=np.array([p.dist_to_reflecting_boundary for p in pts], np.float32),
            n_walks=np.array(nw, np.int32),
            seed=np.array([p.seed for p in pts], np.uint64),
            first_sphere_radius=np.array([p.first_sphere_radius for p in pts], np.float32),
            estimate_normal_aligned=np.array([int(p.estimate_boundary_normal_aligned) for p in pts], np.int32),
            solution_mean=np.array([s.solution_mean for s in stats], np.float64),
            solution_m2=np.array([s.solution_m2 for s in stats], np.float64),
            n_solution_estimates=np.array([s.n_solution_estimates for s in stats], np.int32),
            total_walk_length=np.array([s.total_walk_length for s in stats], np.int64),
            total_splits=np.array([s.total_splits for s in stats], np.int64),
        )
        if any(p.estimation_quantity == EstimationQuantity.SolutionAndGradient for p in pts):
            # estimateSolutionAndGradient: per-dimension gradient moments
            arr["gradient_mean"] = np.array([s.gradient_mean if s.gradient_mean is not None else [0.0] * D
                                             for s in stats], np.float64).reshape(n, D)
            arr["gradient_m2"] = np.array([s.gradient_m2 if s.gradient_m2 is not None else [0.0] * D
                                           for s in stats], np.float64).reshape(n, D)
            arr["n_gradient_estimates"] = np.array([s.n_gradient_estimates for s in stats], np.int32)
            arr["direction_for_derivative"] = np.array([p.direction_for_derivative for p in pts],
                                                       np.float32).reshape(n, D)
            arr["total_first_source_contribution"] = np.array([s.total_first_source_contribution for s in stats],
                                                              np.float64)
            arr["total_derivative_contribution"] = np.array([s.total_derivative_contribution for s in stats],
                                                            np.float64)
        rep = self.solve_arrays(pde, walk_settings, SampleArrays(**arr))
        for i, (p, s) in enumerate(zip(pts, stats)):
            p.first_sphere_radius = float(arr["first_sphere_radius"][i])
            s.solution_mean = float(arr["solution_mean"][i])
            s.solution_m2 = float(arr["solution_m2"][i])
            s.n_solution_estimates = int(arr["n_solution_estimates"][i])
            s.total_walk_length = int(arr["total_walk_length"][i])
            s.total_splits = int(arr["total_splits"][i])
            if "gradient_mean" in arr:
                s.gradient_mean = [float(v) for v in arr["gradient_mean"][i]]
                s.gradient_m2 = [float(v) for v in arr["gradient_m2"][i]]
                s.n_gradient_estimates = int(arr["n_gradient_estimates"][i])
                s.total_first_source_contribution = float(arr["total_first_source_contribution"][i])
                s.total_derivative_contribution = float(arr["total_derivative_contribution"][i])
        if report_progress is not None:
            report_progress(n, 0)
        return rep


class WalkOnSpheres(_Solver):
    """WalkOnSpheres<T,DIM> (point_estimation/walk_on_spheres.h:20-92)."""
    solver_id = A.ZGPU_SOLVER_WALK_ON_SPHERES


class WalkOnStars(_Solver):
    """WalkOnStars<T,DIM> (point_estimation/walk_on_stars.h:22-... )."""
    solver_id = A.ZGPU_SOLVER_WALK_ON_STARS


# ----------------------------------------------------------------- neural cache
class NeuralCache:
    """Hash-grid + MLP cache of the solution, trained on the GPU (zgpu_cache_*).  No
    counterpart in the reference.  Parameters live on the device; x / targets may be numpy
    arrays (host) or CUDA tensors (device)."""

    PARAM_NAMES = ("table", "W1", "b1", "W2", "b2", "w3", "b3")

    def __init__(self, dim, domain_min, domain_max, n_levels=16, log2_table_size=19, base_resolution=4.0,
                 max_resolution=None, learning_rate_grid=1e-2, learning_rate_mlp=1e-3, beta1=0.9, beta2=0.99,
                 epsilon=1e-15, seed=0, padding=0.02, context=None):
        _validate(dim)
        self.ctx = context or default_context()
        self.dim = dim
        lo = np.asarray(domain_min, np.float64)[:dim]
        hi = np.asarray(domain_max, np.float64)[:dim]
        pad = padding * (hi - lo)
        cfg = A.CacheConfig()
        cfg.dim = dim
        cfg.n_levels = n_levels
        cfg.log2_table_size = log2_table_size
        cfg.base_resolution = base_resolution
        # the solution of an elliptic problem is smooth: a coarse finest level keeps many
        # training estimates per cell, which averages their noise instead of memorising it
        cfg.max_resolution = max_resolution if max_resolution is not None else (64.0 if dim == 3 else 128.0)
        for i in range(dim):
            cfg.domain_min[i] = lo[i] - pad[i]
            cfg.domain_max[i] = hi[i] + pad[i]
        cfg.learning_rate_grid = learning_rate_grid
        cfg.learning_rate_mlp = learning_rate_mlp
        cfg.beta1, cfg.beta2, cfg.epsilon = beta1, beta2, epsilon
        cfg.seed = seed
        self.config = cfg
        h = C.c_void_p()
        check(lib().zgpu_cache_create(self.ctx.h, C.byref(cfg), C.byref(h)))
        self.h = h
        _live_caches.add(self)
        off = np.zeros(8, np.int64)
        check(lib().zgpu_cache_layout(self.h, A.ptr(off)))
        self.offsets = off
        res = np.zeros(n_levels, np.float32)
        check(lib().zgpu_cache_resolutions(self.h, A.ptr(res)))
        self.resolutions = res

    @property
    def n_parameters(self):
        return int(self.offsets[7])

    def _mem(self, a):
        return A.ZGPU_MEM_DEVICE if hasattr(a, "is_cuda") and a.is_cuda else A.ZGPU_MEM_HOST

    def _prep(self, a, dtype=np.float32):
        if hasattr(a, "is_cuda") and a.is_cuda:
            return a.contiguous()
        return np.ascontiguousarray(a, dtype)

    def train(self, x, target, steps, batch_size=1 << 16):
        """`steps` Adam steps on consecutive batches of the training set (random order expected);
        returns the mean squared error over those batches."""
        x, t = self._prep(x), self._prep(target)
        loss = C.c_float()
        check(lib().zgpu_cache_train(self.h, int(t.shape[0]), A.ptr(x), A.ptr(t), self._mem(x), int(steps),
                                     int(batch_size), C.byref(loss)))
        return loss.value

    def evaluate(self, x):
        x = self._prep(x)
        n = int(x.shape[0])
        if self._mem(x) == A.ZGPU_MEM_DEVICE:
            import torch
            y = torch.empty(n, dtype=torch.float32, device=x.device)
        else:
            y = np.zeros(n, np.float32)
        check(lib().zgpu_cache_evaluate(self.h, n, A.ptr(x), A.ptr(y), self._mem(x)))
        return y

    def encode(self, x):
        """FP32 hash-grid encoding [n, 32] (host arrays)."""
        x = np.ascontiguousarray(x, np.float32).reshape(-1, self.dim)
        enc = np.zeros((x.shape[0], 32), np.float32)
        check(lib().zgpu_cache_encode(self.h, x.shape[0], A.ptr(x), A.ptr(enc), A.ZGPU_MEM_HOST))
        return enc

    def gradients(self, x, target):
        """Gradient of the mean squared error over all points (no update): (loss, flat grads)."""
        x, t = self._prep(x), self._prep(target)
        g = np.zeros(self.n_parameters, np.float32)
        loss = C.c_double()
        check(lib().zgpu_cache_gradients(self.h, int(t.shape[0]), A.ptr(x), A.ptr(t), self._mem(x), A.ptr(g),
                                         C.byref(loss)))
        return loss.value, g

    def set_learning_rates(self, grid, mlp):
        check(lib().zgpu_cache_set_learning_rates(self.h, float(grid), float(mlp)))

    def get_parameters(self):
        p = np.zeros(self.n_parameters, np.float32)
        check(lib().zgpu_cache_get_parameters(self.h, A.ptr(p)))
        return p

    def set_parameters(self, p):
        p = np.ascontiguousarray(p, np.float32)
        assert p.shape[0] == self.n_parameters
        check(lib().zgpu_cache_set_parameters(self.h, A.ptr(p)))

    def split(self, flat):
        """Views of a flat parameter (or gradient) vector by name."""
        o = self.offsets
        L = self.config.n_levels
        return dict(table=flat[o[0]:o[1]].reshape(L, -1, 2), W1=flat[o[1]:o[2]].reshape(64, 32),
                    b1=flat[o[2]:o[3]], W2=flat[o[3]:o[4]].reshape(64, 64), b2=flat[o[4]:o[5]],
                    w3=flat[o[5]:o[6]], b3=flat[o[6]:o[7]])

    def close(self):
        if getattr(self, "h", None):
            lib().zgpu_cache_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
