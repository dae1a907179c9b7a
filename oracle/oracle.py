"""ctypes wrapper of the CPU oracle -- TEST INFRASTRUCTURE, NOT PRODUCT CODE.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg import this module,
and only as the checker.  The oracle restates rohan-sawhney/zombie's walk hot path on the
CPU (see oracle_core.h for what it follows and how it is pinned: parity against the
reference binary is unpinned because the reference cannot be built; analytic solutions,
brute-force queries and Green's-function identities pin it instead).
"""
import ctypes as C
import os
import subprocess

import numpy as np

from zombie_gb300 import _abi as A

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "liboracle.so")
SOURCES = ["oracle.cpp", "oracle_core.h", "oracle_geometry.h", "oracle_walk.h", "oracle_cache.h"]


def build(force=False):
    """Compiles oracle/_build/liboracle.so with g++ (portable flags: runs on x86 and Arm)."""
    os.makedirs(os.path.dirname(LIB_PATH), exist_ok=True)
    hdr = os.path.join(HERE, "..", "include", "zgpu.h")
    srcs = [os.path.join(HERE, s) for s in SOURCES] + [hdr]
    if not force and os.path.exists(LIB_PATH):
        lib_m = os.path.getmtime(LIB_PATH)
        if all(os.path.getmtime(s) <= lib_m for s in srcs):
            return LIB_PATH
    cmd = ["g++", "-std=c++17", "-O3", "-fPIC", "-shared", "-o", LIB_PATH + ".tmp",
           os.path.join(HERE, "oracle.cpp"), "-lpthread"]
    subprocess.check_call(cmd)
    os.replace(LIB_PATH + ".tmp", LIB_PATH)
    return LIB_PATH


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(LIB_PATH)
        vp, i32, i64, f32, u64 = C.c_void_p, C.c_int, C.c_int64, C.c_float, C.c_uint64
        L.orc_boundary_create.restype = vp
        L.orc_boundary_create.argtypes = [i32, vp, i32, vp, i32, i32, vp, vp, i32, f32, i32]
        L.orc_boundary_destroy.argtypes = [vp]
        L.orc_boundary_flags.argtypes = [vp, vp, vp]
        L.orc_signed_volume.restype = C.c_double
        L.orc_signed_volume.argtypes = [vp]
        L.orc_closest_point.argtypes = [vp, i64, vp, vp, vp, vp, vp]
        L.orc_intersect.argtypes = [vp, i64, vp, vp, vp, vp, vp, vp, vp, vp, vp, vp]
        L.orc_count_hits.argtypes = [vp, i64, vp, vp, vp, vp]
        L.orc_star_radius.argtypes = [vp, i64, vp, vp, vp, f32, vp, vp]
        L.orc_occluded.argtypes = [vp, i64, vp, vp, vp, vp, vp, vp, vp]
        L.orc_sample.argtypes = [vp, i64, vp, vp, vp, vp, vp, vp, vp]
        L.orc_greens_norm.restype = f32
        L.orc_greens_norm.argtypes = [i32, i32, f32, f32]
        L.orc_greens_evaluate.restype = f32
        L.orc_greens_evaluate.argtypes = [i32, i32, f32, f32, f32]
        L.orc_greens_sample_radii.argtypes = [i32, i32, f32, f32, u64, i32, vp]
        L.orc_bessel.restype = C.c_double
        L.orc_bessel.argtypes = [i32, C.c_double]
        L.orc_pcg32.argtypes = [u64, u64, i32, vp, vp]
        L.orc_offset_point.argtypes = [i32, vp, vp, vp]
        L.orc_eval_pde.argtypes = [i32, vp, i64, vp, vp, i32, vp, vp, vp, vp]
        L.orc_solve.argtypes = [i32, vp, vp, vp, vp, vp, i32, C.POINTER(C.c_uint64)]
        L.orc_bvc_splat.argtypes = [i32, C.c_float, vp, C.c_float, C.c_float, C.c_float, C.c_float, C.c_float, vp, i32]
        L.orc_rws_solve.argtypes = [vp, vp, vp, vp, C.c_float, C.c_float, C.c_float, C.c_uint64, vp, i32]
        L.orc_rws_solve.restype = C.c_uint64
        L.orc_hardware_threads.restype = i32
        L.orc_counters.argtypes = [vp]
        L.orc_cache_forward.argtypes = [i32, i32, i32, vp, vp, vp, vp, vp, vp, vp, vp, vp, f32, i64, vp, vp, vp]
        L.orc_cache_corners.argtypes = [i32, i32, i32, vp, vp, vp, i64, vp, vp, vp]
        L.orc_cache_grads.restype = C.c_double
        L.orc_cache_grads.argtypes = [i32, i32, i32, vp, vp, vp, vp, vp, vp, vp, vp, vp, f32, i32, vp, vp,
                                      vp, vp, vp, vp, vp, vp, vp]
        _lib = L
    return _lib


def _f32(a):
    return np.ascontiguousarray(a, dtype=np.float32)


def _i32(a):
    return np.ascontiguousarray(a, dtype=np.int32)


class Boundary:
    """One boundary part (absorbing / Neumann / Robin) with a binary SAH BVH or brute force."""

    def __init__(self, dim, positions, indices, kind=A.ZGPU_BOUNDARY_ABSORBING, kmin=None, kmax=None,
                 solve_double_sided=False, silhouette_precision=1e-3, use_bvh=True):
        self.dim = dim
        self.positions = _f32(positions).reshape(-1, dim)
        self.indices = _i32(indices).reshape(-1, dim)
        self.kmin = None if kmin is None else _f32(kmin)
        self.kmax = None if kmax is None else _f32(kmax)
        self.n_prims = self.indices.shape[0]
        self.h = lib().orc_boundary_create(dim, A.ptr(self.positions), self.positions.shape[0],
                                           A.ptr(self.indices), self.n_prims, kind, A.ptr(self.kmin),
                                           A.ptr(self.kmax), int(solve_double_sided),
                                           float(silhouette_precision), int(use_bvh))

    def __del__(self):
        if getattr(self, "h", None):
            lib().orc_boundary_destroy(self.h)
            self.h = None

    def flags(self):
        has = np.zeros((self.n_prims, self.dim), np.int32)
        ign = np.zeros((self.n_prims, self.dim), np.int32)
        lib().orc_boundary_flags(self.h, A.ptr(has), A.ptr(ign))
        return has, ign

    def signed_volume(self):
        return lib().orc_signed_volume(self.h)

    def closest_point(self, x):
        x = _f32(x).reshape(-1, self.dim)
        n = x.shape[0]
        pt = np.zeros_like(x); nrm = np.zeros_like(x)
        d = np.zeros(n, np.float32); prim = np.zeros(n, np.int32)
        lib().orc_closest_point(self.h, n, A.ptr(x), A.ptr(pt), A.ptr(nrm), A.ptr(d), A.ptr(prim))
        return pt, nrm, d, prim

    def intersect(self, origin, normal, direction, tmax, on_boundary):
        o = _f32(origin).reshape(-1, self.dim); nn = _f32(normal).reshape(-1, self.dim)
        dr = _f32(direction).reshape(-1, self.dim); tm = _f32(tmax); ob = _i32(on_boundary)
        n = o.shape[0]
        hit = np.zeros(n, np.int32); pt = np.zeros_like(o); nrm = np.zeros_like(o)
        dist = np.zeros(n, np.float32); prim = np.zeros(n, np.int32)
        lib().orc_intersect(self.h, n, A.ptr(o), A.ptr(nn), A.ptr(dr), A.ptr(tm), A.ptr(ob), A.ptr(hit),
                            A.ptr(pt), A.ptr(nrm), A.ptr(dist), A.ptr(prim))
        return hit, pt, nrm, dist, prim

    def count_hits(self, origin, direction, tmax):
        o = _f32(origin).reshape(-1, self.dim); dr = _f32(direction).reshape(-1, self.dim); tm = _f32(tmax)
        out = np.zeros(o.shape[0], np.int32)
        lib().orc_count_hits(self.h, o.shape[0], A.ptr(o), A.ptr(dr), A.ptr(tm), A.ptr(out))
        return out

    def star_radius(self, x, min_r, max_r, precision, flip):
        x = _f32(x).reshape(-1, self.dim)
        out = np.zeros(x.shape[0], np.float32)
        lib().orc_star_radius(self.h, x.shape[0], A.ptr(x), A.ptr(_f32(min_r)), A.ptr(_f32(max_r)),
                              float(precision), A.ptr(_i32(flip)), A.ptr(out))
        return out

    def occluded(self, xi, xj, ni, nj, oi, oj):
        xi = _f32(xi).reshape(-1, self.dim)
        out = np.zeros(xi.shape[0], np.int32)
        lib().orc_occluded(self.h, xi.shape[0], A.ptr(xi), A.ptr(_f32(xj)), A.ptr(_f32(ni)), A.ptr(_f32(nj)),
                           A.ptr(_i32(oi)), A.ptr(_i32(oj)), A.ptr(out))
        return out

    def sample(self, x, radius, u):
        x = _f32(x).reshape(-1, self.dim)
        n = x.shape[0]
        found = np.zeros(n, np.int32); pt = np.zeros_like(x); nrm = np.zeros_like(x); pdf = np.zeros(n, np.float32)
        lib().orc_sample(self.h, n, A.ptr(x), A.ptr(_f32(radius)), A.ptr(_f32(u)), A.ptr(found), A.ptr(pt),
                         A.ptr(nrm), A.ptr(pdf))
        return found, pt, nrm, pdf


QUERY_KINDS = ("closest_point", "first_hit", "line_of_sight", "star_radius", "sample")


def counters():
    """Traversal work of the solves since the last call: per query kind calls, nodes, prims."""
    out = np.zeros(15, np.uint64)
    lib().orc_counters(A.ptr(out))
    return {k: dict(calls=int(out[i]), nodes=int(out[5 + i]), prims=int(out[10 + i]))
            for i, k in enumerate(QUERY_KINDS)}


def pcg32(seed, stream, n):
    u = np.zeros(n, np.uint32); f = np.zeros(n, np.float32)
    lib().orc_pcg32(seed, stream, n, A.ptr(u), A.ptr(f))
    return u, f


def bessel(which, x):
    return lib().orc_bessel({"i0": 0, "i1": 1, "k0": 2, "k1": 3}[which], float(x))


def eval_pde(dim, pde, x, normals=None, aligned=False, with_robin_coeff=False):
    """source, dirichlet, robin (and the Robin coefficient) of the oracle's PDE at x."""
    x = _f32(x).reshape(-1, dim)
    n = x.shape[0]
    src = np.zeros(n, np.float32); dr = np.zeros(n, np.float32); rb = np.zeros(n, np.float32)
    kp = np.zeros(n, np.float32)
    nn = None if normals is None else _f32(normals).reshape(-1, dim)
    lib().orc_eval_pde(dim, C.byref(pde), n, A.ptr(x), A.ptr(nn), int(aligned), A.ptr(src), A.ptr(dr), A.ptr(rb),
                       A.ptr(kp))
    return (src, dr, rb, kp) if with_robin_coeff else (src, dr, rb)


def solve(solver, dim, absorbing, reflecting, domain_min, domain_max, pde, settings, points, stats,
          n_threads=None):
    """Runs the CPU restatement of WalkOnSpheres/WalkOnStars::solve.

    points / stats: dicts of numpy arrays with the zgpu_sample_points / statistics fields.
    Returns the number of executed walk steps.
    """
    q = A.GeometricQueriesC()
    q.dim = dim
    q.domain_is_watertight = 1
    for i in range(dim):
        q.domain_min[i] = float(domain_min[i]); q.domain_max[i] = float(domain_max[i])
    q.absorbing = absorbing.h if absorbing is not None else None
    q.reflecting = reflecting.h if reflecting is not None else None
    sp = A.SamplePointsC()
    sp.n = points["pt"].shape[0]
    sp.memory = A.ZGPU_MEM_HOST
    for name in ("pt", "normal", "type", "estimation_quantity", "dist_to_absorbing", "dist_to_reflecting",
                 "n_walks", "seed", "first_sphere_radius", "estimate_normal_aligned", "scene_id",
                 "direction_for_derivative"):
        setattr(sp, name, A.ptr(points.get(name)))
    st = A.SampleStatisticsC()
    st.memory = A.ZGPU_MEM_HOST
    for name in ("solution_mean", "solution_m2", "n_solution_estimates", "total_walk_length", "total_splits",
                 "gradient_mean", "gradient_m2", "n_gradient_estimates", "total_first_source_contribution",
                 "total_derivative_contribution"):
        setattr(st, name, A.ptr(stats.get(name)))
    steps = C.c_uint64(0)
    if n_threads is None:
        n_threads = max(1, lib().orc_hardware_threads())
    lib().orc_solve(solver, C.byref(q), C.byref(pde), C.byref(settings), C.byref(sp), C.byref(st),
                    int(n_threads), C.byref(steps))
    return int(steps.value)


class CacheModel:
    """The neural cache's definition (oracle_cache.h) with parameters given as numpy arrays:
    table [levels, T, 2], W1 [64, 2L], b1 [64], W2 [64, 64], b2 [64], w3 [64], b3 scalar."""

    def __init__(self, dim, res, lo, inv, table, W1, b1, W2, b2, w3, b3):
        self.dim = dim
        self.res = _f32(res)
        self.levels = len(self.res)
        self.table = _f32(table).reshape(self.levels, -1, 2)
        self.log2T = int(np.log2(self.table.shape[1]))
        self.lo = _f32(np.resize(lo, 3))
        self.inv = _f32(np.resize(inv, 3))
        self.W1, self.b1, self.W2, self.b2, self.w3 = (_f32(a) for a in (W1, b1, W2, b2, w3))
        self.b3 = float(b3)

    def _args(self):
        return (self.dim, self.levels, self.log2T, A.ptr(self.res), A.ptr(self.lo), A.ptr(self.inv),
                A.ptr(self.table), A.ptr(self.W1), A.ptr(self.b1), A.ptr(self.W2), A.ptr(self.b2),
                A.ptr(self.w3), self.b3)

    def forward(self, x, with_encoding=False):
        x = _f32(x).reshape(-1, self.dim)
        y = np.zeros(x.shape[0])
        enc = np.zeros((x.shape[0], 2 * self.levels)) if with_encoding else None
        lib().orc_cache_forward(*self._args(), x.shape[0], A.ptr(x), A.ptr(y), A.ptr(enc))
        return (y, enc) if with_encoding else y

    def corners(self, x):
        x = _f32(x).reshape(-1, self.dim)
        C_ = 1 << self.dim
        idx = np.zeros((x.shape[0], self.levels, C_), np.uint32)
        w = np.zeros((x.shape[0], self.levels, C_))
        lib().orc_cache_corners(self.dim, self.levels, self.log2T, A.ptr(self.res), A.ptr(self.lo), A.ptr(self.inv),
                                x.shape[0], A.ptr(x), A.ptr(idx), A.ptr(w))
        return idx, w

    def loss_and_grads(self, x, target):
        x = _f32(x).reshape(-1, self.dim)
        t = _f32(target)
        g = dict(table=np.zeros(self.table.shape), W1=np.zeros(self.W1.shape), b1=np.zeros(64),
                 W2=np.zeros(self.W2.shape), b2=np.zeros(64), w3=np.zeros(64), b3=np.zeros(1))
        loss = lib().orc_cache_grads(*self._args(), x.shape[0], A.ptr(x), A.ptr(t), A.ptr(g["table"]), A.ptr(g["W1"]),
                                     A.ptr(g["b1"]), A.ptr(g["W2"]), A.ptr(g["b2"]), A.ptr(g["w3"]), A.ptr(g["b3"]))
        return loss, g


def bvc_splat(dim, absorption, samples, evals, radius_clamp=1e-3, kernel_regularization=0.0,
              robin_coeff_cutoff=float("inf"), cutoff_absorbing=0.0, cutoff_reflecting=0.0, n_threads=None):
    """BoundaryValueCaching::splat on the CPU: samples / evals are dicts of numpy arrays with the
    zgpu_bvc_samples / zgpu_bvc_eval_points fields; the evaluation statistics are updated in place."""
    s = A.BvcSamplesC()
    s.n = samples["pt"].shape[0]
    for name in ("pt", "normal", "pdf", "type", "estimate_normal_aligned", "solution", "normal_derivative",
                 "contribution", "robin_coeff"):
        setattr(s, name, A.ptr(samples.get(name)))
    e = A.BvcEvalPointsC()
    e.n = evals["pt"].shape[0]
    for name in ("pt", "type", "dist_to_absorbing", "dist_to_reflecting", "mean", "m2", "count", "gradient_mean",
                 "gradient_m2"):
        setattr(e, name, A.ptr(evals.get(name)))
    if n_threads is None:
        n_threads = max(1, lib().orc_hardware_threads())
    lib().orc_bvc_splat(dim, float(absorption), C.byref(s), float(radius_clamp), float(kernel_regularization),
                        float(robin_coeff_cutoff), float(cutoff_absorbing), float(cutoff_reflecting), C.byref(e),
                        int(n_threads))


def rws_solve(dim, absorbing, reflecting, domain_min, domain_max, pde, settings, samples, evals, normal_offset,
              radius_clamp=1e-3, kernel_regularization=0.0, stream=0, n_threads=None, watertight=True):
    """The reverse walks of ReverseWalkOnStarsSolver::solve on the CPU: samples / evals are dicts
    of numpy arrays with the zgpu_rws_samples / zgpu_rws_eval_points fields; evals["totals"] is
    added to.  Returns the number of walk steps."""
    q = A.GeometricQueriesC()
    q.dim = dim
    q.domain_is_watertight = int(watertight)
    for i in range(dim):
        q.domain_min[i] = float(domain_min[i]); q.domain_max[i] = float(domain_max[i])
    q.absorbing = absorbing.h if absorbing is not None else None
    q.reflecting = reflecting.h if reflecting is not None else None
    s = A.RwsSamplesC()
    s.n = samples["pt"].shape[0]
    for name in ("pt", "normal", "type", "estimate_normal_aligned", "pdf", "contribution", "dist_to_absorbing", "seed"):
        setattr(s, name, A.ptr(samples.get(name)))
    e = A.RwsEvalPointsC()
    e.n = evals["pt"].shape[0]
    for name in ("pt", "normal", "type", "totals"):
        setattr(e, name, A.ptr(evals.get(name)))
    if n_threads is None:
        n_threads = max(1, lib().orc_hardware_threads())
    return int(lib().orc_rws_solve(C.byref(q), C.byref(pde), C.byref(settings), C.byref(s), float(normal_offset),
                                   float(radius_clamp), float(kernel_regularization), int(stream), C.byref(e),
                                   int(n_threads)))
