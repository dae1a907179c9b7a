"""Loads the in-tree CUDA library (zombie_gb300/lib/libzgpu.so) and declares its C ABI.

There is no CPU fallback: if the library is missing or cannot be loaded, every entry point
raises.  Call zombie_gb300.build.build() (or __graft_entry__.build()) to compile it.
"""
import ctypes as C
import os

from . import _abi as A

LIB_PATH = os.path.join(os.path.dirname(os.path.abspath(__file__)), "lib", "libzgpu.so")


class ZgpuError(RuntimeError):
    def __init__(self, status, message):
        super().__init__(f"{A.STATUS_NAMES.get(status, status)}: {message}")
        self.status = status


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ZgpuError(A.ZGPU_ERR_CUDA, f"CUDA library not built: {LIB_PATH} is missing "
                                             "(run python -c 'import __graft_entry__ as g; g.build()')")
        L = C.CDLL(LIB_PATH)
        vp, i32, i64, f32 = C.c_void_p, C.c_int, C.c_int64, C.c_float
        pp = C.POINTER(C.c_void_p)
        L.zgpu_abi_version.restype = i32
        L.zgpu_last_error.restype = C.c_char_p
        L.zgpu_context_create.argtypes = [i32, pp]
        L.zgpu_context_destroy.argtypes = [vp]
        L.zgpu_context_synchronize.argtypes = [vp]
        L.zgpu_context_stream.argtypes = [vp]
        L.zgpu_context_stream.restype = vp
        L.zgpu_boundary_create.argtypes = [vp, i32, vp, i32, vp, i32, i32, vp, vp, i32, f32, i32, pp]
        L.zgpu_boundary_destroy.argtypes = [vp]
        L.zgpu_boundary_create_on_device.argtypes = [vp, i32, vp, i32, vp, i32, i32, vp, vp, i32, f32, i32, pp]
        L.zgpu_boundary_update_robin_coefficients.argtypes = [vp, vp, vp]
        L.zgpu_pde_evaluate.argtypes = [vp, i32, vp, i64, vp, vp, vp, i32, vp, vp, vp, vp]
        L.zgpu_bvc_splat.argtypes = [vp, i32, vp, vp, f32, f32, f32, f32, f32, vp, i32]
        L.zgpu_rws_solve.argtypes = [vp, vp, vp, vp, vp, f32, f32, f32, C.c_uint64, vp, i32, vp]
        L.zgpu_boundary_info.argtypes = [vp, C.POINTER(C.c_int64), C.POINTER(C.c_int32), C.POINTER(C.c_int64),
                                         C.POINTER(C.c_int64)]
        L.zgpu_boundary_signed_volume.argtypes = [vp, C.POINTER(C.c_float)]
        L.zgpu_boundary_set_query_mode.argtypes = [vp, i32]
        L.zgpu_query_closest_point.argtypes = [vp, i64, vp, i32, vp, vp, vp, vp, i32]
        L.zgpu_query_intersect.argtypes = [vp, i64, vp, vp, vp, vp, vp, vp, vp, vp, vp, vp, i32]
        L.zgpu_query_count_hits.argtypes = [vp, i64, vp, vp, vp, vp, i32]
        L.zgpu_query_star_radius.argtypes = [vp, i64, vp, vp, vp, f32, vp, vp, i32]
        L.zgpu_query_occluded.argtypes = [vp, i64, vp, vp, vp, vp, vp, vp, vp, i32]
        L.zgpu_query_sample_boundary.argtypes = [vp, i64, vp, vp, vp, vp, vp, vp, vp, i32]
        L.zgpu_solve.argtypes = [vp, i32, vp, vp, vp, vp, vp, vp, vp]
        L.zgpu_last_solve_launches.argtypes = [vp, vp]
        L.zgpu_solve_batched.argtypes = [vp, i32, i32, vp, vp, vp, vp, vp, vp, vp]
        L.zgpu_autotune.argtypes = [vp, i32, vp, vp, vp, vp, i32, i32, vp, C.POINTER(C.c_float)]
        L.zgpu_solve_static.argtypes = [vp, i32, vp, vp, vp, vp, vp, vp]
        L.zgpu_cache_create.argtypes = [vp, vp, pp]
        L.zgpu_cache_destroy.argtypes = [vp]
        L.zgpu_cache_layout.argtypes = [vp, vp]
        L.zgpu_cache_resolutions.argtypes = [vp, vp]
        L.zgpu_cache_get_parameters.argtypes = [vp, vp]
        L.zgpu_cache_set_learning_rates.argtypes = [vp, f32, f32]
        L.zgpu_cache_set_parameters.argtypes = [vp, vp]
        L.zgpu_cache_train.argtypes = [vp, i64, vp, vp, i32, i32, i32, C.POINTER(C.c_float)]
        L.zgpu_cache_gradients.argtypes = [vp, i64, vp, vp, i32, vp, C.POINTER(C.c_double)]
        L.zgpu_cache_evaluate.argtypes = [vp, i64, vp, vp, i32]
        L.zgpu_cache_encode.argtypes = [vp, i64, vp, vp, i32]
        L.zgpu_solve_cached.argtypes = [vp, i32, vp, vp, vp, vp, vp, vp, vp, f32, vp]
        if L.zgpu_abi_version() != A.ZGPU_ABI_VERSION:
            raise ZgpuError(A.ZGPU_ERR_INVALID_ARG, "ABI version mismatch between libzgpu.so and zombie_gb300")
        _lib = L
    return _lib


def check(status):
    if status != A.ZGPU_OK:
        msg = lib().zgpu_last_error()
        raise ZgpuError(status, msg.decode() if msg else "")
    return status


def exported_symbols():
    """Names of the zgpu_* functions declared in include/zgpu.h."""
    import re
    hdr = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include", "zgpu.h")
    with open(hdr) as f:
        txt = f.read()
    return sorted(set(re.findall(r"\b(zgpu_[a-z0-9_]+)\s*\(", txt)))
