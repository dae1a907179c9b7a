"""The C ABI: struct layouts of include/zgpu.h match the ctypes mirrors, and the built
library exports every declared entry point (no GPU needed)."""
import ctypes as C
import os
import subprocess
import tempfile

import pytest

from zombie_gb300 import _abi as A

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

STRUCTS = {
    "zgpu_analytic": A.Analytic, "zgpu_grid": A.Grid, "zgpu_pde": A.Pde, "zgpu_walk_settings": A.WalkSettingsC,
    "zgpu_sample_points": A.SamplePointsC, "zgpu_sample_statistics": A.SampleStatisticsC,
    "zgpu_solve_options": A.SolveOptions, "zgpu_solve_report": A.SolveReport,
    "zgpu_geometric_queries": A.GeometricQueriesC, "zgpu_cache_config": A.CacheConfig,
}


def test_struct_layouts_match_header():
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "zgpu.h"', "int main(void) {"]
    for cname, py in STRUCTS.items():
        lines.append(f'printf("{cname} %zu\\n", sizeof({cname}));')
        for fname, _ in py._fields_:
            lines.append(f'printf("{cname}.{fname} %zu\\n", offsetof({cname}, {fname}));')
    lines.append("return 0; }")
    with tempfile.TemporaryDirectory() as d:
        src = os.path.join(d, "layout.c")
        exe = os.path.join(d, "layout")
        open(src, "w").write("\n".join(lines))
        subprocess.check_call(["gcc", "-std=c99", "-I", os.path.join(ROOT, "include"), src, "-o", exe])
        out = subprocess.check_output([exe], text=True).split("\n")
    got = dict(l.rsplit(" ", 1) for l in out if l)
    for cname, py in STRUCTS.items():
        assert int(got[cname]) == C.sizeof(py), cname
        for fname, _ in py._fields_:
            assert int(got[f"{cname}.{fname}"]) == getattr(py, fname).offset, f"{cname}.{fname}"


def test_constants_match_header():
    """Every ZGPU_* constant of the ctypes layer has the header's value (macros and enums)."""
    names = [k for k in dir(A) if k.startswith("ZGPU_") and isinstance(getattr(A, k), int)]
    lines = ['#include <stdio.h>', '#include "zgpu.h"', "int main(void) {"]
    lines += [f'printf("{k} %lld\\n", (long long)({k}));' for k in names]
    lines.append("return 0; }")
    with tempfile.TemporaryDirectory() as d:
        src = os.path.join(d, "consts.c")
        exe = os.path.join(d, "consts")
        open(src, "w").write("\n".join(lines))
        subprocess.check_call(["gcc", "-std=c99", "-I", os.path.join(ROOT, "include"), src, "-o", exe])
        out = subprocess.check_output([exe], text=True).split("\n")
    got = dict(l.rsplit(" ", 1) for l in out if l)
    assert len(got) == len(names) > 30
    for k in names:
        assert int(got[k]) == getattr(A, k), k


def test_header_compiles_as_cpp():
    with tempfile.TemporaryDirectory() as d:
        src = os.path.join(d, "h.cpp")
        open(src, "w").write('#include "zgpu.h"\nint main() { return zgpu_abi_version == nullptr; }\n')
        subprocess.check_call(["g++", "-std=c++17", "-fsyntax-only", "-I", os.path.join(ROOT, "include"), src])


def test_library_exports_every_declared_symbol():
    from zombie_gb300 import _lib, build
    path = build.build()
    assert os.path.exists(path)
    lib = C.CDLL(path)   # loading needs no GPU
    missing = [s for s in _lib.exported_symbols() if not hasattr(lib, s)]
    assert not missing, missing
    assert len(_lib.exported_symbols()) >= 19
    assert lib.zgpu_abi_version() == A.ZGPU_ABI_VERSION


def test_library_is_built_for_sm103a():
    from zombie_gb300 import build
    assert "arch=compute_103a,code=sm_103a" in " ".join(build.ARCH)
