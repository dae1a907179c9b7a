"""Builds the in-tree CUDA library zombie_gb300/lib/libzgpu.so for sm_103a.

Translation units are compiled in parallel with nvcc (one -gencode, no cmake) and linked
into a shared library that exports the C ABI of include/zgpu.h.
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIBDIR = os.path.join(HERE, "lib")
LIB = os.path.join(LIBDIR, "libzgpu.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
SOURCES = ["zgpu_walk_2d_wos.cu", "zgpu_walk_2d_wost.cu", "zgpu_walk_3d_wos.cu", "zgpu_walk_3d_wost.cu",
           "zgpu_kernels2.cu", "zgpu_kernels3.cu", "zgpu_dispatch.cu", "zgpu_api.cu", "zgpu_build.cpp", "zgpu_static.cu",
           "zgpu_cache.cu", "zgpu_devbuild.cu", "zgpu_bvc.cu", "zgpu_rws.cu"]
HEADERS = ["zgpu_kernels.cuh", "zgpu_wave.cuh", "zgpu_scene.cuh", "zgpu_math.cuh", "zgpu_internal.h", "zgpu_build.h", "zgpu_cache.cuh",
           "zgpu_umma.cuh"]


def nvcc():
    exe = shutil.which("nvcc")
    if exe:
        return exe
    cand = "/usr/local/cuda/bin/nvcc"
    if os.path.exists(cand):
        return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build zombie_gb300")


def _compile(src, extra):
    obj = os.path.join(BUILD, os.path.basename(src) + ".o")
    cmd = [nvcc()] + ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-O3",
                             "-I", os.path.join(ROOT, "include"), "-c", os.path.join(CSRC, src), "-o", obj] + extra
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
    return obj, r.stderr


def _stale():
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    deps = [os.path.join(CSRC, f) for f in SOURCES + HEADERS] + [os.path.join(ROOT, "include", "zgpu.h")]
    return any(os.path.getmtime(d) > t for d in deps)


def build(force=False, verbose=False, extra_flags=()):
    """Compiles and links libzgpu.so; returns its path."""
    if not force and not _stale():
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    os.makedirs(LIBDIR, exist_ok=True)
    extra = list(extra_flags)
    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        futs = [ex.submit(_compile, s, extra) for s in SOURCES]
        objs = []
        for f in futs:
            obj, log = f.result()
            objs.append(obj)
            if verbose and log:
                sys.stderr.write(log)
    tmp = LIB + ".tmp"
    cmd = [nvcc()] + ARCH + ["-shared", "-o", tmp] + objs + ["-Xcompiler", "-fPIC"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
