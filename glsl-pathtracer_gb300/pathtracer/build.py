"""Build of libptgb.so (the CUDA path) from csrc/, in-tree.

nvcc compiles each translation unit for sm_103a only
(-gencode arch=compute_103a,code=sm_103a) in parallel; the host-side BVH
collapse is plain C++.  No cmake, no torch extension machinery.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess

# the package root (glsl-pathtracer_gb300/), as pathtracer.capi has it
PKG_DIR = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(PKG_DIR, "csrc")
OBJ = os.path.join(CSRC, "_build")
LIB = os.path.join(CSRC, "libptgb.so")

NVCC_FLAGS = ["-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-lineinfo", "-std=c++17",
              "-Xcompiler", "-fPIC", "-Xcompiler", "-O2", "--expt-relaxed-constexpr"]
CU_SOURCES = ["pt_kernels.cu", "pt_wavefront.cu", "pt_capi.cu", "pt_bvh_gpu.cu"]
# The path-tracing kernels divide and take square roots as a GPU runs GLSL:
# a / b within 2 ulp and sqrt as the hardware approximation
# (-prec-div=false -prec-sqrt=false; GLSL allows 2.5 ulp for a / b and
# defines sqrt through inversesqrt), not the IEEE-rounded results.  The
# shading stage takes a third less time.  Hits do not depend on it: the
# triangle test and the ray-origin offsets use explicitly rounded
# operations (__fdiv_rn, __fmul_rn, __fmaf_rn ...), which no flag changes,
# and the slab test's reciprocal ray direction is __frcp_rn.
_GLSL_PRECISION = ["-prec-div=false", "-prec-sqrt=false"]
FILE_FLAGS = {"pt_kernels.cu": _GLSL_PRECISION, "pt_wavefront.cu": _GLSL_PRECISION}
CPP_SOURCES = ["bvh8_build.cpp", "cuda_renderer.cpp"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed: " + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    return r.stdout + r.stderr


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build_library(force: bool = False, verbose: bool = False, extra_flags: list[str] | None = None) -> str:
    os.makedirs(OBJ, exist_ok=True)
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    headers.append(os.path.join(os.path.dirname(PKG_DIR), "include", "pt_cuda.h"))
    nv = nvcc()
    jobs = []
    objs = []
    for src in CU_SOURCES + CPP_SOURCES:
        path = os.path.join(CSRC, src)
        if not os.path.exists(path):
            continue
        obj = os.path.join(OBJ, src + ".o")
        objs.append(obj)
        if not force and not _stale(obj, [path, __file__] + headers):
            continue
        if src.endswith(".cu"):
            cmd = [nv] + NVCC_FLAGS + FILE_FLAGS.get(src, []) + (extra_flags or []) + ["-c", path, "-o", obj]
        else:
            cmd = ["g++", "-std=c++17", "-O2", "-fPIC", "-I/usr/local/cuda/include", "-c", path, "-o", obj]
        jobs.append(cmd)
    with cf.ThreadPoolExecutor(max_workers=max(1, len(jobs))) as ex:
        for out in ex.map(_run, jobs):
            if verbose and out.strip():
                print(out)
    if force or _stale(LIB, objs):
        _run([nv, "-shared", "-gencode", "arch=compute_103a,code=sm_103a"] + objs + ["-o", LIB, "-lcudart"])
    return LIB


if __name__ == "__main__":
    print(build_library(verbose=True))
