"""Build of the native parts, in-tree and without cmake.

``build_lib()``     -> mrfmap_gb300/_lib/libmrfmap_gb300.so  (CUDA kernels + C ABI)
``build_pymodule()`` -> mrfmap_gb300/_lib/GVDBPyModules*.so   (pybind11 mirror of
                        the reference's Python module, over the C ABI)

Every translation unit is compiled for sm_103a only, in parallel.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
import sysconfig

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
OUT = os.path.join(PKG, "_lib")
OBJ = os.path.join(OUT, "obj")
INCLUDE = os.path.join(ROOT, "include")
LIBNAME = "libmrfmap_gb300.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "--expt-relaxed-constexpr", "-Xcompiler", "-fPIC",
              "-Xcompiler", "-ffp-contract=off", "-Xcompiler", "-fvisibility=hidden"]

CU_SOURCES = ["mrf_build.cu", "mrf_bp.cu", "mrf_like.cu", "mrf_capi.cu", "mrf_noalloc.cu",
              "mrf_render.cu", "mrf_warmnet.cu"]
HEADERS = ["mrf_internal.h", "mrf_geometry.cuh", "mrf_like_pixel.cuh"]


def nvcc() -> str:
    cand = os.environ.get("NVCC") or shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    return cand


def _stale(target: str, deps: list[str]) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def _run(cmd: list[str]):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    return r


def build_lib(force: bool = False, verbose: bool = False) -> str:
    os.makedirs(OBJ, exist_ok=True)
    hdrs = [os.path.join(CSRC, h) for h in HEADERS] + [os.path.join(INCLUDE, "mrfmap_gb300.h")]
    jobs = []
    objs = []
    for src in CU_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(OBJ, src.replace(".cu", ".o"))
        objs.append(o)
        if force or _stale(o, [s] + hdrs):
            jobs.append([nvcc(), *ARCH, *NVCC_FLAGS, "-I", INCLUDE, "-c", s, "-o", o])
    if jobs:
        with cf.ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
            for r in ex.map(_run, jobs):
                if verbose and r.stderr:
                    print(r.stderr, file=sys.stderr)
    lib = os.path.join(OUT, LIBNAME)
    if force or jobs or _stale(lib, objs):
        _run([nvcc(), *ARCH, "-shared", "-o", lib, *objs, "-Xcompiler", "-fPIC"])
    return lib


def _torch_pybind_include() -> str | None:
    # pybind11 headers ship with torch; this avoids a pybind11 install
    try:
        import torch  # noqa: F401
        inc = os.path.join(os.path.dirname(torch.__file__), "include")
        if os.path.isdir(os.path.join(inc, "pybind11")):
            return inc
    except Exception:
        pass
    try:
        import pybind11
        return pybind11.get_include()
    except Exception:
        return None


def pymodule_path() -> str:
    suffix = sysconfig.get_config_var("EXT_SUFFIX") or ".so"
    return os.path.join(OUT, "GVDBPyModules" + suffix)


def build_pymodule(force: bool = False) -> str:
    lib = build_lib()
    inc = _torch_pybind_include()
    if inc is None:
        raise RuntimeError("pybind11 headers not found")
    srcs = [os.path.join(CSRC, "shim", f) for f in ("GVDBShim.cpp", "GVDBPyModules.cpp", "KeyframeSelector.cpp")]
    hdrs = [os.path.join(ROOT, "include", "mrfmap", h) for h in
            ("GVDBParams.h", "GVDBImage.h", "GVDBInference.h", "GVDBMapLikelihoodEstimator.h",
             "GVDBMRFMap.h", "MatrixArgs.h")]
    out = pymodule_path()
    if not force and not _stale(out, srcs + hdrs + [lib]):
        return out
    cmd = [os.environ.get("CXX", "g++"), "-O2", "-std=c++17", "-shared", "-fPIC", "-fvisibility=hidden",
           "-I", INCLUDE, "-I", inc, "-I", sysconfig.get_paths()["include"], *srcs,
           "-L", OUT, "-lmrfmap_gb300", "-Wl,-rpath,$ORIGIN", "-o", out]
    _run(cmd)
    return out


if __name__ == "__main__":
    print(build_lib(force="--force" in sys.argv, verbose=True))
