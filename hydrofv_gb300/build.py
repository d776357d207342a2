"""Build recipe for libhydro_gb300.so (sm_103a only, in-tree).

    python -m hydrofv_gb300.build          # or hydrofv_gb300.build.build()

Compiles the CUDA translation units with nvcc for sm_103a and the host C
layer with gcc, in parallel, then links one shared library next to this file.
The FP64 step kernels are compiled with ``--fmad=false`` and all host code
with ``-ffp-contract=off``: the drop-in path must perform the same IEEE-754
operations as the reference CPU solver (aarch64 gcc would otherwise fuse
a*b+c).  Object files go to ``hydrofv_gb300/_build/``.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
BUILD = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "libhydro_gb300.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# Extra nvcc flags for every CUDA translation unit, e.g. a tile-shape define
# (-DMH2D_THREADS_FP64=96 -DMH2D_CTAS_FP64=6) when sweeping launch shapes.
EXTRA_NVCC = os.environ.get("HYDRO_NVCC_FLAGS", "").split()
INCLUDES = ["-I" + os.path.join(ROOT, "include"), "-I" + os.path.join(CSRC, "gpu"),
            "-I" + os.path.join(CSRC, "host")]

# (source, extra nvcc flags)
CUDA_SOURCES = [
    ("gpu/mh2d.cu", ["--fmad=false"]),
    ("gpu/mh2d_lim_minmod.cu", ["--fmad=false"]),
    ("gpu/mh2d_lim_vanleer.cu", ["--fmad=false"]),
    ("gpu/mh2d_lim_mc.cu", ["--fmad=false"]),
    ("gpu/mh2d_lim_first_order.cu", ["--fmad=false"]),
    # the FP32 state form: approximate FP32 divide and square root (at most
    # 2 ulp); the FP64 translation units are untouched
    ("gpu/mh2d_fp32.cu", ["-prec-div=false", "-prec-sqrt=false"]),
    ("gpu/runtime2d.cu", []),
    ("gpu/runtime_batch.cu", []),
    ("gpu/host_numerics.cu", ["--fmad=false"]),
    ("gpu/source_term_host.cu", ["--fmad=false"]),
    ("gpu/calibrate.cu", []),
    ("gpu/noalloc2d.cu", []),
    ("gpu/run1d.cu", ["--fmad=false"]),
    ("gpu/adjoint2d.cu", ["--fmad=false"]),
    ("gpu/ad_pointwise.cu", ["--fmad=false"]),
    ("gpu/fx_check.cu", ["--fmad=false"]),
]
C_SOURCES = [
    "host/error.c",
    "host/system.c",
    "host/boundary.c",
    "host/params.c",
    "host/utils.c",
    "host/storing.c",
    "host/progress_bar.c",
    "host/integrate_gpu.c",
]


def _nvcc() -> str:
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(cand):
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libhydro_gb300")
    return cand


def _run(cmd: list[str]) -> str:
    p = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if p.returncode != 0:
        raise RuntimeError("build step failed:\n  " + " ".join(cmd) + "\n" + p.stdout)
    return p.stdout


def _obj(src: str) -> str:
    return os.path.join(BUILD, src.replace("/", "_").rsplit(".", 1)[0] + ".o")


def _stale(obj: str, deps: list[str]) -> bool:
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    return any(os.path.getmtime(d) > t for d in deps)


def _headers() -> list[str]:
    out = []
    for d in (os.path.join(ROOT, "include"), os.path.join(CSRC, "gpu"), os.path.join(CSRC, "host")):
        for f in os.listdir(d):
            if f.endswith((".h", ".cuh")):
                out.append(os.path.join(d, f))
    return out


def build(verbose: bool = False, force: bool = False) -> str:
    """Compile (incrementally) and link; returns the library path."""
    os.makedirs(BUILD, exist_ok=True)
    nvcc = _nvcc()
    headers = _headers()
    jobs = []
    for src, extra in CUDA_SOURCES:
        path = os.path.join(CSRC, src)
        obj = _obj(src)
        if force or _stale(obj, [path, __file__] + headers):
            jobs.append([nvcc, *ARCH, "-O3", "-lineinfo", "-std=c++17", *extra, *EXTRA_NVCC, *INCLUDES,
                         "-Xcompiler", "-fPIC,-ffp-contract=off,-Wall",
                         "-Xptxas", "-v", "-c", path, "-o", obj])
    for src in C_SOURCES:
        path = os.path.join(CSRC, src)
        obj = _obj(src)
        if force or _stale(obj, [path, __file__] + headers):
            jobs.append(["gcc", "-std=gnu11", "-O2", "-fPIC", "-ffp-contract=off", "-Wall",
                         "-Wextra", *INCLUDES, "-c", path, "-o", obj])
    with cf.ThreadPoolExecutor(max_workers=max(2, os.cpu_count() or 2)) as ex:
        for out in ex.map(_run, jobs):
            if verbose and out.strip():
                print(out)
    objs = [_obj(s) for s, _ in CUDA_SOURCES] + [_obj(s) for s in C_SOURCES]
    if force or _stale(LIB, objs):
        _run([nvcc, *ARCH, "-shared", "-cudart", "static", "-o", LIB, *objs, "-lm"])
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, force="-f" in sys.argv))
