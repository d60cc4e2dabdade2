"""Build libcfdwavemaker_gb300.so in-tree with nvcc for sm_103a.

    python -m cfdwavemaker_gb300.build          (or cfdwavemaker_gb300.build.build())

Each translation unit is compiled in parallel to an object under
cfdwavemaker_gb300/_build/, then linked into a shared library with the static
CUDA runtime, so the library needs only the driver (libcuda) at run time.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libcfdwavemaker_gb300.so")
NVCC = os.environ.get("NVCC", "/usr/local/cuda/bin/nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-fvisibility=hidden",
         "-I" + os.path.join(os.path.dirname(HERE), "include")]
SOURCES = ["parser.cpp", "irregular.cu", "sgrid.cu", "regular.cu", "api.cu", "noalloc.cu", "qform.cu",
           "surrogate.cu", "depthform.cu", "vtu.cpp", "smit.cu", "spectrum.cu", "shard.cpp", "convtc.cu"]


def _compile(src):
    obj = os.path.join(BUILD, os.path.splitext(src)[0] + ".o")
    path = os.path.join(CSRC, src)
    deps = [path, os.path.join(CSRC, "cfdwm.h"), os.path.join(CSRC, "sgrid_geom.cuh"), os.path.join(CSRC, "ffmath.cuh"),
            os.path.join(CSRC, "tc05.cuh"), os.path.join(CSRC, "ramp.cuh"),
            os.path.join(os.path.dirname(HERE), "include", "cfdwavemaker_gb300.h")]
    if os.path.exists(obj) and all(os.path.getmtime(obj) >= os.path.getmtime(d) for d in deps):
        return obj, ""
    cmd = [NVCC] + ARCH + FLAGS + ["-c", path, "-o", obj]
    if src.endswith(".cpp"):
        cmd = [NVCC] + FLAGS + ["-x", "c++", "-c", path, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("nvcc failed for %s:\n%s\n%s" % (src, " ".join(cmd), r.stderr))
    return obj, r.stderr


def build(verbose: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        results = list(ex.map(_compile, SOURCES))
    objs = [o for o, _ in results]
    if verbose:
        for _, log in results:
            if log:
                sys.stderr.write(log)
    if (not os.path.exists(LIB)) or any(os.path.getmtime(o) > os.path.getmtime(LIB) for o in objs):
        cmd = [NVCC] + ARCH + ["-shared", "-cudart", "static", "-o", LIB] + objs
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("link failed:\n%s\n%s" % (" ".join(cmd), r.stderr))
    return LIB


if __name__ == "__main__":
    print(build(verbose=True))
