"""Build libphotons_fmm.so (sm_103a) in-tree: one nvcc process per
translation unit, in parallel, then a shared-library link.

    python build.py [--force]
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OBJ = os.path.join(HERE, "_build")
LIBDIR = os.path.join(HERE, "lib")
LIB = os.path.join(LIBDIR, "libphotons_fmm.so")
INCLUDE = os.path.join(ROOT, "include")

SOURCES = ["scan.cu", "tree.cu", "walk.cu", "p2p.cu", "multipole.cu", "api.cu", "legacy.cu", "direct.cu", "noalloc.cu", "domain.cu", "integrate.cu", "snapshot.cu", "pm.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# host code is not contracted into FMAs (the host operators and integrals
# follow the reference's separately rounded arithmetic on every host CPU)
FLAGS = ["-std=c++17", "-O3", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-fvisibility=default",
         "-Xcompiler", "-ffp-contract=off",
         "-I" + INCLUDE, "-I" + CSRC, "-diag-suppress", "177"]


def nvcc():
    cand = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "bin", "nvcc")
    return cand if os.path.exists(cand) else "nvcc"


def _deps_newer(obj, src):
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    for f in os.listdir(CSRC):
        if f.endswith((".cuh", ".h")) and os.path.getmtime(os.path.join(CSRC, f)) > t:
            return True
    if os.path.getmtime(os.path.join(INCLUDE, "photons_fmm.h")) > t:
        return True
    return os.path.getmtime(src) > t


def _compile(src, force):
    s = os.path.join(CSRC, src)
    o = os.path.join(OBJ, src.replace(".cu", ".o"))
    if not force and not _deps_newer(o, s):
        return o, ""
    cmd = [nvcc()] + ARCH + FLAGS + ["-c", s, "-o", o]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("nvcc failed for %s:\n%s\n%s" % (src, " ".join(cmd), r.stdout + r.stderr))
    return o, r.stderr


def build(force=False, verbose=False):
    os.makedirs(OBJ, exist_ok=True)
    os.makedirs(LIBDIR, exist_ok=True)
    with cf.ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 4)) as ex:
        results = list(ex.map(lambda s: _compile(s, force), SOURCES))
    objs = [o for o, _ in results]
    if verbose:
        for _, err in results:
            if err.strip():
                print(err)
    if force or not os.path.exists(LIB) or any(os.path.getmtime(o) > os.path.getmtime(LIB) for o in objs):
        cmd = [nvcc()] + ARCH + ["-shared", "-o", LIB] + objs + ["-lcudart", "-lcufft"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("link failed:\n%s\n%s" % (" ".join(cmd), r.stdout + r.stderr))
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
