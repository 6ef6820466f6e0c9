"""Build of the in-tree CUDA library ``libgbdycore.so`` for sm_103a.

Every translation unit is compiled by nvcc with
``-gencode arch=compute_103a,code=sm_103a -lineinfo -O3`` in parallel, then
linked into a shared library next to this file (git-ignored).
"""
import concurrent.futures as cf
import os
import shutil
import subprocess

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)                      # climaatmos.jl_gb300/
CSRC = os.path.join(ROOT, "csrc")
INCLUDE = os.path.join(os.path.dirname(ROOT), "include")
BUILD = os.path.join(ROOT, "_build")
LIB = os.path.join(PKG, "libgbdycore.so")
SOURCES = ["context.cu", "kernels_se.cu", "kernels_col.cu", "kernels_colg.cu", "columns.cu", "adjoint_se.cu", "adjoint_col.cu", "kernels_misc.cu", "kernels_topo.cu", "geometry.cpp"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc():
    p = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(p):
        raise RuntimeError("nvcc not found: the gbdycore CUDA library cannot be built")
    return p


def _deps():
    files = [os.path.join(CSRC, f) for f in os.listdir(CSRC)] + [os.path.join(INCLUDE, "gbdycore.h")]
    return max(os.path.getmtime(f) for f in files)


def build(force=False, verbose=False, extra=()):
    """Compile (if stale) and return the path of libgbdycore.so."""
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= _deps():
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    cc = nvcc()
    common = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-I", INCLUDE, "-I", CSRC] + list(extra)

    def one(src):
        obj = os.path.join(BUILD, os.path.splitext(src)[0] + ".o")
        cmd = [cc, "-c", os.path.join(CSRC, src), "-o", obj] + common
        if src.endswith(".cu"):
            cmd += ARCH
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed for %s:\n%s%s" % (src, r.stdout, r.stderr))
        if verbose and (r.stdout or r.stderr):
            print(r.stdout + r.stderr)
        return obj

    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(one, SOURCES))
    tmp = LIB + ".tmp"
    cmd = [cc, "-shared", "-o", tmp] + objs + ARCH + ["-ldl"]   # -ldl: NVTX's injection loader
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n%s%s" % (r.stdout, r.stderr))
    os.replace(tmp, LIB)
    return LIB
