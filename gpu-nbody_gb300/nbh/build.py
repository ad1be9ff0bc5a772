"""In-tree build of libnbh.so for sm_103a (GB300).

Each translation unit is compiled in parallel with nvcc
(-gencode arch=compute_103a,code=sm_103a, -O3, -lineinfo) and linked into
gpu-nbody_gb300/nbh/libnbh.so.  Rebuilds only when a source is newer than the library.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess

PKG = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(os.path.dirname(PKG), "csrc")
ROOT = os.path.dirname(os.path.dirname(PKG))
INCLUDE = os.path.join(ROOT, "include")
OBJ_DIR = os.path.join(os.path.dirname(PKG), "_build")
LIB = os.path.join(PKG, "libnbh.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
SOURCES = ["nbh_api.cu", "nbh_tree.cu", "nbh_force.cu", "nbh_theta.cu", "nbh_aux.cu", "nbh_diag.cu",
           "nbh_host.cpp"]


def nvcc() -> str:
    for c in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    raise FileNotFoundError("nvcc not found")


def _deps():
    out = [os.path.join(CSRC, f) for f in os.listdir(CSRC)]
    out.append(os.path.join(INCLUDE, "nbh.h"))
    return out


def up_to_date() -> bool:
    if not os.path.exists(LIB):
        return False
    t = os.path.getmtime(LIB)
    return all(os.path.getmtime(d) <= t for d in _deps())


def _compile(src: str, verbose: bool) -> str:
    obj = os.path.join(OBJ_DIR, os.path.splitext(src)[0] + ".o")
    cmd = [nvcc(), "-std=c++17", "-O3", "-lineinfo", "-Xcompiler", "-fPIC", "-I", INCLUDE,
           "-c", os.path.join(CSRC, src), "-o", obj] + ARCH
    if src.endswith(".cu"):
        cmd += ["--expt-relaxed-constexpr"]
        if verbose:
            cmd += ["-Xptxas", "-v"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("nvcc failed on %s:\n%s\n%s" % (src, " ".join(cmd), r.stderr))
    if verbose and r.stderr:
        print(r.stderr)
    return obj


def build(force: bool = False, verbose: bool = False) -> str:
    if not force and up_to_date():
        return LIB
    os.makedirs(OBJ_DIR, exist_ok=True)
    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(lambda s: _compile(s, verbose), SOURCES))
    tmp = LIB + ".tmp%d" % os.getpid()
    cmd = [nvcc(), "-shared", "-o", tmp] + objs + ARCH + ["-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n%s\n%s" % (" ".join(cmd), r.stderr))
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    import sys
    print(build(force=True, verbose="-v" in sys.argv))
