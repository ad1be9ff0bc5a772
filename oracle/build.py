"""Build recipe of the oracle (test infrastructure only).

``build_oracle()`` compiles oracle/refbh.c into oracle/_build/liboracle.so with
-ffp-contract=off, so every multiply-add in the restatement is either an explicit fmaf
or a separately rounded multiply and add, on x86 and Arm alike.

``build_reference(n)`` compiles the reference project's own OpenCL kernels
(kernels/nbody/{boundingbox,buildtree,summarizetree,sort,calculateforce,integrate}.cl)
as C++ through oracle/ref_shim.hpp, for a body count n (NBODIES is a compile-time
constant of those kernels), into oracle/_ref/libref_<n>.so.  It needs the reference
sources, so it only runs where they are mounted; the .so never travels.
"""
from __future__ import annotations

import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD_DIR = os.path.join(HERE, "_build")
REF_DIR = os.path.join(HERE, "_ref")
REFERENCE_ROOT = os.environ.get("NBH_REFERENCE_ROOT", "/root/reference")

REF_KERNELS = [
    ("boundingbox", "boundingBox"),
    ("buildtree", "buildTree"),
    ("summarizetree", "summarizeTree"),
    ("sort", "sort"),
    ("calculateforce", "calculateForce"),
    ("integrate", "integrate"),
]


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("oracle build failed: %s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))


def oracle_lib_path() -> str:
    return os.path.join(BUILD_DIR, "liboracle.so")


def build_oracle(force: bool = False) -> str:
    out = oracle_lib_path()
    src = os.path.join(HERE, "refbh.c")
    hdr = os.path.join(HERE, "refbh.h")
    deps = [src, hdr]
    if not force and os.path.exists(out) and all(os.path.getmtime(out) >= os.path.getmtime(d) for d in deps):
        return out
    os.makedirs(BUILD_DIR, exist_ok=True)
    tmp = out + ".tmp%d" % os.getpid()
    _run(["gcc", "-O2", "-std=c11", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off",
          "-fno-fast-math", "-Wall", "-o", tmp, src, "-lm"])
    os.replace(tmp, out)
    return out


def reference_available() -> bool:
    return all(os.path.exists(os.path.join(REFERENCE_ROOT, "kernels", "nbody", f + ".cl"))
               for f, _ in REF_KERNELS)


def reference_number_of_nodes(n: int) -> int:
    # GPUBarnesHutNBodySimulation.java:219-227 with maxComputeUnits = 16, WARPSIZE = 16.
    nn = 2 * n
    if nn < 1024 * 16:
        nn = 1024 * 16
    while nn & 15:
        nn += 1
    return nn


def ref_lib_path(n: int) -> str:
    return os.path.join(REF_DIR, "libref_%d.so" % n)


def build_reference(n: int, force: bool = False) -> str:
    """Compile the reference kernels for NBODIES = n.  Raises if the sources are absent."""
    if not reference_available():
        raise FileNotFoundError("reference kernels not found under %s" % REFERENCE_ROOT)
    out = ref_lib_path(n)
    shim = os.path.join(HERE, "ref_shim.hpp")
    runner = os.path.join(HERE, "ref_emul.cpp")
    if not force and os.path.exists(out) and all(
            os.path.getmtime(out) >= os.path.getmtime(d) for d in (shim, runner)):
        return out
    os.makedirs(REF_DIR, exist_ok=True)
    nn = reference_number_of_nodes(n)
    # Launch geometry of the reference host: 16 groups of 16 work-items
    # (GPUBarnesHutNBodySimulation.java:47-49,126-129,207-217).
    defs = ["-DNUMBER_OF_NODES=%d" % nn, "-DNBODIES=%d" % n, "-DWORKGROUP_SIZE=16",
            "-DNUM_WORK_GROUPS=16"]
    common = ["g++", "-std=c++17", "-fPIC", "-pthread", "-ffp-contract=off",
              "-w", "-I", REFERENCE_ROOT, "-I", HERE] + defs
    objs = []
    for stem, kname in REF_KERNELS:
        obj = os.path.join(REF_DIR, "ref_%s_%d.o" % (stem, n))
        cl = os.path.join(REFERENCE_ROOT, "kernels", "nbody", stem + ".cl")
        # buildtree.cl:47-49 declares currentR, body position and depth inside the retry
        # loop and reads them again after a failed lock; at -O0 each keeps its own stack
        # slot across iterations, which is the behaviour the kernel relies on.
        opt = "-O0" if stem == "buildtree" else "-O2"
        lock = ["-DREF_LOCKSTEP"] if stem == "calculateforce" else []
        _run(common + [opt] + lock + ["-x", "c++", "-include", shim, "-DREF_KERNEL_NAME=" + kname,
                       "-DREF_KERNEL_FILE=\"%s\"" % cl, "-c", os.path.join(HERE, "ref_kernel_tu.cpp"),
                       "-o", obj])
        objs.append(obj)
    robj = os.path.join(REF_DIR, "ref_emul_%d.o" % n)
    _run(common + ["-O2", "-c", runner, "-o", robj])
    tmp = out + ".tmp%d" % os.getpid()
    _run(["g++", "-shared", "-pthread", "-o", tmp] + objs + [robj])
    os.replace(tmp, out)
    return out


if __name__ == "__main__":
    print(build_oracle(force=True))
    for arg in sys.argv[1:]:
        print(build_reference(int(arg), force=True))
