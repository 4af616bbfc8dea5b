"""Builds the GB300 library (and, for the tests, the CPU oracle) in-tree.

    python -m miniamr_gb300.build

compiles miniamr_gb300/csrc/*.cu (+ host_init.cpp) for sm_103a with nvcc,
one translation unit per process in parallel, and links
miniamr_gb300/_build/libminiamr_gb300.so.  Objects are rebuilt only when a
source or header is newer.  FP64 bit-exactness needs -fmad=false: no
multiply-add is contracted anywhere (the correctly rounded divisions use
explicit __fma_rn, which the flag does not touch).
"""
from __future__ import annotations

import glob
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libminiamr_gb300.so")
INCLUDE = os.path.join(REPO, "include")
ORACLE_DIR = os.path.join(REPO, "oracle")
ORACLE_LIB = os.path.join(ORACLE_DIR, "_build", "libmamr_oracle.so")

NVCC = os.environ.get("NVCC", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVFLAGS = ARCH + ["-O3", "-lineinfo", "-fmad=false", "-std=c++17",
                  "-Xcompiler", "-fPIC", "-Xcompiler", "-fopenmp",
                  "-I" + INCLUDE, "-I" + CSRC]


def _sources():
    return sorted(glob.glob(os.path.join(CSRC, "*.cu")) +
                  glob.glob(os.path.join(CSRC, "*.cpp")))


def _headers():
    return (glob.glob(os.path.join(CSRC, "*.h")) +
            glob.glob(os.path.join(CSRC, "*.cuh")) +
            [os.path.join(INCLUDE, "miniamr_gb300.h")])


def _newer(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("command failed: " + " ".join(cmd) + "\n" +
                           r.stdout + r.stderr)
    return r


def build_library(verbose: bool = False) -> str:
    os.makedirs(OUT, exist_ok=True)
    headers = _headers()
    jobs = []
    objs = []
    for src in _sources():
        obj = os.path.join(OUT, os.path.basename(src) + ".o")
        objs.append(obj)
        if _newer(obj, [src] + headers):
            jobs.append([NVCC] + NVFLAGS + ["-c", src, "-o", obj])
    if jobs:
        with ThreadPoolExecutor(max_workers=min(8, len(jobs))) as ex:
            for r in ex.map(_run, jobs):
                if verbose and (r.stdout or r.stderr):
                    print(r.stdout + r.stderr)
    if jobs or _newer(LIB, objs):
        _run([NVCC] + ARCH + ["-shared", "-Xcompiler", "-fPIC",
                              "-Xcompiler", "-fopenmp", "-o", LIB] +
             objs + ["-cudart", "static"])
    return LIB


def build_oracle() -> str:
    """The CPU oracle (test infrastructure): plain gcc, no reference needed."""
    _run(["make", "-s", "-C", ORACLE_DIR, "oracle"])
    return ORACLE_LIB


def reference_sources() -> str | None:
    """The reference's ref/ directory: MAMR_REFERENCE_SRC, else the ref/
    directory of a miniAMR checkout named "reference" beside this
    repository; None when neither exists."""
    ref = os.environ.get("MAMR_REFERENCE_SRC")
    if not ref:
        ref = os.path.join(os.path.dirname(REPO), "reference", "ref")
    ok = os.path.isfile(os.path.join(ref, "stencil.c"))
    return ref if ok else None


def build_reference_binaries() -> bool:
    """oracle/_ref/ binaries, from the reference sources when present."""
    ref = reference_sources()
    if ref is None:
        return False
    _run(["make", "-s", "-j8", "-C", ORACLE_DIR, "ref", "hybrid",
          "REF=" + ref])
    return True


def main(argv=None):
    lib = build_library(verbose=True)
    print(lib)
    print(build_oracle())
    if build_reference_binaries():
        print("reference binaries built under oracle/_ref/")


if __name__ == "__main__":
    sys.exit(main())
