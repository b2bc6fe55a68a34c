"""Build recipe of the in-tree CUDA library ``libbnsn_gb300.so`` (sm_103a).

Every ``csrc/*.cu`` is compiled by nvcc for ``sm_103a`` only and the host
utilities by g++, in parallel, then linked into one shared library next to
this file.  Objects go to ``_build/`` (git-ignored).  Rebuilds only what is
older than its sources.
"""

import glob
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(os.path.dirname(HERE), "_build")
LIB = os.path.join(HERE, "libbnsn_gb300.so")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")

NVCC = os.environ.get("NVCC", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVFLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-I", INCLUDE,
           "-Xptxas", "-warn-spills"]
# No floating-point contraction in host code: the synthetic generator and the
# Gauss-Legendre nodes then round alike on x86-64 and aarch64.
CXXFLAGS = ["-O2", "-std=c++17", "-ffp-contract=off", "-fPIC", "-fopenmp", "-I", INCLUDE]


def _deps():
    return glob.glob(os.path.join(CSRC, "*.h")) + glob.glob(os.path.join(CSRC, "*.cuh")) + \
        glob.glob(os.path.join(INCLUDE, "*.h"))


def _stale(target, sources):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(s) > t for s in sources)


def build(verbose=False):
    """Compile and link; returns the library path."""
    os.makedirs(BUILD, exist_ok=True)
    deps = _deps()
    jobs, objs = [], []
    for src in sorted(glob.glob(os.path.join(CSRC, "*.cu"))):
        obj = os.path.join(BUILD, os.path.basename(src) + ".o")
        objs.append(obj)
        if _stale(obj, [src] + deps):
            jobs.append([NVCC] + ARCH + NVFLAGS + ["-c", src, "-o", obj])
    for src in sorted(glob.glob(os.path.join(CSRC, "*.cpp"))):
        obj = os.path.join(BUILD, os.path.basename(src) + ".o")
        objs.append(obj)
        if _stale(obj, [src] + deps):
            jobs.append(["g++"] + CXXFLAGS + ["-c", src, "-o", obj])
    procs = []
    for cmd in jobs:
        if verbose:
            print(" ".join(cmd))
        procs.append((cmd, subprocess.Popen(cmd, stdout=subprocess.PIPE,
                                            stderr=subprocess.STDOUT, text=True)))
    failed = []
    for cmd, p in procs:
        out, _ = p.communicate()
        if p.returncode != 0:
            failed.append((cmd, out))
        elif verbose and out.strip():
            print(out)
    if failed:
        msg = "\n".join(f"$ {' '.join(c)}\n{o}" for c, o in failed)
        raise RuntimeError(f"bns_nurates_gb300 build failed:\n{msg}")
    if jobs or _stale(LIB, objs):
        link = [NVCC] + ARCH + ["-shared", "-o", LIB] + objs + ["-Xcompiler", "-fopenmp"]
        if verbose:
            print(" ".join(link))
        subprocess.check_call(link)
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
