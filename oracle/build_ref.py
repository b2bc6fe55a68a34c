"""Build recipe for oracle/_ref: the reference bns_nurates compiled from its
own headers where they lie, in their no-Kokkos shim mode.

Test infrastructure only.  Everything it writes goes to oracle/_ref/ (git
ignored).  Steps:

1. ``oracle/_ref/gen/GP19Table.hpp``: the GP19 table header is a missing large
   blob in the reference (``.MISSING_LARGE_BLOBS``), so a header carrying the
   synthetic table of ``bns_nurates_gb300/gp19_synthetic.py`` is generated, with
   every value written as an exact hex-float literal.  The GPU path and the
   oracle restatement load the very same numbers.
2. ``oracle/_ref/gen40/bns_nurates.hpp``: ``BS_N_MAX`` is hard-wired to 20 in
   ``include/bns_nurates.hpp:68`` (no ``#ifndef`` guard), which limits the
   reference to n <= 10 quadrature nodes per half-interval.  A generated copy of
   that one header with ``BS_N_MAX 40`` is force-included first (``-include``);
   its include guard then shadows the original, so n = 20 runs too.  Results at
   n <= 10 are identical to the unmodified build.
3. ``libbnsn_ref.so`` from ``oracle/ref_driver.cpp`` and ``ref_layout`` (struct
   layout probe, built against the unmodified headers).

Flags: ``-O2 -ffp-contract=off`` (no FMA contraction, so results do not depend
on the host ISA), OpenMP for the batch drivers.

Timing build (``build_native``): the same driver and headers compiled the way
a user builds the reference for speed, ``-O3 -march=native`` (``-mcpu=native``
on aarch64) with OpenMP, into ``oracle/_ref/libbnsn_ref_native.so``.  The
benchmark times it as the CPU baseline.  Because the benchmark host has no
reference checkout, ``stage()`` keeps a copy of the reference's ``include/``
headers in the git-ignored ``oracle/_ref/src/include`` (it travels with the
working tree, never into the repository's history); ``build_native`` compiles
from the checkout when present, else from that staged copy.
"""

import glob
import importlib.util
import os
import platform
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
# The reference checkout: BNSN_REFERENCE_DIR, else a sibling of this repository.
REF = os.environ.get("BNSN_REFERENCE_DIR") or os.path.join(os.path.dirname(REPO), "reference")
OUT = os.path.join(HERE, "_ref")


def _load_gp19():
    path = os.path.join(REPO, "bns_nurates_gb300", "gp19_synthetic.py")
    spec = importlib.util.spec_from_file_location("gp19_synthetic", path)
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod.table()


def _arr(name, vals):
    body = ",\n    ".join(float(v).hex() for v in vals)
    return f"inline constexpr BS_REAL {name}[{len(vals)}] = {{\n    {body}}};\n"


def write_gp19_header(path):
    t = _load_gp19()
    nbd, yed, td, wd = t["dims"]
    src = [
        "// Generated by oracle/build_ref.py: SYNTHETIC stand-in for the GP19 table.\n",
        "#ifndef BNSN_SYNTH_GP19_TABLE_HPP_\n#define BNSN_SYNTH_GP19_TABLE_HPP_\n",
        f"inline constexpr int GP19_nb_dims = {nbd};\n",
        f"inline constexpr int GP19_Ye_dims = {yed};\n",
        f"inline constexpr int GP19_T_dims = {td};\n",
        f"inline constexpr int GP19_w_dims = {wd};\n",
        _arr("GP19_nb_axis", t["nb"]),
        _arr("GP19_lognb_axis", t["lognb"]),
        _arr("GP19_Ye_axis", t["ye"]),
        _arr("GP19_T_axis", t["t"]),
        _arr("GP19_w_axis", t["w"]),
        _arr("GP19_logw_axis", t["logw"]),
        _arr("GP19_data", t["data"]),
        "#endif\n",
    ]
    with open(path, "w") as f:
        f.write("".join(src))


def write_nmax40_header(path, inc):
    with open(os.path.join(inc, "bns_nurates.hpp")) as f:
        text = f.read()
    old = "#define BS_N_MAX 20"
    if old not in text:
        raise RuntimeError("BS_N_MAX definition not found in reference header")
    with open(path, "w") as f:
        f.write(text.replace(old, "#define BS_N_MAX 40", 1))


STAGED = os.path.join(OUT, "src", "include")
NATIVE_SO = os.path.join(OUT, "libbnsn_ref_native.so")


def _include_dir():
    """The reference headers: the checkout, else the staged copy, else None."""
    for d in (os.path.join(REF, "include"), STAGED):
        if os.path.isfile(os.path.join(d, "m1_opacities.hpp")):
            return d
    return None


def stage():
    """Copy the checkout's include/*.hpp into oracle/_ref/src/include."""
    src = os.path.join(REF, "include")
    if not os.path.isdir(src):
        return False
    os.makedirs(STAGED, exist_ok=True)
    for f in glob.glob(os.path.join(src, "*.hpp")):
        dst = os.path.join(STAGED, os.path.basename(f))
        if os.path.exists(dst):
            os.chmod(dst, 0o644)
        shutil.copyfile(f, dst)
    return True


def _generated(inc):
    gen = os.path.join(OUT, "gen")
    gen40 = os.path.join(OUT, "gen40")
    os.makedirs(gen, exist_ok=True)
    os.makedirs(gen40, exist_ok=True)
    write_gp19_header(os.path.join(gen, "GP19Table.hpp"))
    write_nmax40_header(os.path.join(gen40, "bns_nurates.hpp"), inc)
    return gen, gen40


def build_native(verbose=False):
    """Optimised build of the reference for timing; returns its path or None."""
    inc = _include_dir()
    if inc is None:
        return None
    drv = os.path.join(HERE, "ref_driver.cpp")
    if os.path.exists(NATIVE_SO) and os.path.getmtime(NATIVE_SO) >= max(
            os.path.getmtime(f) for f in glob.glob(os.path.join(inc, "*.hpp")) + [drv]):
        return NATIVE_SO
    gen, gen40 = _generated(inc)
    arch = "-mcpu=native" if platform.machine() in ("aarch64", "arm64") else "-march=native"
    cmd = ["g++", "-std=c++17", "-O3", arch, "-fopenmp", "-fPIC", "-shared", "-w",
           "-include", os.path.join(gen40, "bns_nurates.hpp"), "-I", gen, "-I", inc,
           drv, "-o", NATIVE_SO]
    if verbose:
        print(" ".join(cmd))
    if subprocess.call(cmd) != 0:
        return None
    return NATIVE_SO


def build(verbose=False):
    if not os.path.isdir(os.path.join(REF, "include")):
        if verbose:
            print(f"build_ref: reference not present at {REF}; skipped")
        return False
    stage()
    inc = os.path.join(REF, "include")
    gen, gen40 = _generated(inc)
    lib = [
        "g++", "-std=c++17", "-O2", "-ffp-contract=off", "-fopenmp", "-fPIC", "-shared",
        "-w", "-include", os.path.join(gen40, "bns_nurates.hpp"),
        "-I", gen, "-I", inc,
        os.path.join(HERE, "ref_driver.cpp"), "-o", os.path.join(OUT, "libbnsn_ref.so"),
    ]
    lay = [
        "g++", "-std=c++17", "-O0", "-w", "-I", inc,
        os.path.join(HERE, "ref_layout.cpp"), "-o", os.path.join(OUT, "ref_layout"),
    ]
    procs = [subprocess.Popen(c) for c in (lib, lay)]
    rcs = [p.wait() for p in procs]
    if any(rcs):
        raise RuntimeError(f"build_ref: compilation failed ({rcs})")
    if verbose:
        print("build_ref: built", OUT)
    return True


if __name__ == "__main__":
    sys.exit(0 if build(verbose=True) else 1)
