"""Operation counts of the reference algorithm (measurement infrastructure).

Compiles ``oracle/opcount.cpp``: the reference's own headers with BS_REAL set
to a counting real type (the reference makes the real type a macro,
``include/bns_nurates.hpp:29-34``).  Every floating-point operation and math
call of a grey point is counted and attributed to the reference function it
happens in (distribution reconstruction, TotalNuF, AbsOpacity/StimAbsOpacity,
IsoScattTotal, PairKernels, the three bremsstrahlung kernels,
InelasticScattKernels) or to the integrand assembly and quadrature sums
around them.

Run with each reaction switched on alone, this gives the reference's work per
point for each reaction, i.e. for each phase kernel of the GPU path:

  work(reaction) = assembly + kernel calls + TotalNuF at distinct arguments

(the reference re-evaluates the reconstructed distribution TotalNuF at the
same energy for many cells; only distinct (energy, species) evaluations are
counted as algorithmic work).  FLOP = add/sub + mul + div + sqrt, one each;
transcendental = exp + log + pow + other libm calls, one each; work = FLOP +
transcendental.  Comparisons, fabs/fmin/fmax and rounding are not counted.

Writes ``profiles/op_counts.json``; the benchmark reads it as the algorithmic
work per point of each phase.  Needs the reference headers (the checkout or
the staged copy of oracle/build_ref.py).

    python oracle/opcount.py [--points 256]
"""

import argparse
import ctypes
import json
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
sys.path.insert(0, REPO)

from oracle import build_ref  # noqa: E402

OUT = os.path.join(build_ref.OUT, "libbnsn_opcount.so")
GEN_COUNT = os.path.join(build_ref.OUT, "gen_count")
FIELDS = ("add", "mul", "div", "sqrt", "exp", "log", "pow", "transc", "cmp", "minmax")
COUNTED = ("assembly", "distr", "TotalNuF", "AbsOpacity", "StimAbsOpacity", "IsoScattTotal",
           "PairKernels", "BremKernelsLegCoeff", "BremKernelsBRT06", "BremKernelAbsGP19",
           "InelasticScattKernels")
SEED = 20261203

WORKLOADS = {
    # name: (flags, pars, n, description)
    "c5": ((1, 1, 1, 1, 1), (1, 0, 1, 1, 1, 2, 1, 0), 20,
           "all reactions (beta+WM+mean field, iso, pair, GP19 brem, NES/NPS), n=20"),
    "c3": ((1, 1, 1, 0, 1), (1, 0, 1, 1, 1, 0, 1, 0), 10, "beta + iso + pair + HR98, n=10"),
}
# reaction -> flags (abs_em, pair, brem, inelastic, iso) and the GPU phase it maps to
REACTIONS = {
    "beta": ((1, 0, 0, 0, 0), "prelude"),
    "iso": ((0, 0, 0, 0, 1), "prelude"),
    "pair": ((0, 1, 0, 0, 0), "pair"),
    "brem": ((0, 0, 1, 0, 0), "brem"),
    "nes": ((0, 0, 0, 1, 0), "neps"),
}


def build():
    inc = build_ref._include_dir()
    if inc is None:
        raise RuntimeError("reference headers not found (checkout or staged copy)")
    gen, gen40 = build_ref._generated(inc)
    os.makedirs(GEN_COUNT, exist_ok=True)
    # Two generated copies of reference headers, included ahead of the
    # originals (their include guards then shadow them).
    # integration.hpp:39-40 assign BS_REAL expressions to double locals; the
    # counting type converts to double only explicitly, so the generated copy
    # adds the two casts (no-ops for the plain double build)
    with open(os.path.join(inc, "integration.hpp")) as f:
        text = f.read()
    for v, op in (("xm", "+"), ("xl", "-")):
        old = f"    {v}    = 0.5 * (quad->x2 {op} quad->x1);"
        if old not in text:
            raise RuntimeError(f"integration.hpp: line of {v} not found")
        text = text.replace(old, f"    {v}    = (double)(0.5 * (quad->x2 {op} quad->x1));")
    with open(os.path.join(GEN_COUNT, "integration.hpp"), "w") as f:
        f.write(text)
    # constants.hpp:204-206 pick the exp cut-off by type (700 for double, 80
    # otherwise); the generated copy gives the counting type double's 700, so
    # the counting build computes exactly what the double build computes
    with open(os.path.join(inc, "constants.hpp")) as f:
        text = f.read()
    start = text.index("inline constexpr BS_REAL kBS_ExpUppLim")
    end = text.index(";", start)
    decl = text[start:end]
    if "? 700 :" not in decl or not decl.rstrip().endswith("80"):
        raise RuntimeError("constants.hpp: kBS_ExpUppLim not in the expected form")
    text = text[:start] + decl.rstrip()[:-2] + "700" + text[end:]
    with open(os.path.join(GEN_COUNT, "constants.hpp"), "w") as f:
        f.write(text)
    subprocess.check_call([
        "g++", "-std=c++20", "-O1", "-ffp-contract=off", "-fPIC", "-shared", "-w",
        "-I", GEN_COUNT, "-I", gen40, "-I", gen, "-I", inc,
        os.path.join(HERE, "opcount.cpp"), "-o", OUT])
    return OUT


def count(lib, eos, m1, flags, pars, x, w):
    n = eos.shape[1]
    calls = np.zeros(len(COUNTED), dtype=np.uint64)
    counts = np.zeros((len(COUNTED), len(FIELDS)), dtype=np.uint64)
    nuf = ctypes.c_uint64(0)
    out = np.zeros((20, n))
    f = lib.opcount_m1
    P = ctypes.c_void_p
    f.argtypes = [ctypes.c_int64, P, P, P, P, ctypes.c_int, P, P, P, P, P, P]
    f.restype = ctypes.c_int
    fl = np.asarray(flags, dtype=np.int32)
    pa = np.asarray(pars, dtype=np.int32)
    rc = f(n, eos.ctypes.data, m1.ctypes.data, fl.ctypes.data, pa.ctypes.data, len(x),
           x.ctypes.data, w.ctypes.data, calls.ctypes.data, counts.ctypes.data,
           ctypes.byref(nuf), out.ctypes.data)
    if rc:
        raise RuntimeError(f"opcount_m1 failed ({rc})")
    return calls.astype(float) / n, counts.astype(float) / n, nuf.value / n, out


def _ops(row):
    d = dict(zip(FIELDS, row))
    flop = d["add"] + d["mul"] + d["div"] + d["sqrt"]
    transc = d["exp"] + d["log"] + d["pow"] + d["transc"]
    return flop, transc, d


def summarise(calls, counts, nuf_distinct, detail=False):
    """Per function: calls per point and operations per call (by kind with
    detail); the reaction's algorithmic work per point (TotalNuF at distinct
    arguments only)."""
    funcs, work_flop, work_tr = {}, 0., 0.
    for k, name in enumerate(COUNTED):
        flop, tr, d = _ops(counts[k])
        c = calls[k] if name != "assembly" else 1.
        if name != "assembly" and c == 0:
            continue
        per = {"calls_per_point": c,
               "flop_per_call": flop / c, "transcendental_per_call": tr / c}
        if detail:
            per["ops_per_call"] = {f: v / c for f, v in d.items()}
        funcs[name] = per
        if name == "TotalNuF":
            per["distinct_calls_per_point"] = nuf_distinct
            work_flop += nuf_distinct * flop / c
            work_tr += nuf_distinct * tr / c
        elif name != "distr":
            work_flop += flop
            work_tr += tr
    executed = [_ops(counts[k]) for k in range(len(COUNTED))]
    return {"functions": funcs,
            "work_per_point": {"flop": work_flop, "transcendental": work_tr,
                               "work": work_flop + work_tr},
            "reference_executed_per_point": {
                "flop": sum(e[0] for e in executed), "transcendental": sum(e[1] for e in executed),
                "note": "everything the reference evaluates for the point, including the "
                        "distribution reconstruction and repeated TotalNuF calls"}}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--points", type=int, default=256)
    ap.add_argument("--out", default=os.path.join(REPO, "profiles", "op_counts.json"))
    args = ap.parse_args()
    import oracle
    oracle.build()
    lib = ctypes.CDLL(build())
    port = oracle.port()
    ref = oracle.ref()
    eos, m1 = port.synthetic_points(SEED, args.points)
    res = {"_doc": __doc__.strip().split("\n\n")[1].replace("\n", " ") + " Command: python "
           "oracle/opcount.py --points %d; sample: the first %d points of the seeded "
           "synthetic workload (seed %d)." % (args.points, args.points, SEED)}
    for wl, (flags, pars, nq, desc) in WORKLOADS.items():
        x, w = port.gauss_legendre(nq)
        entry = {"workload": desc, "points": args.points, "reactions": {}, "phases": {}}
        calls, counts, nuf, out = count(lib, eos, m1, flags, pars, x, w)
        entry["all_reactions"] = summarise(calls, counts, nuf, detail=True)
        if ref is not None:
            want = ref.m1_opacities(eos, m1, flags, pars, (x, w))
            entry["outputs_equal_plain_build"] = float(np.mean(out == want))
        # distribution reconstruction: once per point, part of the prelude
        distr = entry["all_reactions"]["functions"]["distr"]
        dwork = distr["flop_per_call"] + distr["transcendental_per_call"]
        for rx, (rflags, phase) in REACTIONS.items():
            on = tuple(a & b for a, b in zip(rflags, flags))
            if not any(on):
                continue
            calls, counts, nuf, _ = count(lib, eos, m1, on, pars, x, w)
            base_calls, base_counts, base_nuf, _ = count(lib, eos, m1, (0, 0, 0, 0, 0), pars,
                                                         x, w)
            r = summarise(calls - base_calls, counts - base_counts, nuf - base_nuf)
            entry["reactions"][rx] = r
            ph = entry["phases"].setdefault(phase, {"flop": 0., "transcendental": 0.,
                                                    "work": 0.})
            for k in ("flop", "transcendental", "work"):
                ph[k] += r["work_per_point"][k]
        # orchestration with every reaction off (the s_beta scale's FDIs,
        # thresholds, zeroed outputs) and the distribution reconstruction
        # belong to the per-point constants of the prelude phase
        _, base_counts, _, _ = count(lib, eos, m1, (0, 0, 0, 0, 0), pars, x, w)
        bflop, btr, _ = _ops(base_counts[0])
        pre = entry["phases"].setdefault("prelude", {"flop": 0., "transcendental": 0.,
                                                     "work": 0.})
        pre["flop"] += distr["flop_per_call"] + bflop
        pre["transcendental"] += distr["transcendental_per_call"] + btr
        pre["work"] += dwork + bflop + btr
        entry["work_per_point"] = sum(p["work"] for p in entry["phases"].values())
        res[wl] = entry
    with open(args.out, "w") as f:
        json.dump(res, f, indent=1, sort_keys=False)
        f.write("\n")
    for wl in WORKLOADS:
        print(wl, {k: round(v["work"]) for k, v in res[wl]["phases"].items()},
              "total", round(res[wl]["work_per_point"]))


if __name__ == "__main__":
    main()
