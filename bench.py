"""Benchmark of the grey M1 opacity path on GB300.

Metric: grey M1 opacity points/s of the mixed-precision path, with the plain
FP64 GPU path timed on the same points and the mixed-vs-FP64 relative error
reported beside it.

One step = the grey M1 opacities (ComputeM1Opacities semantics: all 20
outputs, 4 species, stimulated absorption) of one batch of points:

  c5 (default) : 256^3 all-reactions workload (beta with weak magnetism and
                 mean-field shift, iso scattering, e+e- pair, GP19 brem on the
                 synthetic table, NES/NPS), n = 20.  A step is one
                 256 x 256 x 16 slab = 1,048,576 points.
  c3           : the 128^3 patch, beta + iso + pair + HR98, n = 10 (whole patch).
  c2           : as c3 (the FP64 configuration of the same patch).
  c1           : 4096 points, beta + iso + pair + HR98, n = 10.

Keys of the JSON line:
  value        : points/s of --precision (default mixed) with inputs and outputs
                 resident in HBM; CUDA events around K steps (max over ranks).
  fp64_gpu     : the plain FP64 path on the same points (--precision mixed).
  accuracy     : max / p99 relative error of mixed vs FP64 over every output.
  e2e          : points/s through the host-buffer C-ABI call
                 bnsn_m1_opacities_host (pinned host buffers, host<->device
                 copies inside the timed region).
  roofline     : the kernel phase with the largest device time, its FP64 work
                 per point from an ncu instruction count
                 (profiles/bench_constants.json) over its event-timed duration,
                 against the FP64 peak measured in this run by a DFMA probe.
  cpu_baseline : the reference algorithm (C restatement in oracle/, pinned
                 bit-for-bit to the reference build) on all host cores, on a
                 bounded sample of the same points.

``--impl reference`` times that CPU implementation alone on the same workload,
each step a bounded sample.
"""

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, REPO)

SEED = 20261203
# The metric of both arms (this library and the reference's CPU code); the
# mixed-vs-FP64 comparison is reported under "fp64_gpu" and "accuracy".
METRIC = "grey M1 opacity points/s"
BREM_NAMES = ["HR98", "BRT06", "GP19"]
WORKLOADS = {
    "c1": dict(npts=4096, flags=(1, 1, 1, 0, 1), brem=0, nq=10,
               desc="4096 points, beta+iso+pair+HR98, n=10"),
    "c2": dict(npts=128 ** 3, flags=(1, 1, 1, 0, 1), brem=0, nq=10,
               desc="128^3 = 2,097,152 points, beta+iso+pair+HR98, n=10"),
    "c3": dict(npts=128 ** 3, flags=(1, 1, 1, 0, 1), brem=0, nq=10,
               desc="128^3 = 2,097,152 points, beta+iso+pair+HR98, n=10"),
    "c4": dict(npts=0, flags=None, brem=None, nq=None,
               desc="1536 AMR blocks, edges {8,16,24,32,48,64} (weights .55/.28/.09/.05/.025/"
                    ".005, ~12.9M points), per block: brem HR98/BRT06/GP19, NES on/off, n=10 "
                    "(rho<1e11) or 20; one step = one replay of the CUDA graph of the tuned "
                    "plan over all blocks"),
    "aux": dict(npts=1 << 24, flags=None, brem=None, nq=None,
                desc="auxiliary batched kernels on 16,777,216 arguments/points: the Fermi-Dirac "
                     "family FDI_m92..FDI_p212, CalculateDistrParamsFromM1, NuEquilibriumParams"),
    "c5": dict(npts=256 * 256 * 16, flags=(1, 1, 1, 1, 1), brem=2, nq=20,
               desc="256^3 all reactions (beta+WM+mean field, iso, pair, GP19 brem, NES/NPS), "
                    "n=20; one step = one 256x256x16 slab = 1,048,576 points"),
}


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="c5", choices=sorted(WORKLOADS))
    ap.add_argument("--precision", default="mixed", choices=["fp64", "mixed"])
    ap.add_argument("--npts", type=int, default=0, help="override the points per step")
    ap.add_argument("--cpu-seconds", type=float, default=15.0,
                    help="target CPU time of the cpu_baseline sample")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-fp64", action="store_true", help="skip the FP64 comparison")
    ap.add_argument("--no-spectral", action="store_true",
                    help="skip the spectral leg of the c2/c5 workloads")
    ap.add_argument("--spectral-npts", type=int, default=262144,
                    help="points of the spectral leg (24 energies each)")
    ap.add_argument("--full-parity", action="store_true",
                    help="check the FP64 GPU path on every point against the CPU oracle "
                         "instead of benchmarking")
    ap.add_argument("--spectral-stride", type=int, default=64,
                    help="spectral sample of --full-parity: every k-th point")
    ap.add_argument("--no-grey-parity", action="store_true",
                    help="--full-parity: spectral part only")
    ap.add_argument("--cond-npts", type=int, default=262144,
                    help="points of the grey conditioning probe")
    return ap.parse_args()


def dist_info():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")
        for line in self.lines:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 8:
                continue
            try:
                sm.append(float(parts[0]))
                mx.append(float(parts[1]))
            except ValueError:
                continue
            for nme, v in zip(names, parts[4:8]):
                if v.lower() == "active":
                    reasons.add(nme)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx),
                "reasons": sorted(reasons), "samples": len(sm)}


def load_json(*path):
    try:
        with open(os.path.join(REPO, *path)) as f:
            return json.load(f)
    except OSError:
        return {}


def cpu_impl():
    """The CPU implementation timed as the baseline: the reference's own
    headers built with -O3 for the host CPU and OpenMP (oracle/build_ref.py,
    kind "reference"), else the C restatement in oracle/ (kind "port")."""
    import oracle
    oracle.build()
    r = oracle.ref_native()
    if r is not None:
        return r, "reference", "reference headers, g++ -O3 -march/-mcpu=native -fopenmp"
    return oracle.port(), "port", "C restatement (oracle/bnsn_oracle.c), gcc -O2 -fopenmp"


def cpu_rate(impl, eos, m1, wl, n, nthreads):
    """Reference algorithm on host cores: points/s of the first n points."""
    q = impl.gauss_legendre(wl["nq"])
    pars = (1, 0, 1, 1, 1, wl["brem"], 1, 0)
    t0 = time.perf_counter()
    impl.m1_opacities(eos[:, :n], m1[:, :n], wl["flags"], pars, q, nthreads=nthreads)
    dt = time.perf_counter() - t0
    return n / dt, dt


def cpu_sample_size(impl, eos, m1, wl, seconds, nthreads, cap):
    """Points the CPU processes in about `seconds` (pilot of 8 points/thread)."""
    pilot = min(cap, 8 * nthreads)
    rate, _ = cpu_rate(impl, eos, m1, wl, pilot, nthreads)
    return int(max(pilot, min(cap, rate * seconds)))


def setup_gp19(bn, wl):
    if wl["brem"] == 2:
        from bns_nurates_gb300 import gp19_synthetic
        bn.set_gp19_table(gp19_synthetic.table())


def run_reference(args, rank, world):
    """The reference arm: the reference's CPU implementation on the host cores.
    Inputs come from the oracle's copy of the seeded generator, so this arm
    loads nothing from the product library."""
    if rank != 0:
        return
    import oracle
    wl = dict(WORKLOADS[args.workload])
    nthreads = os.cpu_count()
    if args.workload == "aux":
        print(json.dumps({"impl": "reference", "unavailable": "the aux workload times library "
                          "kernels only; the reference has no batched form of them"}))
        return
    impl, kind, how = cpu_impl()
    if args.workload == "c4":
        run_reference_blocks(args, wl, nthreads, impl, kind, how)
        return
    if args.npts:
        wl["npts"] = args.npts
    cap = min(wl["npts"], 1 << 18)
    eos, m1 = oracle.port().synthetic_points(SEED, cap)
    per_step = max(2.0, min(args.cpu_seconds, 150.0 / max(1, args.steps + args.warmup)))
    n = cpu_sample_size(impl, eos, m1, wl, per_step, nthreads, cap)
    for _ in range(args.warmup):
        cpu_rate(impl, eos, m1, wl, min(n, 4 * nthreads), nthreads)
    rates = [cpu_rate(impl, eos, m1, wl, n, nthreads)[0] for _ in range(args.steps)]
    value = statistics.median(rates)
    sample = f"first {n} points of the {args.workload} workload per step"
    line = {
        "impl": "reference", "metric": METRIC, "value": value,
        "unit": "points/s", "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * n / value, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded generator)",
        "config": {"workload": wl["desc"], "sample_points_per_step": n,
                   "reactions": wl["flags"], "brem": BREM_NAMES[wl["brem"]], "nquad": wl["nq"],
                   "precision": "fp64 (reference CPU algorithm)", "build": how},
        "cpu_baseline": {"value": value, "unit": "points/s", "cores": nthreads, "kind": kind,
                         "sample": sample, "build": how},
        "e2e": {"value": value, "unit": "points/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))


def run_reference_blocks(args, wl, nthreads, impl, kind, how):
    """Reference algorithm on the host cores for the AMR-block workload: per
    block (its reactions, brem and n) over the leading blocks, up to about
    --cpu-seconds of work per step."""
    import oracle
    blocks, n = c4_blocks(SEED, 1536, None)
    cap = min(n, 1 << 17)
    eos, m1 = oracle.port().synthetic_points(SEED, cap)
    rho = eos[0] * 1.66053906892e-24 * 1e21
    port = impl

    def sample(npts):
        done, t0 = 0, time.perf_counter()
        for first, count, flags, brem, _ in blocks:
            if first + count > cap or done >= npts:
                break
            nq = 10 if rho[first] < 1e11 else 20
            sl = slice(first, first + count)
            port.m1_opacities(np.ascontiguousarray(eos[:, sl]), np.ascontiguousarray(m1[:, sl]),
                              flags, (1, 0, 1, 1, 1, brem, 1, 0), port.gauss_legendre(nq),
                              nthreads=nthreads)
            done += count
        return done, time.perf_counter() - t0

    d, dt = sample(4096)
    target = max(1024, int(d / dt * max(2.0, min(args.cpu_seconds, 150.0 /
                                                   max(1, args.steps + args.warmup)))))
    for _ in range(args.warmup):
        sample(1024)
    rates = []
    for _ in range(args.steps):
        d, dt = sample(target)
        rates.append(d / dt)
    value = statistics.median(rates)
    print(json.dumps({
        "impl": "reference", "metric": METRIC, "value": value,
        "unit": "points/s", "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * d / value, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded generator)",
        "config": {"workload": wl["desc"], "sample": f"leading blocks, ~{target} points per step",
                   "precision": "fp64 (reference CPU algorithm)", "build": how},
        "cpu_baseline": {"value": value, "unit": "points/s", "cores": nthreads, "kind": kind,
                         "sample": f"leading blocks of the AMR workload, ~{target} points",
                         "build": how},
        "e2e": {"value": value, "unit": "points/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0}}))


def rel_err(a, b):
    """|a - b| / |b| elementwise, 0 where both are equal (including zeros)."""
    with np.errstate(divide="ignore", invalid="ignore"):
        r = np.abs(a - b) / np.abs(b)
    r[a == b] = 0.
    r[~np.isfinite(r)] = np.inf
    return r


# op-count table entry (profiles/op_counts.json) of each grey workload
OPCOUNT_WORKLOAD = {"c5": "c5", "c3": "c3", "c2": "c3", "c1": "c3"}
SPECIES = ("nue", "anue", "nux", "anux")
GREY_NAMES = [f"{f}[{sp}]" for f in ("eta_0", "kappa_0_a", "eta", "kappa_a", "kappa_s")
              for sp in SPECIES]
SPEC_NAMES = [f"{f}[{sp}]" for f in ("j", "kappa", "j_s", "kappa_s") for sp in SPECIES]
M_U_G = 1.66053906892e-24   # atomic mass unit [g]: rho = nb * m_u * 1e21


def degenerate_corner(eos_h):
    """Points of the degenerate corner T < 2 MeV, rho > 1e14 g/cm^3."""
    return (eos_h[1] < 2.) & (eos_h[0] * M_U_G * 1e21 > 1e14)


def _stats(x):
    x = np.asarray(x).reshape(-1)
    if x.size == 0:
        return None
    return {"max": float(x.max()), "p99": float(np.percentile(x, 99))}


def error_report(r, names, corner):
    """Max and p99 of the relative error r[output, point, ...] per output, over
    all points and over the degenerate corner."""
    rc = r[:, corner]
    return {
        "per_output": {nm: _stats(r[k]) for k, nm in enumerate(names)},
        "degenerate_corner": {"criterion": "T < 2 MeV and rho > 1e14 g/cm^3",
                              "points": int(corner.sum()), "all_outputs": _stats(rc),
                              "per_output": {nm: _stats(rc[k]) for k, nm in enumerate(names)}},
    }


def timed_steps(step, steps, stream, torch):
    """Device ms of `steps` calls between events on `stream`."""
    t0 = torch.cuda.Event(enable_timing=True)
    t1 = torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    t0.record(stream)
    for _ in range(steps):
        step()
    t1.record(stream)
    torch.cuda.synchronize()
    return t0.elapsed_time(t1)


def run_aux(args, rank):
    """Throughput of the auxiliary batched kernels on inputs larger than L2:
    every order of the Fermi-Dirac family (bnsn_fdi, 8 B in + 8 B out per
    argument, arguments uniform in [-50, 150] so that every regime is hit),
    distribution parameters from M1 moments (96 B in, 224 B out per point) and
    the equilibrium distribution with its M1 densities (32 B in, 320 B out)."""
    import torch
    import bns_nurates_gb300 as bn
    from bns_nurates_gb300 import build as libbuild
    libbuild.build()
    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
    n = args.npts or WORKLOADS["aux"]["npts"]
    stream = torch.cuda.current_stream(dev)
    warmup = max(args.warmup, 3)
    gen = torch.Generator(device=dev).manual_seed(SEED)
    x = torch.rand(n, dtype=torch.float64, device=dev, generator=gen) * 200. - 50.
    y = torch.empty_like(x)
    peaks = load_json("MEASURED_PEAKS.json")
    hbm = peaks.get("hbm_gbs")
    fp64_peak = bn.fp64_peak_tflops()
    res = {}

    def timed(fn, nbytes, count):
        for _ in range(warmup):
            fn()
        ms = timed_steps(fn, args.steps, stream, torch) / args.steps
        gbs = nbytes * count / (ms * 1e-3) / 1e9
        return {"ms": ms, "per_s": count / (ms * 1e-3), "gbs": gbs,
                "hbm_frac": gbs / hbm if hbm else None}

    l0 = bn.kernel_launches()
    fdi = {}
    for k2 in sorted(bn.FDI_NAMES):
        r = timed(lambda: bn.fdi(k2 / 2, x, out=y, stream=stream), 16, n)
        fdi[bn.FDI_NAMES[k2]] = {"args_per_s": r["per_s"], "ms": r["ms"], "gbs": r["gbs"],
                                 "hbm_frac": r["hbm_frac"]}
    # one point per workload row: distribution parameters and equilibrium
    npts = min(n, 1 << 22)
    eos_h, m1_h = bn.synthetic_points(SEED, npts)
    eos = torch.from_numpy(eos_h).to(dev)
    m1 = torch.from_numpy(m1_h).to(dev)
    d_out = torch.empty((28, npts), dtype=torch.float64, device=dev)
    res["distr_from_m1"] = timed(lambda: bn.distr_from_m1(m1, out=d_out, stream=stream),
                                 12 * 8 + 28 * 8, npts)
    res["nu_equilibrium"] = timed(lambda: bn.nu_equilibrium(eos, stream=stream),
                                  4 * 8 + 40 * 8, npts)
    launches = bn.kernel_launches() - l0
    rates = [v["args_per_s"] for v in fdi.values()]
    line = {
        "metric": "auxiliary kernels throughput", "workload": "aux", "unit": "arguments/s",
        "value": statistics.median(rates), "n_gpus": 1, "steps": args.steps, "warmup": warmup,
        "higher_is_better": True, "dtype": "f64", "data": "synthetic (uniform arguments; seeded "
        "generator points)", "config": {"workload": WORKLOADS["aux"]["desc"], "fdi_arguments": n,
        "points": npts, "l2": "inputs and outputs (256 MB per FDI call) larger than L2"},
        "fdi": fdi, "distr_from_m1": res["distr_from_m1"], "nu_equilibrium": res["nu_equilibrium"],
        "peaks": {"hbm_gbs": hbm, "fp64_tflops_probe": fp64_peak},
        "gpu_launches": launches,
    }
    if rank == 0:
        print(json.dumps(line))


C4_EDGES = (8, 16, 24, 32, 48, 64)
C4_WEIGHTS = (0.55, 0.28, 0.09, 0.05, 0.025, 0.005)


def c4_blocks(seed, nblocks, eos_first_rho):
    """Block table of the AMR workload: edge^3 points per block, reactions
    beta+iso+pair always, brem variant uniform, NES on/off, n by density."""
    rng = np.random.default_rng(seed)
    blocks, first = [], 0
    for _ in range(nblocks):
        e = int(rng.choice(C4_EDGES, p=C4_WEIGHTS))
        count = e ** 3
        brem = int(rng.integers(0, 3))
        nes = int(rng.integers(0, 2))
        blocks.append([first, count, (1, 1, 1, nes, 1), brem, None])
        first += count
    return blocks, first


def run_blocks(args, rank, world, local):
    """The batched-AMR workload through bnsn_blocks_plan_create / _run in a
    CUDA graph."""
    import torch
    import bns_nurates_gb300 as bn
    from bns_nurates_gb300 import build as libbuild
    from bns_nurates_gb300 import shards
    if rank == 0:
        libbuild.build()
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
        dist.barrier()
        libbuild.build()
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    from bns_nurates_gb300 import gp19_synthetic
    bn.set_gp19_table(gp19_synthetic.table())
    blocks, n = c4_blocks(SEED + rank, 1536, None)
    if args.npts:   # smaller runs: keep the first blocks up to npts points
        keep, tot = [], 0
        for b in blocks:
            if tot + b[1] > args.npts:
                break
            keep.append(b)
            tot += b[1]
        blocks, n = keep, tot
    first, _ = shards.rank_points(n, rank)
    t0 = time.perf_counter()
    eos_h, m1_h = bn.synthetic_points(SEED, n, first=first)
    gen_s = time.perf_counter() - t0
    rho = eos_h[0] * 1.66053906892e-24 * 1e21   # nb [nm^-3] -> rho [g cm^-3]
    for b in blocks:
        b[4] = 10 if rho[b[0]] < 1e11 else 20
    eos = torch.from_numpy(eos_h).to(dev)
    m1 = torch.from_numpy(m1_h).to(dev)
    out = torch.empty((20, n), dtype=torch.float64, device=dev)
    stream = torch.cuda.Stream(dev)
    warmup = max(args.warmup, 3)
    plans, graphs, outs, tune_s = {}, {}, {}, {}
    precs = [args.precision] + (["fp64"] if args.precision == "mixed" and not args.no_fp64 else [])
    for prec in precs:
        o = out if prec == args.precision else torch.empty_like(out)
        t0 = time.perf_counter()
        plans[prec] = bn.BlocksPlan(blocks, eos, m1, o, precision=prec, tune=True, stream=stream)
        torch.cuda.synchronize()
        tune_s[prec] = time.perf_counter() - t0
        with torch.cuda.stream(stream):
            plans[prec].run(eos, m1, o, stream=stream)
        torch.cuda.synchronize()
        g = torch.cuda.CUDAGraph()
        l0 = bn.kernel_launches()
        with torch.cuda.graph(g, stream=stream):
            plans[prec].run(eos, m1, o, stream=stream)
        per_replay = bn.kernel_launches() - l0   # library kernels captured in the graph
        graphs[prec], outs[prec] = g, o
        if prec == args.precision:
            launches_per_step = per_replay

    def timed(prec, steps):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record(stream)
        with torch.cuda.stream(stream):
            for _ in range(steps):
                graphs[prec].replay()
        e1.record(stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / steps

    for _ in range(warmup):
        timed(args.precision, 1)
    if world > 1:
        torch.distributed.barrier()
    with ClockSampler(local) as clk:
        ms = timed(args.precision, args.steps)
    ms = shards.max_over_ranks(ms, dev)
    value = world * n / (ms * 1e-3)
    res = outs[args.precision].cpu().numpy()
    fp64 = accuracy = None
    if "fp64" in graphs and args.precision == "mixed":
        timed("fp64", 1)
        ms64 = timed("fp64", 1)
        fp64 = {"value": world * n / (ms64 * 1e-3), "unit": "points/s", "ms_per_step": ms64,
                "steps": 1, "warmup": 1, "mixed_over_fp64": ms64 / ms}
        r64 = outs["fp64"].cpu().numpy()
        r = rel_err(res, r64)
        accuracy = {"vs": "plain FP64 GPU path (same plan, FP64), every output of every point",
                    "max_rel": float(r.max()), "p99_rel": float(np.percentile(r, 99)),
                    "p999_rel": float(np.percentile(r, 99.9)),
                    "frac_above_1e-6": float(np.mean(r > 1e-6)),
                    **error_report(r, GREY_NAMES, degenerate_corner(eos_h))}

        # conditioning: the FP64 plan's own change under +2 ulp of T or mu_e
        # (where the reference's pair Psi formula is rounding noise, eta - s
        # between ~35 and 200, the FP64 outputs move by orders of magnitude)
        def grey64(e, o):
            plans["fp64"].run(e, m1, o, stream=stream)

        accuracy.update(conditioned_error(torch, eos, grey64, (20, n), r, r64, GREY_NAMES))
    # end to end: pinned host inputs -> device, graph replay, outputs -> host
    e2e = None
    if not args.no_e2e:
        eos_p = torch.from_numpy(eos_h).pin_memory()
        m1_p = torch.from_numpy(m1_h).pin_memory()
        out_p = torch.empty((20, n), dtype=torch.float64).pin_memory()
        ksteps = max(1, min(args.steps, 2))
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(ksteps):
            with torch.cuda.stream(stream):
                eos.copy_(eos_p, non_blocking=True)
                m1.copy_(m1_p, non_blocking=True)
                graphs[args.precision].replay()
                out_p.copy_(outs[args.precision], non_blocking=True)
            stream.synchronize()
        dt = shards.max_over_ranks((time.perf_counter() - t0) / ksteps, dev)
        e2e = {"value": world * n / dt, "unit": "points/s",
               "h2d_bytes_per_step": int(23 * 8 * n), "d2h_bytes_per_step": int(20 * 8 * n),
               "call": "BlocksPlan.run in a CUDA graph with host-buffer copies"}
    groups = plans[args.precision].groups()
    if rank == 0:
        nq20 = sum(1 for b in blocks if b[4] == 20)
        line = {
            "metric": METRIC,
            "comparison": "mixed-precision path vs plain FP64 GPU path (fp64_gpu, accuracy)",
            "value": value, "unit": "points/s", "n_gpus": world, "steps": args.steps,
            "warmup": warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64" if args.precision == "fp64" else "f32+f64",
            "data": "synthetic (seeded generator with the reference's input ranges)",
            "config": {"workload": WORKLOADS["c4"]["desc"], "blocks": len(blocks),
                       "points_per_step_per_gpu": n, "blocks_n20": nq20,
                       "precision": args.precision, "groups": len(groups),
                       "l2": "inputs (%.0f MB per GPU) larger than L2 (129 MB)"
                             % (23 * 8 * n / 1e6),
                       "parallelism": f"{world} independent point shards"},
            "fp64_gpu": fp64, "accuracy": accuracy, "e2e": e2e,
            "autotuner": {"plan_create_s": tune_s, "groups": groups,
                          "layout": plans[args.precision].layout(),
                          "knobs": "points per step (16k, 33k, 65k, 131k over all groups), "
                                   "then persistent-grid scale (points per CTA, 4 or 2), each "
                                   "timed on the first four steps of the data"},
            "launches_per_replay": launches_per_step,
            "clocks": clk.summary(), "gpu_launches": launches_per_step * args.steps,
            "generator_s": gen_s,
        }
        print(json.dumps(line))
    for p_ in plans.values():
        p_.close()
    if world > 1:
        torch.distributed.destroy_process_group()


SPEC_ENERGIES = np.logspace(0., np.log10(300.), 24)
SPEC_WARMUP, SPEC_STEPS = 3, 5


def spectral_leg(args, bn, torch, eos, m1, eos_h, flags, params, q, stream, world, dev):
    """Spectral opacities (16 outputs x 24 energies per point) of the first
    --spectral-npts points: device-timed points/s of --precision and, for the
    mixed path, of the plain FP64 path on the same points, the mixed-vs-FP64
    error and the mixed path's FP64-recomputation statistics."""
    ns = min(eos.shape[1], args.spectral_npts)
    eo, mo = eos[:, :ns].contiguous(), m1[:, :ns].contiguous()
    precs = [args.precision] + (["fp64"] if args.precision == "mixed" else [])
    outs, legs = {}, {}
    for prec in precs:
        o = torch.empty((16, ns, SPEC_ENERGIES.size), dtype=torch.float64, device=dev)

        def sstep(prec=prec, o=o):
            bn.spectral_opacities(eo, mo, flags, params, q, SPEC_ENERGIES, precision=prec,
                                  out=o, stream=stream)

        for _ in range(SPEC_WARMUP):
            sstep()
        if prec == "mixed":
            bn.spectral_mixed_stats(reset=True)
        ms = timed_steps(sstep, SPEC_STEPS, stream, torch) / SPEC_STEPS
        legs[prec] = {"value": world * ns / (ms * 1e-3), "unit": "points/s", "ms": ms,
                      "steps": SPEC_STEPS, "warmup": SPEC_WARMUP}
        if prec == "mixed":
            st = bn.spectral_mixed_stats(reset=True)   # totals over the SPEC_STEPS calls
            legs[prec]["fp64_recomputed"] = {k: v / max(1, st["evaluated"])
                                             for k, v in st.items() if k != "evaluated"}
        outs[prec] = o
    res = {"points": ns, "energies": int(SPEC_ENERGIES.size),
           "energy_range_mev": [1.0, 300.0], "outputs_per_energy": 16, **legs}
    if "fp64" in outs and args.precision == "mixed":
        a, b = outs["mixed"].cpu().numpy(), outs["fp64"].cpu().numpy()
        r = rel_err(a, b)
        res["mixed_over_fp64"] = legs["fp64"]["ms"] / legs["mixed"]["ms"]
        res["accuracy"] = {"vs": "plain FP64 GPU path, every output, point and energy",
                           "max_rel": float(r.max()), "p99_rel": float(np.percentile(r, 99)),
                           "p999_rel": float(np.percentile(r, 99.9)),
                           "frac_above_1e-6": float(np.mean(r > 1e-6)),
                           **error_report(r, SPEC_NAMES, degenerate_corner(eos_h[:, :ns]))}

        def spec64(e, o):
            bn.spectral_opacities(e, mo, flags, params, q, SPEC_ENERGIES, precision="fp64",
                                  out=o, stream=stream)

        res["accuracy"].update(conditioned_error(torch, eo, spec64, tuple(outs["fp64"].shape),
                                                 r, b, SPEC_NAMES))
    return res


def conditioned_error(torch, eos, run64, shape, r, ref, names):
    """Splits the mixed-vs-FP64 error by the conditioning of each output: an
    output is well conditioned when the FP64 path moves by at most 1e-9
    (relative) under a two-ulp change of T or of mu_e; there the contract is
    1e-6, elsewhere the reference's own result is not reproducible to that
    level."""
    sens = np.zeros(shape)
    for row in (1, 7):
        e2 = eos.clone()
        e2[row] *= 1. + 2. ** -51
        o = torch.empty(shape, dtype=torch.float64, device=eos.device)
        run64(e2, o)
        torch.cuda.synchronize()
        sens = np.maximum(sens, rel_err(o.cpu().numpy(), ref))
    well = sens <= 1e-9
    rw = np.where(well, r, 0.)
    return {"well_conditioned": {"criterion": "FP64 output moves <= 1e-9 under +2 ulp in T "
                                              "or mu_e",
                                 "points": int(shape[1]), "fraction": float(well.mean()),
                                 "max_rel": float(rw.max()),
                                 "p999_rel": float(np.percentile(r[well], 99.9))
                                 if well.any() else None,
                                 "max_rel_per_output": {nm: float(rw[k].max())
                                                        for k, nm in enumerate(names)}}}


def _probe_sens(fn, fn_fma, eos_h, want, fn_fdi=None):
    """Largest relative change of the oracle under its FMA build, its build
    with Fermi integrals moved by one part in 2^52, and T or mu_e moved by two
    ulps: how far the reference's own result is reproducible."""
    sens = rel_err(fn_fma(eos_h), want)
    if fn_fdi is not None:
        sens = np.maximum(sens, rel_err(fn_fdi(eos_h), want))
    for row in (1, 7):
        e2 = eos_h.copy()
        e2[row] *= 1. + 2. ** -51
        sens = np.maximum(sens, rel_err(fn(e2), want))
    return sens


def _parity_summary(r, sens, names, got=None, want=None, worst=0):
    """Parity figures of GPU-vs-oracle errors r with probe spreads sens; with
    worst > 0 also the `worst` elements of largest error-to-spread ratio
    (index into r, output name, values)."""
    above = r > 1e-12
    with np.errstate(divide="ignore", invalid="ignore"):
        ratio = np.where(above, r / sens, 0.)
    well = sens <= 1e-13
    top = []
    if worst:
        flat = np.argsort(ratio, axis=None)[::-1][:worst]
        for f in flat:
            idx = np.unravel_index(f, r.shape)
            top.append({"index": [int(i) for i in idx], "output": names[idx[0]],
                        "rel_err": float(r[idx]), "spread": float(sens[idx]),
                        "gpu": float(got[idx]), "oracle": float(want[idx])})
    return {
        "worst_elements": top,
        "elements": int(r.size), "max_rel": float(r.max()),
        "frac_within_1e-12": float(1. - above.mean()),
        "oracle_frac_reproducible_1e-12": float(np.mean(sens <= 1e-12)),
        "worst_error_to_spread": float(ratio.max()),
        "well_conditioned": {"criterion": "oracle probe spread <= 1e-13",
                             "fraction": float(well.mean()),
                             "max_rel": float(np.max(np.where(well, r, 0.)))},
        "max_rel_per_output": {nm: float(r[k].max()) for k, nm in enumerate(names)},
    }


def run_full_parity(args):
    """--full-parity: the plain FP64 GPU path on every point of the workload
    (c2: the 2,097,152-point 128^3 patch) against the CPU oracle, with the
    oracle's three conditioning probes; spectral opacities at 24 energies on
    every 64th point.  Reports the fraction of elements within 1e-12 and the
    largest ratio of error to probe spread (the smallest safety factor the
    parity tests could use)."""
    import torch
    import oracle
    import bns_nurates_gb300 as bn
    from bns_nurates_gb300 import build as libbuild
    libbuild.build()
    oracle.build()
    wl = dict(WORKLOADS[args.workload])
    n = args.npts or wl["npts"]
    setup_gp19(bn, wl)
    port, pfma, pfdi = oracle.port(), oracle.port_fma(), oracle.port_fdi()
    nthreads = os.cpu_count()
    t0 = time.perf_counter()
    eos_h, m1_h = bn.synthetic_points(SEED, n)
    flags, params = bn.opacity_flags(*wl["flags"]), bn.opacity_params(brem_implementation=wl["brem"])
    q = bn.gauss_legendre(wl["nq"])
    eos, m1 = torch.from_numpy(eos_h).cuda(), torch.from_numpy(m1_h).cuda()
    got = bn.m1_opacities(eos, m1, flags, params, q, precision="fp64").cpu().numpy()
    qo = port.gauss_legendre(wl["nq"])
    pars = (1, 0, 1, 1, 1, wl["brem"], 1, 0)

    def grey(impl):
        return lambda e: impl.m1_opacities(e, m1_h, wl["flags"], pars, qo, nthreads=nthreads)

    res = {"workload": wl["desc"], "points": n}
    if not args.no_grey_parity:
        want = grey(port)(eos_h)
        sens = _probe_sens(grey(port), grey(pfma), eos_h, want, grey(pfdi))
        res["grey"] = _parity_summary(rel_err(got, want), sens, GREY_NAMES, got, want, worst=8)
    # spectral: every 64th point (--spectral-stride), 24 log-spaced energies 1-300 MeV
    idx = np.arange(0, n, args.spectral_stride)
    es, ms_ = np.ascontiguousarray(eos_h[:, idx]), np.ascontiguousarray(m1_h[:, idx])
    gs = bn.spectral_opacities(torch.from_numpy(es).cuda(), torch.from_numpy(ms_).cuda(), flags,
                               params, q, SPEC_ENERGIES, precision="fp64").cpu().numpy()

    def spec(impl):
        return lambda e: impl.spectral(e, ms_, wl["flags"], pars, qo, SPEC_ENERGIES,
                                       nthreads=nthreads)

    ws = spec(port)(es)
    ss = _probe_sens(spec(port), spec(pfma), es, ws, spec(pfdi))
    res["spectral"] = {"points": int(idx.size), "energies": int(SPEC_ENERGIES.size),
                       "sample": "every 64th point of the workload (index = [output, "
                                 "sample, energy]; workload point = 64 * sample)",
                       **_parity_summary(rel_err(gs, ws), ss, SPEC_NAMES, gs, ws, worst=8)}
    res["wall_s"] = time.perf_counter() - t0
    res["cores"] = nthreads
    print(json.dumps({"full_parity": res}))


def main():
    args = parse()
    rank, world, local = dist_info()
    if args.impl == "reference":
        run_reference(args, rank, world)
        return
    if args.full_parity:
        run_full_parity(args)
        return
    if args.workload == "c4":
        run_blocks(args, rank, world, local)
        return
    if args.workload == "aux":
        run_aux(args, rank)
        return

    import torch
    import bns_nurates_gb300 as bn
    from bns_nurates_gb300 import build as libbuild
    if rank == 0:
        libbuild.build()
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
        dist.barrier()
        libbuild.build()
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)

    wl = dict(WORKLOADS[args.workload])
    if args.npts:
        wl["npts"] = args.npts
    n = wl["npts"]
    q = bn.gauss_legendre(wl["nq"])
    flags = bn.opacity_flags(*wl["flags"])
    params = bn.opacity_params(brem_implementation=wl["brem"])
    setup_gp19(bn, wl)
    warmup = max(args.warmup, 3)

    # per-rank shard of points (weak scaling): rank r owns points [r n, (r+1) n)
    from bns_nurates_gb300 import shards
    first, _ = shards.rank_points(n, rank)
    t0 = time.perf_counter()
    eos_h, m1_h = bn.synthetic_points(SEED, n, first=first)
    gen_s = time.perf_counter() - t0
    eos = torch.from_numpy(eos_h).to(dev)
    m1 = torch.from_numpy(m1_h).to(dev)
    out = torch.empty((20, n), dtype=torch.float64, device=dev)
    stream = torch.cuda.current_stream(dev)

    def step(precision=args.precision, o=out):
        bn.m1_opacities(eos, m1, flags, params, q, out=o, precision=precision, stream=stream)

    for _ in range(warmup):
        step()
    torch.cuda.synchronize()

    # timed region: K steps, per-phase events around every kernel launch
    if world > 1:
        torch.distributed.barrier()
    bn.phase_times()
    bn.phase_timing(True)
    bn.grey_mixed_stats(reset=True)
    launches0 = bn.kernel_launches()
    with ClockSampler(local) as clk:
        total_ms = timed_steps(step, args.steps, stream, torch)
    launches = bn.kernel_launches() - launches0
    mstats = bn.grey_mixed_stats(reset=True)   # totals over the timed steps
    fallbacks = ({k: v / max(1, mstats["evaluated"]) for k, v in mstats.items() if k != "evaluated"}
                 if args.precision == "mixed" else None)
    bn.phase_timing(False)
    phases = bn.phase_times()
    if world > 1:
        torch.distributed.barrier()
        total_ms = shards.max_over_ranks(total_ms, dev)
    ms_per_step = total_ms / args.steps
    value = world * n / (ms_per_step * 1e-3)
    assert torch.isfinite(out).all().item(), "non-finite outputs"
    res = out.cpu().numpy()

    # plain FP64 GPU path on the same points
    fp64 = accuracy = None
    if args.precision == "mixed" and not args.no_fp64:
        out64 = torch.empty_like(out)
        step("fp64", out64)
        k64 = max(1, min(2, args.steps))
        ms64 = timed_steps(lambda: step("fp64", out64), k64, stream, torch) / k64
        fp64 = {"value": world * n / (ms64 * 1e-3), "unit": "points/s", "ms_per_step": ms64,
                "steps": k64, "warmup": 1, "mixed_over_fp64": ms64 / ms_per_step}
        r64 = out64.cpu().numpy()
        r = rel_err(res, r64)
        accuracy = {"vs": "plain FP64 GPU path, every output of every point",
                    "max_rel": float(r.max()), "p99_rel": float(np.percentile(r, 99)),
                    "p999_rel": float(np.percentile(r, 99.9)),
                    "frac_above_1e-6": float(np.mean(r > 1e-6)),
                    **error_report(r, GREY_NAMES, degenerate_corner(eos_h))}
        # conditioning of each output: the FP64 path's own change when T or
        # mu_e moves by two ulps, on the first points of the batch
        nc = min(n, args.cond_npts)

        def grey64(e, o):
            bn.m1_opacities(e, m1[:, :nc].contiguous(), flags, params, q, out=o,
                            precision="fp64", stream=stream)

        accuracy.update(conditioned_error(torch, eos[:, :nc].contiguous(), grey64,
                                          (20, nc), r[:, :nc], r64[:, :nc], GREY_NAMES))

    # end to end through the host-buffer C-ABI call, pinned host memory
    e2e = None
    if not args.no_e2e:
        eos_p = torch.from_numpy(eos_h).pin_memory()
        m1_p = torch.from_numpy(m1_h).pin_memory()
        out_p = torch.empty((20, n), dtype=torch.float64).pin_memory()
        e_np, m_np, o_np = eos_p.numpy(), m1_p.numpy(), out_p.numpy()
        bn.m1_opacities_host(e_np, m_np, flags, params, q, out=o_np, precision=args.precision)
        ksteps = max(1, min(args.steps, 2))
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(ksteps):
            bn.m1_opacities_host(e_np, m_np, flags, params, q, out=o_np,
                                 precision=args.precision)
        dt = (time.perf_counter() - t0) / ksteps
        if world > 1:
            dt = shards.max_over_ranks(dt, dev)
        e2e = {"value": world * n / dt, "unit": "points/s",
               "h2d_bytes_per_step": int(23 * 8 * n), "d2h_bytes_per_step": int(20 * 8 * n),
               "call": "bnsn_m1_opacities_host"}
        assert np.array_equal(o_np, res), "host-buffer and device paths differ"

    # roofline of the dominant kernel phase: its pipe (FP64 for the plain path,
    # FP32 for the mixed path's double-float phases) and its work per point from
    # an ncu instruction count (profiles/bench_constants.json)
    peaks = load_json("MEASURED_PEAKS.json")
    consts = load_json("profiles", "bench_constants.json").get(args.workload, {}).get(
        args.precision, {})
    top = max(phases, key=lambda k: phases[k][0])
    top_ms, top_launches = phases[top]
    c = consts.get(top, {})
    bound = c.get("bound", "fp64")
    probe = bn.fp64_peak_tflops if bound == "fp64" else bn.fp32_peak_tflops
    peak = probe()
    chunks = max(1, top_launches)                # one launch of the phase per scratch chunk
    pts_per_launch = n * args.steps / chunks
    top_launch_ms = top_ms / chunks
    roofline = {"kernel": f"grey phase '{top}'", "bound": bound, "unit": "TFLOP/s",
                "achieved": None, "peak": peak, "frac": None, "traffic": None,
                "peak_source": f"{bound.upper()} FMA-chain probe run in this process "
                               f"(bnsn_{bound}_peak_probe); MEASURED_PEAKS.json has no "
                               f"{bound.upper()} figure",
                "launch_ms": top_launch_ms, "launches": top_launches,
                "share_of_step": top_ms / total_ms if total_ms else None}
    # numerator: the reference algorithm's work per point for this phase,
    # counted by the op-counting build of the reference (oracle/opcount.py ->
    # profiles/op_counts.json); the phase's executed FLOP on its pipe (ncu
    # instruction count) is kept beside it
    opc = load_json("profiles", "op_counts.json").get(OPCOUNT_WORKLOAD.get(args.workload), {})
    alg = opc.get("phases", {}).get(top, {}).get("work")
    executed = c.get(f"{bound}_flop_per_point")
    if alg:
        ach = alg * pts_per_launch / (top_launch_ms * 1e-3) / 1e12
        roofline["achieved"] = ach
        roofline["frac"] = ach / peak if peak else None
        roofline["work_per_point"] = alg
        roofline["work_source"] = ("profiles/op_counts.json: reference operations per point "
                                   "of the reaction this phase computes (FLOP + "
                                   "transcendental calls, one each)")
    if executed:
        ex = executed * pts_per_launch / (top_launch_ms * 1e-3) / 1e12
        roofline["executed_per_point"] = executed
        roofline["executed_tflops"] = ex
        roofline["executed_frac"] = ex / peak if peak else None
        roofline["executed_source"] = c.get("source")
    if c.get("dram_bytes_per_point"):
        roofline["traffic"] = c["dram_bytes_per_point"] * pts_per_launch
    hbm = peaks.get("hbm_gbs")
    io_gbs = (23 + 20) * 8 * n / (ms_per_step * 1e-3) / 1e9
    roofline["hbm_secondary"] = {"achieved_gbs": io_gbs, "peak_gbs": hbm,
                                 "frac": io_gbs / hbm if hbm else None,
                                 "note": "algorithmic I/O bytes (23 inputs + 20 outputs "
                                         "x 8 B per point) over the step time"}

    # spectral leg (c2, c5: grey plus spectral opacities at 24 log-spaced
    # energies 1-300 MeV) on the first points of the step's batch
    spectral = None
    if args.workload in ("c2", "c5") and not args.no_spectral:
        spectral = spectral_leg(args, bn, torch, eos, m1, eos_h, flags, params, q, stream, world,
                                dev)

    cpu = None
    if rank == 0 and not args.no_cpu:
        impl, kind, how = cpu_impl()
        nthreads = os.cpu_count()
        ns = cpu_sample_size(impl, eos_h, m1_h, wl, args.cpu_seconds, nthreads, n)
        rate, dt = cpu_rate(impl, eos_h, m1_h, wl, ns, nthreads)
        cpu = {"value": rate, "unit": "points/s", "cores": nthreads, "kind": kind,
               "sample": f"first {ns} points of the step's batch, {dt:.1f} s", "build": how}

    if rank == 0:
        line = {
            "metric": METRIC,
            "comparison": "mixed-precision path vs plain FP64 GPU path (fp64_gpu, accuracy)",
            "value": value, "unit": "points/s",
            "n_gpus": world, "steps": args.steps, "warmup": warmup,
            "ms_per_step": ms_per_step, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64" if args.precision == "fp64" else "f32+f64",
            "data": "synthetic (seeded generator with the reference's input ranges)",
            "config": {"workload": wl["desc"], "points_per_step_per_gpu": n,
                       "reactions": {"abs_em": wl["flags"][0], "pair": wl["flags"][1],
                                     "brem": wl["flags"][2], "inelastic": wl["flags"][3],
                                     "iso": wl["flags"][4]},
                       "brem": BREM_NAMES[wl["brem"]], "nquad": wl["nq"],
                       "precision": args.precision, "stim_abs": 1,
                       "l2": "inputs (%.0f MB per GPU) larger than L2 (129 MB)"
                             % (23 * 8 * n / 1e6),
                       "parallelism": f"{world} independent point shards"},
            "fp64_gpu": fp64, "accuracy": accuracy,
            "e2e": e2e, "roofline": roofline, "cpu_baseline": cpu, "spectral": spectral,
            "clocks": clk.summary(), "gpu_launches": launches,
            "phases_ms": {k: {"ms": v[0], "launches": v[1]} for k, v in phases.items() if v[1]},
            "fallback_fraction": fallbacks,
            "generator_s": gen_s,
        }
        print(json.dumps(line))
    if world > 1:
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
