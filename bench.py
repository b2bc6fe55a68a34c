"""Benchmark of the grey M1 opacity path on GB300.

One step = the grey M1 opacities (ComputeM1Opacities semantics, all 20
outputs, 4 species) of every point of the workload, one kernel launch.

  value : points/s with inputs and outputs resident in HBM, device time of K
          launches between CUDA events (max over ranks).
  e2e   : points/s through the host-buffer C-ABI call bnsn_m1_opacities_host
          (pinned host buffers, host->device and device->host copies inside
          the timed region).
  roofline / cpu_baseline / clocks / gpu_launches: see the design doc.

Workloads (synthetic, seeded; the reference's inputs are CCSN/BNS tables):
  c2  : 128^3 = 2,097,152 points, beta + iso + pair + HR98, n = 10
  c5  : 256^3 = 16,777,216 points, all reactions, GP19 (synthetic table), n = 20
  c1  : 4096 points, beta + iso + pair + HR98, n = 10

``--impl reference`` times the reference algorithm on the host cores (the
CPU oracle, oracle/) for the same workload on a bounded sample per step.
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
WORKLOADS = {
    "c1": dict(npts=4096, flags=(1, 1, 1, 0, 1), brem=0, nq=10),
    "c2": dict(npts=128 ** 3, flags=(1, 1, 1, 0, 1), brem=0, nq=10),
    "c5": dict(npts=256 ** 3, flags=(1, 1, 1, 1, 1), brem=2, nq=20),
}
# Per-point FP64 work of the grey kernel, in FLOP (a DFMA counts 2), from an
# ncu count of the kernel's FP64 instructions over a sample of the workload
# (profiles/grey_fp64_c2.md); the kernel evaluates each distinct quantity
# once, so this is the algorithm's work, not repeated work.
FP64_FLOP_PER_POINT = {"c2": None, "c5": None, "c1": None}


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="c2", choices=sorted(WORKLOADS))
    ap.add_argument("--precision", default="fp64", choices=["fp64", "mixed"])
    ap.add_argument("--npts", type=int, default=0, help="override the point count")
    ap.add_argument("--cpu-sample", type=int, default=16384)
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
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


def load_peaks():
    try:
        with open(os.path.join(REPO, "MEASURED_PEAKS.json")) as f:
            return json.load(f)
    except OSError:
        return {}


def load_profile_numbers():
    """FP64 FLOP/point and DRAM bytes/point recorded from ncu (profiles/)."""
    try:
        with open(os.path.join(REPO, "profiles", "bench_constants.json")) as f:
            return json.load(f)
    except OSError:
        return {}


def cpu_sample_rate(eos, m1, wl, nsample, nthreads):
    """Reference algorithm (CPU oracle, restatement of the reference C++) on
    host cores: points/s over a bounded sample of the workload."""
    import oracle
    port = oracle.port()
    q = port.gauss_legendre(wl["nq"])
    pars = (1, 0, 1, 1, 1, wl["brem"], 1, 0)
    idx = slice(0, nsample)
    t0 = time.perf_counter()
    port.m1_opacities(eos[:, idx], m1[:, idx], wl["flags"], pars, q, nthreads=nthreads)
    dt = time.perf_counter() - t0
    return nsample / dt, dt


def run_reference(args, rank, world):
    if rank != 0:
        return
    import oracle
    oracle.build()
    import bns_nurates_gb300 as bn
    from bns_nurates_gb300 import build as libbuild
    libbuild.build()
    wl = WORKLOADS[args.workload]
    nthreads = os.cpu_count()
    n = args.cpu_sample
    eos, m1 = bn.synthetic_points(SEED, n)
    for _ in range(args.warmup):
        cpu_sample_rate(eos, m1, wl, min(n, 512), nthreads)
    rates = []
    for _ in range(args.steps):
        r, _ = cpu_sample_rate(eos, m1, wl, n, nthreads)
        rates.append(r)
    value = statistics.median(rates)
    line = {
        "impl": "reference", "metric": "grey M1 opacity points/s", "value": value,
        "unit": "points/s", "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * n / value, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded generator)",
        "config": {"workload": f"{args.workload}: sample of {n} points per step",
                   "reactions": wl["flags"], "brem": ["HR98", "BRT06", "GP19"][wl["brem"]],
                   "nquad": wl["nq"]},
        "cpu_baseline": {"value": value, "unit": "points/s", "cores": nthreads, "kind": "port",
                         "sample": f"{n} points of the {args.workload} workload per step"},
        "e2e": {"value": value, "unit": "points/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))


def main():
    args = parse()
    rank, world, local = dist_info()
    if args.impl == "reference":
        run_reference(args, rank, world)
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
    if wl["brem"] == 2:
        from bns_nurates_gb300 import gp19_synthetic
        bn.set_gp19_table(gp19_synthetic.table())

    # per-rank shard of points (weak scaling): rank r owns points [r n, (r+1) n)
    t0 = time.perf_counter()
    eos_h, m1_h = bn.synthetic_points(SEED, n, first=rank * n)
    gen_s = time.perf_counter() - t0
    eos = torch.from_numpy(eos_h).to(dev)
    m1 = torch.from_numpy(m1_h).to(dev)
    out = torch.empty((20, n), dtype=torch.float64, device=dev)
    stream = torch.cuda.current_stream(dev)

    def step():
        bn.m1_opacities(eos, m1, flags, params, q, out=out, precision=args.precision,
                        stream=stream)

    for _ in range(max(args.warmup, 3)):
        step()
    torch.cuda.synchronize()

    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    with ClockSampler(local) as clk:
        t_all0 = torch.cuda.Event(enable_timing=True)
        t_all1 = torch.cuda.Event(enable_timing=True)
        t_all0.record(stream)
        for k in range(args.steps):
            starts[k].record(stream)
            step()
            ends[k].record(stream)
        t_all1.record(stream)
        torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    total_ms = t_all0.elapsed_time(t_all1)
    launch_ms = [s.elapsed_time(e) for s, e in zip(starts, ends)]
    if world > 1:
        tt = torch.tensor([total_ms], device=dev)
        torch.distributed.all_reduce(tt, op=torch.distributed.ReduceOp.MAX)
        total_ms = float(tt.item())
    ms_per_step = total_ms / args.steps
    value = world * n / (ms_per_step * 1e-3)
    assert torch.isfinite(out).all().item(), "non-finite outputs"

    # end to end through the host-buffer C-ABI call, pinned host memory
    e2e = None
    if not args.no_e2e:
        eos_p = torch.from_numpy(eos_h).pin_memory()
        m1_p = torch.from_numpy(m1_h).pin_memory()
        out_p = torch.empty((20, n), dtype=torch.float64).pin_memory()
        e_np, m_np, o_np = eos_p.numpy(), m1_p.numpy(), out_p.numpy()
        bn.m1_opacities_host(e_np, m_np, flags, params, q, out=o_np, precision=args.precision)
        ksteps = max(1, min(args.steps, 3))
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(ksteps):
            bn.m1_opacities_host(e_np, m_np, flags, params, q, out=o_np,
                                 precision=args.precision)
        dt = (time.perf_counter() - t0) / ksteps
        if world > 1:
            tt = torch.tensor([dt], device=dev)
            torch.distributed.all_reduce(tt, op=torch.distributed.ReduceOp.MAX)
            dt = float(tt.item())
        e2e = {"value": world * n / dt, "unit": "points/s",
               "h2d_bytes_per_step": int(23 * 8 * n), "d2h_bytes_per_step": int(20 * 8 * n)}
        assert np.array_equal(o_np, out.cpu().numpy()), "host and device paths differ"

    peaks = load_peaks()
    prof = load_profile_numbers().get(args.workload, {})
    kernel_ms = statistics.median(launch_ms)
    flop_pt = prof.get("fp64_flop_per_point")
    fp64_peak = bn.fp64_peak_tflops()
    roofline = {"bound": "fp64", "unit": "TFLOP/s", "achieved": None, "peak": fp64_peak,
                "frac": None, "traffic": None,
                "peak_source": "measured in this run: DFMA-chain probe (bnsn_fp64_peak_probe)"}
    if flop_pt:
        ach = flop_pt * n / (kernel_ms * 1e-3) / 1e12
        roofline["achieved"] = ach
        if fp64_peak:
            roofline["frac"] = ach / fp64_peak
    if prof.get("dram_bytes_per_point"):
        roofline["traffic"] = prof["dram_bytes_per_point"] * n
    hbm = peaks.get("hbm_gbs")
    alg_bytes = (23 + 20) * 8 * n
    roofline["hbm"] = {"achieved_gbs": alg_bytes / (kernel_ms * 1e-3) / 1e9,
                       "peak_gbs": hbm, "frac": (alg_bytes / (kernel_ms * 1e-3) / 1e9 / hbm)
                       if hbm else None, "note": "secondary: algorithmic I/O bytes only"}

    cpu = None
    if rank == 0 and not args.no_cpu:
        import oracle
        oracle.build()
        ns = min(args.cpu_sample, n)
        rate, dt = cpu_sample_rate(eos_h, m1_h, wl, ns, os.cpu_count())
        cpu = {"value": rate, "unit": "points/s", "cores": os.cpu_count(), "kind": "port",
               "sample": f"first {ns} points of the workload, {dt:.1f} s"}

    if rank == 0:
        line = {
            "metric": "grey M1 opacity points/s", "value": value, "unit": "points/s",
            "n_gpus": world, "steps": args.steps, "warmup": max(args.warmup, 3),
            "ms_per_step": ms_per_step, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64" if args.precision == "fp64" else "f32+f64",
            "data": "synthetic (seeded generator, reference-shaped inputs)",
            "config": {"workload": f"{args.workload}: {n} points per GPU",
                       "reactions": {"abs_em": wl["flags"][0], "pair": wl["flags"][1],
                                     "brem": wl["flags"][2], "inelastic": wl["flags"][3],
                                     "iso": wl["flags"][4]},
                       "brem": ["HR98", "BRT06", "GP19"][wl["brem"]], "nquad": wl["nq"],
                       "precision": args.precision, "stim_abs": 1,
                       "l2": "inputs (%.0f MB/GPU) larger than L2" % (23 * 8 * n / 1e6),
                       "parallelism": f"{world} independent point shards"},
            "e2e": e2e, "roofline": roofline, "cpu_baseline": cpu,
            "clocks": clk.summary(), "gpu_launches": args.steps,
            "kernel_ms": {"median": kernel_ms, "min": min(launch_ms), "max": max(launch_ms)},
            "generator_s": gen_s,
        }
        print(json.dumps(line))
    if world > 1:
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
