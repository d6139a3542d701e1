#!/usr/bin/env python
"""Benchmark of the fused neutron-propagation kernel on GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

A step is one pass of the hot path over one batch: `--ncount` Monte-Carlo
neutrons (default 1e8) through the guide-chain instrument (disc source ->
10 m guide -> 5 m tapered guide -> 100x100 PSD + 200-bin energy monitor).
The headline `value` is FP32-fused neutrons/s over all ranks (each rank
runs its own neutron index range: weak scaling); the FP64 plain kernel is
timed the same way beside it, and chi^2/dof between the two histograms
(independent streams) is reported.  `e2e` repeats the FP32 measurement
through the public API with host buffers: tallies copied host->device
before and device->host after every step.

--impl reference times the CPU restatement of the reference algorithm (the
oracle: the reference itself is Python/Numba and its CPU engine is not
installable here) on all host cores, on the same workload and metric.
"""

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

METRIC = ("neutrons/s, FP32 fused vs FP64 plain on 1 GB300 at "
          "χ²/dof≤1.1; bwd/fwd cost")
UNIT = "neutrons/s"

WORKLOADS = {
    "guide_chain": (
        "guide_chain: disc source r=5cm E 5-100 meV -> 10 m guide 5x5 cm m=3 "
        "-> 5 m taper 5->2 cm -> PSD 100x100 +-3 cm + energy 200 bins 0-100 "
        "meV"),
    "sphere_theta_tof": (
        "sphere_theta_tof: disc source -> isotropic sphere r=1cm -> 4pi shell "
        "r=3m theta 180 x tof 200"),
    "sqe_hollow_cylinder": (
        "sqe_hollow_cylinder: 60 meV 1x1 cm beam -> hollow cylinder with "
        "200x200 S(Q,E) -> 3 m cylinder I(Q,E) 100x100"),
    "sns_source_chain": (
        "sns_source_chain: SNS moderator source (the reference's moderator "
        "file, 5-20 meV, 3x3 cm) -> PSD 100x100 + energy 100 bins at 5 m"),
    "tapered_guide_chain": (
        "tapered_guide_chain: 3x3 cm source, 10 +- 9.5 A -> 10.99 m "
        "segmented tapered guide (100 elliptic segments, m=6) -> "
        "position-divergence monitor 250x250"),
    "ms_hollow_cylinder": (
        "ms_hollow_cylinder: 1x1 cm source, 10 +- 9.5 A -> isotropic hollow "
        "cylinder r 1-2 cm with multiple scattering (<= 16 outputs per "
        "neutron, 2 x 5 loops) -> 4pi PSD 90x90"),
    "powder_banked": (
        "powder_banked: the guide_chain guides -> powder cylinder r=0.5 cm "
        "h=4 cm, 50 peaks -> banked detector R=3 m, 8 banks x 128 tubes x "
        "256 pixels x 1000 tof bins (2.62e8 bins)"),
    "constant_qe_box": (
        "constant_qe_box: 1x1 cm source 70 meV -> Al block 6x10x1 cm, "
        "constant (Q, E) = (3 /A, 30 meV) kernel -> I(Q,E) monitor 160x120"),
    "e_q_box": (
        "e_q_box: 1x1 cm source 70 meV -> Al block 6x10x1 cm, E(Q) kernel "
        "E = 30 + 20 sin(Q), S = 1, Q 0-10 /A -> I(Q,E) monitor 160x120"),
    "un_ms": (
        "un_ms: 1x1 cm source 500 meV -> UN cylinder r=5.64 mm h=1 cm, "
        "multiple scattering (<= 33 outputs per neutron) through a "
        "composite of 8 E(Q) kernels -> I(Q,E) monitor 150x100"),
    "composite_box": (
        "composite_box: 70 meV -> Al block 6x10x1 cm, composite kernel "
        "(E(Q), constant (Q, E), isotropic; weights 2:1:1) -> I(Q,E) "
        "160x120"),
    "sans2d_grid": (
        "sans2d_grid: 0.3x0.3 mm source, 10 +- 0.65 A -> Al plate 3x3 cm "
        "x 0.2 mm with S(Qx,Qy) on a 1475x1100 grid -> PSD 250x250 at "
        "10 m"),
    "anyshape_guide_chain": (
        "anyshape_guide_chain: 3x3 cm source, 10 +- 9.5 A -> 10 m guide "
        "from an OFF mesh (4 faces, 3.5x3.5 cm), m=3 -> PSD 250x250 + "
        "position-divergence x and y 250x250"),
    "verdi": (
        "verdi: the VERDI instrument (26 components): SNS moderator "
        "(source_rot2_cdr_cyl_3x3_20190417.dat, 0.1-1000 meV) -> 2 elliptic "
        "mirrors as 4 tapered guides of 499 segments, m=6, with shields -> "
        "secondary-source slit -> 5x5 mm sample mask; 11 wavelength, "
        "position-divergence and PSD monitors"),
}

# Per-neutron counts of the FP32 path-regeneration kernel on this workload,
# from one ncu --set full capture of a 1e7-neutron launch (456 blocks x 256
# threads): executed FP32 arithmetic (2*FFMA + FADD + FMUL, thread level),
# warp instructions issued, and the DRAM bytes of that launch (tally bins
# touched; it does not grow with the neutron count).
KERNEL_COUNTS = {
    "guide_chain": {"fp32_flops_per_neutron": 169.32,
                    "warp_inst_per_neutron": 35.23,
                    "thread_inst_per_neutron": 823.2,
                    "dram_bytes_per_launch": 135936,
                    "captured_neutrons": 10_000_000,
                    "kernel": "mcv::regen_kernel<float>",
                    "traffic_note": "the tally bins, independent of the "
                                    "neutron count"},
    # the multiple-scattering tree kernel (608 blocks x 256 threads on a
    # 1e6-neutron launch); its DRAM traffic is
    # the local-memory working set (tree lists and spills of 1024 lanes an
    # SM) leaving L2, and grows with the neutron count
    "un_ms": {"warp_inst_per_neutron": 919.4,
              "thread_inst_per_neutron": 919.4 * 15.35,
              "dram_bytes_per_neutron": 1438.0,
              "captured_neutrons": 1_000_000,
              "kernel": "mcv::ms_chain_kernel<float>",
              "traffic_note": "local memory (tree lists, spills) evicted "
                              "from L2, 1.44 KB per incident neutron; 76 B "
                              "at 2 blocks an SM (16% slower), 0.69 KB at "
                              "3 (9% slower)"},
}


def parse_args(argv=None):
    ap = argparse.ArgumentParser(description=__doc__)
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--workload", choices=sorted(WORKLOADS),
                    default="guide_chain")
    ap.add_argument("--ncount", type=float, default=1e8)
    ap.add_argument("--seed", type=int, default=2024)
    ap.add_argument("--cpu-seconds", type=float, default=12.0,
                    help="CPU baseline sample length")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-batched", action="store_true")
    ap.add_argument("--no-grad", action="store_true")
    a = ap.parse_args(argv)
    if a.warmup < 0 or a.steps < 1:
        ap.error("need --steps >= 1 and --warmup >= 0")
    return a


def build_instrument(name):
    from acc_gb300 import instruments
    return getattr(instruments, name)()


# ---------------------------------------------------------------- clocks
class ClockSampler:
    """nvidia-smi clock/throttle samples taken during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,"
              "clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, device_index):
        self.dev = device_index
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.dev}",
                 f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200", "-f", self.path],
                stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [],
                    "note": "nvidia-smi unavailable"}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons, power = [], [], set(), []
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown",
                 "sw_power_cap"]
        try:
            for line in open(self.path):
                f = [x.strip() for x in line.split(",")]
                if len(f) < 9:
                    continue
                try:
                    sm.append(float(f[1]))
                    smax.append(float(f[2]))
                    power.append(float(f[3]))
                except ValueError:
                    continue
                for n, v in zip(names, f[5:9]):
                    if v.lower() == "active":
                        reasons.add(n)
        finally:
            os.unlink(self.path)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [],
                    "note": "no samples"}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(smax),
                "power_w_max": max(power) if power else None,
                "samples": len(sm), "reasons": sorted(reasons)}


# --------------------------------------------------------- GPU timing
def time_chain(chain, ncount, steps, warmup, floattype, seed, first0, world,
               rank, flush, variant=None):
    """Warm up, then time exactly `steps` launches with CUDA events on the
    launching stream (L2 flushed between launches, outside the events).
    Returns per-step milliseconds."""
    import torch
    import torch.distributed as dist
    from acc_gb300 import engine
    from acc_gb300.sharding import shard_range

    def block(k):
        # step k covers world * ncount neutrons; this rank's block of them
        first, count = shard_range(world * ncount, rank, world)
        assert count == ncount
        return first0 + k * world * ncount + first

    stream = torch.cuda.current_stream()
    for w in range(warmup):
        engine.run_chain(chain, ncount, seed=seed, floattype=floattype,
                         first=block(w), sync=False, variant=variant)
    engine.read_status(expected=warmup * ncount if warmup else 0)
    evs = [(torch.cuda.Event(enable_timing=True),
            torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
    if world > 1:
        dist.barrier()
    torch.cuda.synchronize()
    for k in range(steps):
        flush.zero_()
        evs[k][0].record(stream)
        engine.run_chain(chain, ncount, seed=seed, floattype=floattype,
                         first=block(warmup + k), sync=False,
                         variant=variant)
        evs[k][1].record(stream)
    torch.cuda.synchronize()
    if world > 1:
        dist.barrier()
    engine.read_status(expected=steps * ncount)
    return [a.elapsed_time(b) for a, b in evs]


def max_over_ranks(x, world):
    if world == 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64, device="cuda")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def e2e_run(ins, ncount, steps, warmup, seed, world, rank):
    """The FP32 run through the public API with host tallies: per step,
    pinned host -> device tally copies, the chain call, device -> host
    copies and the status check (which synchronises)."""
    import torch
    from acc_gb300 import engine
    from acc_gb300.components.monitors.MonitorBase import MonitorBase
    chain = engine.chain_for_instrument(ins)
    mons = [c for c in ins.components if isinstance(c, MonitorBase)]
    dev = [m._device_tally for m in mons]
    host = [torch.zeros(t.numel(), dtype=torch.float64).pin_memory()
            for t in dev]
    h2d = sum(t.numel() * 8 for t in dev) + __import__("ctypes").sizeof(chain)
    d2h = sum(t.numel() * 8 for t in dev)

    def step(k):
        for h, d in zip(host, dev):
            d.copy_(h, non_blocking=True)
        engine.run_chain(chain, ncount, seed=seed, floattype="float32",
                         first=(k * world + rank) * ncount, sync=False)
        for h, d in zip(host, dev):
            h.copy_(d, non_blocking=True)
        engine.read_status(expected=ncount)

    for k in range(warmup):
        step(k)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for k in range(steps):
        step(warmup + k)
    torch.cuda.synchronize()
    dt = time.perf_counter() - t0
    return dt, h2d, d2h


def batched_run(world, rank, replays=3):
    """64 variants of the sphere chain (Ei log-uniform 20-500 meV, counts
    log-uniform 1e6-1e8, own seed and 180x200 histogram) in one persistent
    FP32 launch replayed from a CUDA graph, launch shape from the
    autotuner."""
    import torch
    from acc_gb300 import autotune, engine, instruments
    ins, counts, seeds = instruments.sphere_variants(64, seed=rank)
    best = autotune.tune_batched(ins, counts, seeds, floattype="float32",
                                 use_cache=False)
    g = engine.BatchedGraph(ins, counts, seeds, floattype="float32",
                            threads_per_block=best["threads_per_block"],
                            blocks=best["blocks"], chunk=best["chunk"])
    g.launch()
    engine.read_status(expected=g.total)
    a = torch.cuda.Event(enable_timing=True)
    b = torch.cuda.Event(enable_timing=True)
    a.record()
    for _ in range(replays):
        g.launch()
    b.record()
    b.synchronize()
    ms = a.elapsed_time(b) / replays
    engine.read_status(expected=replays * g.total)
    ms = max_over_ranks(ms, world)
    g.close()
    return {"variants": 64, "neutrons_per_launch": g.total,
            "value": world * g.total / (ms / 1e3), "unit": UNIT,
            "ms_per_launch": ms, "replays": replays, "dtype": "f32",
            "launch": {k: best[k] for k in
                       ("threads_per_block", "blocks", "chunk")},
            "note": "one persistent launch per CUDA-graph replay"}


def grad_cost(name, ncount, params, reps=2):
    """Kernel time of the FP32 forward (mcv_run_chain) and of the backward
    replay (mcv_backward) on one workload, CUDA events, after a warm-up."""
    import torch
    from acc_gb300 import engine
    from acc_gb300.autograd import GradRun
    ins = build_instrument(name) if isinstance(name, str) else name
    mon = [c for c in ins.components if hasattr(c, "hist_shape")][-1]
    run = GradRun(ins, mon, ncount, seed=11, floattype="float32",
                  params=params(ins))
    dout = torch.randn(mon.nbins(), dtype=torch.float64, device="cuda")
    dparam = {}
    dtable = {}
    for kind, target in run.params.values():
        k = run._index(target[0] if isinstance(target, list) else target)
        c = run.chain.comp[k]
        if kind in ("sqe_table", "powder_F2"):
            n = c.ip[4] * c.ip[5] if kind == "sqe_table" else c.ip[4]
            dtable[k] = torch.zeros(n, dtype=torch.float64, device="cuda")
        else:
            dparam[k] = torch.zeros(3, dtype=torch.float64, device="cuda")

    def fwd():
        engine.run_chain(run.chain, ncount, seed=11, floattype="float32",
                         sync=False)

    def bwd():
        engine.backward(run.chain, ncount, {run.mon_index: dout}, dparam,
                        dtable, seed=11, floattype="float32")

    out = {}
    for label, fn in (("forward_ms", fwd), ("backward_ms", bwd)):
        fn()
        torch.cuda.synchronize()
        best = float("inf")
        for _ in range(reps):
            a = torch.cuda.Event(enable_timing=True)
            b = torch.cuda.Event(enable_timing=True)
            a.record()
            fn()
            b.record()
            b.synchronize()
            best = min(best, a.elapsed_time(b))
        engine.read_status()
        out[label] = best
    out["bwd_over_fwd"] = out["backward_ms"] / out["forward_ms"]
    out["neutrons"] = ncount
    out["monitor_bins"] = mon.nbins()
    return out


def powder_atomic_roofline(ncount=int(1e9), reps=3):
    """Config 5's forward (guide chain -> powder cylinder -> banked detector
    of 2.62e8 bins) in FP32: its rate, and its tally atomics against the
    measured L2 atomic throughput (mcv_probe_atomic_rate: FP64 atomicAdd
    into random bins of an array the size of the detector's tally).  Each
    detected neutron makes three FP64 atomics (N, sum p, sum p^2)."""
    import torch
    from acc_gb300 import engine, instruments
    ins = instruments.powder_banked()
    chain = engine.chain_for_instrument(ins)
    det = ins.components[-1]
    nb = det.nbins()
    engine.run_chain(chain, ncount, seed=7, floattype="float32", sync=False)
    engine.read_status(expected=ncount)
    det._device_tally.zero_()
    a = torch.cuda.Event(enable_timing=True)
    b = torch.cuda.Event(enable_timing=True)
    a.record()
    for r in range(reps):
        engine.run_chain(chain, ncount, seed=7, floattype="float32",
                         first=(r + 1) * ncount, sync=False)
    b.record()
    b.synchronize()
    engine.read_status(expected=reps * ncount)
    s = a.elapsed_time(b) / 1e3 / reps
    detected = float(det._device_tally[:nb].sum()) / reps
    peak = engine.probe_atomic_rate(3 * nb)
    got = 3 * detected / s
    return {"value": ncount / s, "unit": UNIT, "ms_per_launch": 1e3 * s,
            "neutrons_per_launch": ncount, "detector_bins": nb,
            "detected_per_launch": detected,
            "roofline": {"bound": "l2_atomics", "achieved": got,
                         "peak": peak, "unit": "FP64 atomics/s",
                         "frac": got / peak,
                         "per_unit": "3 FP64 atomics per detected neutron",
                         "peak_source": "mcv_probe_atomic_rate over "
                                        f"{3 * nb} doubles (random bins)"}}


def grad_costs():
    from acc_gb300 import instruments
    sqe = grad_cost(
        "sqe_hollow_cylinder", int(1e8),
        lambda ins: {"S": ("sqe_table", ins.components[1]),
                     "mu": ("hss_mu", ins.components[1])})
    pw = grad_cost(
        instruments.powder_banked(), int(1e9),
        lambda ins: {"F2": ("powder_F2", ins.components[5]),
                     "m": ("guide_m", [ins.components[1],
                                       ins.components[2]])})
    return {"sqe_hollow_cylinder": sqe, "powder_banked": pw}


# ---------------------------------------------------------- CPU baseline
def cpu_oracle_rate(workload, seconds, seed, nthreads=0):
    """Neutrons/s of the CPU oracle's timed-baseline build on a bounded
    sample of the workload."""
    from acc_gb300.engine import chain_for_instrument
    from acc_gb300.memory import HostBinder
    from oracle import binding as O
    ins = build_instrument(workload)
    ch = chain_for_instrument(ins, HostBinder())
    nthreads = nthreads or os.cpu_count() or 1
    chunk = 1_000_000
    O.run_chain(ch, 100_000, seed=seed, nthreads=nthreads, timing=True)
    done, t0 = 0, time.perf_counter()
    while True:
        O.run_chain(ch, chunk, seed=seed, first=done, nthreads=nthreads,
                    timing=True)
        done += chunk
        el = time.perf_counter() - t0
        if el >= seconds:
            break
        if el > 0.5 and done / el * (seconds - el) > 4 * chunk:
            chunk *= 2
    return done / el, done, nthreads


def cpu_model():
    try:
        for line in open("/proc/cpuinfo"):
            if line.lower().startswith(("model name", "cpu model")):
                return line.split(":", 1)[1].strip()
        out = subprocess.run(["lscpu"], capture_output=True, text=True).stdout
        for line in out.splitlines():
            if line.startswith("Model name"):
                return line.split(":", 1)[1].strip()
    except OSError:
        pass
    return "unknown"


# ------------------------------------------------------------- arms
def reference_arm(a, rank, world):
    """The reference's CPU path (its restatement: the oracle's timed build)
    on all host cores: each step is the GPU arm's step, --ncount neutrons
    of the same workload."""
    if rank != 0:
        return 0
    sample = int(a.ncount)
    from acc_gb300.engine import chain_for_instrument
    from acc_gb300.memory import HostBinder
    from oracle import binding as O
    from oracle import build as OB
    ins = build_instrument(a.workload)
    ch = chain_for_instrument(ins, HostBinder())
    nthreads = os.cpu_count() or 1
    for w in range(a.warmup):
        O.run_chain(ch, sample, seed=a.seed, first=w * sample,
                    nthreads=nthreads, timing=True)
    t = []
    for k in range(a.steps):
        t0 = time.perf_counter()
        O.run_chain(ch, sample, seed=a.seed, first=(a.warmup + k) * sample,
                    nthreads=nthreads, timing=True)
        t.append(time.perf_counter() - t0)
    value = sample * a.steps / sum(t)
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT,
        "n_gpus": world, "steps": a.steps, "warmup": a.warmup,
        "ms_per_step": 1e3 * sum(t) / a.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic: seeded Philox neutrons, no input data",
        "config": {"workload": WORKLOADS[a.workload],
                   "neutrons_per_step": sample},
        "cpu_baseline": {
            "value": value, "unit": UNIT, "cores": nthreads, "kind": "port",
            "sample": f"{sample} neutrons per step of the same workload "
                      f"(the GPU arm's step), CPU FP64 restatement of the "
                      f"reference chain (mcvine/acc is Python+Numba; its "
                      f"CPU engine mcvine-core is not installable offline) "
                      f"built {OB.describe(timing=True)}, {nthreads} "
                      f"threads; host {cpu_model()}"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))
    return 0


def ours_arm(a, rank, world, local_rank):
    import torch
    import torch.distributed as dist
    from acc_gb300 import _build, engine
    from acc_gb300.components.monitors.MonitorBase import MonitorBase
    _build.build_engine()
    torch.cuda.set_device(local_rank)
    ncount = int(a.ncount)
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32,
                        device="cuda")

    # FP32 fused (headline)
    ins32 = build_instrument(a.workload)
    chain32 = engine.chain_for_instrument(ins32)
    ins64 = build_instrument(a.workload)
    chain64 = engine.chain_for_instrument(ins64)
    clocks = ClockSampler(torch.cuda.current_device())
    clocks.start()
    ms32 = time_chain(chain32, ncount, a.steps, a.warmup, "float32", a.seed,
                      0, world, rank, flush)
    t32 = max_over_ranks(sum(ms32) / 1e3, world)
    # FP64 plain (the clock samples span the three timed regions): the
    # kernel with contracted multiply-adds, and the one that rounds every
    # multiply and add separately (the oracle-parity build)
    ins64f = build_instrument(a.workload)
    chain64f = engine.chain_for_instrument(ins64f)
    ms64f = time_chain(chain64f, ncount, a.steps, a.warmup, "float64",
                       a.seed + 1, 0, world, rank, flush, variant="fp64_fma")
    ms64 = time_chain(chain64, ncount, a.steps, a.warmup, "float64",
                      a.seed + 1, 0, world, rank, flush)
    clk = clocks.stop()
    t64 = max_over_ranks(sum(ms64) / 1e3, world)
    t64f = max_over_ranks(sum(ms64f) / 1e3, world)
    # the FP32 kernel without path regeneration, for comparison
    ins_t = build_instrument(a.workload)
    ms_t = time_chain(engine.chain_for_instrument(ins_t), ncount, a.steps,
                      a.warmup, "float32", a.seed, 0, world, rank, flush,
                      variant="thread")
    t_thread = max_over_ranks(sum(ms_t) / 1e3, world)

    # all ranks' tallies summed (the one collective of the sharded path)
    tallies = []
    for ins in (ins32, ins64):
        ts = [c._device_tally for c in ins.components
              if isinstance(c, MonitorBase)]
        if world > 1:
            for t in ts:
                dist.all_reduce(t)
        tallies.append(ts)

    e2e = None
    if not a.no_e2e:
        ins_e = build_instrument(a.workload)
        engine.chain_for_instrument(ins_e)
        dt, h2d, d2h = e2e_run(ins_e, ncount, a.steps, a.warmup, a.seed + 2,
                               world, rank)
        dt = max_over_ranks(dt, world)
        e2e = {"value": world * ncount * a.steps / dt, "unit": UNIT,
               "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h}

    batched = None
    if not a.no_batched:
        batched = batched_run(world, rank)
    grads = None if a.no_grad or rank != 0 else grad_costs()
    powder = None if a.no_grad or rank != 0 else powder_atomic_roofline()

    if rank != 0:
        return 0

    from acc_gb300.stats import chi2_per_dof, z_summary
    chi2 = {}
    mons = [c for c in ins32.components if isinstance(c, MonitorBase)]
    for mon, g32, g64 in zip(mons, tallies[0], tallies[1]):
        shape = (3,) + tuple(getattr(mon, "shape4", mon.hist_shape))
        h32 = g32.cpu().numpy().reshape(shape)
        h64 = g64.cpu().numpy().reshape(shape)
        c2, dof = chi2_per_dof(h32, h64)
        entry = {"chi2_per_dof": c2, "bins": dof}
        if dof < 100 and len(shape) > 3:
            # too sparse at this neutron count: compare the projection on
            # the first and last axes (sums of N, p, p^2 over the others)
            axes = tuple(range(2, len(shape) - 1))
            h32, h64 = h32.sum(axis=axes), h64.sum(axis=axes)
            c2, dof = chi2_per_dof(h32, h64)
            entry = {"chi2_per_dof": c2, "bins": dof,
                     "projection": "first and last axes"}
        entry["z"] = z_summary(h32, h64)
        chi2[mon.name] = entry

    fp32_peak = engine.probe_fma_peak(32)
    fp64_peak = engine.probe_fma_peak(64)
    sfu_rate = engine.probe_sfu_rate()
    mean_s = statistics.mean(ms32) / 1e3
    counts = KERNEL_COUNTS.get(a.workload, {})
    fpn = counts.get("fp32_flops_per_neutron")
    achieved = fpn * ncount / mean_s / 1e12 if fpn else None
    fp32_pipe = {
        "achieved": achieved, "peak": fp32_peak, "unit": "TFLOP/s",
        "frac": achieved / fp32_peak if achieved else None,
        "per_unit": f"{fpn} executed FP32 flops per neutron (ncu count)",
        "peak_source": "FP32 FMA peak measured in this run "
                       "(mcv_probe_fma_peak); the measured peak file has "
                       "HBM and bf16-tensor peaks only",
        "fp64_peak_tflops": fp64_peak,
        "sfu_peak_ops_per_s": sfu_rate,
        "sfu_peak_source": "mcv_probe_sfu_rate: FP32 ex2.approx chains on "
                           "every SM, measured in this run",
    }
    # the binding limit: one warp instruction per cycle per SM sub-partition
    # (4 per SM); divergence (SIMT efficiency) sets how many warp
    # instructions a neutron costs.  The FP32 pipe is far from its peak
    # (fp32_pipe): the kernel issues control flow, compares and loads
    # between its multiply-adds.
    wpn = counts.get("warp_inst_per_neutron")
    sms = torch.cuda.get_device_properties(
        torch.cuda.current_device()).multi_processor_count
    mhz = (clk or {}).get("sm_mhz") or 2070.0
    peak_issue = sms * 4 * mhz * 1e6
    got = wpn * ncount / mean_s if wpn else None
    traffic = counts.get("dram_bytes_per_launch")
    if traffic is None and counts.get("dram_bytes_per_neutron"):
        traffic = counts["dram_bytes_per_neutron"] * ncount
    roofline = {
        "bound": "issue",
        "achieved": got, "peak": peak_issue, "unit": "warp-inst/s",
        "frac": got / peak_issue if got else None,
        "traffic": traffic,
        "kernel": counts.get("kernel"),
        "per_unit": f"{wpn} warp instructions per neutron (ncu count), "
                    f"{counts.get('thread_inst_per_neutron')} thread "
                    "instructions",
        "peak_source": "SMs x 4 issue slots x median SM clock sampled "
                       "during the timed region",
        "traffic_note": "DRAM bytes from ncu on a "
                        f"{counts.get('captured_neutrons')}-neutron launch, "
                        f"per launch of this run: {counts.get('traffic_note')}",
        "fp32_pipe": fp32_pipe,
    }
    cpu = None
    if world == 1 and not a.no_cpu_baseline:
        from oracle import build as OB
        rate, n, cores = cpu_oracle_rate(a.workload, a.cpu_seconds, a.seed)
        cpu = {"value": rate, "unit": UNIT, "cores": cores, "kind": "port",
               "sample": f"{n} neutrons of the same workload through the CPU "
                         f"FP64 oracle (C, OpenMP, {cores} threads, built "
                         f"{OB.describe(timing=True)}), host {cpu_model()}"}
    value = world * ncount * a.steps / t32
    v64 = world * ncount * a.steps / t64
    v64f = world * ncount * a.steps / t64f
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
        "steps": a.steps, "warmup": a.warmup,
        "ms_per_step": 1e3 * t32 / a.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic: seeded Philox neutrons, no input data",
        "config": {"workload": WORKLOADS[a.workload],
                   "neutrons_per_step_per_gpu": ncount,
                   "precision": "FP32 fused kernel; tof as a compensated "
                                "float pair, tallies FP64",
                   "l2": "512 MiB write between timed launches, outside "
                         "the CUDA events",
                   "parallelism": f"{world} replica(s), disjoint neutron "
                                  "index ranges, one tally all-reduce"},
        "fp64_plain": {"value": v64f, "unit": UNIT,
                       "ms_per_step": 1e3 * t64f / a.steps, "dtype": "f64",
                       "build": "multiply-adds contracted "
                                "(MCV_VARIANT_FP64_FMA)"},
        "fp64_plain_no_fma": {"value": v64, "unit": UNIT,
                              "ms_per_step": 1e3 * t64 / a.steps,
                              "dtype": "f64",
                              "build": "--fmad=false: every multiply and "
                                       "add rounded, as the oracle"},
        "fp32_over_fp64": value / v64f,
        "fp32_over_fp64_basis": "fp64_plain (contracted, the faster FP64 "
                                "kernel)",
        "fp32_over_fp64_no_fma": value / v64,
        "fp32_one_neutron_per_thread": {
            "value": world * ncount * a.steps / t_thread, "unit": UNIT,
            "ms_per_step": 1e3 * t_thread / a.steps,
            "note": "launch variant 1: one neutron per thread to the end "
                    "of the chain (no path regeneration, no multiple-"
                    "scattering tree state machine)"},
        "chi2_fp32_vs_fp64": chi2,
        "bwd_over_fwd": grads,
        "powder_banked_forward": powder,
        "batched": batched,
        "e2e": e2e,
        "roofline": roofline,
        "cpu_baseline": cpu,
        "clocks": clk,
        "gpu_launches": a.steps,
    }
    print(json.dumps(line))
    return 0


def main(argv=None):
    a = parse_args(argv)
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))
    if a.impl == "reference":
        return reference_arm(a, rank, world)
    if world > 1:
        import torch
        import torch.distributed as dist
        torch.cuda.set_device(local_rank)
        dist.init_process_group("nccl")
    try:
        return ours_arm(a, rank, world, local_rank)
    finally:
        if world > 1:
            import torch.distributed as dist
            dist.destroy_process_group()


if __name__ == "__main__":
    sys.exit(main())
