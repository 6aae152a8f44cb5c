#!/usr/bin/env python
"""Benchmark of the receiver-side ping reduction on GB300.

A step is one ping of one synthetic sample buffer. Default workload: the
dense-directivity precision ping (2^24 samples, 512 bearings x 4096 ranges,
1.2 MHz carrier phase and spreading applied on the device); --config selects
another. On 2D workloads with an echo model both forms are timed: the
tensor-core precision form (rtacx_reduce_precision: bin first, BF16x3
contraction over bearings, FP32 range filter) is the headline and the plain
form (rtacx_reduce: sort + bin + per-sample sparse PSF gather) is reported
beside it; otherwise the plain form is the headline.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--config NAME]
  python bench.py --impl reference ...   # the reference algorithm on the host cores

`value` is device throughput with the samples resident in HBM (samples/s);
`e2e` is the same metric through the C ABI with pinned host buffers, the
host->device copy of the samples and the device->host copy of the ping inside
the timed region. The sample buffer (268 MB at 2^24 samples) is larger than
L2 (129 MB), so every step reads it from HBM. Under torchrun each rank runs
an independent replica on its own GPU (pings are independent; no collective
on the data path): `value` is the sum of the ranks' pings over the max time.
"""
from __future__ import annotations

import argparse
import datetime
import inspect
import json
import math
import os
import shutil
import statistics
import subprocess
import sys
import tempfile
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

from rtac_simulation_gb300 import workloads  # noqa: E402

DEFAULT_CONFIG = "precision_2d"
# DRAM bytes per launch (dram__bytes_read.sum + dram__bytes_write.sum) from
# ncu captures of the default workload, each taken with
#   ncu --set full --clock-control none -k regex:<kernel> -s <n> -c 1 \
#       python bench.py --steps 2 --warmup 3 --no-cpu-baseline [--no-next-rows]
# on a GB300. Reported as `traffic` beside the live `achieved` numbers.
NCU_TRAFFIC_BYTES = {
    "k_prec_accumulate_staged": 336.287e6 + 5.313e6,
    "k_gemm_tn": 78.715e6 + 4.004e6,
    "sort_bin": (268.531e6 + 3.186e6) + (273.130e6 + 220.672e6),   # k_count + k_scatter_pipe
}
# The accumulation's bound is the L2's reduction throughput, not HBM: ncu on
# the default workload (profiles/k_prec_accumulate_staged_precision_2d.md)
# shows 1.50 L2 reduction requests (1.57 sectors) per sample and the L2 at
# 65 % of its peak throughput while DRAM carries the algorithmic bytes once.
NCU_ACCUMULATE_L2 = {"l2_throughput_pct": 64.7, "l2_red_sectors_pct": 40.6, "red_sectors_per_sample": 1.57,
                     "red_requests_per_sample": 1.50}

# Plain form: count, bin scan, scatter, windows, then (2D) the tile plan and
# the split gather or (1D) the row gather.
KERNELS_PER_PING = {1: 5, 2: 6}
PRECISION_KERNELS_PER_PING = 5   # clear, staged accumulate, operand split, tensor-core GEMM, range filter


def parse_args():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=None,
                   help="timed steps (default: 500 for this implementation's pings, 3 for the host reference)")
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", choices=["ours", "reference"], default="ours")
    p.add_argument("--config", default=DEFAULT_CONFIG, choices=sorted(workloads.CONFIGS))
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--no-reference-kernel", action="store_true",
                   help="reference arm: skip timing the reference's own CUDA kernel")
    p.add_argument("--no-next-rows", action="store_true",
                   help="skip the timing of the echo-sample epilogue, directivity tables and rasteriser")
    return p.parse_args()


def dist_env():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def init_dist(world):
    if world <= 1:
        return None
    import torch.distributed as dist
    os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
    dist.init_process_group("gloo")
    return dist


def max_over_ranks(dist, x: float) -> float:
    if dist is None:
        return x
    import torch
    t = torch.tensor([x], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 20 ms."""

    QUERY = ("timestamp,index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu: int):
        self.gpu = gpu
        self.proc = None
        self.path = None
        self.t_begin = self.t_end = None

    def begin(self):
        """Marks the start of the timed region (host wall clock)."""
        self.t_begin = datetime.datetime.now()

    def end(self):
        self.t_end = datetime.datetime.now()

    def start(self):
        if not shutil.which("nvidia-smi"):
            return
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.QUERY}",
                                      "--format=csv,noheader,nounits", "-lms", "20"],
                                     stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        time.sleep(0.3)

    def stop(self) -> dict | None:
        if self.proc is None:
            return None
        time.sleep(0.25)
        self.proc.terminate()
        self.proc.wait()
        rows = [l.split(",") for l in open(self.path).read().strip().split("\n") if l.strip()]
        os.unlink(self.path)
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        parsed = []
        for r in rows:
            r = [x.strip() for x in r]
            try:
                ts = datetime.datetime.strptime(r[0], "%Y/%m/%d %H:%M:%S.%f")
                parsed.append((ts, float(r[2]), float(r[3]), [n for n, v in zip(names, r[6:10]) if v.lower() == "active"]))
            except (ValueError, IndexError):
                continue
        region = []
        if self.t_begin and self.t_end:      # the samples taken during the timed region
            lo = self.t_begin - datetime.timedelta(milliseconds=25)
            hi = self.t_end + datetime.timedelta(milliseconds=25)
            region = [p for p in parsed if lo <= p[0] <= hi]
        inside = region or parsed
        if not inside:
            return None
        return {"sm_mhz": statistics.median(p[1] for p in inside), "sm_max_mhz": max(p[2] for p in inside),
                "reasons": sorted({n for p in inside for n in p[3]}), "samples": len(inside),
                "in_timed_region": bool(region)}


def measured_peaks() -> dict:
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return {"hbm_gbs": d["hbm_gbs"], "bf16_tflops": d["bf16_tflops"], "source": "measured",
                "sm_max_mhz": d.get("sm_max_mhz", 2070.0)}
    return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "source": "fallback", "sm_max_mhz": 2070.0}


def useful_pairs(wk) -> float:
    """Algorithmic work of the gather: sum over samples of (output rows inside
    the pulse support) x (bearings inside the beam support)."""
    s = wk.sensor
    R = workloads.linspace(s["range_min"], s["range_max"], s["range_count"]).astype(np.float64)
    scale = float(np.float32(1.0) / np.float32(np.float32(s["pulse_duration"]) * np.float32(s["sound_celerity"])))
    half_r = 0.5 / scale * (1.0 + 1.0 / len(s["pulse"]))
    t = wk.samples[:, 2].astype(np.float64)
    rows = np.searchsorted(R, t + half_r, "left") - np.searchsorted(R, t - half_r, "right")
    if wk.dims == 1:
        return float(rows.sum())
    th = np.sort(np.asarray(s["bearings"], np.float64))
    half_b = 0.5 * s["beam_span"] * (1.0 + 1.0 / len(s["beam"]))
    b = wk.samples[:, 3].astype(np.float64)
    cols = np.searchsorted(th, b + half_b, "left") - np.searchsorted(th, b - half_b, "right")
    return float((rows * cols).sum())


# Samples of the bounded ping the host arms reduce per step: the same
# geometry, tables and sample distributions as the GPU workload, fewer
# samples (the per-sample cost of the reference algorithm -- the gather over
# the PSF support -- does not depend on the sample count).
CPU_PING_SAMPLES = 1 << 17


def full_samples(config: str) -> int:
    """Sample count of a configuration's full ping (its builder's default)."""
    return int(inspect.signature(workloads.CONFIGS[config]).parameters["n_samples"].default)


def cpu_workload(config: str, echo_mode: int = 1):
    """The bounded host ping of a configuration, with the echo epilogue applied
    in the reference's float arithmetic (its ray generator does it before
    this path)."""
    from oracle import oracle
    wk = workloads.CONFIGS[config](n_samples=min(full_samples(config), CPU_PING_SAMPLES))
    if wk.echo:
        wk.samples = oracle.apply_echo(wk.samples, wk.sensor, wk.echo, mode=echo_mode)
    return wk


def cpu_reference_step(wk, threads: int) -> float:
    """Seconds of the reference algorithm (oracle, FP32 reference arithmetic)
    on the host for one whole ping: travel sort, keys, segments, windows and
    the per-sample PSF gather of every output cell."""
    from oracle import oracle
    t0 = time.perf_counter()
    oracle.reduce(wk.samples, wk.sensor, mode=1, threads=threads)
    return time.perf_counter() - t0


def cpu_model() -> str:
    """Host CPU model: lscpu's model name, else /proc/cpuinfo's, else the Arm
    part number's name."""
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.lower().startswith("model name:"):
                return line.split(":", 1)[1].strip()
    except (OSError, subprocess.SubprocessError):
        pass
    arm_parts = {"0xd4f": "Neoverse-V2", "0xd40": "Neoverse-V1", "0xd49": "Neoverse-N2", "0xd0c": "Neoverse-N1"}
    try:
        for line in open("/proc/cpuinfo"):
            key, _, val = line.partition(":")
            if key.strip().lower() == "model name":
                return val.strip()
            if key.strip().lower() == "cpu part":
                return arm_parts.get(val.strip().lower(), f"Arm part {val.strip()}")
    except OSError:
        pass
    return "unknown"


def reference_gpu_kernel(config: str) -> dict:
    """The reference's own 2D reduction kernel (do_sparse_convolve_2d_f,
    src/SensorInstance2D.cu:44-83), compiled from the reference's source for
    sm_103a where the reference tree is (oracle/_ref/ref_sparse2d.cubin) and
    launched as SensorInstance2D::do_reduce does, on this GPU and the full
    workload: CUDA-event time per launch with the samples already
    travel-sorted and binned (its Thrust sort and do_make_bins are not
    included). Reported beside the host arm, not timed as it."""
    from oracle import ref_kernel
    if not ref_kernel.CUBIN.exists():
        return {"unavailable": "oracle/_ref/ref_sparse2d.cubin was not built (no reference tree where it was built)"}
    if config in ("echosounder_1d", "ea400_reference_1d"):
        return {"unavailable": "1D: this arm times the reference's 2D kernel only"}
    with tempfile.TemporaryDirectory() as d:
        tmp = Path(d)
        exe = ref_kernel.build_harness(tmp)
        _, ms, wk = ref_kernel.run_case(exe, tmp, config, config, {}, reps=2)
    return {"ms_per_launch": ms, "samples": int(wk.n), "samples_per_s": wk.n / (ms / 1e3),
            "what": "do_sparse_convolve_2d_f from the reference's source, one 512-thread CTA per output cell, "
                    "PSF texture (linear filter, border); sort and binning excluded; mean of 2 launches after 1"}


def run_reference(args, world, rank):
    if rank != 0:
        return
    if args.config == "batched_mix":
        return run_reference_batch(args)
    wk = cpu_workload(args.config)
    full_desc = wk_desc(wk).replace(f": {wk.n} samples", f": {full_samples(args.config)} samples", 1)
    threads = os.cpu_count() or 1
    for _ in range(args.warmup):
        cpu_reference_step(wk, threads)
    times = [cpu_reference_step(wk, threads) for _ in range(args.steps)]
    t = statistics.median(times)
    value = wk.n / t
    sample = (f"per step: one whole ping of {wk.n} samples with the workload's geometry ({full_desc}): "
              f"sort, keys, segments, windows and the FP32 per-sample PSF gather of all "
              f"{int(np.prod(wk.out_shape))} output cells, nothing extrapolated; median of {args.steps}")
    line = {
        "impl": "reference", "metric": "samples/s", "value": value, "unit": "samples/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * t,
        "pings_per_s": 1.0 / t, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32", "data": "synthetic (seeded)",
        "config": {"workload": full_desc, "form": "reference algorithm, host CPU",
                   "host_ping": f"{wk.n} samples per step (same geometry and distributions)"},
        "cpu_baseline": {"value": value, "unit": "samples/s", "cores": threads, "kind": "port",
                         "sample": sample, "cpu": cpu_model()},
        "e2e": {"value": value, "unit": "samples/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    if not args.no_reference_kernel:
        try:
            line["reference_cuda_kernel"] = reference_gpu_kernel(args.config)
        except Exception as e:   # the host arm stands on its own
            line["reference_cuda_kernel"] = {"unavailable": f"{type(e).__name__}: {e}"[:200]}
    print(json.dumps(line))


def run_reference_batch(args):
    """Reference algorithm on the host for the batched mix, bounded: every
    step reduces 8 of the 64 pings in full (sort, bin and the gather of every
    output cell), each capped at CPU_PING_SAMPLES samples."""
    pings = workloads.batched_mix()
    sample = []
    for wk in pings[::8]:
        if wk.n > CPU_PING_SAMPLES:
            wk = workloads.Workload(wk.name, wk.dims, wk.sensor, wk.samples[:CPU_PING_SAMPLES], wk.meta)
        sample.append(wk)
    threads = os.cpu_count() or 1
    times = []
    for step in range(args.warmup + args.steps):
        t = sum(cpu_reference_step(wk, threads) for wk in sample)
        if step >= args.warmup:
            times.append(t)
    t = statistics.median(times)
    n = sum(wk.n for wk in sample)
    value = n / t
    print(json.dumps({
        "impl": "reference", "metric": "samples/s", "value": value, "unit": "samples/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * t, "pings_per_s": len(sample) / t,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded)",
        "config": {"workload": "batched_mix (8 of the 64 pings per step, each reduced in full, at most "
                               f"{CPU_PING_SAMPLES} samples each)", "form": "reference algorithm, host CPU"},
        "cpu_baseline": {"value": value, "unit": "samples/s", "cores": threads, "kind": "port",
                         "sample": f"8 of the 64 pings ({n} samples) fully reduced per step", "cpu": cpu_model()},
        "e2e": {"value": value, "unit": "samples/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}))


def wk_desc(wk) -> str:
    s = wk.sensor
    if wk.dims == 1:
        return f"{wk.name}: {wk.n} samples, 1D {s['range_count']} ranges, {len(s['pulse'])}-tap pulse"
    return (f"{wk.name}: {wk.n} samples, {len(s['bearings'])} bearings x {s['range_count']} ranges, "
            f"{len(s['pulse'])}-tap pulse x {len(s['beam'])}-tap beam")


def time_form(ctx, form, d_in, n, out, host_in, host_out, steps, warmup, dist, local, torch, echo=None, alt=None):
    """Device time of `steps` pings (samples resident), per-stage event times
    and the end-to-end time with pinned host buffers, for one form. The form
    "precision_compensated" is the precision form with the carrier phase
    reduced in compensated float arithmetic instead of FP64. With `alt` (a
    second context, its host and device ping buffers) the precision forms are
    also timed with two pings in flight: consecutive pings alternate between
    the two contexts on two streams, as a streaming caller double-buffers;
    the timed throughput is the single-stream one (one ping at a time, which
    is also the latency), the two-in-flight time is reported beside it (it
    swings between 0.28 and 0.32 ms per ping from box to box, around the
    single-stream 0.29-0.30 ms, as the two pings' grids share the L2)."""
    from rtac_simulation_gb300 import _lib
    if echo:
        extra = _lib.RTACX_ECHO_PHASE_COMPENSATED if form == "precision_compensated" else 0
        for c in (ctx, alt[0]) if alt else (ctx,):
            c.set_echo_model(echo["carrier_hz"], echo["flags"] | extra)
    call = ctx.reduce if form == "plain" else ctx.reduce_precision
    stream = torch.cuda.current_stream()
    for _ in range(max(warmup, 3)):
        call(d_in, n, out, stream=stream)
    ctx.stream_status(stream)
    clocks = ClockSampler(local)
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    clocks.start()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    dev_lanes = [(ctx, stream, out)]
    if alt and form != "plain":
        dev_lanes.append((alt[0], torch.cuda.Stream(), alt[2]))
    # Single stream, one ping after the other: the timed throughput and the
    # per-ping latency.
    clocks.begin()
    ev0.record(stream)
    for _ in range(steps):
        call(d_in, n, out, stream=stream)
    ev1.record(stream)
    torch.cuda.synchronize()
    clocks.end()
    t_single = max_over_ranks(dist, ev0.elapsed_time(ev1) / 1e3)
    # Two pings in flight (precision forms), reported beside it: consecutive
    # pings alternate between two contexts on two streams.

    def dev_step(i):
        c, s, o = dev_lanes[i % len(dev_lanes)]
        (c.reduce if form == "plain" else c.reduce_precision)(d_in, n, o, stream=s)

    for i in range(max(warmup, 3) * len(dev_lanes)):
        dev_step(i)
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    ev0.record(stream)
    for _, s, _ in dev_lanes[1:]:
        s.wait_event(ev0)
    for i in range(steps):
        dev_step(i)
    for _, s, _ in dev_lanes[1:]:
        done = torch.cuda.Event()
        done.record(s)
        stream.wait_event(done)
    ev1.record(stream)
    torch.cuda.synchronize()
    clk = clocks.stop()
    for c, s, _ in dev_lanes:
        c.stream_status(s)
    ctx.stream_status(stream)
    t_two = max_over_ranks(dist, ev0.elapsed_time(ev1) / 1e3)
    t_dev = t_single

    ctx.set_tracing(True)
    names = _lib.STAGES if form == "plain" else _lib.PRECISION_STAGES
    stage = {k: 0.0 for k in names}
    traced = min(steps, 20)
    for _ in range(traced):
        call(d_in, n, out, stream=stream)
        for k, v in ctx.stage_times(precision=(form != "plain")).items():
            stage[k] += v / traced
    ctx.set_tracing(False)

    # End to end from pinned host memory through the public C ABI: the
    # precision forms use rtacx_reduce_precision_host (chunked host->device
    # copies overlapped with the accumulation, ping copied back) with two
    # pings in flight (two contexts on two streams, as a streaming caller
    # double-buffers: one ping's filter, GEMM and read-back overlap the next
    # ping's copies); the plain form copies the samples in, runs rtacx_reduce
    # and copies the ping out.
    lanes = [(ctx, stream, host_out)]
    if alt and form != "plain":
        lanes.append((alt[0], torch.cuda.Stream(), alt[1]))

    def e2e_step(i):
        if form == "plain":
            d_in.copy_(host_in, non_blocking=True)
            call(d_in, n, out, stream=stream)
            host_out.copy_(out, non_blocking=True)
        else:
            c, s, h = lanes[i % len(lanes)]
            c.reduce_precision_host(host_in, n, h, stream=s)

    for i in range(len(lanes)):
        e2e_step(i)
    torch.cuda.synchronize()
    for c, s, _ in lanes:
        c.stream_status(s)
    if dist:
        dist.barrier()
    ev0.record(stream)
    for _, s, _ in lanes[1:]:
        s.wait_event(ev0)
    for i in range(steps):
        e2e_step(i)
    for _, s, _ in lanes[1:]:
        done = torch.cuda.Event()
        done.record(s)
        stream.wait_event(done)
    ev1.record(stream)
    torch.cuda.synchronize()
    for c, s, _ in lanes:
        c.stream_status(s)
    t_e2e = max_over_ranks(dist, ev0.elapsed_time(ev1) / 1e3)
    # Serial reference points of one step: host->device copy of the samples,
    # the device-resident ping, device->host copy of the ping.
    evs = [torch.cuda.Event(enable_timing=True) for _ in range(4)]
    evs[0].record(stream)
    d_in.copy_(host_in, non_blocking=True)
    evs[1].record(stream)
    call(d_in, n, out, stream=stream)
    evs[2].record(stream)
    host_out.copy_(out, non_blocking=True)
    evs[3].record(stream)
    torch.cuda.synchronize()
    e2e_split = {"h2d_ms": evs[0].elapsed_time(evs[1]), "ping_ms": evs[1].elapsed_time(evs[2]),
                 "d2h_ms": evs[2].elapsed_time(evs[3]), "e2e_step_ms": 1e3 * t_e2e / steps}
    return dict(t_dev=t_dev, t_single=t_single, t_two=t_two, stage=stage, t_e2e=t_e2e, clocks=clk,
                e2e_split=e2e_split, lanes=len(dev_lanes))


def time_next_rows(torch, local, peaks, reps=20, warmup=3):
    """CUDA-event times of the rows either side of the ping reduction, each
    through its C ABI entry point on device-resident inputs:
      make_samples   2^24 ray hits (24 B) -> SimSample2D records (16 B), the
                     ray generator's carrier phase, spreading and receiver
                     directivity lookup (rtacx_make_samples);
      directivity    a rectangle and a disk receiver table (host call + kernel);
      rasterize      a 1.05M-triangle seafloor + sphere at 2048 x 1536 pixels
                     (rtacx_rasterize), and the same followed by the plain
                     ping of an Oculus-like 256-bearing receiver (the GL
                     simulation's per-ping path)."""
    from rtac_simulation_gb300 import _lib, scene
    stream = torch.cuda.current_stream()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)

    def timed(fn):
        for _ in range(warmup):
            fn()
        torch.cuda.synchronize()
        ev0.record(stream)
        for _ in range(reps):
            fn()
        ev1.record(stream)
        torch.cuda.synchronize()
        return ev0.elapsed_time(ev1) / 1e3 / reps

    hbm = peaks["hbm_gbs"]
    res = {"timing": f"CUDA events on the launching stream, {warmup} warm-up + {reps} timed calls, mean per call"}

    # Receiver directivity tables.
    rect = [1.56e-3, 8e-3, 1.25e-3, 1.0, 8.0]
    disk = [6e-3, 1.25e-3, 1.0, 8.0]
    tabs = {}
    # The call includes the host size query and the output allocation.
    bounds = {"rectangle": "launch (size query, allocation and one short kernel)",
              "disk": "FP64 pipe (double sin, cos, atan2, sqrt and j1 per entry, as the reference builder; not profiled)"}
    for name, kind, par in (("rectangle", _lib.RTACX_DIRECTIVITY_RECTANGLE, rect),
                            ("disk", _lib.RTACX_DIRECTIVITY_DISK, disk)):
        t = timed(lambda: _lib.directivity_table(kind, par, stream=stream))
        tabs[name] = _lib.directivity_table(kind, par, stream=stream)
        e = tabs[name].numel()
        res[f"directivity_{name}"] = {"entries": e, "us_per_table": 1e6 * t, "entries_per_s": e / t,
                                      "params": par, "bound": bounds[name]}

    # Echo-sample epilogue on 2^24 hits.
    wk = workloads.oculus_reference_2d(n_samples=16)
    ctx = _lib.Context(local)
    ctx.configure_2d(**wk.sensor)
    ctx.configure_receiver(np.eye(3), tabs["rectangle"].cpu().numpy(), carrier_hz=1.2e6,
                           flags=_lib.RTACX_ECHO_PHASE | _lib.RTACX_ECHO_SPREADING)
    n = 1 << 24
    g = torch.Generator(device="cuda")
    g.manual_seed(7)
    hits = torch.empty((n, 6), dtype=torch.float32, device="cuda")
    hits[:, 0:2].normal_(generator=g)
    hits[:, 2].uniform_(0.2, 6.0, generator=g)
    az = torch.empty(n, device="cuda").uniform_(-1.3, 1.3, generator=g)
    el = torch.empty(n, device="cuda").uniform_(-0.4, 0.4, generator=g)
    hits[:, 3], hits[:, 4], hits[:, 5] = torch.cos(el) * torch.cos(az), torch.cos(el) * torch.sin(az), torch.sin(el)
    del az, el
    smp = torch.empty((n, 4), dtype=torch.float32, device="cuda")
    t = timed(lambda: ctx.make_samples(hits, n, smp, stream=stream))
    ctx.stream_status(stream)
    gbs = n * 40 / t / 1e9
    res["make_samples"] = {"hits": n, "ms": 1e3 * t, "hits_per_s": n / t,
                           "roofline": {"bound": "hbm", "achieved": gbs, "peak": hbm, "unit": "GB/s", "frac": gbs / hbm,
                                        "algorithmic": "24 B hit read + 16 B sample written per hit",
                                        "peak_source": peaks["source"]},
                           "l2": "inputs larger than L2 (671 MB per call)"}
    del hits, smp

    # Rasteriser.
    V, N, T = scene.seafloor_and_sphere(grid=724)
    W, H = 2048, 1536
    S = (scene.perspective(70.0, W / H, 0.1, 100.0)).astype(np.float32)
    L = np.eye(4, dtype=np.float32)
    dV, dN = torch.from_numpy(V).cuda(), torch.from_numpy(N).cuda()
    dT = torch.from_numpy(T.view(np.int32)).cuda()
    px = torch.empty((H * W, 4), dtype=torch.float32, device="cuda")
    raster = lambda: ctx.rasterize(dV, dN, dT, L, S, np.zeros(3, np.float32), W, H, px, stream=stream)
    t = timed(raster)
    ctx.stream_status(stream)
    covered = int((px[:, 2] > 0).sum().item())
    # Lower bound of the DRAM bytes: visibility buffer cleared, read by the
    # resolve (8 B each) and one sample written per pixel (16 B); vertices
    # read (24 B) and transformed (48 B); triangle indices read (12 B).
    alg = W * H * (8 + 8 + 16) + V.shape[0] * (24 + 48) + T.shape[0] * 12
    gbs = alg / t / 1e9
    res["rasterize"] = {"triangles": int(T.shape[0]), "vertices": int(V.shape[0]), "pixels": W * H,
                        "covered_pixels": covered, "ms": 1e3 * t, "pixels_per_s": W * H / t,
                        "triangles_per_s": T.shape[0] / t,
                        "roofline": {"bound": "hbm", "achieved": gbs, "peak": hbm, "unit": "GB/s", "frac": gbs / hbm,
                                     "algorithmic": "32 B per pixel + 72 B per vertex + 12 B per triangle (lower bound)",
                                     "peak_source": peaks["source"]}}
    # Mesh -> ping: rasterised samples reduced by a receiver ranged to the
    # scene (1 .. 45 m, adaptive pulse), as the GL simulation does per ping.
    rmin, rmax, c = 1.0, 45.0, 1500.0
    duration = workloads.adaptive_duration(rmin, rmax, 500, c)
    sensor = dict(wk.sensor)
    sensor.update(range_min=rmin, range_max=rmax, pulse_duration=float(duration),
                  margin=float(workloads.F32(workloads.F32(c) * duration)),
                  pulse=workloads.waveform_sine(1.2e6, float(duration), 8))
    ctx.configure_2d(**sensor)
    ping = torch.empty((sensor["range_count"], len(sensor["bearings"]), 2), dtype=torch.float32, device="cuda")

    def mesh_to_ping():
        raster()
        ctx.reduce(px, W * H, ping, stream=stream)

    t = timed(mesh_to_ping)
    ctx.stream_status(stream)
    res["mesh_to_ping"] = {"ms": 1e3 * t, "pings_per_s": 1.0 / t,
                           "receiver": f"{sensor['range_count']} ranges x {len(sensor['bearings'])} bearings, 1-45 m, "
                                       "plain form"}
    return res


def to_complex(t):
    o = t.cpu().numpy()
    return o[..., 0].astype(np.float64) + 1j * o[..., 1]


def run_ours(args, world, rank, local):
    import torch
    from rtac_simulation_gb300 import _lib

    dist = init_dist(world)
    torch.cuda.set_device(local)
    wk = workloads.CONFIGS[args.config]()
    n = wk.n
    ctx = _lib.Context(local)
    if wk.dims == 1:
        ctx.configure_1d(**wk.sensor)
    else:
        ctx.configure_2d(**wk.sensor)
    if wk.echo:
        ctx.set_echo_model(wk.echo["carrier_hz"], wk.echo["flags"])
    forms = ["plain"]
    steer = wk.precision.get("steer", 0.0)
    if wk.dims == 2 and wk.echo:
        tab = workloads.precision_tables(wk.sensor, **wk.precision)
        ctx.configure_precision(**tab)
        forms = ["precision", "precision_compensated", "precision_fp16", "plain"]
        if args.config == "stress_2d":   # the clustered ping: also with the hot-range replicas
            forms.insert(3, "precision_hot")
    ctx.reserve(n)
    host_in = torch.from_numpy(wk.samples.reshape(-1)).pin_memory()
    d_in = host_in.to("cuda")
    # The plain form reads the samples rotated by exp(i kappa sin theta_s):
    # its ping rotated by exp(-i kappa sin theta_b) is then the per-sample
    # counterpart of the precision form's steered complex directivity (the
    # work per ping does not depend on the values).
    if steer:
        plain_host = torch.from_numpy(workloads.steer_samples(wk.samples, steer).reshape(-1)).pin_memory()
        plain_dev = plain_host.to("cuda")
    else:
        plain_host, plain_dev = host_in, d_in
    outs = {f: torch.empty(wk.out_shape + (2,), dtype=torch.float32, device="cuda") for f in forms}
    host_out = torch.empty(wk.out_shape + (2,), dtype=torch.float32).pin_memory()
    alt = None
    if "precision" in forms:   # second context: two pings in flight in the end-to-end loop
        ctx2 = _lib.Context(local)
        ctx2.configure_2d(**wk.sensor)
        ctx2.configure_precision(**tab)
        alt = (ctx2, torch.empty(wk.out_shape + (2,), dtype=torch.float32).pin_memory(),
               torch.empty(wk.out_shape + (2,), dtype=torch.float32, device="cuda"))
    res = {}
    for f in forms:
        if f in ("precision_fp16", "precision_hot"):   # FP16 contraction / hot-range replicas, FP64 phase
            fl = _lib.RTACX_PRECISION_FP16_ROWSCALE if f == "precision_fp16" else _lib.RTACX_PRECISION_HOT_RANGE
            for c in (ctx, alt[0]):
                c.configure_precision(**tab, flags=fl)
        # The plain form (~72 ms per ping here) is timed over at most 20 steps
        # when it is not the headline form.
        steps_f = min(args.steps, 20) if (f == "plain" and forms[0] != "plain") else args.steps
        src_dev, src_host = (plain_dev, plain_host) if f == "plain" else (d_in, host_in)
        res[f] = time_form(ctx, f, src_dev, n, outs[f], src_host, host_out, steps_f, args.warmup, dist, local, torch,
                           wk.echo, alt)
        res[f]["steps"] = steps_f
        if f in ("precision_fp16", "precision_hot"):
            for c in (ctx, alt[0]):
                c.configure_precision(**tab)
    if rank != 0:
        return
    head = forms[0]
    peaks = measured_peaks()
    rec_in = 16 if wk.dims == 2 else 12

    def form_line(f):
        r = res[f]
        return {"samples_per_s": world * n * r["steps"] / r["t_dev"], "ms_per_step": 1e3 * r["t_dev"] / r["steps"],
                "ms_per_step_two_in_flight": 1e3 * r["t_two"] / r["steps"] if r["lanes"] > 1 else None,
                "e2e_samples_per_s": world * n * r["steps"] / r["t_e2e"], "steps": r["steps"],
                "stage_ms": {k: round(v, 4) for k, v in r["stage"].items()},
                "e2e_step_ms": {k: round(v, 4) for k, v in r["e2e_split"].items()},
                "clocks": r["clocks"]}

    line = {
        "metric": "samples/s", "value": world * n * args.steps / res[head]["t_dev"], "unit": "samples/s",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * res[head]["t_dev"] / args.steps,
        "pings_per_s": world * args.steps / res[head]["t_dev"],
        "latency_ms": 1e3 * res[head]["t_single"] / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded)",
        "config": {"workload": wk_desc(wk),
                   "form": ("precision: bin onto range nodes two bins apart x a 4x bearing grid, BF16x3 tcgen05 "
                            "complex contraction (K split in two), FP32 polyphase range filter, FP64 carrier phase"
                            if head == "precision" else "plain (FP32 SIMT sparse PSF gather)"),
                   "l2": ("inputs larger than L2 (%.0f MB of samples)" if n * rec_in > 129e6 else
                          "inputs smaller than L2 (%.0f MB of samples): timed warm, not flushed") % (n * rec_in / 1e6),
                   "timing": ("one ping at a time on one stream (two pings in flight on two contexts and "
                              "two streams measured beside it: forms.*.ms_per_step_two_in_flight, within "
                              "+/-10 % of it from box to box as the two pings' grids share the L2)"
                              if head == "precision" else "one ping at a time on one stream"),
                   "e2e_path": ("rtacx_reduce_precision_host from pinned host memory, two pings in flight "
                                "(two contexts, two streams)" if head == "precision" else
                                "pinned H2D copy + rtacx_reduce + D2H copy"),
                   "parallelism": f"replicas x{world}"},
        "forms": {f: form_line(f) for f in forms},
    }
    if "precision" in forms:
        line["precision_speedup_vs_plain"] = ((res["plain"]["t_dev"] / res["plain"]["steps"]) /
                                              (res["precision"]["t_dev"] / res["precision"]["steps"]))

    # Rooflines. Plain gather: 8 flop per useful (sample, cell) pair.
    st = res["plain"]["stage"]
    pairs = useful_pairs(wk)
    gather_s = st["reduce"] / 1e3
    fp32_peak = 152 * 128 * 2 * peaks["sm_max_mhz"] * 1e6 / 1e12
    gather_tf = 8.0 * pairs / gather_s / 1e12 if gather_s > 0 else 0.0
    roof_plain = {"bound": "fp32" if wk.dims == 1 else "issue (operand construction of the tensor-core gather)",
                  "achieved": gather_tf, "peak": fp32_peak, "unit": "TFLOP/s",
                  "frac": gather_tf / fp32_peak, "traffic": None,
                  "kernel": "k_gather_tc (TF32 x3 tcgen05)" if wk.dims == 2 else "k_gather_1d",
                  "peak_source": "nominal FP32 SIMT (152 SMs x 128 FMA x max clock), the FP32-equivalent "
                                 "denominator of the useful work; no measured FP32 peak",
                  "algorithmic": "8 flop per useful (sample, output cell) pair, %.3e pairs" % pairs}
    bin_bytes = n * (rec_in + 16)
    bin_s = (st["count"] + st["reset"] + st["binscan"] + st["scatter"] + st["windows"]) / 1e3
    bin_gbs = bin_bytes / bin_s / 1e9 if bin_s > 0 else 0.0
    ncu = NCU_TRAFFIC_BYTES if args.config == DEFAULT_CONFIG else {}
    line["roofline_sort_bin"] = {"bound": "hbm", "achieved": bin_gbs, "peak": peaks["hbm_gbs"], "unit": "GB/s",
                                 "frac": bin_gbs / peaks["hbm_gbs"], "traffic": ncu.get("sort_bin"),
                                 "peak_source": peaks["source"],
                                 "algorithmic": f"{rec_in}+16 bytes per sample over count+reset+binscan+scatter+windows"}
    if "precision" in forms:
        ps = res["precision"]["stage"]
        nR, nB = wk.sensor["range_count"], len(wk.sensor["bearings"])
        cells = tab["grid_count"]
        rows_g = (nR - 1) // 2 + 1 + np.asarray(tab["range_taps"]).reshape(2, -1).shape[1] + 1
        # Accumulate: one read of every sample (16 B) + the binned grid (one
        # 16-byte {left, right} pair per node and bearing interval) written once.
        acc_bytes = n * rec_in + rows_g * cells * 16
        acc_gbs = acc_bytes / (ps["accumulate"] / 1e3) / 1e9
        Mp, Np, Kp = -(-rows_g // 128) * 128, -(-2 * nB // 256) * 256, -(-6 * cells // 64) * 64
        gemm_tf = 2.0 * Mp * Np * Kp / (ps["gemm"] / 1e3) / 1e12
        roof_acc = {"bound": "hbm", "achieved": acc_gbs, "peak": peaks["hbm_gbs"], "unit": "GB/s",
                    "frac": acc_gbs / peaks["hbm_gbs"], "traffic": ncu.get("k_prec_accumulate_staged"),
                    "kernel": "k_prec_accumulate_staged",
                    "peak_source": peaks["source"],
                    "algorithmic": f"{rec_in} B per sample read + 16 B per grid interval ({rows_g} x {cells})",
                    "l2_bound": dict(NCU_ACCUMULATE_L2, reductions_per_s=NCU_ACCUMULATE_L2["red_sectors_per_sample"]
                                     * n / (ps["accumulate"] / 1e3),
                                     note="bound by the L2's reduction rate (two 16-byte vector reductions "
                                          "per sample into a 68 MB L2-resident grid, lane pairs sending a sample's "
                                          "two node rows as one sector when they share it: 1.5 requests per "
                                          "sample); HBM carries the samples once")}
        roof_gemm = {"bound": "tensor", "achieved": gemm_tf, "peak": peaks["bf16_tflops"], "unit": "TFLOP/s",
                     "frac": gemm_tf / peaks["bf16_tflops"], "traffic": ncu.get("k_gemm_tn"), "kernel": "k_gemm_tn",
                     "peak_source": peaks["source"],
                     "algorithmic": f"2*M*N*K with M={Mp} N={Np} K={Kp} (three BF16 split products as one K)"}
        dominant = max(("accumulate", "gemm", "filter", "split"), key=lambda k: ps[k])
        line["roofline"] = roof_gemm if dominant == "gemm" else roof_acc
        line["roofline"]["dominant_stage"] = dominant
        line["roofline_gemm"] = roof_gemm
        line["roofline_accumulate"] = roof_acc
        line["roofline_plain_gather"] = roof_plain
    else:
        line["roofline"] = roof_plain
    r = res[head]
    line["e2e"] = {"value": world * n * args.steps / r["t_e2e"], "unit": "samples/s",
                   "h2d_bytes_per_step": n * rec_in, "d2h_bytes_per_step": int(np.prod(wk.out_shape)) * 8}
    line["gpu_launches"] = (PRECISION_KERNELS_PER_PING if head == "precision" else KERNELS_PER_PING[wk.dims]) * args.steps
    line["clocks"] = r["clocks"]
    if world == 1 and args.config == DEFAULT_CONFIG and not args.no_next_rows:
        line["next_rows"] = time_next_rows(torch, local, peaks)

    if world == 1 and not args.no_cpu_baseline:
        from oracle import oracle
        threads = os.cpu_count() or 1
        cpu_wk = cpu_workload(args.config)
        t_cpu = statistics.median(cpu_reference_step(cpu_wk, threads) for _ in range(3))
        line["cpu_baseline"] = {
            "value": cpu_wk.n / t_cpu, "unit": "samples/s", "cores": threads, "kind": "port",
            "sample": (f"oracle FP32 reference arithmetic (per-sample PSF, float carrier phase as the reference): "
                       f"one whole ping of {cpu_wk.n} samples with this workload's geometry, all "
                       f"{int(np.prod(cpu_wk.out_shape))} output cells, median of 3, nothing extrapolated"),
            "cpu": cpu_model()}
        # Bit-exact bin counts of this ping against the oracle's keys.
        s_ = wk.sensor
        keys, side = oracle.range_keys(s_["range_count"], s_["range_min"], s_["range_max"], s_["margin"],
                                       wk.samples[:, 2])
        want_counts = np.bincount(keys[keys != 0xFFFFFFFF].astype(np.int64), minlength=s_["range_count"])
        g_counts = torch.empty(s_["range_count"], dtype=torch.int32, device="cuda")
        g_oor = torch.empty(2, dtype=torch.int64, device="cuda")
        ctx.bin(d_in, n, wk.dims, counts=g_counts, oor=g_oor, stream=torch.cuda.current_stream())
        ctx.stream_status(torch.cuda.current_stream())
        line["bin_counts_bit_exact"] = bool(
            np.array_equal(g_counts.cpu().numpy().view(np.uint32), want_counts.astype(np.uint32)) and
            g_oor.cpu().tolist() == [int((side < 0).sum()), int((side > 0).sum())])
        # Accuracy of this run's pings against their FP64 oracles on bands of rows.
        nR = wk.sensor["range_count"]
        exact = oracle.apply_echo(wk.samples, wk.sensor, wk.echo) if wk.echo else wk.samples
        exact_steered = workloads.steer_samples(exact, steer) if steer else exact
        acc = {}
        bands = [(0, 16), (nR // 3, nR // 3 + 16), (nR // 2, nR // 2 + 16)] if wk.dims == 2 else [(0, nR)]
        got_plain = to_complex(outs["plain"])
        if steer:
            got_plain = workloads.steer_ping(got_plain, wk.sensor["bearings"], steer)
        for b0, b1 in bands:
            # The per-sample PSF in FP64 (the steered counterpart where the directivity is steered).
            want = oracle.reduce(exact_steered, wk.sensor, mode=0, rows=(b0, b1), threads=threads)
            if steer:
                want = workloads.steer_ping(want, wk.sensor["bearings"], steer)
            if not np.linalg.norm(want) > 0:      # no echo in this band
                continue
            rel = lambda a_, b_: float(np.linalg.norm(a_ - b_) / np.linalg.norm(b_))
            acc.setdefault("plain_rel_l2_vs_fp64", []).append(rel(got_plain[b0:b1], want))
            if "precision" in forms:
                want_b = oracle.reduce_binned(exact, wk.sensor, tab, rows=(b0, b1), threads=threads)
                for f in [f_ for f_ in forms if f_.startswith("precision")]:
                    got_p = to_complex(outs[f])
                    acc.setdefault(f"{f}_rel_l2_vs_fp64_binned", []).append(rel(got_p[b0:b1], want_b))
                acc.setdefault("precision_rel_l2_vs_fp64_per_sample", []).append(
                    rel(to_complex(outs["precision"])[b0:b1], want))
                acc.setdefault("precision_rel_l2_vs_plain_fp32_path", []).append(
                    rel(to_complex(outs["precision"])[b0:b1], got_plain[b0:b1]))
                acc.setdefault("binned_vs_per_sample_model_rel_l2", []).append(rel(want_b, want))
        acc["rows_checked"] = bands
        acc["note"] = ("fp64_binned: the FP64 oracle of the binned model the precision form computes; "
                       "fp64_per_sample / binned_vs_per_sample: against the reference's per-sample PSF in FP64")
        line["accuracy"] = acc
    print(json.dumps(line))


def run_batch(args, world, rank, local):
    """Batched mixed-sensor set: 64 heterogeneous pings in one CUDA graph
    (rtacx_batch_*, autotuned); pings/s, per-ping device latency."""
    import torch
    from rtac_simulation_gb300 import _lib

    dist = init_dist(world)
    torch.cuda.set_device(local)
    pings = workloads.batched_mix()
    ctxs, host_in, d_in, outs, host_out = [], [], [], [], []
    for wk in pings:
        c = _lib.Context(local)
        (c.configure_1d if wk.dims == 1 else c.configure_2d)(**wk.sensor)
        c.reserve(wk.n)
        ctxs.append(c)
        h = torch.from_numpy(wk.samples.reshape(-1)).pin_memory()
        host_in.append(h)
        d_in.append(h.to("cuda"))
        outs.append(torch.empty(wk.out_shape + (2,), device="cuda"))
        host_out.append(torch.empty(wk.out_shape + (2,)).pin_memory())
    batch = _lib.Batch(local)
    plan_args = [(c, d, wk.n, o) for wk, c, d, o in zip(pings, ctxs, d_in, outs)]
    stream = torch.cuda.current_stream()
    # The staged form (one launch per binning stage + persistent gather),
    # timed first for comparison; then the fused single-launch form.
    batch.plan(plan_args, autotune=True, staged=True)
    staged = {"tuning": batch.tuning(), "graph_kernels": batch.graph_kernels()}
    for _ in range(max(args.warmup, 3)):
        batch.run(stream)
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    for _ in range(args.steps):
        batch.run(stream)
    ev1.record(stream)
    batch.status(stream)
    staged["ms_per_step"] = ev0.elapsed_time(ev1) / args.steps
    batch.plan(plan_args, autotune=True)
    kernels = batch.graph_kernels()
    for _ in range(max(args.warmup, 3)):
        batch.run(stream)
    batch.status(stream)
    torch.cuda.synchronize()
    clocks = ClockSampler(local)
    if dist:
        dist.barrier()
    clocks.start()
    clocks.begin()
    ev0.record(stream)
    for _ in range(args.steps):
        batch.run(stream)
    ev1.record(stream)
    torch.cuda.synchronize()
    clocks.end()
    clk = clocks.stop()
    batch.status(stream)
    t_dev = max_over_ranks(dist, ev0.elapsed_time(ev1) / 1e3)
    # Per-ping device latency: each ping alone through rtacx_reduce.
    lat = []
    for wk, c, d, o in zip(pings, ctxs, d_in, outs):
        c.reduce(d, wk.n, o, stream=stream)
        ev0.record(stream)
        c.reduce(d, wk.n, o, stream=stream)
        ev1.record(stream)
        torch.cuda.synchronize()
        lat.append(ev0.elapsed_time(ev1))
    batch.run(stream)
    torch.cuda.synchronize()
    ev0.record(stream)
    for _ in range(args.steps):
        for h, d in zip(host_in, d_in):
            d.copy_(h, non_blocking=True)
        batch.run(stream)
        for o, h in zip(outs, host_out):
            h.copy_(o, non_blocking=True)
    ev1.record(stream)
    torch.cuda.synchronize()
    t_e2e = max_over_ranks(dist, ev0.elapsed_time(ev1) / 1e3)
    if rank != 0:
        return
    total = sum(wk.n for wk in pings)
    pairs = sum(useful_pairs(wk) for wk in pings)
    peaks = measured_peaks()
    fp32_peak = 152 * 128 * 2 * peaks["sm_max_mhz"] * 1e6 / 1e12
    tf = 8.0 * pairs * args.steps / t_dev / 1e12
    rec_bytes = sum(wk.n * (16 if wk.dims == 2 else 12) for wk in pings)
    line = {
        "metric": "samples/s", "value": world * total * args.steps / t_dev, "unit": "samples/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * t_dev / args.steps,
        "pings_per_s": world * len(pings) * args.steps / t_dev,
        "per_ping_latency_ms": {"median": float(np.median(lat)), "p90": float(np.percentile(lat, 90)),
                                "max": float(np.max(lat)), "batched_amortised": 1e3 * t_dev / args.steps / len(pings)},
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded)",
        "config": {"workload": f"batched_mix: {len(pings)} pings, {total} samples (log-uniform 2^14..2^22), "
                               "50% 512-bearing 2D, 25% 256-bearing 2D, 25% 1D 2048 ranges",
                   "form": "plain, batched: one cooperative persistent kernel (zero, count, scan, windows, "
                           "scatter, gather of every ping, bounded grid barriers) in one CUDA graph",
                   "tuning": batch.tuning(), "graph_kernels": kernels, "parallelism": f"replicas x{world}"},
        "staged_form": staged,
        "roofline": {"bound": "fp32", "achieved": tf, "peak": fp32_peak, "unit": "TFLOP/s", "frac": tf / fp32_peak,
                     "traffic": None, "kernel": "k_batch_fused (the whole batch)",
                     "peak_source": "nominal FP32 SIMT", "algorithmic": "8 flop per useful (sample, cell) pair, %.3e pairs" % pairs},
        "e2e": {"value": world * total * args.steps / t_e2e, "unit": "samples/s",
                "h2d_bytes_per_step": rec_bytes, "d2h_bytes_per_step": sum(int(np.prod(wk.out_shape)) * 8 for wk in pings)},
        "gpu_launches": kernels * args.steps, "clocks": clk,
    }
    print(json.dumps(line))


def main():
    args = parse_args()
    if args.steps is None:   # the host reference's steps take seconds, a batch ~70 ms, a precision ping ~0.2 ms
        args.steps = 3 if args.impl == "reference" else (20 if args.config == "batched_mix" else 500)
    world, rank, local = dist_env()
    if args.impl == "reference":
        run_reference(args, world, rank)
        return
    if args.config == "batched_mix":
        run_batch(args, world, rank, local)
        return
    run_ours(args, world, rank, local)


if __name__ == "__main__":
    main()
