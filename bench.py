#!/usr/bin/env python
"""Benchmark of the receiver-side ping reduction on GB300.

A step is one ping: sort + bin + sparse PSF reduction of one synthetic sample
buffer (rtacx_reduce). Default workload: the dense-directivity precision ping
(2^24 samples, 512 bearings x 4096 ranges); --config selects another.

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
KERNELS_PER_PING = 6   # count, colscan, binscan, scatter, windows, gather


def parse_args():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=20)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", choices=["ours", "reference"], default="ours")
    p.add_argument("--config", default=DEFAULT_CONFIG, choices=sorted(workloads.CONFIGS))
    p.add_argument("--no-cpu-baseline", action="store_true")
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
    """nvidia-smi clocks and throttle reasons sampled every 200 ms."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu: int):
        self.gpu = gpu
        self.proc = None
        self.path = None

    def start(self):
        if not shutil.which("nvidia-smi"):
            return
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.QUERY}",
                                      "--format=csv,noheader,nounits", "-lms", "200"],
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
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            r = [x.strip() for x in r]
            try:
                sm.append(float(r[1]))
                mx.append(float(r[2]))
            except (ValueError, IndexError):
                continue
            for name, v in zip(names, r[5:9]):
                if v.lower() == "active":
                    reasons.add(name)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


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


def cpu_reference_step(wk, rows_per_step: int, threads: int) -> tuple[float, int]:
    """Time the reference algorithm (oracle, FP32 reference arithmetic) on the
    host: full sort + bin of all samples plus the gather of `rows_per_step`
    output rows; extrapolate the gather to every row. Returns seconds per
    ping and the row count actually reduced."""
    from oracle import oracle
    nR = wk.sensor["range_count"]
    r0 = nR // 2 - rows_per_step // 2
    t0 = time.perf_counter()
    oracle.reduce(wk.samples, wk.sensor, mode=1, rows=(r0, r0), threads=threads)
    t_bin = time.perf_counter() - t0
    t0 = time.perf_counter()
    oracle.reduce(wk.samples, wk.sensor, mode=1, rows=(r0, r0 + rows_per_step), threads=threads)
    t_rows = max(time.perf_counter() - t0 - t_bin, 1e-9)
    return t_bin + t_rows * nR / rows_per_step, rows_per_step


def cpu_model() -> str:
    try:
        for line in open("/proc/cpuinfo"):
            if line.lower().startswith(("model name", "cpu part")):
                return line.split(":", 1)[1].strip()
    except OSError:
        pass
    return "unknown"


def run_reference(args, world, rank):
    if rank != 0:
        return
    wk = workloads.CONFIGS[args.config]()
    threads = os.cpu_count() or 1
    rows = 16 if wk.dims == 2 else max(64, wk.sensor["range_count"] // 8)
    for _ in range(args.warmup):
        cpu_reference_step(wk, rows, threads)
    times = [cpu_reference_step(wk, rows, threads)[0] for _ in range(args.steps)]
    t = statistics.median(times)
    value = wk.n / t
    sample = (f"per step: sort+bin of all {wk.n} samples and the FP32 gather of {rows} of "
              f"{wk.sensor['range_count']} output rows, extrapolated to the full ping; median of {args.steps}")
    print(json.dumps({
        "impl": "reference", "metric": "samples/s", "value": value, "unit": "samples/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * t,
        "pings_per_s": 1.0 / t, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32", "data": "synthetic (seeded)",
        "config": {"workload": wk_desc(wk), "form": "reference algorithm, host CPU"},
        "cpu_baseline": {"value": value, "unit": "samples/s", "cores": threads, "kind": "port",
                         "sample": sample, "cpu": cpu_model()},
        "e2e": {"value": value, "unit": "samples/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }))


def wk_desc(wk) -> str:
    s = wk.sensor
    if wk.dims == 1:
        return f"{wk.name}: {wk.n} samples, 1D {s['range_count']} ranges, {len(s['pulse'])}-tap pulse"
    return (f"{wk.name}: {wk.n} samples, {len(s['bearings'])} bearings x {s['range_count']} ranges, "
            f"{len(s['pulse'])}-tap pulse x {len(s['beam'])}-tap beam")


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
    ctx.reserve(n)
    host_in = torch.from_numpy(wk.samples.reshape(-1)).pin_memory()
    d_in = host_in.to("cuda")
    out = torch.empty(wk.out_shape + (2,), dtype=torch.float32, device="cuda")
    host_out = torch.empty(out.shape, dtype=torch.float32).pin_memory()
    stream = torch.cuda.current_stream()

    for _ in range(max(args.warmup, 3)):
        ctx.reduce(d_in, n, out, stream=stream)
    ctx.stream_status(stream)

    # Timed region: K pings, samples resident in HBM.
    clocks = ClockSampler(local)
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    clocks.start()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    for _ in range(args.steps):
        ctx.reduce(d_in, n, out, stream=stream)
    ev1.record(stream)
    torch.cuda.synchronize()
    clk = clocks.stop()
    ctx.stream_status(stream)
    t_dev = max_over_ranks(dist, ev0.elapsed_time(ev1) / 1e3)
    if dist:
        dist.barrier()

    # Per-stage device times on the launching stream (separate pass).
    ctx.set_tracing(True)
    stage = {k: 0.0 for k in _lib.STAGES}
    for _ in range(args.steps):
        ctx.reduce(d_in, n, out, stream=stream)
        for k, v in ctx.stage_times().items():
            stage[k] += v / args.steps
    ctx.set_tracing(False)

    # End to end through the C ABI: pinned host samples in, ping out.
    ctx.reduce(d_in, n, out, stream=stream)
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    ev0.record(stream)
    for _ in range(args.steps):
        d_in.copy_(host_in, non_blocking=True)
        ctx.reduce(d_in, n, out, stream=stream)
        host_out.copy_(out, non_blocking=True)
    ev1.record(stream)
    torch.cuda.synchronize()
    ctx.stream_status(stream)
    t_e2e = max_over_ranks(dist, ev0.elapsed_time(ev1) / 1e3)

    if rank != 0:
        return
    value = world * n * args.steps / t_dev
    e2e_value = world * n * args.steps / t_e2e
    peaks = measured_peaks()

    # Roofline of the dominant kernel (the PSF gather): algorithmic FP32 flops
    # (8 per useful sample x output-cell pair) over its mean launch time.
    pairs = useful_pairs(wk)
    gather_s = stage["reduce"] / 1e3
    fp32_peak = 152 * 128 * 2 * peaks["sm_max_mhz"] * 1e6 / 1e12
    achieved = 8.0 * pairs / gather_s / 1e12 if gather_s > 0 else 0.0
    # Sort / bin: one read of every input record and one write of every sorted
    # record (the survey's algorithmic bytes), over count + scatter + scans.
    rec_in = 16 if wk.dims == 2 else 12
    bin_bytes = n * (rec_in + 16)
    bin_s = (stage["count"] + stage["colscan"] + stage["binscan"] + stage["scatter"] + stage["windows"]) / 1e3
    bin_gbs = bin_bytes / bin_s / 1e9 if bin_s > 0 else 0.0

    line = {
        "metric": "samples/s", "value": value, "unit": "samples/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * t_dev / args.steps,
        "pings_per_s": world * args.steps / t_dev,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded)",
        "config": {"workload": wk_desc(wk), "form": "plain (FP32 SIMT sparse PSF gather)",
                   "l2": "inputs larger than L2 (%.0f MB of samples)" % (n * rec_in / 1e6),
                   "parallelism": f"replicas x{world}"},
        "stage_ms": {k: round(v, 4) for k, v in stage.items()},
        "roofline": {"bound": "fp32", "achieved": achieved, "peak": fp32_peak, "unit": "TFLOP/s",
                     "frac": achieved / fp32_peak, "traffic": None, "kernel": "k_gather_2d" if wk.dims == 2 else "k_gather_1d",
                     "peak_source": "nominal FP32 SIMT (152 SMs x 128 FMA x max clock); no measured FP32 peak",
                     "algorithmic": "8 flop per useful (sample, output cell) pair, %.3e pairs" % pairs},
        "roofline_bin": {"bound": "hbm", "achieved": bin_gbs, "peak": peaks["hbm_gbs"], "unit": "GB/s",
                         "frac": bin_gbs / peaks["hbm_gbs"], "traffic": None,
                         "peak_source": peaks["source"],
                         "algorithmic": f"{rec_in}+16 bytes per sample over count+colscan+binscan+scatter+windows"},
        "e2e": {"value": e2e_value, "unit": "samples/s", "h2d_bytes_per_step": n * rec_in,
                "d2h_bytes_per_step": int(np.prod(wk.out_shape)) * 8},
        "gpu_launches": KERNELS_PER_PING * args.steps,
        "clocks": clk,
    }
    if world == 1 and not args.no_cpu_baseline:
        threads = os.cpu_count() or 1
        rows = 32 if wk.dims == 2 else max(64, wk.sensor["range_count"] // 8)
        t_cpu, rows = cpu_reference_step(wk, rows, threads)
        line["cpu_baseline"] = {
            "value": n / t_cpu, "unit": "samples/s", "cores": threads, "kind": "port",
            "sample": (f"oracle FP32 reference arithmetic: sort+bin of all {n} samples plus the gather of "
                       f"{rows} of {wk.sensor['range_count']} rows, extrapolated"),
            "cpu": cpu_model()}
        # Accuracy of this run's ping against the FP64 oracle on a band of rows.
        from oracle import oracle
        nR = wk.sensor["range_count"]
        r0 = nR // 3
        band = (r0, r0 + (8 if wk.dims == 2 else nR - r0))
        ref = oracle.reduce(wk.samples, wk.sensor, mode=0, rows=band, threads=threads)
        o = out.cpu().numpy()
        got = (o[..., 0].astype(np.float64) + 1j * o[..., 1])[band[0]:band[1]]
        line["accuracy"] = {"rel_l2_vs_fp64": float(np.linalg.norm(got - ref) / np.linalg.norm(ref)),
                            "rows_checked": list(band)}
    print(json.dumps(line))


def main():
    args = parse_args()
    world, rank, local = dist_env()
    if args.impl == "reference":
        run_reference(args, world, rank)
        return
    run_ours(args, world, rank, local)


if __name__ == "__main__":
    main()
