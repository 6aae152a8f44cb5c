"""Runs the reference's own 2D reduction kernel on a GPU machine.

TEST INFRASTRUCTURE ONLY. do_sparse_convolve_2d_f (src/SensorInstance2D.cu:
44-83) is compiled from the reference tree into oracle/_ref/ref_sparse2d.cubin
by oracle/ref_build.sh (where the reference tree is), against the stand-ins
of oracle/ref_stubs_cuda. oracle/ref_sparse_harness.cpp launches it as
SensorInstance2D::do_reduce does (src/SensorInstance2D.cu:85-119). The
inputs are a seeded workload's samples, sorted by travel, and the reference
bin views of the oracle (bit-exact against the reference's own key
arithmetic). Used by tests/golden/make_ref_pings.py (golden pings) and bench.py's
reference arm (the kernel's time on the same GPU). run_case_1d does the same
for the reference's 1D kernel (oracle/_ref/ref_sparse1d.cubin).
"""
from __future__ import annotations

import os
import struct
import subprocess
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))

from oracle import oracle  # noqa: E402
from rtac_simulation_gb300 import workloads as wl  # noqa: E402

CUBIN = HERE / "_ref" / "ref_sparse2d.cubin"
CUBIN_1D = HERE / "_ref" / "ref_sparse1d.cubin"
HARNESS_SRC = HERE / "ref_sparse_harness.cpp"


def require_cubin(path: Path = CUBIN) -> None:
    if not path.exists():
        raise SystemExit(f"{path} is missing: build it with oracle/ref_build.sh where the reference tree is")


def build_harness(out: Path) -> Path:
    cuda = Path(os.environ.get("CUDA_HOME", "/usr/local/cuda"))
    exe = out / "ref_sparse_harness"
    subprocess.run(["g++", "-std=c++17", "-O1", "-I", str(HERE / "ref_stubs_cuda"),
                    "-I", str(cuda / "include"), str(HARNESS_SRC), "-L", str(cuda / "lib64"),
                    "-L", str(cuda / "lib64" / "stubs"), "-lcudart", "-lcuda", "-o", str(exe)], check=True)
    return exe


def case_inputs(builder: str, kwargs: dict):
    """(workload, travel-sorted samples, bin views, PSF image, x scale, y scale)."""
    wk = getattr(wl, builder)(**kwargs)
    s = wk.sensor
    order = np.argsort(wk.samples[:, 2], kind="stable")
    sorted_smp = np.ascontiguousarray(wk.samples[order], dtype=np.float32)
    views = oracle.bin_samples(sorted_smp, s)["windows"].astype(np.uint64)
    pulse = np.asarray(s["pulse"], dtype=np.complex64)
    beam = np.asarray(s["beam"], dtype=np.float32)
    # generate_psf_data: PSF[h][w] = waveform[h] * beam[w], in float.
    psf = (pulse[:, None] * beam[None, :].astype(np.complex64)).astype(np.complex64)
    xscale = np.float32(np.float32(1.0) / np.float32(s["beam_span"]))
    yscale = oracle.pulse_scale(s)
    return wk, sorted_smp, views, psf, xscale, yscale


def run_case(exe: Path, tmp: Path, name: str, builder: str, kwargs: dict, reps: int = 0):
    """(the reference kernel's ping (complex64 [nR][nB]), with reps > 0 its
    mean time per launch in ms (else None), the workload)."""
    wk, smp, views, psf, xscale, yscale = case_inputs(builder, kwargs)
    s = wk.sensor
    bear = np.asarray(s["bearings"], dtype=np.float32)
    nB, nR = bear.size, s["range_count"]
    H, W = psf.shape
    src, dst = tmp / f"{name}.in", tmp / f"{name}.out"
    with open(src, "wb") as f:
        f.write(struct.pack("<5IQ", 0x474E5052, nB, nR, W, H, smp.shape[0]))
        f.write(np.array([s["range_min"], s["range_max"], xscale, yscale], dtype=np.float32).tobytes())
        f.write(bear.tobytes())
        f.write(psf.tobytes())
        f.write(smp.tobytes())
        f.write(np.ascontiguousarray(views).tobytes())
    cmd = [str(exe), str(CUBIN), str(src), str(dst)] + ([str(reps)] if reps else [])
    res = subprocess.run(cmd, check=True, capture_output=True, text=True)
    ms = None
    for line in res.stdout.splitlines():
        if line.startswith("ref_kernel_ms "):
            ms = float(line.split()[1])
    if reps and ms is None:
        raise SystemExit(f"{name}: the harness printed no time")
    ping = np.fromfile(dst, dtype=np.complex64).reshape(nR, nB)
    src.unlink()
    dst.unlink()
    return ping, ms, wk


# Address modes of the 1D pulse texture the harness can bind (the reference's
# own 1D texture takes rtac_base defaults, which are not vendored).
ADDRESS_BORDER, ADDRESS_CLAMP = 0, 1


def run_case_1d(exe: Path, tmp: Path, name: str, samples: np.ndarray, sensor: dict, literal: bool, address: int,
                reps: int = 0):
    """The reference's 1D kernel (do_sparse_convolve_1d_f,
    src/SensorInstance1D.cu:35-72) on these SimSample1D records: (ping
    complex64 [nR], mean ms per launch with reps > 0 else None). The PSF
    scaling is the reference's literal 1.0f / duration * c
    (src/SensorInstance1D.cu:30) with literal=True, else its evident intent
    1 / (duration * c); `address` selects border or clamp addressing of the
    1D pulse texture (linear filter, normalized coordinates)."""
    s = sensor
    order = np.argsort(samples[:, 2], kind="stable")
    smp = np.ascontiguousarray(samples[order], dtype=np.float32)
    views = oracle.bin_samples(smp, s)["windows"].astype(np.uint64)
    pulse = np.ascontiguousarray(s["pulse"], dtype=np.complex64)
    nR = s["range_count"]
    src, dst = tmp / f"{name}.in", tmp / f"{name}.out"
    with open(src, "wb") as f:
        f.write(struct.pack("<4IQ", 0x314E5052, nR, pulse.size, address, smp.shape[0]))
        f.write(np.array([s["range_min"], s["range_max"], oracle.pulse_scale(s, literal_1d=literal)],
                         dtype=np.float32).tobytes())
        f.write(pulse.tobytes())
        f.write(smp.tobytes())
        f.write(np.ascontiguousarray(views).tobytes())
    cmd = [str(exe), str(CUBIN_1D), str(src), str(dst)] + ([str(reps)] if reps else [])
    res = subprocess.run(cmd, check=True, capture_output=True, text=True)
    ms = None
    for line in res.stdout.splitlines():
        if line.startswith("ref_kernel_ms "):
            ms = float(line.split()[1])
    ping = np.fromfile(dst, dtype=np.complex64)
    src.unlink()
    dst.unlink()
    return ping, ms
