"""Golden 2D pings from the reference's own reduction kernel.

do_sparse_convolve_2d_f (src/SensorInstance2D.cu:44-83) is compiled from the
reference tree into oracle/_ref/ref_sparse2d.cubin by oracle/ref_build.sh
(here, where the reference tree is), with the stand-ins of
oracle/ref_stubs_cuda for the non-vendored rtac_base. This script runs on a
machine with a GPU: it builds oracle/ref_sparse_harness.cpp, feeds it the
travel-sorted samples and the reference bin views (the oracle's windows,
which are bit-exact against the reference's own key arithmetic) of each
case, and stores the kernel's ping with the case parameters:

    python tests/golden/make_ref_pings.py OUT_DIR

writes OUT_DIR/ref_pings_2d.npz; copy it to tests/golden/. The samples are
not stored: each case is rebuilt from its seeded workload.
"""
import os
import struct
import subprocess
import sys
import tempfile
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

from oracle import oracle  # noqa: E402
from rtac_simulation_gb300 import workloads as wl  # noqa: E402

CUBIN = ROOT / "oracle" / "_ref" / "ref_sparse2d.cubin"
HARNESS_SRC = ROOT / "oracle" / "ref_sparse_harness.cpp"

# name -> (workload builder, keyword arguments, stored row step)
CASES = {
    "oculus_reference": ("oculus_reference_2d", dict(n_samples=20000, seed=4), 4),
    "oculus_small": ("oculus_2d", dict(n_samples=8192, seed=11, n_bearings=64, n_ranges=128), 1),
}


def build_harness(out: Path) -> Path:
    cuda = Path(os.environ.get("CUDA_HOME", "/usr/local/cuda"))
    exe = out / "ref_sparse_harness"
    subprocess.run(["g++", "-std=c++17", "-O1", "-I", str(ROOT / "oracle" / "ref_stubs_cuda"),
                    "-I", str(cuda / "include"), str(HARNESS_SRC), "-L", str(cuda / "lib64"),
                    "-L", str(cuda / "lib64" / "stubs"), "-lcudart", "-lcuda", "-o", str(exe)], check=True)
    return exe


def case_inputs(builder: str, kwargs: dict):
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


def run_case(exe: Path, tmp: Path, name: str, builder: str, kwargs: dict) -> np.ndarray:
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
    subprocess.run([str(exe), str(CUBIN), str(src), str(dst)], check=True)
    return np.fromfile(dst, dtype=np.complex64).reshape(nR, nB)


def main(out_dir: str) -> None:
    out = Path(out_dir)
    out.mkdir(parents=True, exist_ok=True)
    if not CUBIN.exists():
        raise SystemExit(f"{CUBIN} is missing: build it with oracle/ref_build.sh where the reference tree is")
    with tempfile.TemporaryDirectory() as d:
        tmp = Path(d)
        exe = build_harness(tmp)
        fields = {}
        for name, (builder, kwargs, step) in CASES.items():
            ping = run_case(exe, tmp, name, builder, kwargs)
            if not np.isfinite(ping).all():
                raise SystemExit(f"{name}: non-finite values in the reference ping")
            fields[f"{name}__ping"] = ping[::step]
            fields[f"{name}__row_step"] = np.int64(step)
            fields[f"{name}__builder"] = np.array(builder)
            fields[f"{name}__kwargs"] = np.array(repr(sorted(kwargs.items())))
    np.savez(out / "ref_pings_2d.npz", **fields)
    print("wrote", out / "ref_pings_2d.npz")


if __name__ == "__main__":
    if len(sys.argv) != 2:
        raise SystemExit("usage: python tests/golden/make_ref_pings.py OUT_DIR")
    main(sys.argv[1])
