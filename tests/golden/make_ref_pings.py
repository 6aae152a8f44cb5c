"""Golden 2D and 1D pings from the reference's own reduction kernels.

do_sparse_convolve_2d_f (src/SensorInstance2D.cu:44-83) is compiled from the
reference tree into oracle/_ref/ref_sparse2d.cubin by oracle/ref_build.sh
(here, where the reference tree is), with the stand-ins of
oracle/ref_stubs_cuda for the non-vendored rtac_base. This script runs on a
machine with a GPU: oracle/ref_kernel.py builds oracle/ref_sparse_harness.cpp
and feeds it the travel-sorted samples and the reference bin views (the
oracle's windows, which are bit-exact against the reference's own key
arithmetic) of each case; the kernel's ping is stored with the case
parameters:

    python tests/golden/make_ref_pings.py OUT_DIR

writes OUT_DIR/ref_pings_2d.npz; copy it to tests/golden/. The samples are
not stored: each case is rebuilt from its seeded workload.

    python tests/golden/make_ref_pings.py --1d OUT_DIR

does the same for the 1D kernel (do_sparse_convolve_1d_f,
src/SensorInstance1D.cu:35-72, oracle/_ref/ref_sparse1d.cubin) into
OUT_DIR/ref_pings_1d.npz. The reference's 1D pulse texture takes rtac_base's
filter and address defaults, which are not vendored: every case is recorded
with linear filtering under both border and clamp addressing, and with both
the reference's literal PSF scaling (1.0f / duration * c) and its evident
intent 1 / (duration * c). The literal scaling only reaches the pulse table
for travels exactly at an output range, so those cases set every eighth
travel there (workloads.on_range_grid).
"""
import sys
import tempfile
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

from oracle import ref_kernel  # noqa: E402

# name -> (workload builder, keyword arguments, stored row step)
CASES = {
    "oculus_reference": ("oculus_reference_2d", dict(n_samples=20000, seed=4), 4),
    "oculus_small": ("oculus_2d", dict(n_samples=8192, seed=11, n_bearings=64, n_ranges=128), 1),
}


# name -> (workload builder, keyword arguments, literal scaling, address mode)
CASES_1D = {
    f"{w}_{'literal' if lit else 'intent'}_{'clamp' if mode else 'border'}": (b, kw, lit, mode)
    for w, b, kw in (("ea400_reference", "ea400_reference_1d", dict(n_samples=20000, seed=5)),
                     ("echosounder", "echosounder_1d", dict(n_samples=65536, seed=1)))
    for lit in (False, True) for mode in (0, 1)
}


def case_samples_1d(builder: str, kwargs: dict, literal: bool):
    """The samples and sensor of a 1D case (rebuilt the same way by the tests)."""
    from rtac_simulation_gb300 import workloads as wl
    wk = getattr(wl, builder)(**kwargs)
    smp = wl.on_range_grid(wk.samples, wk.sensor) if literal else wk.samples
    return smp, wk.sensor


def main_1d(out_dir: str) -> None:
    out = Path(out_dir)
    out.mkdir(parents=True, exist_ok=True)
    ref_kernel.require_cubin(ref_kernel.CUBIN_1D)
    with tempfile.TemporaryDirectory() as d:
        tmp = Path(d)
        exe = ref_kernel.build_harness(tmp)
        fields = {}
        for name, (builder, kwargs, literal, mode) in CASES_1D.items():
            smp, sensor = case_samples_1d(builder, kwargs, literal)
            ping, _ = ref_kernel.run_case_1d(exe, tmp, name, smp, sensor, literal, mode)
            if not np.isfinite(ping).all():
                raise SystemExit(f"{name}: non-finite values in the reference ping")
            fields[f"{name}__ping"] = ping
            fields[f"{name}__builder"] = np.array(builder)
            fields[f"{name}__kwargs"] = np.array(repr(sorted(kwargs.items())))
            fields[f"{name}__literal"] = np.int64(literal)
            fields[f"{name}__address"] = np.int64(mode)
    np.savez(out / "ref_pings_1d.npz", **fields)
    print("wrote", out / "ref_pings_1d.npz")


def main(out_dir: str) -> None:
    out = Path(out_dir)
    out.mkdir(parents=True, exist_ok=True)
    ref_kernel.require_cubin()
    with tempfile.TemporaryDirectory() as d:
        tmp = Path(d)
        exe = ref_kernel.build_harness(tmp)
        fields = {}
        for name, (builder, kwargs, step) in CASES.items():
            ping, _, _ = ref_kernel.run_case(exe, tmp, name, builder, kwargs)
            if not np.isfinite(ping).all():
                raise SystemExit(f"{name}: non-finite values in the reference ping")
            fields[f"{name}__ping"] = ping[::step]
            fields[f"{name}__row_step"] = np.int64(step)
            fields[f"{name}__builder"] = np.array(builder)
            fields[f"{name}__kwargs"] = np.array(repr(sorted(kwargs.items())))
    np.savez(out / "ref_pings_2d.npz", **fields)
    print("wrote", out / "ref_pings_2d.npz")


if __name__ == "__main__":
    if len(sys.argv) == 3 and sys.argv[1] == "--1d":
        main_1d(sys.argv[2])
    elif len(sys.argv) == 2:
        main(sys.argv[1])
    else:
        raise SystemExit("usage: python tests/golden/make_ref_pings.py [--1d] OUT_DIR")
