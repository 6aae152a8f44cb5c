"""Golden 2D pings from the reference's own reduction kernel.

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
    if len(sys.argv) != 2:
        raise SystemExit("usage: python tests/golden/make_ref_pings.py OUT_DIR")
    main(sys.argv[1])
