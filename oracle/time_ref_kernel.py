"""Times the reference's own 2D reduction kernel beside this project's plain
form, on the same GPU and the same pings.

TEST INFRASTRUCTURE ONLY (the reference kernel is compiled from the reference
tree into oracle/_ref/ref_sparse2d.cubin by oracle/ref_build.sh; see
oracle/ref_kernel.py). For each workload it records:
  * the reference kernel do_sparse_convolve_2d_f (src/SensorInstance2D.cu:
    44-83), launched as SensorInstance2D::do_reduce does (one CTA per output
    cell, 512 threads, the PSF on the texture unit), CUDA-event time per launch
    with the samples already sorted and binned (the reference's Thrust sort
    and do_make_bins are not included);
  * this project's plain form through rtacx_reduce on the same samples: the
    gather stage alone (the counterpart of the kernel above) and the whole
    call (counting sort, windows and gather), with exact bilinear PSF weights
    and with RTACX_FLAG_TEXTURE_PSF (the reference's texture evaluation);
  * the relative L2 distance of both pings to the reference kernel's ping.

    python oracle/time_ref_kernel.py OUT_JSON [WORKLOAD ...]

WORKLOAD names a builder of rtac_simulation_gb300.workloads (default:
oculus_reference_2d oculus_2d precision_2d).
"""
from __future__ import annotations

import json
import sys
import tempfile
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parent))

from oracle import ref_kernel  # noqa: E402

DEFAULT = ("oculus_reference_2d", "oculus_2d", "precision_2d")


def rel_l2(a: np.ndarray, b: np.ndarray) -> float:
    return float(np.linalg.norm((a - b).ravel()) / max(np.linalg.norm(b.ravel()), 1e-30))


def time_plain(wk, flags: int, reps: int):
    """(ping, gather ms, whole-call ms) of rtacx_reduce on this workload."""
    import torch
    from rtac_simulation_gb300 import _lib
    ctx = _lib.Context(0)
    ctx.configure_2d(**wk.sensor, flags=flags)
    d = torch.from_numpy(np.ascontiguousarray(wk.samples).reshape(-1)).cuda()
    out = torch.empty(tuple(wk.out_shape) + (2,), dtype=torch.float32, device="cuda")
    stream = torch.cuda.current_stream()
    ctx.reduce(d, wk.n, out, stream=stream)
    ctx.stream_status(stream)
    ping = out.cpu().numpy()
    ping = ping[..., 0] + 1j * ping[..., 1]
    ctx.set_tracing(True)
    gather = []
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    total = 0.0
    for _ in range(reps):
        torch.cuda.synchronize()
        e0.record(stream)
        ctx.reduce(d, wk.n, out, stream=stream)
        e1.record(stream)
        torch.cuda.synchronize()
        total += e0.elapsed_time(e1)
        gather.append(ctx.stage_times()["reduce"])
    ctx.stream_status(stream)
    ctx.close()
    return ping, float(np.mean(gather)), total / reps


def main(out_json: str, names) -> None:
    from rtac_simulation_gb300 import _lib
    ref_kernel.require_cubin()
    res = {"timing": "CUDA events on the launching stream after one untimed launch; samples resident on the device"}
    with tempfile.TemporaryDirectory() as d:
        tmp = Path(d)
        exe = ref_kernel.build_harness(tmp)
        for name in names:
            reps = 3 if name in ("precision_2d", "stress_2d") else 10
            ref_ping, ref_ms, wk = ref_kernel.run_case(exe, tmp, name, name, {}, reps=reps)
            exact, g_exact, t_exact = time_plain(wk, 0, reps)
            tex, g_tex, t_tex = time_plain(wk, _lib.RTACX_FLAG_TEXTURE_PSF, reps)
            res[name] = {
                "samples": int(wk.n), "bearings": int(wk.out_shape[1]), "ranges": int(wk.out_shape[0]),
                "reps": reps,
                "reference_kernel_ms": ref_ms,
                "plain_gather_ms": g_exact, "plain_call_ms": t_exact,
                "plain_texture_psf_gather_ms": g_tex, "plain_texture_psf_call_ms": t_tex,
                "gather_speedup_vs_reference_kernel": ref_ms / g_exact,
                "rel_l2_plain_vs_reference_kernel": rel_l2(exact, ref_ping),
                "rel_l2_texture_psf_vs_reference_kernel": rel_l2(tex, ref_ping),
            }
            print(name, json.dumps(res[name]), flush=True)
    Path(out_json).write_text(json.dumps(res, indent=1) + "\n")


if __name__ == "__main__":
    if len(sys.argv) < 2:
        raise SystemExit("usage: python oracle/time_ref_kernel.py OUT_JSON [WORKLOAD ...]")
    main(sys.argv[1], sys.argv[2:] or DEFAULT)
