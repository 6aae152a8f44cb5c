"""Shared helpers of the GPU parity tests: run the C-ABI path on device
buffers and bring the results back for comparison with the oracle."""
import numpy as np
import torch

from rtac_simulation_gb300 import _lib


def make_context(wk, flags=0):
    ctx = _lib.Context(0)
    if wk.dims == 1:
        ctx.configure_1d(**wk.sensor, flags=flags)
    else:
        ctx.configure_2d(**wk.sensor, flags=flags)
    return ctx


def to_device(samples: np.ndarray, offset_floats: int = 0) -> torch.Tensor:
    flat = np.ascontiguousarray(samples, dtype=np.float32).reshape(-1)
    buf = torch.zeros(flat.size + offset_floats + 4, dtype=torch.float32, device="cuda")
    buf[offset_floats:offset_floats + flat.size] = torch.from_numpy(flat).cuda()
    return buf[offset_floats:]


def gpu_bin(ctx, samples: np.ndarray, dims: int, nR: int, offset_floats: int = 0):
    n = samples.shape[0]
    d = to_device(samples, offset_floats)
    keys = torch.empty(max(n, 1), dtype=torch.int32, device="cuda")
    seg = torch.empty((nR, 2), dtype=torch.int32, device="cuda")
    win = torch.empty((nR, 2), dtype=torch.int32, device="cuda")
    cnt = torch.empty(nR, dtype=torch.int32, device="cuda")
    oor = torch.empty(2, dtype=torch.int64, device="cuda")
    stream = torch.cuda.current_stream()
    ctx.bin(d, n, dims, keys, seg, win, cnt, oor, stream=stream)
    ctx.stream_status(stream)
    u32 = lambda t: t.cpu().numpy().view(np.uint32)
    return dict(keys=u32(keys)[:n], segments=u32(seg), windows=u32(win), counts=u32(cnt),
                oor=oor.cpu().numpy().astype(np.uint64))


def gpu_reduce(ctx, samples: np.ndarray, out_shape, offset_floats: int = 0, repeat: int = 1):
    d = to_device(samples, offset_floats)
    out = torch.full(tuple(out_shape) + (2,), float("nan"), dtype=torch.float32, device="cuda")
    stream = torch.cuda.current_stream()
    for _ in range(repeat):
        ctx.reduce(d, samples.shape[0], out, stream=stream)
    ctx.stream_status(stream)
    o = out.cpu().numpy()
    return o[..., 0].astype(np.float64) + 1j * o[..., 1].astype(np.float64)


def rel_l2(a, b) -> float:
    nb = np.linalg.norm(b)
    if nb == 0:
        return float(np.linalg.norm(a))
    return float(np.linalg.norm(a - b) / nb)
