"""ctypes wrapper of the oracle (oracle/rtacx_oracle.cpp).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the
CPU-baseline / reference arm of bench.py, never by the product package.
Parity status: pinned for the range key and pulse table (the reference's own
headers), the receiver directivity tables (the reference's own
src/Directivity.cpp, bit for bit) and for the 2D reduction (the reference's own kernel run on a GB300:
reduce(mode=2) reproduces its pings, tests/golden/ref_pings_2d.npz); the 1D
reduction is a restatement.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB_PATH = HERE / "librtacx_oracle.so"

_P = ctypes.c_void_p
_U32 = ctypes.c_uint32
_U64 = ctypes.c_uint64
_F = ctypes.c_float
_I = ctypes.c_int

_lib = None


def build() -> Path:
    subprocess.run(["make", "-s", "-C", str(HERE), "librtacx_oracle.so"], check=True)
    return LIB_PATH


def load() -> ctypes.CDLL:
    global _lib
    if _lib is not None:
        return _lib
    src = HERE / "rtacx_oracle.cpp"
    if not LIB_PATH.exists() or LIB_PATH.stat().st_mtime < src.stat().st_mtime:
        build()
    lib = ctypes.CDLL(str(LIB_PATH))
    lib.rtacx_oracle_key_params.argtypes = [_U32, _F, _F, _F, ctypes.POINTER(_F), ctypes.POINTER(_F),
                                            ctypes.POINTER(_F), ctypes.POINTER(_F)]
    lib.rtacx_oracle_key_params.restype = None
    lib.rtacx_oracle_range_keys.argtypes = [_U32, _F, _F, _F, _P, _U64, _U32, _P, _P]
    lib.rtacx_oracle_range_keys.restype = None
    lib.rtacx_oracle_bin_overlap.argtypes = [_F, _F, _U32, _F]
    lib.rtacx_oracle_bin_overlap.restype = _I
    lib.rtacx_oracle_linspace_at.argtypes = [_F, _F, _U32, _U32]
    lib.rtacx_oracle_linspace_at.restype = _F
    lib.rtacx_oracle_bearing_bins.argtypes = [_F, _F, _U32, _P, _U64, _U32, _P]
    lib.rtacx_oracle_bearing_bins.restype = None
    lib.rtacx_oracle_bin.argtypes = [_P, _U64, _U32, _U32, _F, _F, _U32, _F, _P, _P, _P,
                                     ctypes.POINTER(_U64), ctypes.POINTER(_U64)]
    lib.rtacx_oracle_bin.restype = _I
    lib.rtacx_oracle_reduce.argtypes = [_U32, _P, _U64, _F, _F, _U32, _F, _F, _P, _U32, _F, _P, _U32,
                                        _P, _U32, _I, _U32, _U32, _I, _P]
    lib.rtacx_oracle_reduce.restype = None
    lib.rtacx_oracle_apply_echo.argtypes = [_P, _U64, _U32, ctypes.c_double, _F, _U32, _I]
    lib.rtacx_oracle_apply_echo.restype = None
    lib.rtacx_oracle_reduce_binned.argtypes = [_P, _U64, _F, _F, _U32, _F, _U32, _F, _F, _U32, _P, _P, _U32, _U32,
                                               _U32, _U32, _I, _P]
    lib.rtacx_oracle_reduce_binned.restype = None
    lib.rtacx_oracle_make_samples.argtypes = [_P, _U64, _P, _P, _U32, _U32, ctypes.c_double, _F, _U32, _U32, _P]
    lib.rtacx_oracle_make_samples.restype = None
    lib.rtacx_oracle_rasterize.argtypes = [_P, _P, _P, _U32, _U32, _P, _P, _P, _U32, _U32, ctypes.c_double, _F, _P, _P]
    lib.rtacx_oracle_rasterize.restype = None
    _lib = lib
    return lib


def key_params(n_bins, min_bin, max_bin, margin):
    lib = load()
    a, b, lo, hi = _F(), _F(), _F(), _F()
    lib.rtacx_oracle_key_params(n_bins, min_bin, max_bin, margin, ctypes.byref(a), ctypes.byref(b),
                                ctypes.byref(lo), ctypes.byref(hi))
    return np.float32(a.value), np.float32(b.value), np.float32(lo.value), np.float32(hi.value)


def range_keys(n_bins, min_bin, max_bin, margin, travel):
    """Range key and out-of-range side (-1, 0, +1) of every travel value."""
    lib = load()
    t = np.ascontiguousarray(travel, dtype=np.float32)
    keys = np.empty(t.size, dtype=np.uint32)
    side = np.empty(t.size, dtype=np.int8)
    lib.rtacx_oracle_range_keys(n_bins, min_bin, max_bin, margin, t.ctypes.data, t.size, 1,
                                keys.ctypes.data, side.ctypes.data)
    return keys, side


def bin_overlap(rmin, rmax, n, margin) -> int:
    return load().rtacx_oracle_bin_overlap(rmin, rmax, n, margin)


def linspace_at(rmin, rmax, n, r) -> np.float32:
    return np.float32(load().rtacx_oracle_linspace_at(rmin, rmax, n, r))


def bearing_bins(scale, offset, count, bearing):
    t = np.ascontiguousarray(bearing, dtype=np.float32)
    out = np.empty(t.size, dtype=np.uint32)
    load().rtacx_oracle_bearing_bins(scale, offset, count, t.ctypes.data, t.size, 1, out.ctypes.data)
    return out


def bin_samples(samples: np.ndarray, sensor: dict):
    """Reference segments, windows, counts and out-of-range counts."""
    lib = load()
    s = np.ascontiguousarray(samples, dtype=np.float32)
    n, stride = s.shape
    nR = sensor["range_count"]
    seg = np.zeros((nR, 2), dtype=np.uint32)
    win = np.zeros((nR, 2), dtype=np.uint32)
    cnt = np.zeros(nR, dtype=np.uint32)
    lo, hi = _U64(), _U64()
    ov = lib.rtacx_oracle_bin(s.ctypes.data, n, stride, 2 if stride == 4 else 1,
                              sensor["range_min"], sensor["range_max"], nR, sensor["margin"],
                              seg.ctypes.data, win.ctypes.data, cnt.ctypes.data,
                              ctypes.byref(lo), ctypes.byref(hi))
    return dict(segments=seg, windows=win, counts=cnt, oor=np.array([lo.value, hi.value], dtype=np.uint64),
                overlap=ov)


def pulse_scale(sensor: dict, literal_1d: bool = False) -> np.float32:
    d, c = np.float32(sensor["pulse_duration"]), np.float32(sensor["sound_celerity"])
    if literal_1d:
        return np.float32(np.float32(np.float32(1.0) / d) * c)
    return np.float32(np.float32(1.0) / np.float32(d * c))


def reduce(samples: np.ndarray, sensor: dict, mode: int = 0, rows=None, threads: int = 0,
           literal_1d: bool = False) -> np.ndarray:
    """Oracle ping. mode 0: FP64 (complex128), mode 1: FP32 reference
    arithmetic (complex64), mode 2: the PSF fetched as the reference's
    texture does on the GPU (coordinate truncated to 21 fractional bits,
    weights rounded to 1/256; border addressing), accumulated in FP64
    (complex128); mode 3 (1D): mode 2 with clamp addressing. rows = (begin,
    end) restricts the output rows."""
    lib = load()
    s = np.ascontiguousarray(samples, dtype=np.float32)
    n, stride = s.shape
    dims = 2 if stride == 4 else 1
    nR = sensor["range_count"]
    r0, r1 = rows if rows is not None else (0, nR)
    pulse = np.ascontiguousarray(sensor["pulse"], dtype=np.complex64)
    if dims == 2:
        beam = np.ascontiguousarray(sensor["beam"], dtype=np.float32)
        bearings = np.ascontiguousarray(sensor["bearings"], dtype=np.float32)
        bscale = np.float32(np.float32(1.0) / np.float32(sensor["beam_span"]))
        nB = bearings.size
    else:
        beam = np.zeros(1, dtype=np.float32)
        bearings = np.zeros(1, dtype=np.float32)
        bscale, nB = np.float32(0.0), 1
    if mode == 3 and dims != 1:
        raise ValueError("the clamp-addressed texture mode is 1D only")
    out = np.zeros((r1 - r0, nB), dtype=np.complex64 if mode == 1 else np.complex128)
    threads = threads or (os.cpu_count() or 1)
    lib.rtacx_oracle_reduce(dims, s.ctypes.data, n, sensor["range_min"], sensor["range_max"], nR,
                            sensor["margin"], pulse_scale(sensor, literal_1d), pulse.ctypes.data, pulse.size,
                            bscale, beam.ctypes.data, beam.size, bearings.ctypes.data, nB,
                            mode, r0, r1, threads, out.ctypes.data)
    return out[:, 0] if dims == 1 else out


def apply_echo(samples: np.ndarray, sensor: dict, echo: dict | None, mode: int = 0) -> np.ndarray:
    """Copy of `samples` with the echo pre-step applied (mode 0 exact FP64,
    mode 1 the reference's float arithmetic)."""
    out = np.array(samples, dtype=np.float32, copy=True, order="C")
    if not echo or not echo.get("flags"):
        return out
    n, stride = out.shape
    load().rtacx_oracle_apply_echo(out.ctypes.data, n, stride, float(echo.get("carrier_hz", 0.0)),
                                   sensor["sound_celerity"], int(echo["flags"]), mode)
    return out


def reduce_binned(samples: np.ndarray, sensor: dict, tables: dict, rows=None, threads: int = 0) -> np.ndarray:
    """FP64 oracle of the binned precision model (complex128 [rows][nB]).
    `tables` holds the precision configuration (workloads.precision_tables):
    directivity [grid_count][nB], range_taps [2][L] (one tap set per output
    row parity), tap_center, grid_count, grid_first, grid_last."""
    lib = load()
    s = np.ascontiguousarray(samples, dtype=np.float32)
    n = s.shape[0]
    nR = sensor["range_count"]
    nB = len(sensor["bearings"])
    D = np.ascontiguousarray(tables["directivity"], dtype=np.complex64)
    t = np.ascontiguousarray(tables["range_taps"], dtype=np.complex64).reshape(2, -1)   # [phase][tap]
    cells = int(tables["grid_count"])
    assert D.shape == (cells, nB)
    r0, r1 = rows if rows is not None else (0, nR)
    out = np.zeros((r1 - r0, nB), dtype=np.complex128)
    lib.rtacx_oracle_reduce_binned(s.ctypes.data, n, sensor["range_min"], sensor["range_max"], nR,
                                   sensor["margin"], nB, tables["grid_first"], tables["grid_last"], cells,
                                   D.ctypes.data, t.ctypes.data, t.shape[1], int(tables["tap_center"]), r0, r1,
                                   threads or (os.cpu_count() or 1), out.ctypes.data)
    return out


def make_samples(hits: np.ndarray, rotation, table, carrier_hz: float, c: float, flags: int, dims: int) -> np.ndarray:
    """Oracle of rtacx_make_samples: hits (n, 6) float32 -> samples (n, 3|4)."""
    h = np.ascontiguousarray(hits, dtype=np.float32)
    R = np.ascontiguousarray(np.asarray(rotation, np.float32).reshape(9))
    tab = None if table is None else np.ascontiguousarray(table, dtype=np.float32)
    out = np.zeros((h.shape[0], 4 if dims == 2 else 3), dtype=np.float32)
    load().rtacx_oracle_make_samples(h.ctypes.data, h.shape[0], R.ctypes.data,
                                     None if tab is None else tab.ctypes.data,
                                     0 if tab is None else tab.shape[1], 0 if tab is None else tab.shape[0],
                                     carrier_hz, c, flags, dims, out.ctypes.data)
    return out


def rasterize(vertices, normals, triangles, world_to_local, world_to_screen, origin, width, height,
              carrier_hz=1.2e6, c=1500.0):
    """Oracle of rtacx_rasterize: (samples (H*W, 4) float32, winner (H*W,) int32)."""
    v = np.ascontiguousarray(vertices, np.float32)
    nrm = np.ascontiguousarray(normals, np.float32)
    t = np.ascontiguousarray(triangles, np.uint32)
    L = np.ascontiguousarray(np.asarray(world_to_local, np.float32).reshape(16))
    S = np.ascontiguousarray(np.asarray(world_to_screen, np.float32).reshape(16))
    o = np.ascontiguousarray(np.asarray(origin, np.float32))
    out = np.zeros((height * width, 4), np.float32)
    win = np.zeros(height * width, np.int32)
    load().rtacx_oracle_rasterize(v.ctypes.data, nrm.ctypes.data, t.ctypes.data, v.shape[0], t.shape[0],
                                  L.ctypes.data, S.ctypes.data, o.ctypes.data, width, height, carrier_hz, c,
                                  out.ctypes.data, win.ctypes.data)
    return out, win


def directivity_table(kind: str, params, baffle: str = "none", oversampling: int = 1) -> np.ndarray:
    """Receiver directivity table (float32 [height][width]) as the reference
    builds it on the host: kind "RECT" (params width, height, wavelength;
    Directivity::rectangle_antenna, src/Directivity.cpp:59-101) or "DISK"
    (params diameter, wavelength; Directivity::disk_antenna,
    src/Directivity.cpp:109-166). Table sizes, the float / double mix and the
    single-sided baffle follow those lines. Where disk_antenna's
    sqrt(1 - y2 - z2) cancels the reference's result depends on its libm's
    last bit (a NaN or a tiny x, both below the 1e-2 cut-off); the exact-math
    limit is taken here, x = 0 and a value of 0."""
    from scipy.special import j1

    f32 = np.float32
    os_ = int(oversampling)
    if kind == "RECT":
        width, height, wl = (f32(p) for p in params)
        half_os = float(f32(f32(0.5) * f32(os_)) * f32(2))          # 0.5f * oversampling * 2 in float
        Nw = 2 * int(half_os * np.pi * float(width) / float(wl) + 1)
        Nh = 2 * int(half_os * np.pi * float(height) / float(wl) + 1)
        elev = np.pi * np.arange(Nh, dtype=np.float64) / Nh
        bear = np.pi * np.arange(Nw, dtype=np.float64) / Nw
        ke = np.pi * float(height) / float(wl)
        kb = np.pi * float(width) / float(wl)
        with np.errstate(divide="ignore", invalid="ignore"):
            e = (np.sin(ke * np.sin(elev)) / (ke * np.sin(elev))).astype(f32)
            b = (np.sin(kb * np.sin(bear)) / (kb * np.sin(bear))).astype(f32)
        e[0] = f32(1)
        b[0] = f32(1)
        data = (e[:, None] * b[None, :]).astype(f32)
    elif kind == "DISK":
        dia, wl = (f32(p) for p in params)
        period = f32(f32(f32(2) * wl) / dia)
        N = max(64, 8 * int(os_ * np.pi / float(period)))
        elev = (np.pi * np.arange(N, dtype=np.float64) / N)[:, None]
        bear = (np.pi * np.arange(N, dtype=np.float64) / N)[None, :]
        cose2, sine2 = np.cos(elev) ** 2, np.sin(elev) ** 2
        cosb2, sinb2 = np.cos(bear) ** 2, np.sin(bear) ** 2
        with np.errstate(divide="ignore", invalid="ignore"):
            denom = 1.0 - sine2 * sinb2
            y2 = cose2 * sinb2 / denom
            z2 = sine2 * cosb2 / denom
            s = 1.0 - y2 - z2
            x = np.where((denom > 0.0) & (s > 0.0), np.sqrt(np.where(s > 0.0, s, 0.0)), 0.0)
            x = np.where((elev > 0.5 * np.pi) | (bear > 0.5 * np.pi), -x, x)
            a = (np.pi * float(dia) / float(wl)) * np.sin(np.arctan2(np.sqrt(y2 + z2), x))
            v = np.where(np.abs(a) < 1.0e-3, 1.0, 2.0 * j1(a) / a)
        data = np.where(np.abs(x) < 1.0e-2, 0.0, v).astype(f32)
    else:
        raise ValueError(f"unknown directivity kind {kind!r}")
    if baffle == "single-sided":
        H, W = data.shape
        data[H // 2 + 1:, :] = 0
        data[:, W // 2 + 1:] = 0
    elif baffle != "none":
        raise ValueError(f"unsupported baffle mode {baffle!r}")
    return data
