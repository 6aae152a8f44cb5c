"""ctypes binding of librtacx.so (include/rtacx.h).

The binding carries plain integers (device pointers, stream handles) across
the C ABI; torch is not needed here. Loading fails loudly when the library has
not been built: there is no fallback path.
"""
from __future__ import annotations

import ctypes
import os
from pathlib import Path

import numpy as np

LIB_PATH = Path(__file__).resolve().parent / "librtacx.so"

RTACX_OK = 0
RTACX_ERR_INVALID_ARGUMENT = 1
RTACX_ERR_NOT_CONFIGURED = 2
RTACX_ERR_CUDA = 3
RTACX_ERR_OUT_OF_MEMORY = 4
RTACX_ERR_DEVICE = 5
RTACX_ERR_UNSUPPORTED = 6
RTACX_KEY_OUT_OF_RANGE = 0xFFFFFFFF
RTACX_SAMPLE_1D = 1
RTACX_SAMPLE_2D = 2
RTACX_FLAG_1D_LITERAL_SCALING = 1
RTACX_FLAG_TEXTURE_PSF = 2
RTACX_FLAG_TEXTURE_CLAMP = 4
RTACX_FLAG_SIMT_GATHER = 8

_STATUS_NAMES = {
    RTACX_OK: "RTACX_OK",
    RTACX_ERR_INVALID_ARGUMENT: "RTACX_ERR_INVALID_ARGUMENT",
    RTACX_ERR_NOT_CONFIGURED: "RTACX_ERR_NOT_CONFIGURED",
    RTACX_ERR_CUDA: "RTACX_ERR_CUDA",
    RTACX_ERR_OUT_OF_MEMORY: "RTACX_ERR_OUT_OF_MEMORY",
    RTACX_ERR_DEVICE: "RTACX_ERR_DEVICE",
    RTACX_ERR_UNSUPPORTED: "RTACX_ERR_UNSUPPORTED",
}

# Every entry point include/rtacx.h declares, with its ctypes signature.
_P = ctypes.c_void_p
_U32 = ctypes.c_uint32
_U64 = ctypes.c_uint64
_I = ctypes.c_int


class Sensor1D(ctypes.Structure):
    _fields_ = [("range_min", ctypes.c_float), ("range_max", ctypes.c_float), ("range_count", _U32),
                ("sound_celerity", ctypes.c_float), ("pulse_duration", ctypes.c_float),
                ("margin", ctypes.c_float), ("pulse", _P), ("pulse_len", _U32), ("flags", _U32)]


class Sensor2D(ctypes.Structure):
    _fields_ = [("range_min", ctypes.c_float), ("range_max", ctypes.c_float), ("range_count", _U32),
                ("sound_celerity", ctypes.c_float), ("pulse_duration", ctypes.c_float),
                ("margin", ctypes.c_float), ("pulse", _P), ("pulse_len", _U32),
                ("beam", _P), ("beam_len", _U32), ("beam_span", ctypes.c_float),
                ("bearings", _P), ("bearing_count", _U32), ("flags", _U32)]


SIGNATURES = {
    "rtacx_version": (ctypes.c_char_p, []),
    "rtacx_create": (_I, [ctypes.POINTER(_P), _I]),
    "rtacx_destroy": (None, [_P]),
    "rtacx_last_error": (ctypes.c_char_p, [_P]),
    "rtacx_configure_1d": (_I, [_P, ctypes.POINTER(Sensor1D)]),
    "rtacx_configure_2d": (_I, [_P, ctypes.POINTER(Sensor2D)]),
    "rtacx_reserve": (_I, [_P, _U64]),
    "rtacx_bin": (_I, [_P, _P, _U64, _I, _P, _P, _P, _P, _P, _P]),
    "rtacx_reduce": (_I, [_P, _P, _U64, _P, _P]),
    "rtacx_stream_status": (_I, [_P, _P]),
    "rtacx_set_tracing": (_I, [_P, _I]),
    "rtacx_diag_drop_accumulation_stage": (_I, [_P, _U32]),
    "rtacx_diag_sorted": (_I, [_P, _P, _U64, _P]),
    "rtacx_stage_times": (_I, [_P, ctypes.POINTER(ctypes.c_float), _I]),
    "rtacx_reduce_noalloc": (_I, [_I, _P, _P, _U64, _P, _P]),
    "rtacx_gemm_bf16_tn": (_I, [_P, _P, _P, _I, _I, _I, _P]),
    "rtacx_set_echo_model": (_I, [_P, _P]),
    "rtacx_configure_precision": (_I, [_P, _P]),
    "rtacx_reduce_precision": (_I, [_P, _P, _U64, _P, _P]),
    "rtacx_reduce_precision_host": (_I, [_P, _P, _U64, _P, _P]),
    "rtacx_configure_receiver": (_I, [_P, _P]),
    "rtacx_make_samples": (_I, [_P, _P, _U64, _P, _P]),
    "rtacx_directivity_table": (_I, [_I, ctypes.POINTER(ctypes.c_float), _P, ctypes.POINTER(_U32),
                                     ctypes.POINTER(_U32), _P]),
    "rtacx_rasterize": (_I, [_P, _P, _P, _P, _P]),
    "rtacx_batch_create": (_I, [ctypes.POINTER(_P), _I]),
    "rtacx_batch_destroy": (None, [_P]),
    "rtacx_batch_last_error": (ctypes.c_char_p, [_P]),
    "rtacx_batch_plan": (_I, [_P, _P, _U32, _U32]),
    "rtacx_batch_run": (_I, [_P, _P]),
    "rtacx_batch_tuning": (_I, [_P, ctypes.POINTER(_U32), ctypes.POINTER(_U32), ctypes.POINTER(_U32),
                                ctypes.POINTER(ctypes.c_float)]),
    "rtacx_batch_status": (_I, [_P, _P]),
    "rtacx_batch_graph_kernels": (_I, [_P, ctypes.POINTER(_U32)]),
    "rtacx_diag_batch_barrier": (_I, [_P, _U32, _U32]),
}

RTACX_BATCH_AUTOTUNE = 1
RTACX_BATCH_STAGED = 2
RTACX_DIRECTIVITY_RECTANGLE = 1
RTACX_DIRECTIVITY_DISK = 2


class Mesh(ctypes.Structure):
    _fields_ = [("vertices", _P), ("normals", _P), ("triangles", _P), ("n_vertices", _U32), ("n_triangles", _U32)]


class RasterView(ctypes.Structure):
    _fields_ = [("world_to_local", ctypes.c_float * 16), ("world_to_screen", ctypes.c_float * 16),
                ("origin", ctypes.c_float * 3), ("width", _U32), ("height", _U32),
                ("carrier_hz", ctypes.c_double), ("sound_celerity", ctypes.c_float)]


class Receiver(ctypes.Structure):
    _fields_ = [("rotation", ctypes.c_float * 9), ("directivity", _P), ("directivity_width", _U32),
                ("directivity_height", _U32), ("carrier_hz", ctypes.c_double), ("flags", _U32)]


def directivity_table_size(kind: int, params):
    """(height, width) of the table rtacx_directivity_table builds for these
    parameters (a host-only query, no device work)."""
    lib = load()
    p = (ctypes.c_float * len(params))(*params)
    w, h = _U32(), _U32()
    st = lib.rtacx_directivity_table(kind, p, None, ctypes.byref(w), ctypes.byref(h), None)
    if st != RTACX_OK:
        raise RtacxError(st, "rtacx_directivity_table (size) failed")
    return h.value, w.value


def directivity_table(kind: int, params, stream=None):
    """Device directivity table (torch tensor [height][width]) built by
    rtacx_directivity_table."""
    import torch
    lib = load()
    p = (ctypes.c_float * len(params))(*params)
    w, h = _U32(), _U32()
    rows, cols = directivity_table_size(kind, params)
    out = torch.empty((rows, cols), dtype=torch.float32, device="cuda")
    st = lib.rtacx_directivity_table(kind, p, out.data_ptr(), ctypes.byref(w), ctypes.byref(h), _stream(stream))
    if st != RTACX_OK:
        raise RtacxError(st, "rtacx_directivity_table failed")
    return out


class PingDesc(ctypes.Structure):
    _fields_ = [("ctx", _P), ("samples", _P), ("n", _U64), ("out", _P)]

RTACX_ECHO_PHASE = 1
RTACX_ECHO_SPREADING = 2
RTACX_ECHO_PHASE_COMPENSATED = 4
RTACX_PRECISION_FP16_ROWSCALE = 1
RTACX_PRECISION_HOT_RANGE = 2
PRECISION_STAGES = ("accumulate", "split", "filter", "gemm", "unused", "clear")


class EchoModel(ctypes.Structure):
    _fields_ = [("carrier_hz", ctypes.c_double), ("flags", _U32)]


class PrecisionDesc(ctypes.Structure):
    _fields_ = [("directivity", _P), ("range_taps", _P), ("tap_count", _U32), ("tap_center", _U32),
                ("flags", _U32), ("grid_count", _U32), ("grid_first", ctypes.c_float), ("grid_last", ctypes.c_float)]

STAGES = ("count", "reset", "binscan", "scatter", "windows", "reduce")

_lib = None


class RtacxError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"{_STATUS_NAMES.get(status, status)}: {message}")
        self.status = status


def load() -> ctypes.CDLL:
    """Load librtacx.so, binding every declared entry point."""
    global _lib
    if _lib is not None:
        return _lib
    if not LIB_PATH.exists():
        raise RuntimeError(f"{LIB_PATH} is missing: build it with `python -m rtac_simulation_gb300.build`")
    lib = ctypes.CDLL(str(LIB_PATH))
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def _ptr(x) -> int | None:
    """Device pointer of a torch tensor, an int, or None."""
    if x is None:
        return None
    if isinstance(x, int):
        return x
    return x.data_ptr()


def _stream(s) -> int | None:
    if s is None:
        return None
    if isinstance(s, int):
        return s
    return s.cuda_stream


class Context:
    """One rtacx context (a configured sensor plus its device scratch)."""

    def __init__(self, device: int = 0):
        self._lib = load()
        h = _P()
        st = self._lib.rtacx_create(ctypes.byref(h), device)
        if st != RTACX_OK:
            raise RtacxError(st, f"rtacx_create(device={device}) failed")
        self._h = h
        self.device = device
        self.dims = 0
        self._keep = []

    def close(self) -> None:
        if getattr(self, "_h", None) is not None and self._h.value:
            self._lib.rtacx_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    @property
    def handle(self) -> int:
        return self._h.value

    def last_error(self) -> str:
        msg = self._lib.rtacx_last_error(self._h)
        return msg.decode() if msg else ""

    def _check(self, st: int) -> None:
        if st != RTACX_OK:
            raise RtacxError(st, self.last_error())

    def configure_1d(self, *, range_min, range_max, range_count, sound_celerity, pulse_duration,
                     margin, pulse, flags=0) -> None:
        p = np.ascontiguousarray(np.asarray(pulse, dtype=np.complex64))
        s = Sensor1D(range_min, range_max, range_count, sound_celerity, pulse_duration, margin,
                     p.ctypes.data, p.size, flags)
        self._check(self._lib.rtacx_configure_1d(self._h, ctypes.byref(s)))
        self.dims = 1

    def configure_2d(self, *, range_min, range_max, range_count, sound_celerity, pulse_duration,
                     margin, pulse, beam, beam_span, bearings, flags=0) -> None:
        p = np.ascontiguousarray(np.asarray(pulse, dtype=np.complex64))
        bm = np.ascontiguousarray(np.asarray(beam, dtype=np.float32))
        br = np.ascontiguousarray(np.asarray(bearings, dtype=np.float32))
        s = Sensor2D(range_min, range_max, range_count, sound_celerity, pulse_duration, margin,
                     p.ctypes.data, p.size, bm.ctypes.data, bm.size, beam_span,
                     br.ctypes.data, br.size, flags)
        self._check(self._lib.rtacx_configure_2d(self._h, ctypes.byref(s)))
        self.dims = 2

    def reserve(self, max_samples: int) -> None:
        self._check(self._lib.rtacx_reserve(self._h, max_samples))

    def bin(self, samples, n: int, kind: int, keys=None, segments=None, windows=None,
            counts=None, oor=None, stream=None) -> None:
        self._check(self._lib.rtacx_bin(self._h, _ptr(samples), n, kind, _ptr(keys), _ptr(segments),
                                        _ptr(windows), _ptr(counts), _ptr(oor), _stream(stream)))

    def reduce(self, samples, n: int, out, stream=None) -> None:
        self._check(self._lib.rtacx_reduce(self._h, _ptr(samples), n, _ptr(out), _stream(stream)))

    def set_echo_model(self, carrier_hz: float = 0.0, flags: int = 0) -> None:
        m = EchoModel(carrier_hz, flags)
        self._check(self._lib.rtacx_set_echo_model(self._h, ctypes.byref(m)))

    def configure_precision(self, directivity=None, range_taps=None, tap_center: int = 0, flags: int = 0,
                            grid_count: int = 0, grid_first: float = 0.0, grid_last: float = 0.0) -> None:
        """rtacx_configure_precision; the keyword arguments are those of
        workloads.precision_tables (directivity [grid_count][nB] complex)."""
        d = None if directivity is None else np.ascontiguousarray(np.asarray(directivity, dtype=np.complex64))
        t = None if range_taps is None else np.ascontiguousarray(np.asarray(range_taps, dtype=np.complex64).reshape(2, -1))
        desc = PrecisionDesc(None if d is None else d.ctypes.data, None if t is None else t.ctypes.data,
                             0 if t is None else t.shape[1], tap_center, flags, grid_count, grid_first, grid_last)
        self._check(self._lib.rtacx_configure_precision(self._h, ctypes.byref(desc)))

    def reduce_precision(self, samples, n: int, out, stream=None) -> None:
        self._check(self._lib.rtacx_reduce_precision(self._h, _ptr(samples), n, _ptr(out), _stream(stream)))

    def reduce_precision_host(self, samples, n: int, out, stream=None) -> None:
        """samples / out: host buffers (pinned for overlapped copies)."""
        self._check(self._lib.rtacx_reduce_precision_host(self._h, _ptr(samples), n, _ptr(out), _stream(stream)))

    def configure_receiver(self, rotation=None, directivity=None, carrier_hz: float = 0.0, flags: int = 0) -> None:
        R = np.eye(3, dtype=np.float32) if rotation is None else np.asarray(rotation, np.float32).reshape(3, 3)
        tab = None if directivity is None else np.ascontiguousarray(np.asarray(directivity, np.float32))
        r = Receiver((ctypes.c_float * 9)(*R.reshape(-1).tolist()), None if tab is None else tab.ctypes.data,
                     0 if tab is None else tab.shape[1], 0 if tab is None else tab.shape[0], carrier_hz, flags)
        self._check(self._lib.rtacx_configure_receiver(self._h, ctypes.byref(r)))

    def make_samples(self, hits, n: int, samples, stream=None) -> None:
        self._check(self._lib.rtacx_make_samples(self._h, _ptr(hits), n, _ptr(samples), _stream(stream)))

    def rasterize(self, vertices, normals, triangles, world_to_local, world_to_screen, origin, width: int,
                  height: int, samples, carrier_hz: float = 1.2e6, sound_celerity: float = 1500.0,
                  stream=None) -> None:
        """vertices / normals / triangles: device tensors; matrices row-major 4x4."""
        L = np.asarray(world_to_local, np.float32).reshape(16)
        S = np.asarray(world_to_screen, np.float32).reshape(16)
        m = Mesh(_ptr(vertices), _ptr(normals), _ptr(triangles), vertices.shape[0], triangles.shape[0])
        v = RasterView((ctypes.c_float * 16)(*L.tolist()), (ctypes.c_float * 16)(*S.tolist()),
                       (ctypes.c_float * 3)(*np.asarray(origin, np.float32).tolist()), width, height,
                       carrier_hz, sound_celerity)
        self._check(self._lib.rtacx_rasterize(self._h, ctypes.byref(m), ctypes.byref(v), _ptr(samples),
                                              _stream(stream)))

    def diag_drop_accumulation_stage(self, stage: int = 0xFFFFFFFF) -> None:
        """Failure-path diagnostic: the staged accumulation skips one stage's
        copy (0xFFFFFFFF: none), so its CTA times out and flags the error word."""
        self._check(self._lib.rtacx_diag_drop_accumulation_stage(self._h, stage))

    def diag_sorted(self, records, max_records: int, stream=None) -> None:
        """Copies the sorted scratch of the last binning (float4 records
        grouped by composite key) into `records`."""
        self._check(self._lib.rtacx_diag_sorted(self._h, _ptr(records), max_records, _stream(stream)))

    def set_tracing(self, enable: bool) -> None:
        self._check(self._lib.rtacx_set_tracing(self._h, 1 if enable else 0))

    def stage_times(self, precision: bool = False) -> dict:
        """Per-stage device milliseconds of the last traced call."""
        names = PRECISION_STAGES if precision else STAGES
        buf = (ctypes.c_float * len(STAGES))()
        k = self._lib.rtacx_stage_times(self._h, buf, len(STAGES))
        if k < 0:
            raise RtacxError(-k, self.last_error())
        return {names[i]: float(buf[i]) for i in range(min(k, len(names)))}

    def stream_status(self, stream=None) -> None:
        self._check(self._lib.rtacx_stream_status(self._h, _stream(stream)))


class Batch:
    """Batched plain form (rtacx_batch_*): many pings, one CUDA graph."""

    def __init__(self, device: int = 0):
        self._lib = load()
        h = _P()
        st = self._lib.rtacx_batch_create(ctypes.byref(h), device)
        if st != RTACX_OK:
            raise RtacxError(st, "rtacx_batch_create failed")
        self._h = h

    def close(self) -> None:
        if getattr(self, "_h", None) is not None and self._h.value:
            self._lib.rtacx_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, st: int) -> None:
        if st != RTACX_OK:
            msg = self._lib.rtacx_batch_last_error(self._h)
            raise RtacxError(st, msg.decode() if msg else "")

    def plan(self, pings, autotune: bool = True, staged: bool = False) -> None:
        """pings: sequence of (Context, samples tensor, n, out tensor). staged:
        one launch per binning stage instead of the fused single launch."""
        arr = (PingDesc * len(pings))()
        for i, (ctx, smp, n, out) in enumerate(pings):
            arr[i] = PingDesc(ctx.handle, _ptr(smp), n, _ptr(out))
        flags = (RTACX_BATCH_AUTOTUNE if autotune else 0) | (RTACX_BATCH_STAGED if staged else 0)
        self._check(self._lib.rtacx_batch_plan(self._h, arr, len(pings), flags))

    def run(self, stream=None) -> None:
        self._check(self._lib.rtacx_batch_run(self._h, _stream(stream)))

    def status(self, stream=None) -> None:
        """Waits for the stream; raises RtacxError (RTACX_ERR_DEVICE) if a
        grid-barrier wait of a run expired."""
        self._check(self._lib.rtacx_batch_status(self._h, _stream(stream)))

    def graph_kernels(self) -> int:
        k = _U32()
        self._check(self._lib.rtacx_batch_graph_kernels(self._h, ctypes.byref(k)))
        return k.value

    def diag_barrier(self, extra_arrivals: int, wait_ms: int = 1000) -> None:
        """Diagnostic (next plan): barriers wait for extra_arrivals more CTAs
        than the launch has; each wait gives up after wait_ms."""
        self._check(self._lib.rtacx_diag_batch_barrier(self._h, extra_arrivals, wait_ms))

    def tuning(self) -> dict:
        r, b, p = _U32(), _U32(), _U32()
        ms = ctypes.c_float()
        self._check(self._lib.rtacx_batch_tuning(self._h, ctypes.byref(r), ctypes.byref(b), ctypes.byref(p),
                                                 ctypes.byref(ms)))
        return {"tile_rows": r.value, "tile_bearings": b.value, "samples_per_cta": p.value, "tuned_ms": ms.value}
