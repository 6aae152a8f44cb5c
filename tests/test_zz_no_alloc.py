"""rtacx_reduce_noalloc: the allocation-free ping.

For callers that cannot call cudaMalloc (allocation-banned sensor loops,
processes whose device memory belongs to another allocator), the library
offers one entry point whose scratch is a fixed file-scope device array.
This test calls it through the C ABI twice in a row and compares each result
with the ordinary rtacx_reduce path at the plain form's tolerance. It sits in
its own file, collected last, and passes alone in a fresh process as well as
after the other tests.
"""
import ctypes

import numpy as np
import pytest

from rtac_simulation_gb300 import _lib
from rtac_simulation_gb300 import workloads as wl

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():
    pytest.skip("needs a GPU", allow_module_level=True)

TOL = 1e-5


def _sensor_struct(wk):
    keep = []
    s = wk.sensor
    pulse = np.ascontiguousarray(s["pulse"], dtype=np.complex64)
    keep.append(pulse)
    if wk.dims == 1:
        st = _lib.Sensor1D(s["range_min"], s["range_max"], s["range_count"], s["sound_celerity"],
                           s["pulse_duration"], s["margin"], pulse.ctypes.data, pulse.size, 0)
        return st, keep
    beam = np.ascontiguousarray(s["beam"], dtype=np.float32)
    bear = np.ascontiguousarray(s["bearings"], dtype=np.float32)
    keep += [beam, bear]
    st = _lib.Sensor2D(s["range_min"], s["range_max"], s["range_count"], s["sound_celerity"],
                       s["pulse_duration"], s["margin"], pulse.ctypes.data, pulse.size,
                       beam.ctypes.data, beam.size, s["beam_span"], bear.ctypes.data, bear.size, 0)
    return st, keep


def _to_complex(t):
    o = t.cpu().numpy()
    return o[..., 0].astype(np.float64) + 1j * o[..., 1]


@pytest.mark.parametrize("maker", [
    lambda: wl.oculus_reference_2d(n_samples=30000),
    lambda: wl.oculus_2d(n_samples=1 << 17, n_ranges=512),
    lambda: wl.echosounder_1d(n_samples=1 << 16, n_ranges=2048),
])
def test_noalloc_matches_reduce_twice(maker):
    wk = maker()
    lib = _lib.load()
    dev = torch.from_numpy(wk.samples.reshape(-1)).cuda()
    stream = torch.cuda.current_stream()

    ctx = _lib.Context(0)
    if wk.dims == 1:
        ctx.configure_1d(**wk.sensor)
    else:
        ctx.configure_2d(**wk.sensor)
    ref_out = torch.empty(wk.out_shape + (2,), dtype=torch.float32, device="cuda")
    ctx.reduce(dev, wk.n, ref_out, stream=stream)
    ctx.stream_status(stream)
    ref = _to_complex(ref_out)
    ctx.close()

    sensor, keep = _sensor_struct(wk)
    kind = _lib.RTACX_SAMPLE_1D if wk.dims == 1 else _lib.RTACX_SAMPLE_2D
    for _ in range(2):
        out = torch.full(wk.out_shape + (2,), float("nan"), dtype=torch.float32, device="cuda")
        st = lib.rtacx_reduce_noalloc(kind, ctypes.byref(sensor), dev.data_ptr(), wk.n, out.data_ptr(),
                                      stream.cuda_stream)
        assert st == _lib.RTACX_OK
        torch.cuda.synchronize()
        got = _to_complex(out)
        assert np.isfinite(got).all()
        err = np.linalg.norm(got - ref) / np.linalg.norm(ref)
        assert err <= TOL, err


def test_noalloc_rejects_sizes_beyond_limits():
    wk = wl.oculus_reference_2d(n_samples=16)
    lib = _lib.load()
    sensor, keep = _sensor_struct(wk)
    dev = torch.zeros(16, dtype=torch.float32, device="cuda")
    out = torch.zeros(wk.out_shape + (2,), dtype=torch.float32, device="cuda")
    too_many = (1 << 18) + 1
    assert lib.rtacx_reduce_noalloc(_lib.RTACX_SAMPLE_2D, ctypes.byref(sensor), dev.data_ptr(), too_many,
                                    out.data_ptr(), None) == _lib.RTACX_ERR_UNSUPPORTED
    sensor.range_count = 4097
    assert lib.rtacx_reduce_noalloc(_lib.RTACX_SAMPLE_2D, ctypes.byref(sensor), dev.data_ptr(), 4,
                                    out.data_ptr(), None) == _lib.RTACX_ERR_UNSUPPORTED


def test_noalloc_rejects_misaligned_buffers():
    """Only 4-byte aligned samples and 8-byte aligned pings are accepted; the
    check comes before any upload or launch."""
    wk = wl.oculus_reference_2d(n_samples=16)
    lib = _lib.load()
    sensor, keep = _sensor_struct(wk)
    dev = torch.zeros(64 + 4, dtype=torch.float32, device="cuda")
    out = torch.zeros(2 * wk.out_shape[0] * wk.out_shape[1] + 2, dtype=torch.float32, device="cuda")
    assert lib.rtacx_reduce_noalloc(_lib.RTACX_SAMPLE_2D, ctypes.byref(sensor), dev.data_ptr(), 16,
                                    out.data_ptr() + 4, None) == _lib.RTACX_ERR_INVALID_ARGUMENT
    assert lib.rtacx_reduce_noalloc(_lib.RTACX_SAMPLE_2D, ctypes.byref(sensor), dev.data_ptr() + 2, 16,
                                    out.data_ptr(), None) == _lib.RTACX_ERR_INVALID_ARGUMENT
    assert torch.count_nonzero(out).item() == 0
