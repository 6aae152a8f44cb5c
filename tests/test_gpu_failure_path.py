"""Failure path of the bounded waits, without a GPU fault: the staged
precision accumulation is told to skip one stage's bulk copy
(rtacx_diag_drop_accumulation_stage), so the CTA waiting for it runs out its
bounded wait (about one second), sets the device error word and stops.
rtacx_stream_status reports it, and the same context then computes a
correct ping."""
import numpy as np
import pytest

from rtac_simulation_gb300 import workloads as wl

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():
    pytest.skip("needs a GPU", allow_module_level=True)

from helpers_gpu import make_context, rel_l2, to_device  # noqa: E402
from rtac_simulation_gb300 import _lib  # noqa: E402


def test_dropped_stage_times_out_and_context_recovers(oracle):
    wk = wl.precision_2d(n_samples=1 << 16, n_bearings=128, n_ranges=512)
    ctx = make_context(wk)
    ctx.set_echo_model(wk.echo["carrier_hz"], wk.echo["flags"])
    tab = wl.precision_tables(wk.sensor, **wk.precision)
    ctx.configure_precision(**tab)
    d = to_device(wk.samples)
    out = torch.empty(tuple(wk.out_shape) + (2,), dtype=torch.float32, device="cuda")
    stream = torch.cuda.current_stream()

    ctx.diag_drop_accumulation_stage(5)
    ctx.reduce_precision(d, wk.n, out, stream=stream)
    with pytest.raises(_lib.RtacxError) as e:
        ctx.stream_status(stream)
    assert e.value.status == _lib.RTACX_ERR_DEVICE
    assert "8" in str(e.value)            # kErrAccumulateTimeout = 1 << 3

    ctx.diag_drop_accumulation_stage()
    ctx.reduce_precision(d, wk.n, out, stream=stream)
    ctx.stream_status(stream)
    o = out.cpu().numpy()
    got = o[..., 0].astype(np.float64) + 1j * o[..., 1]
    want = oracle.reduce_binned(oracle.apply_echo(wk.samples, wk.sensor, wk.echo), wk.sensor, tab)
    assert rel_l2(got, want) <= 1e-4
