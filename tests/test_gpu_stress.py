"""Contention stress ping (half of the samples in ~1% of the range bins):
bit-exact bin counts, segments and windows at the full 2^27-sample size, the
precision form against the FP64 oracle of its binned model on every row of
the full ping, and both forms against their FP64 oracles on a reduced copy
with the same structure (the hot tiles are split across CTAs by the
persistent gather)."""
import numpy as np
import pytest

from rtac_simulation_gb300 import workloads as wl

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():
    pytest.skip("needs a GPU", allow_module_level=True)

from helpers_gpu import gpu_bin, gpu_reduce, make_context, rel_l2  # noqa: E402
from test_gpu_precision import gpu_precision, precision_context  # noqa: E402


def reference_segments_windows(counts, low, overlap):
    """do_make_segments / do_make_bins restated on bin counts (numpy)."""
    nR = counts.size
    starts = low + np.concatenate([[0], np.cumsum(counts)[:-1]]).astype(np.int64)
    seg = np.zeros((nR, 2), np.uint32)
    ne = counts > 0
    seg[ne, 0] = starts[ne]
    seg[ne, 1] = starts[ne] + counts[ne]
    win = np.zeros((nR, 2), np.uint32)
    nz = np.flatnonzero(ne)
    for r in range(nR):
        lo, hi = max(0, r - overlap), min(nR - 1, r + overlap)
        i0 = np.searchsorted(nz, lo)
        i1 = np.searchsorted(nz, hi, side="right") - 1
        if i0 <= i1 and nz[i0] < nz[i1]:
            f, l = nz[i0], nz[i1]
            win[r] = (starts[f], starts[l] + counts[l] - starts[f])
    return seg, win


def test_stress_full_size_binning_bit_exact(oracle):
    wk = wl.stress_2d()
    s = wk.sensor
    ctx = make_context(wk)
    got = gpu_bin(ctx, wk.samples, 2, s["range_count"])
    keys, side = oracle.range_keys(s["range_count"], s["range_min"], s["range_max"], s["margin"], wk.samples[:, 2])
    np.testing.assert_array_equal(got["keys"], keys)
    valid = keys != 0xFFFFFFFF
    counts = np.bincount(keys[valid].astype(np.int64), minlength=s["range_count"]).astype(np.uint32)
    np.testing.assert_array_equal(got["counts"], counts)
    low, high = int((side < 0).sum()), int((side > 0).sum())
    assert got["oor"].tolist() == [low, high]
    ov = oracle.bin_overlap(s["range_min"], s["range_max"], s["range_count"], s["margin"])
    seg, win = reference_segments_windows(counts.astype(np.int64), low, ov)
    np.testing.assert_array_equal(got["segments"], seg)
    np.testing.assert_array_equal(got["windows"], win)
    # The cluster really is hot: half of the samples in about 1% of the bins.
    top = np.sort(counts)[::-1][: s["range_count"] // 100].sum()
    assert top > 0.45 * wk.n


@pytest.mark.parametrize("hot", [False, True])
def test_stress_full_size_precision_every_row(oracle, hot):
    """2^27 samples, 1024 x 8192, the 271 MB grid larger than the L2, with
    and without the hot-range replicas: every row against the binned FP64
    oracle."""
    from rtac_simulation_gb300 import _lib
    wk = wl.stress_2d()
    ctx = precision_context(wk, flags=_lib.RTACX_PRECISION_HOT_RANGE if hot else 0)
    got = gpu_precision(ctx, wk.samples, wk.out_shape)
    ctx.close()
    tab = wl.precision_tables(wk.sensor, **wk.precision)
    want = oracle.reduce_binned(oracle.apply_echo(wk.samples, wk.sensor, wk.echo), wk.sensor, tab)
    assert np.isfinite(got).all()
    assert rel_l2(got, want) <= 1e-4


def test_stress_reduced_plain_matches_oracle(oracle):
    wk = wl.stress_2d(n_samples=1 << 20, n_ranges=2048)
    ctx = make_context(wk)
    ctx.set_echo_model(wk.echo["carrier_hz"], wk.echo["flags"])
    got = gpu_reduce(ctx, wk.samples, wk.out_shape)
    want = oracle.reduce(oracle.apply_echo(wk.samples, wk.sensor, wk.echo), wk.sensor)
    assert rel_l2(got, want) <= 1e-5


def test_stress_reduced_precision_matches_oracle(oracle):
    wk = wl.stress_2d(n_samples=1 << 20, n_ranges=2048)
    ctx = precision_context(wk)
    got = gpu_precision(ctx, wk.samples, wk.out_shape)
    tab = wl.precision_tables(wk.sensor, **wk.precision)
    want = oracle.reduce_binned(oracle.apply_echo(wk.samples, wk.sensor, wk.echo), wk.sensor, tab)
    assert rel_l2(got, want) <= 1e-4


@pytest.mark.parametrize("flags_name", ["RTACX_PRECISION_HOT_RANGE", "RTACX_PRECISION_HOT_RANGE|FP16"])
def test_stress_reduced_precision_hot_range_matches_oracle(oracle, flags_name):
    """Clustered ping with the hot-range replicas (the densest 128 range
    nodes, 256 output bins, accumulate into 8 replicas added back before the
    contraction): same oracle bar, through the device and the host-buffer
    entry points."""
    from rtac_simulation_gb300 import _lib
    from test_gpu_precision import gpu_precision_host
    flags = _lib.RTACX_PRECISION_HOT_RANGE
    if "FP16" in flags_name:
        flags |= _lib.RTACX_PRECISION_FP16_ROWSCALE
    wk = wl.stress_2d(n_samples=1 << 20, n_ranges=2048)
    ctx = precision_context(wk, flags=flags)
    tab = wl.precision_tables(wk.sensor, **wk.precision)
    want = oracle.reduce_binned(oracle.apply_echo(wk.samples, wk.sensor, wk.echo), wk.sensor, tab)
    got = gpu_precision(ctx, wk.samples, wk.out_shape)
    assert rel_l2(got, want) <= 1e-4
    host = gpu_precision_host(ctx, wk.samples, wk.out_shape)
    assert rel_l2(host, want) <= 1e-4


def test_uniform_ping_with_hot_range_flag_unchanged():
    """No dense interval on a uniform ping: the flag changes nothing but the
    order of float additions."""
    from rtac_simulation_gb300 import _lib
    wk = wl.precision_2d(n_samples=1 << 18, n_bearings=128, n_ranges=2048)
    a = gpu_precision(precision_context(wk), wk.samples, wk.out_shape)
    b = gpu_precision(precision_context(wk, flags=_lib.RTACX_PRECISION_HOT_RANGE), wk.samples, wk.out_shape)
    assert rel_l2(b, a) <= 1e-5
