"""Sort + bin parity (bit-exact): keys, counts, segments, windows and
out-of-range counts of rtacx_bin against the oracle's literal restatement of
Binner::Key / do_make_segments / do_make_bins."""
import numpy as np
import pytest

from rtac_simulation_gb300 import workloads as wl

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():
    pytest.skip("needs a GPU", allow_module_level=True)

from helpers_gpu import gpu_bin, make_context  # noqa: E402


def check_bin(oracle, wk, offset_floats=0):
    ctx = make_context(wk)
    got = gpu_bin(ctx, wk.samples, wk.dims, wk.sensor["range_count"], offset_floats)
    s = wk.sensor
    keys, _ = oracle.range_keys(s["range_count"], s["range_min"], s["range_max"], s["margin"], wk.samples[:, 2])
    want = oracle.bin_samples(wk.samples, s)
    np.testing.assert_array_equal(got["keys"], keys)
    np.testing.assert_array_equal(got["counts"], want["counts"])
    np.testing.assert_array_equal(got["oor"], want["oor"])
    np.testing.assert_array_equal(got["segments"], want["segments"])
    np.testing.assert_array_equal(got["windows"], want["windows"])
    ctx.close()


@pytest.mark.parametrize("maker", [
    lambda: wl.echosounder_1d(),
    lambda: wl.ea400_reference_1d(),
    lambda: wl.oculus_reference_2d(),
    lambda: wl.oculus_2d(n_samples=1 << 17),
    lambda: wl.precision_2d(n_samples=1 << 16),
])
def test_bin_matches_oracle(oracle, maker):
    check_bin(oracle, maker())


def test_bin_full_size_precision_ping(oracle):
    check_bin(oracle, wl.precision_2d())


def test_bin_unaligned_records(oracle):
    # A 2D buffer that is 4-byte but not 16-byte aligned takes the scalar-load path.
    check_bin(oracle, wl.oculus_reference_2d(n_samples=3000), offset_floats=1)


@pytest.mark.parametrize("n", [0, 1, 2, 31, 33, 1000])
def test_bin_small_counts(oracle, n):
    wk = wl.oculus_reference_2d(n_samples=max(n, 1))
    wk.samples = wk.samples[:n]
    check_bin(oracle, wk)


def test_bin_hot_bins_and_nulls(oracle):
    wk = wl.oculus_2d(n_samples=1 << 16)
    smp = wk.samples
    R = wl.linspace(wk.sensor["range_min"], wk.sensor["range_max"], wk.sensor["range_count"])
    smp[: 1 << 14, 2] = R[100]          # one hot bin
    smp[1 << 14: 1 << 15, 2] = R[101]   # its neighbour
    smp[-1000:, :] = 0.0
    smp[-1000:, 2] = -1.0                # null samples (travel -1)
    check_bin(oracle, wk)


def test_bin_degenerate_sensors(oracle):
    for nR in (1, 2, 3):
        wk = wl.oculus_reference_2d(n_samples=500)
        wk.sensor["range_count"] = nR
        check_bin(oracle, wk)
    wk = wl.oculus_reference_2d(n_samples=500)
    wk.sensor["margin"] = 0.0
    check_bin(oracle, wk)


def test_bin_special_travels(oracle):
    wk = wl.oculus_reference_2d(n_samples=64)
    wk.samples[:8, 2] = [np.inf, -np.inf, 1e30, -1e30, 0.0, -0.0, 3e9, -3e9]
    ctx = make_context(wk)
    got = gpu_bin(ctx, wk.samples, 2, wk.sensor["range_count"])
    s = wk.sensor
    keys, _ = oracle.range_keys(s["range_count"], s["range_min"], s["range_max"], s["margin"], wk.samples[:, 2])
    np.testing.assert_array_equal(got["keys"], keys)
