"""Known-answer tests of the oracle's restatement of the reference path.

No reference test pins this part of the path (the reference has no asserting
tests), so these cases are derived by hand from the cited reference code:
do_make_segments / do_make_bins (src/Binner.cu:51-136) and the texture
lookup of KernelView2D (include/rtac_simulation/ReductionKernel.h:44-73).
"""
import math

import numpy as np
import pytest

from rtac_simulation_gb300 import workloads as wl


def small_sensor(nR=64, nB=8, taps=9, beam_taps=17, extent_bins=9.0, span=0.2):
    rmin, rmax, c = 1.0, 11.0, 1500.0
    res = float(wl.linspace_resolution(rmin, rmax, nR))
    pulse = (np.arange(taps) + 1 + 1j * (np.arange(taps) - 3)).astype(np.complex64)
    beam = (1.0 + np.arange(beam_taps, dtype=np.float32)) / beam_taps
    bearings = np.linspace(-0.3, 0.3, nB).astype(np.float32)
    return wl.sensor_2d(rmin, rmax, nR, c, pulse, extent_bins * res, beam, span, bearings)


def samples2d(travel, bearing, value):
    travel = np.asarray(travel, np.float32)
    out = np.zeros((travel.size, 4), np.float32)
    out[:, 0] = np.real(value)
    out[:, 1] = np.imag(value)
    out[:, 2] = travel
    out[:, 3] = bearing
    return out


def test_segments_follow_sorted_keys(oracle):
    s = small_sensor()
    R = wl.linspace(s["range_min"], s["range_max"], s["range_count"])
    t = np.array([R[5], R[3], R[5], R[40], 0.1, 50.0, R[3]], np.float32)
    b = oracle.bin_samples(samples2d(t, 0.0, 1.0), s)
    keys, side = oracle.range_keys(s["range_count"], s["range_min"], s["range_max"], s["margin"], t)
    assert b["oor"].tolist() == [int((side < 0).sum()), int((side > 0).sum())]
    low = int(b["oor"][0])
    # Sorted by travel: low out-of-range first, then bins in order.
    order = sorted(k for k in keys.tolist() if k != 0xFFFFFFFF)
    for k in set(order):
        first = low + order.index(k)
        assert b["segments"][k].tolist() == [first, first + order.count(k)]
    assert b["counts"].sum() == len(order)
    empty = [k for k in range(s["range_count"]) if k not in order]
    assert np.all(b["segments"][empty] == 0)


def test_single_nonempty_bin_gives_empty_windows(oracle):
    # do_make_bins: a window with exactly one non-empty bin shrinks to
    # istart == iend and yields an empty view (src/Binner.cu:90-102).
    s = small_sensor()
    R = wl.linspace(s["range_min"], s["range_max"], s["range_count"])
    smp = samples2d([R[20]] * 3, 0.0, 1.0 + 1.0j)
    b = oracle.bin_samples(smp, s)
    assert b["overlap"] > 0
    assert np.all(b["windows"] == 0)
    assert np.all(oracle.reduce(smp, s) == 0)


def test_zero_overlap_gives_zero_ping(oracle):
    s = small_sensor()
    s["margin"] = 0.5 * float(wl.linspace_resolution(s["range_min"], s["range_max"], s["range_count"]))
    assert oracle.bin_overlap(s["range_min"], s["range_max"], s["range_count"], s["margin"]) == 0
    wk = wl.oculus_2d(n_samples=2000, n_bearings=8, n_ranges=64, rmin=1.0, rmax=11.0)
    wk.sensor["margin"] = s["margin"]
    assert np.all(oracle.reduce(wk.samples, wk.sensor) == 0)


def test_empty_and_out_of_range_inputs(oracle):
    s = small_sensor()
    assert np.all(oracle.reduce(np.zeros((0, 4), np.float32), s) == 0)
    smp = samples2d([-1.0, 0.0, 1e6, np.inf], 0.0, 1.0)
    b = oracle.bin_samples(smp, s)
    assert b["counts"].sum() == 0 and b["oor"].sum() == 4
    assert np.all(oracle.reduce(smp, s) == 0)


def test_two_sample_psf_value(oracle):
    # Sample A exactly on output range r and bearing b, sample B (value 0)
    # in the next bin so that the window is not empty: out(r, b) is
    # v_A * pulse[centre] * beam[centre] for odd table sizes.
    s = small_sensor()
    R = wl.linspace(s["range_min"], s["range_max"], s["range_count"])
    r, b = 30, 3
    th = s["bearings"][b]
    smp = samples2d([R[r], R[r + 1]], th, np.array([2.0 - 1.0j, 0.0]))
    out = oracle.reduce(smp, s)
    H, W = len(s["pulse"]), len(s["beam"])
    want = (2.0 - 1.0j) * complex(s["pulse"][H // 2]) * float(s["beam"][W // 2])
    # The texel coordinate of d = 0 is exactly the centre tap only up to the
    # float rounding of the pulse scale.
    assert abs(out[r, b] - want) < 1e-5 * abs(want)


def test_psf_is_linear_interpolation(oracle):
    # Half-way between two texels the PSF is the mean of the two taps.
    s = small_sensor(taps=9, extent_bins=9.0)
    R = wl.linspace(s["range_min"], s["range_max"], s["range_count"])
    r, b = 30, 2
    th = s["bearings"][b]
    ext = 1.0 / float(np.float32(np.float32(1.0) / np.float32(np.float32(s["pulse_duration"]) * np.float32(s["sound_celerity"]))))
    d = ext / 9.0 * 0.5
    smp = samples2d([R[r] + d, R[r + 2]], th, np.array([1.0, 0.0]))
    out = oracle.reduce(smp, s)
    H = len(s["pulse"])
    want = 0.5 * (complex(s["pulse"][H // 2]) + complex(s["pulse"][H // 2 + 1])) * float(s["beam"][len(s["beam"]) // 2])
    assert abs(out[r, b] - want) < 2e-4 * abs(want)


def test_fp32_reference_arithmetic_close_to_fp64(oracle):
    wk = wl.oculus_2d(n_samples=20000, n_bearings=64, n_ranges=128)
    o64 = oracle.reduce(wk.samples, wk.sensor, mode=0)
    o32 = oracle.reduce(wk.samples, wk.sensor, mode=1)
    err = np.linalg.norm(o32 - o64) / np.linalg.norm(o64)
    assert 0 < err < 1e-3


def test_permutation_invariance(oracle):
    wk = wl.oculus_reference_2d(n_samples=5000)
    perm = np.random.default_rng(0).permutation(wk.n)
    a = oracle.reduce(wk.samples, wk.sensor)
    b = oracle.reduce(wk.samples[perm], wk.sensor)
    assert np.linalg.norm(a - b) <= 1e-12 * np.linalg.norm(a)


@pytest.mark.parametrize("maker", [wl.ea400_reference_1d, lambda: wl.echosounder_1d(n_samples=4000, n_ranges=512)])
def test_1d_oracle_runs(oracle, maker):
    wk = maker()
    out = oracle.reduce(wk.samples, wk.sensor)
    assert out.shape == (wk.sensor["range_count"],)
    assert np.isfinite(out).all() and np.abs(out).max() > 0
