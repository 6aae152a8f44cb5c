"""The C++ host mirror of the reference's receiver API
(include/rtacx/simulation.hpp) driven by a C++ program written the way a
reference user writes it (tests/cpp/sensor_instance_demo.cpp): SensorInfo +
Waveform_Sine (adaptive or fixed duration, 8x oversampling) + beam table ->
SensorInstance -> compute_output(). Its ping must match the FP64 oracle."""
import subprocess

import numpy as np
import pytest

from rtac_simulation_gb300 import build
from rtac_simulation_gb300 import workloads as wl

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():
    pytest.skip("needs a GPU", allow_module_level=True)


def run_demo(tmp_path, wk, frequency, duration, fixed, sink=None, texture_psf=False):
    if not build.DEMO_BIN.exists():
        build.build_demo()
    s = wk.sensor
    lines = [f"dims {wk.dims}", f"range_min {s['range_min']!r}", f"range_max {s['range_max']!r}",
             f"range_count {s['range_count']}", f"celerity {s['sound_celerity']!r}", f"frequency {frequency!r}",
             f"duration {duration!r}", f"fixed {1 if fixed else 0}", "oversampling 8",
             f"texture_psf {1 if texture_psf else 0}"]
    if wk.dims == 2:
        lines.append(f"beam_span {s['beam_span']!r}")
        lines.append("beam %d %s" % (len(s["beam"]), " ".join(repr(float(x)) for x in s["beam"])))
        lines.append("bearings %d %s" % (len(s["bearings"]), " ".join(repr(float(x)) for x in s["bearings"])))
    (tmp_path / "params.txt").write_text("\n".join(lines) + "\n")
    wk.samples.astype(np.float32).tofile(tmp_path / "samples.bin")
    res = subprocess.run([str(build.DEMO_BIN), str(tmp_path / "params.txt"), str(tmp_path / "samples.bin"),
                          str(tmp_path / "out.bin")] + ([str(sink)] if sink else []), capture_output=True, text=True)
    assert res.returncode == 0, res.stderr
    return np.fromfile(tmp_path / "out.bin", dtype=np.complex64).reshape(wk.out_shape)


def test_cpp_mirror_2d_adaptive_waveform(tmp_path, oracle):
    wk = wl.oculus_reference_2d(n_samples=30000)
    got = run_demo(tmp_path, wk, 1.2e6, 1.0, fixed=False)      # duration ignored: adaptive
    want = oracle.reduce(wk.samples, wk.sensor)
    assert np.linalg.norm(got - want) / np.linalg.norm(want) <= 1e-5


def test_cpp_mirror_1d_fixed_waveform(tmp_path, oracle):
    wk = wl.ea400_reference_1d(n_samples=30000)
    got = run_demo(tmp_path, wk, 38.0e3, 128.0e-6, fixed=True)
    want = oracle.reduce(wk.samples, wk.sensor)
    assert np.linalg.norm(got - want) / np.linalg.norm(want) <= 1e-5


def test_cpp_file_sink_records(tmp_path, oracle):
    """SensorInstance2D_2<Complex> (the reference factory's type) read through
    get_ping(), and two FileSink records of its pings."""
    from rtac_simulation_gb300.sink import read_pings
    wk = wl.oculus_reference_2d(n_samples=20000)
    got = run_demo(tmp_path, wk, 1.2e6, 1.0, fixed=False, sink=tmp_path / "pings.bin")
    want = oracle.reduce(wk.samples, wk.sensor)
    assert np.linalg.norm(got - want) / np.linalg.norm(want) <= 1e-5
    recs = read_pings(tmp_path / "pings.bin")
    assert len(recs) == 2
    for r in recs:
        assert r["ping"].shape == wk.out_shape
        np.testing.assert_array_equal(r["bearings"], np.asarray(wk.sensor["bearings"], np.float32))
        assert np.linalg.norm(r["ping"] - got) <= 1e-6 * np.linalg.norm(got)
        assert r["range_min"] == np.float32(wk.sensor["range_min"]) and r["range_max"] == np.float32(wk.sensor["range_max"])


def test_cpp_mirror_2d_texture_psf_matches_reference_texture_model(tmp_path, oracle):
    """set_texture_psf(true) on the C++ mirror: the PSF is fetched from a
    texture as the reference's SensorInstance2D does, and the ping matches
    the oracle's texture-unit model (which reproduces the reference's own
    kernel, tests/test_oracle_golden.py) to float round-off."""
    wk = wl.oculus_reference_2d(n_samples=20000)
    got = run_demo(tmp_path, wk, wk.meta["frequency"], 0.0, False, texture_psf=True).astype(np.complex128)
    want = oracle.reduce(wk.samples, wk.sensor, mode=2)
    assert np.linalg.norm(got - want) / np.linalg.norm(want) <= 1e-6
