"""The reference-side binding (the statements a maintainer adds to the
reference's SensorInstance2D, tests/cpp/binding/sensor_instance2d_rtacx.inc):
it compiles against the reference's own headers and links to librtacx.so
(oracle/binding_check.sh, where the reference tree is present), and the same
statements, run on a GPU in a stand-in of the class, give the oracle's ping."""
import subprocess
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]


def test_binding_compiles_against_the_reference_headers():
    from rtac_simulation_gb300 import build
    if not build.LIB.exists():
        build.build_library()
    res = subprocess.run([str(ROOT / "oracle" / "binding_check.sh")], capture_output=True, text=True, timeout=300)
    assert res.returncode == 0, res.stdout + res.stderr
    if "nothing checked" in res.stdout:
        pytest.skip("no reference tree on this machine")
    so = ROOT / "oracle" / "_ref" / "binding_real_headers.so"
    undefined = subprocess.run(["nm", "-D", "--undefined-only", str(so)], capture_output=True, text=True).stdout
    for sym in ("rtacx_create", "rtacx_configure_2d", "rtacx_reduce", "rtacx_stream_status", "rtacx_destroy"):
        assert sym in undefined, sym
    exported = subprocess.run(["nm", "-D", "--defined-only", str(build.LIB)], capture_output=True, text=True).stdout
    for sym in ("rtacx_create", "rtacx_configure_2d", "rtacx_reduce", "rtacx_stream_status", "rtacx_destroy"):
        assert f" T {sym}" in exported, sym


def _run_binding(tmp_path, wk, texture=False):
    from rtac_simulation_gb300 import build
    if not build.BINDING_BIN.exists() or build.BINDING_BIN.stat().st_mtime < build.BINDING_SRC.stat().st_mtime:
        build.build_binding()
    s = wk.sensor
    p = np.asarray(s["pulse"], dtype=np.complex64)
    pairs = np.stack([p.real, p.imag], axis=-1).reshape(-1)
    n_taps = p.size
    lines = [f"range_min {s['range_min']!r}", f"range_max {s['range_max']!r}", f"range_count {s['range_count']}",
             f"celerity {s['sound_celerity']!r}", f"duration {s['pulse_duration']!r}", f"beam_span {s['beam_span']!r}",
             "pulse %d %s" % (n_taps, " ".join(repr(float(x)) for x in pairs)),
             "beam %d %s" % (len(s["beam"]), " ".join(repr(float(x)) for x in s["beam"])),
             "bearings %d %s" % (len(s["bearings"]), " ".join(repr(float(x)) for x in s["bearings"]))]
    (tmp_path / "params.txt").write_text("\n".join(lines) + "\n")
    wk.samples.astype(np.float32).tofile(tmp_path / "samples.bin")
    res = subprocess.run([str(build.BINDING_BIN), str(tmp_path / "params.txt"), str(tmp_path / "samples.bin"),
                          str(tmp_path / "out.bin")] + (["texture"] if texture else []),
                         capture_output=True, text=True, timeout=120)
    assert res.returncode == 0, res.stderr
    margin = float(res.stdout.split()[1])
    return np.fromfile(tmp_path / "out.bin", dtype=np.complex64).reshape(wk.out_shape), margin


@pytest.mark.gpu
def test_binding_ping_matches_the_oracle(tmp_path, oracle):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("needs a GPU")
    from helpers_gpu import rel_l2
    from rtac_simulation_gb300 import workloads as wl
    wk = wl.oculus_reference_2d(n_samples=20000)
    got, margin = _run_binding(tmp_path, wk)
    sensor = dict(wk.sensor, margin=margin)
    want = oracle.reduce(wk.samples, sensor)
    assert np.isfinite(got).all()
    assert rel_l2(got, want) <= 1e-5
