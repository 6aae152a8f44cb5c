"""The C-ABI library loads and exports every entry point include/rtacx.h
declares, with the struct layouts the header defines. No GPU needed: no call
here launches device work."""
import ctypes
import re
import subprocess
import tempfile
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
HEADER = ROOT / "include" / "rtacx.h"


@pytest.fixture(scope="module")
def lib():
    from rtac_simulation_gb300 import _lib, build
    srcs = build.sources()
    if not _lib.LIB_PATH.exists() or any(s.stat().st_mtime > _lib.LIB_PATH.stat().st_mtime for s in srcs):
        build.build_library()
    return _lib


def declared_functions():
    text = HEADER.read_text()
    return sorted(set(re.findall(r"^\s*(?:rtacx_status|void|int|const char\*)\s+(rtacx_\w+)\s*\(", text, re.M)))


def test_header_declares_entry_points():
    names = declared_functions()
    assert {"rtacx_create", "rtacx_destroy", "rtacx_configure_1d", "rtacx_configure_2d",
            "rtacx_bin", "rtacx_reduce", "rtacx_stream_status"} <= set(names)


def test_library_exports_every_declared_symbol(lib):
    so = ctypes.CDLL(str(lib.LIB_PATH))
    for name in declared_functions():
        assert hasattr(so, name), name
        assert name in lib.SIGNATURES, f"{name} has no ctypes signature"
    nm = subprocess.run(["nm", "-D", "--defined-only", str(lib.LIB_PATH)], capture_output=True, text=True).stdout
    exported = set(re.findall(r"\b(rtacx_\w+)\b", nm))
    assert set(declared_functions()) <= exported


def test_struct_layout_matches_header(lib):
    fields = {"rtacx_sensor_1d": lib.Sensor1D, "rtacx_sensor_2d": lib.Sensor2D}
    lines = ['#include <stdio.h>', '#include <stddef.h>', f'#include "{HEADER}"', "int main(void) {"]
    for cname, py in fields.items():
        lines.append(f'printf("{cname} size %zu\\n", sizeof({cname}));')
        for f, _ in py._fields_:
            lines.append(f'printf("{cname} {f} %zu\\n", offsetof({cname}, {f}));')
    lines.append("return 0; }")
    with tempfile.TemporaryDirectory() as d:
        src, exe = Path(d) / "probe.c", Path(d) / "probe"
        src.write_text("\n".join(lines))
        subprocess.run(["gcc", "-std=c99", str(src), "-o", str(exe)], check=True)
        out = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split("\n")
    got = {}
    for line in out:
        if line:
            parts = line.split()
            got[(parts[0], parts[1])] = int(parts[2])
    for cname, py in fields.items():
        assert got[(cname, "size")] == ctypes.sizeof(py)
        for f, _ in py._fields_:
            assert got[(cname, f)] == getattr(py, f).offset, (cname, f)


def test_version_string(lib):
    so = lib.load()
    assert b"sm_103a" in so.rtacx_version()


def test_create_without_gpu_fails_cleanly(lib):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    so = lib.load()
    h = ctypes.c_void_p()
    assert so.rtacx_create(ctypes.byref(h), 0) != lib.RTACX_OK
    assert not h.value


def test_directivity_table_sizes_without_a_gpu(lib):
    # The size query does no device work: the table sides follow the
    # reference builders (src/Directivity.cpp:63-64, 113-114), checked against
    # the tables the reference's own code produced.
    import json
    from pathlib import Path
    cases = json.loads((Path(__file__).resolve().parent / "golden" / "ref_directivity.json").read_text())["cases"]
    for c in cases:
        par = [float.fromhex(x) for x in c["params"]]
        baffle = 1.0 if c["baffle"] == "single-sided" else 0.0
        kind = lib.RTACX_DIRECTIVITY_RECTANGLE if c["kind"] == "RECT" else lib.RTACX_DIRECTIVITY_DISK
        assert lib.directivity_table_size(kind, par + [baffle, float(c["oversampling"])]) == (c["height"], c["width"])


def test_directivity_table_rejects_bad_parameters(lib):
    rect, disk = lib.RTACX_DIRECTIVITY_RECTANGLE, lib.RTACX_DIRECTIVITY_DISK
    for kind, par, status in [
        (rect, [0.0, 0.01, 0.00125, 0.0, 1.0], lib.RTACX_ERR_INVALID_ARGUMENT),
        (rect, [0.01, 0.01, 0.00125, 0.0, 0.5], lib.RTACX_ERR_INVALID_ARGUMENT),
        (rect, [float("nan"), 0.01, 0.00125, 0.0, 1.0], lib.RTACX_ERR_INVALID_ARGUMENT),
        (rect, [1e30, 0.01, 0.00125, 0.0, 1.0], lib.RTACX_ERR_UNSUPPORTED),
        (rect, [0.01, 0.01, 0.00125, 0.0, 1e30], lib.RTACX_ERR_UNSUPPORTED),
        (rect, [3.0, 3.0, 0.00125, 0.0, 1.0], lib.RTACX_ERR_UNSUPPORTED),
        (disk, [1e30, 0.00125, 0.0, 1.0], lib.RTACX_ERR_UNSUPPORTED),
        (disk, [0.1, 0.00125, 0.0, float("inf")], lib.RTACX_ERR_UNSUPPORTED),
        (disk, [0.1, -1.0, 0.0, 1.0], lib.RTACX_ERR_INVALID_ARGUMENT),
        (7, [0.1, 0.00125, 0.0, 1.0], lib.RTACX_ERR_INVALID_ARGUMENT),
    ]:
        with pytest.raises(lib.RtacxError) as e:
            lib.directivity_table_size(kind, par)
        assert e.value.status == status, (kind, par)


def test_cpp_mirror_without_a_gpu_reports_the_failure(lib, tmp_path):
    # The C++ mirror (include/rtacx/simulation.hpp) turns a failing status
    # into std::runtime_error, as the reference's API throws: without a GPU
    # the sensor's constructor cannot create its context, and the demo
    # program written against the mirror exits with that message.
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    from rtac_simulation_gb300 import build
    srcs = build.sources() + [build.DEMO_SRC, ROOT / "include" / "rtacx" / "simulation.hpp"]
    if not build.DEMO_BIN.exists() or any(s.stat().st_mtime > build.DEMO_BIN.stat().st_mtime for s in srcs):
        build.build_demo()
    (tmp_path / "params.txt").write_text("dims 1\nrange_min 0.5\nrange_max 100.0\nrange_count 64\n"
                                         "celerity 1500.0\nfrequency 38000.0\nduration 0.0001\nfixed 0\n"
                                         "oversampling 8\ntexture_psf 0\n")
    (tmp_path / "samples.bin").write_bytes(bytes(48))
    res = subprocess.run([str(build.DEMO_BIN), str(tmp_path / "params.txt"), str(tmp_path / "samples.bin"),
                          str(tmp_path / "out.bin")], capture_output=True, text=True, timeout=60)
    assert res.returncode != 0
    assert "cannot create a context on CUDA device 0" in res.stderr
    assert not (tmp_path / "out.bin").exists()
