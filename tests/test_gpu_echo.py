"""Echo-sample epilogue and receiver directivity tables on the device.

rtacx_directivity_table is compared with the tables the reference's own
src/Directivity.cpp builds (tests/golden/ref_directivity.json);
rtacx_make_samples with the oracle's FP64 restatement of the ray generator's
and receiver's per-hit arithmetic."""
import json
from pathlib import Path

import numpy as np
import pytest

from rtac_simulation_gb300 import _lib
from rtac_simulation_gb300 import workloads as wl

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():
    pytest.skip("needs a GPU", allow_module_level=True)

from helpers_gpu import make_context, rel_l2  # noqa: E402

GOLDEN = Path(__file__).resolve().parent / "golden" / "ref_directivity.json"


@pytest.mark.parametrize("case", range(4))
def test_directivity_tables_match_reference(case):
    c = json.loads(GOLDEN.read_text())["cases"][case]
    par = [float.fromhex(x) for x in c["params"]]
    baffle = 1.0 if c["baffle"] == "single-sided" else 0.0
    if c["kind"] == "RECT":
        tab = _lib.directivity_table(_lib.RTACX_DIRECTIVITY_RECTANGLE, par + [baffle, float(c["oversampling"])])
    else:
        tab = _lib.directivity_table(_lib.RTACX_DIRECTIVITY_DISK, par + [baffle, float(c["oversampling"])])
    got = tab.cpu().numpy()
    assert got.shape == (c["height"], c["width"])
    want = np.array([float.fromhex(x) for x in c["values"]], np.float32).reshape(c["height"], c["width"])
    # disk_antenna takes sqrt(1 - y2 - z2) where the terms cancel (and 0/0 at
    # elevation = bearing = pi/2): the reference table holds NaNs whose
    # positions depend on the host libm's last bit. The device builder keeps
    # the exact-math limit there, 0.
    assert np.isfinite(got).all()
    want = np.where(np.isnan(want), np.float32(0.0), want)
    assert np.max(np.abs(got - want)) <= 2e-6


def random_hits(n, seed):
    rng = np.random.default_rng(seed)
    az = rng.uniform(-1.3, 1.3, n)
    el = rng.uniform(-0.4, 0.4, n)
    d = np.stack([np.cos(el) * np.cos(az), np.cos(el) * np.sin(az), np.sin(el)], axis=1)
    hits = np.empty((n, 6), np.float32)
    hits[:, 0] = rng.normal(size=n)
    hits[:, 1] = rng.normal(size=n)
    hits[:, 2] = rng.uniform(0.2, 6.0, n)
    hits[: n // 50, 2] = rng.uniform(0.0, 9e-5, n // 50)      # misses / too close: null samples
    hits[:, 3:] = d
    return hits


def rotation(seed):
    rng = np.random.default_rng(seed)
    q, _ = np.linalg.qr(rng.normal(size=(3, 3)))
    return (q * np.sign(np.linalg.det(q))).astype(np.float32)


@pytest.mark.parametrize("maker,dims", [(wl.oculus_reference_2d, 2), (wl.ea400_reference_1d, 1)])
def test_make_samples_matches_oracle(oracle, maker, dims):
    wk = maker(n_samples=16)
    ctx = make_context(wk)
    table = _lib.directivity_table(_lib.RTACX_DIRECTIVITY_RECTANGLE, [1.56e-3, 8e-3, 1.25e-3, 1.0, 8.0]).cpu().numpy()
    R = rotation(3)
    ctx.configure_receiver(R, table, carrier_hz=1.2e6, flags=3)
    hits = random_hits(100000, 5)
    d_hits = torch.from_numpy(hits.reshape(-1)).cuda()
    out = torch.full((hits.shape[0], 4 if dims == 2 else 3), float("nan"), device="cuda")
    ctx.make_samples(d_hits, hits.shape[0], out, stream=torch.cuda.current_stream())
    ctx.stream_status(torch.cuda.current_stream())
    got = out.cpu().numpy()
    want = oracle.make_samples(hits, R, table, 1.2e6, wk.sensor["sound_celerity"], 3, dims)
    np.testing.assert_array_equal(got[:, 2], want[:, 2])                 # travel / null marker
    assert rel_l2(got[:, 0] + 1j * got[:, 1], want[:, 0] + 1j * want[:, 1]) <= 1e-5
    if dims == 2:
        assert np.max(np.abs(got[:, 3] - want[:, 3])) <= 2e-6
    null = hits[:, 2] < 1e-4
    assert np.all(got[null, 2] == -1.0) and np.all(got[null, :2] == 0.0)


def test_make_samples_then_reduce(oracle):
    # Device-produced samples feed the ping directly.
    wk = wl.oculus_reference_2d(n_samples=16)
    ctx = make_context(wk)
    ctx.configure_receiver(np.eye(3), None, carrier_hz=1.2e6, flags=3)
    hits = random_hits(50000, 9)
    d_hits = torch.from_numpy(hits.reshape(-1)).cuda()
    smp = torch.empty((hits.shape[0], 4), device="cuda")
    stream = torch.cuda.current_stream()
    ctx.make_samples(d_hits, hits.shape[0], smp, stream=stream)
    out = torch.empty(wk.out_shape + (2,), device="cuda")
    ctx.reduce(smp, hits.shape[0], out, stream=stream)
    ctx.stream_status(stream)
    want_smp = oracle.make_samples(hits, np.eye(3), None, 1.2e6, wk.sensor["sound_celerity"], 3, 2)
    want = oracle.reduce(want_smp, wk.sensor)
    o = out.cpu().numpy()
    assert rel_l2(o[..., 0] + 1j * o[..., 1], want) <= 2e-5
