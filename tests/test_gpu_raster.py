"""Rasterised echo samples (the GL ray caster's shader math on CUDA) against
the oracle's restatement: identical coverage (integer edge functions, top-left
rule, depth ties to the first triangle) and the fragment arithmetic within
float tolerance; then the samples feed a ping."""
import math

import numpy as np
import pytest

from rtac_simulation_gb300 import scene
from rtac_simulation_gb300 import workloads as wl

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():
    pytest.skip("needs a GPU", allow_module_level=True)

from helpers_gpu import make_context, rel_l2  # noqa: E402


def setup(width=256, height=192, yaw=0.15):
    V, N, T = scene.seafloor_and_sphere()
    R = np.array([[math.cos(yaw), 0, math.sin(yaw), 0], [0, 1, 0, 0], [-math.sin(yaw), 0, math.cos(yaw), 0], [0, 0, 0, 1]])
    L = R                                     # world -> local (rotation about y)
    S = scene.perspective(70.0, width / height, 0.1, 100.0) @ R
    return V, N, T, L.astype(np.float32), S.astype(np.float32), np.zeros(3, np.float32), width, height


@pytest.mark.parametrize("yaw", [0.0, 0.15, -0.4])
def test_raster_matches_oracle(oracle, yaw):
    V, N, T, L, S, o, W, H = setup(yaw=yaw)
    wk = wl.oculus_reference_2d(n_samples=16)
    ctx = make_context(wk)
    out = torch.full((H * W, 4), float("nan"), device="cuda")
    ctx.rasterize(torch.from_numpy(V).cuda(), torch.from_numpy(N).cuda(), torch.from_numpy(T.view(np.int32)).cuda(),
                  L, S, o, W, H, out, stream=torch.cuda.current_stream())
    ctx.stream_status(torch.cuda.current_stream())
    got = out.cpu().numpy()
    want, winner = oracle.rasterize(V, N, T, L, S, o, W, H)
    covered = winner >= 0
    assert covered.sum() > 0.3 * W * H
    np.testing.assert_array_equal(got[:, 2] > 0, covered)          # same coverage
    np.testing.assert_allclose(got[covered, 2], want[covered, 2], rtol=2e-6, atol=1e-6)   # range
    np.testing.assert_allclose(got[covered, 3], want[covered, 3], rtol=0, atol=2e-6)      # bearing
    assert rel_l2(got[:, 0] + 1j * got[:, 1], want[:, 0] + 1j * want[:, 1]) <= 1e-5
    assert np.all(got[~covered] == 0)


def test_rasterised_samples_make_a_ping(oracle):
    V, N, T, L, S, o, W, H = setup()
    # Oculus receiver re-ranged to the scene (1 .. 45 m) with its adaptive
    # pulse: a fixed pulse shorter than the range step would give binOverlap
    # 0 and, as in the reference, an all-empty ping.
    wk = wl.oculus_reference_2d(n_samples=16)
    rmin, rmax, c = 1.0, 45.0, 1500.0
    duration = wl.adaptive_duration(rmin, rmax, 500, c)
    wk.sensor.update(range_min=rmin, range_max=rmax, pulse_duration=float(duration),
                     margin=float(wl.F32(wl.F32(c) * duration)), pulse=wl.waveform_sine(1.2e6, float(duration), 8))
    assert oracle.bin_overlap(rmin, rmax, 500, wk.sensor["margin"]) >= 1
    ctx = make_context(wk)
    smp = torch.empty((H * W, 4), device="cuda")
    stream = torch.cuda.current_stream()
    ctx.rasterize(torch.from_numpy(V).cuda(), torch.from_numpy(N).cuda(), torch.from_numpy(T.view(np.int32)).cuda(),
                  L, S, o, W, H, smp, stream=stream)
    out = torch.empty(wk.out_shape + (2,), device="cuda")
    ctx.reduce(smp, H * W, out, stream=stream)
    ctx.stream_status(stream)
    want_smp, _ = oracle.rasterize(V, N, T, L, S, o, W, H)
    want = oracle.reduce(want_smp, wk.sensor)
    g = out.cpu().numpy()
    assert np.linalg.norm(want) > 0
    assert rel_l2(g[..., 0] + 1j * g[..., 1], want) <= 2e-5
