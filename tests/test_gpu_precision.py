"""Precision (tensor-core) form against the FP64 oracle of the binned model
at <= 1e-4 relative L2, the FP64 echo pre-step of the plain form at 1e-5, and
the binned model against the per-sample PSF of the plain form at <= 1e-2."""
import numpy as np
import pytest

from rtac_simulation_gb300 import workloads as wl

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():
    pytest.skip("needs a GPU", allow_module_level=True)

from helpers_gpu import gpu_reduce, make_context, rel_l2, to_device  # noqa: E402

TOL = 1e-4


def gpu_precision(ctx, samples, out_shape):
    d = to_device(samples)
    out = torch.full(tuple(out_shape) + (2,), float("nan"), dtype=torch.float32, device="cuda")
    stream = torch.cuda.current_stream()
    ctx.reduce_precision(d, samples.shape[0], out, stream=stream)
    ctx.stream_status(stream)
    o = out.cpu().numpy()
    return o[..., 0].astype(np.float64) + 1j * o[..., 1]


def tables(wk, **kw):
    """The workload's precision configuration (its steered complex
    directivity where it has one)."""
    return wl.precision_tables(wk.sensor, **{**wk.precision, **kw})


def precision_context(wk, explicit=True, flags=0):
    ctx = make_context(wk)
    if wk.echo:
        ctx.set_echo_model(wk.echo["carrier_hz"], wk.echo["flags"])
    if explicit:
        ctx.configure_precision(**tables(wk), flags=flags)
    else:
        ctx.configure_precision(flags=flags)
    return ctx


@pytest.mark.parametrize("maker", [
    lambda: wl.precision_2d(n_samples=1 << 16, n_bearings=128, n_ranges=512),
    lambda: wl.precision_2d(n_samples=1 << 18, n_ranges=1024),
    lambda: wl.precision_2d(n_samples=1 << 14, n_bearings=100, n_ranges=300),
    lambda: wl.oculus_2d(n_samples=1 << 16, n_ranges=256, n_bearings=256),
])
def test_precision_matches_binned_fp64_oracle(oracle, maker):
    wk = maker()
    ctx = precision_context(wk)
    got = gpu_precision(ctx, wk.samples, wk.out_shape)
    tab = tables(wk)
    smp = oracle.apply_echo(wk.samples, wk.sensor, wk.echo)
    want = oracle.reduce_binned(smp, wk.sensor, tab)
    assert np.isfinite(got).all()
    err = rel_l2(got, want)
    assert err <= TOL, err



def test_precision_contexts_of_different_shapes_interleave(oracle):
    # A second, smaller precision context configured after the first must not
    # shrink the first one's per-kernel shared-memory limits.
    big = wl.precision_2d(n_samples=1 << 16, n_ranges=1024)
    small = wl.precision_2d(n_samples=1 << 12, n_bearings=100, n_ranges=300)
    cb = precision_context(big)
    cs = precision_context(small)
    for wk, ctx in ((small, cs), (big, cb)):
        got = gpu_precision(ctx, wk.samples, wk.out_shape)
        tab = tables(wk)
        want = oracle.reduce_binned(oracle.apply_echo(wk.samples, wk.sensor, wk.echo), wk.sensor, tab)
        assert rel_l2(got, want) <= TOL

def test_precision_full_size_every_row(oracle):
    """The headline ping (2^24 samples, 512 x 4096) against the FP64 oracle
    of the binned model on every one of its 4096 rows, as a whole and row by
    row (the worst row within 10x the bar)."""
    wk = wl.precision_2d()
    ctx = precision_context(wk)
    got = gpu_precision(ctx, wk.samples, wk.out_shape)
    tab = tables(wk)
    smp = oracle.apply_echo(wk.samples, wk.sensor, wk.echo)
    want = oracle.reduce_binned(smp, wk.sensor, tab)
    assert np.isfinite(got).all()
    assert rel_l2(got, want) <= TOL
    norms = np.linalg.norm(want, axis=1)
    live = norms > 1e-6 * norms.max()
    per_row = np.linalg.norm(got - want, axis=1)[live] / norms[live]
    assert per_row.max() <= 10 * TOL, per_row.max()


def test_precision_derived_tables_match_explicit():
    wk = wl.precision_2d(n_samples=1 << 15, n_bearings=128, n_ranges=512)
    wk.precision = {}                  # the library derives the real (unsteered) directivity
    a = gpu_precision(precision_context(wk, explicit=True), wk.samples, wk.out_shape)
    b = gpu_precision(precision_context(wk, explicit=False), wk.samples, wk.out_shape)
    assert rel_l2(b, a) <= 1e-6


def test_precision_unaligned_shape_uses_copy_out(oracle):
    wk = wl.precision_2d(n_samples=1 << 14, n_bearings=77, n_ranges=130)
    ctx = precision_context(wk)
    got = gpu_precision(ctx, wk.samples, wk.out_shape)
    tab = tables(wk)
    want = oracle.reduce_binned(oracle.apply_echo(wk.samples, wk.sensor, wk.echo), wk.sensor, tab)
    assert rel_l2(got, want) <= TOL


def test_plain_form_with_fp64_echo(oracle):
    wk = wl.precision_2d(n_samples=1 << 14, n_ranges=1024)
    ctx = make_context(wk)
    ctx.set_echo_model(wk.echo["carrier_hz"], wk.echo["flags"])
    got = gpu_reduce(ctx, wk.samples, wk.out_shape)
    want = oracle.reduce(oracle.apply_echo(wk.samples, wk.sensor, wk.echo), wk.sensor)
    assert rel_l2(got, want) <= 1e-5


@pytest.mark.parametrize("form", ["plain", "precision"])
def test_compensated_phase_matches_fp64_oracle(oracle, form):
    # RTACX_ECHO_PHASE_COMPENSATED reduces the carrier phase without FP64;
    # the FP64 oracle must not tell the difference.
    wk = wl.precision_2d(n_samples=1 << 16, n_ranges=1024)
    flags = wk.echo["flags"] | 4
    exact = oracle.apply_echo(wk.samples, wk.sensor, wk.echo)
    if form == "plain":
        ctx = make_context(wk)
        ctx.set_echo_model(wk.echo["carrier_hz"], flags)
        got = gpu_reduce(ctx, wk.samples, wk.out_shape)
        assert rel_l2(got, oracle.reduce(exact, wk.sensor)) <= 1e-5
    else:
        ctx = make_context(wk)
        ctx.set_echo_model(wk.echo["carrier_hz"], flags)
        tab = tables(wk)
        ctx.configure_precision(**tab)
        got = gpu_precision(ctx, wk.samples, wk.out_shape)
        assert rel_l2(got, oracle.reduce_binned(exact, wk.sensor, tab)) <= TOL


def gpu_precision_host(ctx, samples, out_shape, pinned=True):
    """The host-buffer entry point: pinned host samples in, host ping out."""
    h = torch.from_numpy(np.ascontiguousarray(samples, dtype=np.float32))
    if pinned:
        h = h.pin_memory()
    out = torch.full(tuple(out_shape) + (2,), float("nan"), dtype=torch.float32)
    if pinned:
        out = out.pin_memory()
    stream = torch.cuda.current_stream()
    ctx.reduce_precision_host(h, samples.shape[0], out, stream=stream)
    ctx.stream_status(stream)
    o = out.numpy()
    return o[..., 0].astype(np.float64) + 1j * o[..., 1]


@pytest.mark.parametrize("n", [0, 1000, (1 << 21) + 17, 5 * (1 << 20) + 3])
def test_precision_host_entry_matches_device_entry(oracle, n):
    """Chunked, copy-overlapped host entry point (1 to 3 staging chunks and
    the empty ping) gives the device entry point's ping."""
    wk = wl.precision_2d(n_samples=max(n, 1), n_bearings=128, n_ranges=512)
    smp = wk.samples[:n]
    ctx = precision_context(wk)
    dev = gpu_precision(ctx, smp, wk.out_shape)
    host = gpu_precision_host(ctx, smp, wk.out_shape)
    assert np.isfinite(host).all()
    if n == 0:
        assert np.all(host == 0) and np.all(dev == 0)
        return
    # Same arithmetic; only the order of the float atomics differs (as between
    # two device runs), which moves the ping by ~1e-6 relative at 5M samples.
    assert rel_l2(host, dev) <= 1e-5
    if n <= 1 << 21:
        tab = tables(wk)
        want = oracle.reduce_binned(oracle.apply_echo(smp, wk.sensor, wk.echo), wk.sensor, tab)
        assert rel_l2(host, want) <= TOL


def test_precision_host_entry_pageable_memory():
    wk = wl.precision_2d(n_samples=1 << 16, n_bearings=128, n_ranges=512)
    ctx = precision_context(wk)
    a = gpu_precision(ctx, wk.samples, wk.out_shape)
    b = gpu_precision_host(ctx, wk.samples, wk.out_shape, pinned=False)
    assert rel_l2(b, a) <= 1e-6


@pytest.mark.parametrize("maker", [
    lambda: wl.precision_2d(n_samples=1 << 16, n_bearings=128, n_ranges=512),
    lambda: wl.precision_2d(n_samples=1 << 14, n_bearings=100, n_ranges=300),
    lambda: wl.oculus_2d(n_samples=1 << 16, n_ranges=256, n_bearings=256),
])
def test_precision_fp16_rowscale_matches_binned_fp64_oracle(oracle, maker):
    """FP16 operands with per-row / per-column power-of-two scaling: 22-bit
    split halves, so the error sits at the FP32 accumulation level, below
    the BF16 split's."""
    from rtac_simulation_gb300 import _lib
    wk = maker()
    tab = tables(wk)
    want = oracle.reduce_binned(oracle.apply_echo(wk.samples, wk.sensor, wk.echo), wk.sensor, tab)
    got16 = gpu_precision(precision_context(wk, flags=_lib.RTACX_PRECISION_FP16_ROWSCALE), wk.samples, wk.out_shape)
    gotbf = gpu_precision(precision_context(wk), wk.samples, wk.out_shape)
    assert np.isfinite(got16).all()
    e16, ebf = rel_l2(got16, want), rel_l2(gotbf, want)
    assert e16 <= TOL, e16
    assert e16 <= ebf * 1.01, (e16, ebf)


def test_precision_fp16_rowscale_wide_dynamic_range(oracle):
    """Rows whose magnitudes differ by ~2^40 (amplitudes scaled per range):
    the per-row scale keeps every row inside the FP16 range."""
    from rtac_simulation_gb300 import _lib
    wk = wl.precision_2d(n_samples=1 << 15, n_bearings=128, n_ranges=512)
    smp = wk.samples.copy()
    t = smp[:, 2]
    scale = np.exp2(40.0 * (t - t.min()) / (t.max() - t.min()) - 20.0).astype(np.float32)
    smp[:, 0] *= scale
    smp[:, 1] *= scale
    tab = tables(wk)
    want = oracle.reduce_binned(oracle.apply_echo(smp, wk.sensor, wk.echo), wk.sensor, tab)
    got = gpu_precision(precision_context(wk, flags=_lib.RTACX_PRECISION_FP16_ROWSCALE), smp, wk.out_shape)
    assert np.isfinite(got).all()
    # per-row relative error, so that the small rows count as much as the large ones
    rows = np.linalg.norm(want, axis=1) > 0
    rel = np.linalg.norm(got - want, axis=1)[rows] / np.linalg.norm(want, axis=1)[rows]
    assert np.median(rel) <= TOL and np.percentile(rel, 99) <= 10 * TOL, (np.median(rel), np.percentile(rel, 99))


@pytest.mark.parametrize("flags", [0, 1])
def test_precision_long_pulse_multi_chunk_filter(oracle, flags):
    """101 range taps: the range filter stages its taps in several chunks."""
    wk = wl.precision_2d(n_samples=1 << 15, n_bearings=128, n_ranges=512, taps=101)
    tab = tables(wk)
    assert tab["range_taps"].shape[1] > 64            # taps per output-row parity
    want = oracle.reduce_binned(oracle.apply_echo(wk.samples, wk.sensor, wk.echo), wk.sensor, tab)
    got = gpu_precision(precision_context(wk, flags=flags), wk.samples, wk.out_shape)
    assert rel_l2(got, want) <= TOL


def test_precision_host_entry_graph_capture():
    """rtacx_reduce_precision_host is stream-ordered with its copy stream
    fork-joined by events, so it can be captured in a CUDA graph and replayed."""
    wk = wl.precision_2d(n_samples=(1 << 21) + 5, n_bearings=128, n_ranges=512)
    ctx = precision_context(wk)
    n = wk.samples.shape[0]
    h = torch.from_numpy(np.ascontiguousarray(wk.samples, dtype=np.float32)).pin_memory()
    out = torch.zeros(tuple(wk.out_shape) + (2,), dtype=torch.float32).pin_memory()
    s = torch.cuda.Stream()
    with torch.cuda.stream(s):
        ctx.reduce_precision_host(h, n, out, stream=s)     # first call allocates the staging buffers
    torch.cuda.synchronize()
    ctx.stream_status(s)
    ref = out.clone()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g, stream=s):
        ctx.reduce_precision_host(h, n, out, stream=s)
    out.fill_(float("nan"))
    torch.cuda.synchronize()
    g.replay()
    torch.cuda.synchronize()
    ctx.stream_status(s)
    a, b = out.numpy(), ref.numpy()
    assert np.isfinite(a).all()
    assert rel_l2(a[..., 0] + 1j * a[..., 1], b[..., 0] + 1j * b[..., 1]) <= 1e-5


def _small_precision():
    return wl.precision_2d(n_samples=1 << 12, n_bearings=128, n_ranges=512)


def _bin_travel(oracle, sensor, r):
    """A travel whose reference key is range bin r."""
    t = np.float32(sensor["range_min"] + r * float(wl.linspace_resolution(sensor["range_min"], sensor["range_max"],
                                                                           sensor["range_count"])))
    keys, _ = oracle.range_keys(sensor["range_count"], sensor["range_min"], sensor["range_max"], sensor["margin"],
                                np.array([t], np.float32))
    assert keys[0] == r
    return t


def test_precision_all_out_of_range_and_single_bin_are_zero(oracle):
    """No in-range sample, or samples in one range bin only: every window is
    the reference's empty view, so the ping is zero (src/Binner.cu:90-102)."""
    wk = _small_precision()
    ctx = precision_context(wk)
    smp = wk.samples.copy()
    smp[:, 2] = np.float32(1e4)                      # above the range
    assert np.all(gpu_precision(ctx, smp, wk.out_shape) == 0)
    smp[:, 2] = _bin_travel(oracle, wk.sensor, 200)   # all in bin 200
    assert np.all(gpu_precision(ctx, smp, wk.out_shape) == 0)


def test_precision_zero_amplitude_samples_open_windows(oracle):
    """A zero-amplitude sample still makes its bin non-empty: bins 200 + 201
    give non-empty windows, bin 200 alone gives the empty view."""
    wk = _small_precision()
    ctx = precision_context(wk)
    tab = tables(wk)
    smp = wk.samples[:64].copy()
    smp[:, 2] = _bin_travel(oracle, wk.sensor, 200)
    zero = smp[:8].copy()
    zero[:, 0] = 0.0
    zero[:, 1] = 0.0
    zero[:, 2] = _bin_travel(oracle, wk.sensor, 201)
    both = np.concatenate([smp, zero])
    got = gpu_precision(ctx, both, wk.out_shape)
    want = oracle.reduce_binned(oracle.apply_echo(both, wk.sensor, wk.echo), wk.sensor, tab)
    assert np.linalg.norm(want) > 0
    assert rel_l2(got, want) <= TOL
    assert np.all(gpu_precision(ctx, smp, wk.out_shape) == 0)


def test_precision_degenerate_bearings_match_oracle(oracle):
    """Out-of-grid bearings clamp to the grid's end bearings; NaN and
    infinite bearings contribute nothing (their bins still count as
    non-empty), in the kernel as in the oracle."""
    wk = _small_precision()
    ctx = precision_context(wk)
    tab = tables(wk)
    smp = wk.samples.copy()
    bad = np.array([np.nan, np.inf, -np.inf, 3.0, -3.0, 1e30], np.float32)
    smp[:bad.size * 64, 3] = np.repeat(bad, 64)
    got = gpu_precision(ctx, smp, wk.out_shape)
    want = oracle.reduce_binned(oracle.apply_echo(smp, wk.sensor, wk.echo), wk.sensor, tab)
    assert np.isfinite(got).all()
    assert rel_l2(got, want) <= TOL


@pytest.mark.parametrize("grid", [None, (768, -1.3, 1.25), (130, 0.0, 0.0)])
def test_precision_grid_edges(oracle, grid):
    """Samples exactly on grid bearings and one ulp below them, outside the
    grid (clamped to its end bearings), on the default grid and on explicit
    ones (a grid wider than the fan, a coarse one), against the oracle's
    restatement of the same float arithmetic."""
    wk = wl.precision_2d(n_samples=1 << 14, n_bearings=128, n_ranges=512)
    kw = {} if grid is None else dict(grid_count=grid[0], grid_first=grid[1], grid_last=grid[2])
    if grid is not None and grid[1] == grid[2]:
        kw = dict(grid_count=grid[0])
    tab = tables(wk, **kw)
    g = wl.grid_points(tab["grid_first"], tab["grid_last"], tab["grid_count"])
    smp = wk.samples.copy()
    on = g[np.arange(smp.shape[0] // 4) % g.size]
    smp[:on.size, 3] = on
    smp[on.size:2 * on.size, 3] = np.nextafter(on, np.float32(-np.inf))
    smp[2 * on.size:2 * on.size + 64, 3] = np.float32(1.5)      # beyond the last grid bearing
    ctx = make_context(wk)
    ctx.set_echo_model(wk.echo["carrier_hz"], wk.echo["flags"])
    ctx.configure_precision(**tab)
    got = gpu_precision(ctx, smp, wk.out_shape)
    want = oracle.reduce_binned(oracle.apply_echo(smp, wk.sensor, wk.echo), wk.sensor, tab)
    assert np.isfinite(got).all()
    assert rel_l2(got, want) <= TOL


@pytest.mark.parametrize("n", [(1 << 14) + 7, 1000, 1])
def test_precision_partial_stage_and_unaligned_records(oracle, n):
    """The staged accumulation copies the samples in stages of 1024 records:
    a ping whose last stage is partial (or that is shorter than one stage)
    matches the oracle, and the same samples at an address that is not
    16-byte aligned (accumulated by the general kernel) give the same ping."""
    wk = wl.precision_2d(n_samples=n, n_bearings=128, n_ranges=512)
    ctx = precision_context(wk)
    tab = tables(wk)
    got = gpu_precision(ctx, wk.samples, wk.out_shape)
    want = oracle.reduce_binned(oracle.apply_echo(wk.samples, wk.sensor, wk.echo), wk.sensor, tab)
    assert np.isfinite(got).all()
    assert rel_l2(got, want) <= TOL
    d = to_device(wk.samples, offset_floats=1)
    out = torch.empty(tuple(wk.out_shape) + (2,), dtype=torch.float32, device="cuda")
    stream = torch.cuda.current_stream()
    ctx.reduce_precision(d, n, out, stream=stream)
    ctx.stream_status(stream)
    o = out.cpu().numpy()
    assert rel_l2(o[..., 0] + 1j * o[..., 1], got) <= 1e-6


def test_precision_consecutive_pings_start_from_a_zero_grid(oracle):
    """Each ping starts from a zeroed binned grid: pings of different samples
    on one context, on the caller's stream and on a second stream, each match
    their own oracle."""
    wk_a = wl.precision_2d(n_samples=1 << 15, n_bearings=128, n_ranges=512, seed=5)
    wk_b = wl.precision_2d(n_samples=1 << 14, n_bearings=128, n_ranges=512, seed=6)
    ctx = precision_context(wk_a)
    tab = tables(wk_a)
    want = {id(w): oracle.reduce_binned(oracle.apply_echo(w.samples, w.sensor, w.echo), w.sensor, tab)
            for w in (wk_a, wk_b)}
    side = torch.cuda.Stream()
    for w, stream in ((wk_a, None), (wk_b, None), (wk_a, side), (wk_b, side), (wk_a, None)):
        d = to_device(w.samples)
        out = torch.empty(tuple(w.out_shape) + (2,), dtype=torch.float32, device="cuda")
        s = stream if stream is not None else torch.cuda.current_stream()
        s.wait_stream(torch.cuda.current_stream())
        ctx.reduce_precision(d, w.samples.shape[0], out, stream=s)
        ctx.stream_status(s)
        o = out.cpu().numpy()
        assert rel_l2(o[..., 0] + 1j * o[..., 1], want[id(w)]) <= TOL


def _random_phase(D, seed=21):
    """D with an independent uniform phase per entry: a complex directivity
    with no structure the contraction could lean on."""
    rng = np.random.default_rng(seed)
    return (D * np.exp(2j * np.pi * rng.random(D.shape))).astype(np.complex64)


@pytest.mark.parametrize("fp16", [False, True])
@pytest.mark.parametrize("kind", ["steered", "random_phase"])
def test_precision_complex_directivity(oracle, fp16, kind):
    """Im D != 0 through both contraction forms: the {dr, -di}, {di, dr}
    layout of the directivity operand (and the FP16 column scales over the
    imaginary rows) against the FP64 oracle of the binned model."""
    from rtac_simulation_gb300 import _lib
    wk = wl.precision_2d(n_samples=1 << 18, n_ranges=1024)
    tab = tables(wk)
    if kind == "random_phase":
        tab["directivity"] = _random_phase(tab["directivity"])
    assert np.abs(tab["directivity"].imag).max() > 0.03
    flags = _lib.RTACX_PRECISION_FP16_ROWSCALE if fp16 else 0
    ctx = make_context(wk)
    ctx.set_echo_model(wk.echo["carrier_hz"], wk.echo["flags"])
    ctx.configure_precision(**tab, flags=flags)
    got = gpu_precision(ctx, wk.samples, wk.out_shape)
    want = oracle.reduce_binned(oracle.apply_echo(wk.samples, wk.sensor, wk.echo), wk.sensor, tab)
    assert np.isfinite(got).all()
    err = rel_l2(got, want)
    assert err <= TOL, err
    # The real-directivity ping differs: the imaginary half is really used.
    ctx.configure_precision(**{**tab, "directivity": tab["directivity"].real.astype(np.complex64)}, flags=flags)
    assert rel_l2(gpu_precision(ctx, wk.samples, wk.out_shape), want) > 100 * TOL


@pytest.mark.parametrize("fp16", [False, True])
def test_precision_complex_directivity_full_size(oracle, fp16):
    """The headline ping (2^24 samples, 512 x 4096, steered complex
    directivity on a 2048-bearing grid) through the FP16 per-row-scaled
    contraction and again through the BF16 one, against the binned FP64
    oracle on every row."""
    from rtac_simulation_gb300 import _lib
    wk = wl.precision_2d()
    tab = tables(wk)
    ctx = make_context(wk)
    ctx.set_echo_model(wk.echo["carrier_hz"], wk.echo["flags"])
    ctx.configure_precision(**tab, flags=_lib.RTACX_PRECISION_FP16_ROWSCALE if fp16 else 0)
    got = gpu_precision(ctx, wk.samples, wk.out_shape)
    smp = oracle.apply_echo(wk.samples, wk.sensor, wk.echo)
    want = oracle.reduce_binned(smp, wk.sensor, tab)
    assert rel_l2(got, want) <= TOL


def per_sample_ping(ctx_plain, wk, steer):
    """The plain form's per-sample ping with the steering phase of the
    precision workload's directivity (samples rotated by exp(i kappa sin
    theta_s), the ping by exp(-i kappa sin theta_b))."""
    got = gpu_reduce(ctx_plain, wl.steer_samples(wk.samples, steer), wk.out_shape)
    return wl.steer_ping(got, wk.sensor["bearings"], steer)


@pytest.mark.parametrize("n_ranges", [1024, 4096])
def test_precision_model_close_to_per_sample_psf(n_ranges):
    """The binned model against the reference's per-sample PSF (the plain
    form, itself within 1e-5 of the FP64 oracle) on the same ping: range
    nodes two bins apart with the projected taps and the bearing grid of
    four cells per output bearing with the projected directivity leave about
    6e-3 to 7e-3 relative L2 (bar: 1e-2)."""
    wk = wl.precision_2d(n_samples=1 << 18, n_ranges=n_ranges)
    prec = gpu_precision(precision_context(wk), wk.samples, wk.out_shape)
    plain_ctx = make_context(wk)
    plain_ctx.set_echo_model(wk.echo["carrier_hz"], wk.echo["flags"])
    plain = per_sample_ping(plain_ctx, wk, wk.precision["steer"])
    diff = rel_l2(prec, plain)
    print(f"binned vs per-sample model ({n_ranges} ranges): rel-L2 {diff:.3e}")
    assert diff <= 1e-2, diff
