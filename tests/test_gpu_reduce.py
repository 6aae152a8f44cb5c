"""Ping parity: rtacx_reduce against the FP64 oracle at <= 1e-5 relative L2
(the plain form's tolerance), plus size-independent properties at the
benchmark's full sizes."""
import numpy as np
import pytest

from rtac_simulation_gb300 import workloads as wl

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():
    pytest.skip("needs a GPU", allow_module_level=True)

from helpers_gpu import to_device, gpu_reduce, make_context, rel_l2  # noqa: E402

TOL = 1e-5


@pytest.mark.parametrize("maker", [
    lambda: wl.echosounder_1d(),
    lambda: wl.ea400_reference_1d(),
    lambda: wl.oculus_reference_2d(),
    lambda: wl.oculus_2d(n_samples=1 << 16),
    lambda: wl.oculus_2d(n_samples=1 << 14, n_bearings=100, n_ranges=300),
    lambda: wl.precision_2d(n_samples=1 << 13, n_ranges=1024),
])
def test_reduce_matches_fp64_oracle(oracle, maker):
    wk = maker()
    ctx = make_context(wk)
    got = gpu_reduce(ctx, wk.samples, wk.out_shape)
    want = oracle.reduce(wk.samples, wk.sensor)
    assert np.isfinite(got).all()
    err = rel_l2(got, want)
    assert err <= TOL, err


@pytest.mark.parametrize("maker", [
    lambda: wl.oculus_reference_2d(),
    lambda: wl.oculus_2d(n_samples=1 << 18),
    lambda: wl.oculus_2d(n_samples=1 << 14, n_bearings=100, n_ranges=300),
    lambda: wl.precision_2d(n_samples=1 << 16, n_ranges=1024),
    lambda: wl.stress_2d(n_samples=1 << 18, n_ranges=2048),
])
def test_tensor_core_gather_matches_simt_gather(oracle, maker):
    """The default 2D gather forms the sample x PSF outer products on the
    tensor cores (TF32 hi / lo operands, three products, FP32 accumulation);
    RTACX_FLAG_SIMT_GATHER selects the FP32 CUDA-core gather. Both meet the
    FP64 oracle's bar, and they agree to float round-off (their sums run in
    different orders)."""
    from rtac_simulation_gb300 import _lib
    wk = maker()
    tc = gpu_reduce(make_context(wk), wk.samples, wk.out_shape)
    simt = gpu_reduce(make_context(wk, flags=_lib.RTACX_FLAG_SIMT_GATHER), wk.samples, wk.out_shape)
    want = oracle.reduce(wk.samples, wk.sensor)
    assert np.isfinite(tc).all()
    assert rel_l2(tc, want) <= TOL, rel_l2(tc, want)
    assert rel_l2(simt, want) <= TOL
    assert rel_l2(tc, simt) <= 5e-6, rel_l2(tc, simt)


def test_reduce_1d_literal_scaling(oracle):
    wk = wl.ea400_reference_1d()
    ctx = make_context(wk, flags=1)
    got = gpu_reduce(ctx, wk.samples, wk.out_shape)
    want = oracle.reduce(wk.samples, wk.sensor, literal_1d=True)
    assert rel_l2(got, want) <= TOL


def test_reduce_zero_cases(oracle):
    wk = wl.oculus_reference_2d(n_samples=3)
    R = wl.linspace(wk.sensor["range_min"], wk.sensor["range_max"], wk.sensor["range_count"])
    wk.samples[:, 2] = R[50]            # one non-empty bin: every window is empty
    ctx = make_context(wk)
    assert np.all(gpu_reduce(ctx, wk.samples, wk.out_shape) == 0)
    assert np.all(gpu_reduce(ctx, wk.samples[:0], wk.out_shape) == 0)



def test_contexts_of_different_shapes_interleave(oracle):
    # Kernel launch limits (dynamic shared memory) are per kernel and device,
    # shared by every context: configuring a smaller sensor after a larger one
    # must leave the larger context's launches valid.
    big = wl.oculus_2d(n_samples=1 << 16)
    small = wl.oculus_2d(n_samples=1 << 12, n_bearings=64, n_ranges=128)
    cb = make_context(big)
    cs = make_context(small)
    got_s = gpu_reduce(cs, small.samples, small.out_shape)
    got_b = gpu_reduce(cb, big.samples, big.out_shape)
    assert rel_l2(got_b, oracle.reduce(big.samples, big.sensor)) <= TOL
    assert rel_l2(got_s, oracle.reduce(small.samples, small.sensor)) <= TOL

def test_reduce_unaligned_matches_aligned():
    wk = wl.oculus_reference_2d(n_samples=5000)
    ctx = make_context(wk)
    a = gpu_reduce(ctx, wk.samples, wk.out_shape)
    b = gpu_reduce(ctx, wk.samples, wk.out_shape, offset_floats=1)
    assert rel_l2(b, a) <= 1e-6


def test_reduce_rejects_misaligned_ping():
    """A ping pointer that is only 4-byte aligned is refused with a status
    before any launch (the gathers store whole complex64 cells)."""
    from rtac_simulation_gb300 import _lib
    wk = wl.oculus_reference_2d(n_samples=64)
    ctx = make_context(wk)
    d = to_device(wk.samples)
    buf = torch.zeros(2 * wk.out_shape[0] * wk.out_shape[1] + 2, dtype=torch.float32, device="cuda")
    lib = _lib.load()
    st = lib.rtacx_reduce(ctx.handle, d.data_ptr(), wk.n, buf.data_ptr() + 4, None)
    assert st == _lib.RTACX_ERR_INVALID_ARGUMENT
    assert "aligned" in ctx.last_error()
    assert torch.count_nonzero(buf).item() == 0


def test_full_size_rows_match_oracle(oracle):
    # 2^24-sample, 512 x 4096 dense-directivity ping: every row's window holds
    # ~2.7e5 samples; check a band of rows against the FP64 oracle.
    wk = wl.precision_2d()
    ctx = make_context(wk)
    got = gpu_reduce(ctx, wk.samples, wk.out_shape)
    rows = (2000, 2008)
    want = oracle.reduce(wk.samples, wk.sensor, rows=rows)
    assert rel_l2(got[rows[0]:rows[1]], want) <= TOL


def test_full_size_properties():
    wk = wl.oculus_2d()
    ctx = make_context(wk)
    base = gpu_reduce(ctx, wk.samples, wk.out_shape)
    # Permutation invariance: the caller's sample order does not matter.
    perm = np.random.default_rng(7).permutation(wk.n)
    assert rel_l2(gpu_reduce(ctx, wk.samples[perm], wk.out_shape), base) <= 1e-6
    # Linearity in the sample values.
    scaled = wk.samples.copy()
    scaled[:, :2] *= np.float32(-0.5)
    assert rel_l2(gpu_reduce(ctx, scaled, wk.out_shape), -0.5 * base) <= 1e-6
    # Repeated calls on the same context are stable.
    assert rel_l2(gpu_reduce(ctx, wk.samples, wk.out_shape, repeat=3), base) <= 1e-6
