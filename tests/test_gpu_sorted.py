"""Sorted scratch of the counting sort (bit-exact): after rtacx_bin, every
in-range sample appears exactly once in the context's sorted scratch,
grouped by composite key (range bin x bearing sub-bins + bearing sub-bin) in
ascending order. Range keys come from the oracle's restatement of
Binner::Key; the bearing sub-bins from the oracle's restatement of the
device formula with the parameters the configuration derives."""
import numpy as np
import pytest

from rtac_simulation_gb300 import workloads as wl

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():
    pytest.skip("needs a GPU", allow_module_level=True)

from helpers_gpu import gpu_bin, make_context  # noqa: E402

KEY_OOR = np.uint32(0xFFFFFFFF)
MAX_SMEM_BINS = 49152


def bearing_subbins(sensor: dict):
    """Bearing sub-bin count, scale and offset as rtacx_configure_2d derives
    them: sub-bins while the beam support stays below a quarter of the fan."""
    b = np.asarray(sensor["bearings"], dtype=np.float32)
    W = len(sensor["beam"])
    sb = 0.5 * float(np.float32(sensor["beam_span"])) * (1.0 + 1.0 / W) * (1.0 + 1e-4) + 1e-6
    lo, hi = float(b.min()) - sb, float(b.max()) + sb
    nbb = 1
    if 4.0 * 2.0 * sb < hi - lo:
        while nbb < 32 and (hi - lo) / (2.0 * nbb) > sb and sensor["range_count"] * nbb * 2 <= MAX_SMEM_BINS:
            nbb *= 2
    if nbb == 1:
        return 1, np.float32(0.0), np.float32(0.0)
    flo, fhi = np.float32(lo), np.float32(hi)
    scale = np.float32(np.float32(nbb) / np.float32(fhi - flo))
    return nbb, scale, np.float32(-flo * scale)


def composite_keys(oracle, wk, records):
    s = wk.sensor
    rk, _ = oracle.range_keys(s["range_count"], s["range_min"], s["range_max"], s["margin"],
                              np.ascontiguousarray(records[:, 2]))
    rk = rk.astype(np.uint32)
    if wk.dims == 1:
        return rk
    nbb, scale, offset = bearing_subbins(s)
    if nbb == 1:
        return rk
    bb = oracle.bearing_bins(scale, offset, nbb, np.ascontiguousarray(records[:, 3]))
    return np.where(rk == KEY_OOR, KEY_OOR, rk * np.uint32(nbb) + bb).astype(np.uint32)


def record_hash(records: np.ndarray) -> np.ndarray:
    w = np.ascontiguousarray(records, dtype=np.float32).view(np.uint32).astype(np.uint64)
    x = w[:, 0] | (w[:, 1] << np.uint64(32))
    y = w[:, 2] | (w[:, 3] << np.uint64(32))
    h = x * np.uint64(0x9E3779B97F4A7C15) ^ y * np.uint64(0xC2B2AE3D27D4EB4F)
    h ^= h >> np.uint64(29)
    h *= np.uint64(0xBF58476D1CE4E5B9)
    return h ^ (h >> np.uint64(32))


def per_key_sums(keys, h, n_keys):
    """Exact per-key sums of the 64-bit hashes, as four 16-bit lanes."""
    return [np.bincount(keys, weights=((h >> np.uint64(16 * q)) & np.uint64(0xFFFF)).astype(np.float64),
                        minlength=n_keys) for q in range(4)]


def check_sorted(oracle, wk, exact_order: bool):
    ctx = make_context(wk)
    n = wk.samples.shape[0]
    got_bin = gpu_bin(ctx, wk.samples, wk.dims, wk.sensor["range_count"])
    recs = np.zeros((n, 4), dtype=np.float32)
    recs[:, :wk.samples.shape[1]] = wk.samples
    ck = composite_keys(oracle, wk, recs)
    inr = ck != KEY_OOR
    m = int(inr.sum())
    assert m == n - int(got_bin["oor"].sum())
    out = torch.empty((max(m, 1), 4), dtype=torch.float32, device="cuda")
    ctx.diag_sorted(out, m, stream=torch.cuda.current_stream())
    ctx.stream_status(torch.cuda.current_stream())
    got = out.cpu().numpy()[:m]
    ctx.close()
    gk = composite_keys(oracle, wk, got)
    assert not np.any(gk == KEY_OOR)
    assert np.all(gk[1:] >= gk[:-1]), "sorted scratch not grouped by ascending composite key"
    want_keys = ck[inr]
    n_keys = int(max(want_keys.max(initial=0), gk.max(initial=0))) + 1
    np.testing.assert_array_equal(np.bincount(gk, minlength=n_keys), np.bincount(want_keys, minlength=n_keys))
    for a, b in zip(per_key_sums(gk, record_hash(got), n_keys), per_key_sums(want_keys, record_hash(recs[inr]), n_keys)):
        np.testing.assert_array_equal(a, b)
    if exact_order:
        def canon(keys, r):
            u = np.ascontiguousarray(r).view(np.uint32)
            order = np.lexsort((u[:, 3], u[:, 2], u[:, 1], u[:, 0], keys))
            return keys[order], u[order]
        ka, ua = canon(gk, got)
        kb, ub = canon(want_keys, recs[inr])
        np.testing.assert_array_equal(ka, kb)
        np.testing.assert_array_equal(ua, ub)


@pytest.mark.parametrize("maker", [
    lambda: wl.echosounder_1d(),
    lambda: wl.oculus_reference_2d(),
    lambda: wl.oculus_2d(n_samples=1 << 20),
    lambda: wl.precision_2d(n_samples=1 << 20),
    lambda: wl.echosounder_1d(n_samples=1 << 20, n_ranges=8192),    # pipelined, reservations in two batches
    lambda: wl.precision_2d(n_samples=1 << 20, n_ranges=12000),     # pipelined, 16 bins per thread
    lambda: wl.oculus_2d(n_samples=1 << 18, n_ranges=512),     # 16384 bins: the unpipelined staged shape
    lambda: wl.oculus_2d(n_samples=1000),
])
def test_sorted_scratch_matches_oracle(oracle, maker):
    check_sorted(oracle, maker(), exact_order=True)


@pytest.mark.parametrize("maker", [lambda: wl.oculus_2d(n_samples=1 << 18),
                                   lambda: wl.precision_2d(n_samples=1 << 18)])
def test_sorted_scratch_hot_bins(oracle, maker):
    wk = maker()
    R = wl.linspace(wk.sensor["range_min"], wk.sensor["range_max"], wk.sensor["range_count"])
    wk.samples[: 1 << 16, 2] = R[100]          # one hot range bin: runs longer than a scatter tile
    wk.samples[-1000:, 2] = -1.0               # out of range
    check_sorted(oracle, wk, exact_order=True)


def test_sorted_scratch_full_size_precision_ping(oracle):
    check_sorted(oracle, wl.precision_2d(), exact_order=False)
