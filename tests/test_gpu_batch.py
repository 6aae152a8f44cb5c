"""Batched plain form (rtacx_batch_*): every ping of a heterogeneous batch
equals the single-ping path, and the single-ping path equals the oracle; the
fused form is one kernel in the graph, and its grid-barrier waits are
bounded (a barrier that cannot complete sets the batch status word and the
run stops without touching the pings)."""
import numpy as np
import pytest

from rtac_simulation_gb300 import _lib
from rtac_simulation_gb300 import workloads as wl

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():
    pytest.skip("needs a GPU", allow_module_level=True)

from helpers_gpu import gpu_reduce, make_context, rel_l2  # noqa: E402


def _complex(t):
    o = t.cpu().numpy()
    return o[..., 0].astype(np.float64) + 1j * o[..., 1]


def single_ping(wk):
    """The single-ping path with the batch's arithmetic: the FP32 CUDA-core
    gather (the batched kernel does not use the tensor-core one)."""
    flags = _lib.RTACX_FLAG_SIMT_GATHER if wk.dims == 2 else 0
    return gpu_reduce(make_context(wk, flags=flags), wk.samples, wk.out_shape)


@pytest.fixture(scope="module")
def batch_setup():
    pings = wl.batched_mix(n_pings=12, seed=11, log2_min=10, log2_max=15)
    ctxs, devs, outs = [], [], []
    for wk in pings:
        ctxs.append(make_context(wk))
        devs.append(torch.from_numpy(wk.samples.reshape(-1)).cuda())
        outs.append(torch.full(wk.out_shape + (2,), float("nan"), device="cuda"))
    return pings, ctxs, devs, outs


@pytest.mark.parametrize("staged", [False, True])
@pytest.mark.parametrize("autotune", [False, True])
def test_batch_equals_single_ping(batch_setup, autotune, staged):
    pings, ctxs, devs, outs = batch_setup
    batch = _lib.Batch(0)
    batch.plan([(c, d, wk.n, o) for wk, c, d, o in zip(pings, ctxs, devs, outs)], autotune=autotune,
               staged=staged)
    stream = torch.cuda.current_stream()
    for _ in range(2):
        for o in outs:
            o.fill_(float("nan"))
        batch.run(stream)
        batch.status(stream)
        torch.cuda.synchronize()
        for wk, o in zip(pings, outs):
            got = _complex(o)
            want = single_ping(wk)
            assert np.isfinite(got).all()
            assert rel_l2(got, want) <= 1e-6, wk.name
    t = batch.tuning()
    assert t["tile_rows"] in (16, 32) and t["tile_bearings"] in (64, 128)
    if autotune:
        assert t["tuned_ms"] > 0


def test_fused_batch_is_one_kernel(batch_setup):
    pings, ctxs, devs, outs = batch_setup
    batch = _lib.Batch(0)
    args = [(c, d, wk.n, o) for wk, c, d, o in zip(pings, ctxs, devs, outs)]
    batch.plan(args, autotune=False)
    assert batch.graph_kernels() == 1
    batch.plan(args, autotune=False, staged=True)
    assert batch.graph_kernels() == 7      # reset, zero, count, scan, scatter, windows, gather
    batch.close()


def test_fused_batch_barrier_wait_is_bounded(batch_setup):
    """The first grid barrier waits for one CTA more than the launch has:
    every CTA gives up after 100 ms, the status word reports it, no ping is
    written, and the next plan runs clean."""
    pings, ctxs, devs, outs = batch_setup
    batch = _lib.Batch(0)
    args = [(c, d, wk.n, o) for wk, c, d, o in zip(pings, ctxs, devs, outs)]
    stream = torch.cuda.current_stream()
    batch.diag_barrier(1, 100)
    batch.plan(args, autotune=False)
    for o in outs:
        o.fill_(float("nan"))
    batch.run(stream)
    with pytest.raises(_lib.RtacxError) as e:
        batch.status(stream)
    assert e.value.status == _lib.RTACX_ERR_DEVICE
    for o in outs:
        assert torch.isnan(o).all()
    batch.status(stream)                   # the word was cleared
    batch.diag_barrier(0, 1000)
    batch.plan(args, autotune=False)
    batch.run(stream)
    batch.status(stream)
    for wk, o in zip(pings, outs):
        assert rel_l2(_complex(o), single_ping(wk)) <= 1e-6, wk.name
    batch.close()


def test_batch_pings_match_oracle(batch_setup, oracle):
    pings, ctxs, devs, outs = batch_setup
    batch = _lib.Batch(0)
    batch.plan([(c, d, wk.n, o) for wk, c, d, o in zip(pings, ctxs, devs, outs)], autotune=False)
    batch.run(torch.cuda.current_stream())
    torch.cuda.synchronize()
    for wk, o in list(zip(pings, outs))[:4]:
        assert rel_l2(_complex(o), oracle.reduce(wk.samples, wk.sensor)) <= 1e-5, wk.name


def test_batch_rejects_shared_context(batch_setup):
    pings, ctxs, devs, outs = batch_setup
    batch = _lib.Batch(0)
    with pytest.raises(_lib.RtacxError):
        batch.plan([(ctxs[0], devs[0], pings[0].n, outs[0]), (ctxs[0], devs[0], pings[0].n, outs[0])])


def test_batch_full_size_mix(oracle):
    """The batched configuration at its size: 64 pings with log-uniform
    sample counts in [2^14, 2^22] (half 512-bearing 2D, a quarter 256-bearing
    2D, a quarter 1D). Every ping equals the single-ping path over the whole
    ping, and the FP64 oracle on a band of 8 rows."""
    pings = wl.batched_mix()
    assert len(pings) == 64
    ctxs, devs, outs = [], [], []
    for wk in pings:
        ctxs.append(make_context(wk))
        devs.append(torch.from_numpy(wk.samples.reshape(-1)).cuda())
        outs.append(torch.full(wk.out_shape + (2,), float("nan"), device="cuda"))
    batch = _lib.Batch(0)
    batch.plan([(c, d, wk.n, o) for wk, c, d, o in zip(pings, ctxs, devs, outs)], autotune=False)
    assert batch.graph_kernels() == 1
    batch.run(torch.cuda.current_stream())
    batch.status(torch.cuda.current_stream())
    torch.cuda.synchronize()
    for wk, o, ctx in zip(pings, outs, ctxs):
        got = _complex(o)
        assert np.isfinite(got).all(), wk.name
        # Same arithmetic as the single-ping path up to the order of the float
        # reductions (the batch splits hot tiles differently).
        assert rel_l2(got, single_ping(wk)) <= 1e-5, wk.name
        nR = wk.sensor["range_count"]
        rows = (nR // 3, nR // 3 + 8)
        want = oracle.reduce(wk.samples, wk.sensor, rows=rows)
        band = got[rows[0]:rows[1]]
        assert rel_l2(band, want) <= 1e-5, wk.name
    batch.close()
    for c in ctxs:
        c.close()
