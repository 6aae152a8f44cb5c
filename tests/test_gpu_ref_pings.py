"""The plain form against pings of the reference's own reduction kernel
(tests/golden/ref_pings_2d.npz, recorded on a GB300 from the reference's
do_sparse_convolve_2d_f). This project evaluates the PSF with exact bilinear
weights; the reference's texture unit holds them in 8-bit fixed point, so
the two differ by that quantization (the oracle's texture mode reproduces
the reference to 1e-7, tests/test_oracle_golden.py)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():
    pytest.skip("needs a GPU", allow_module_level=True)

from helpers_gpu import gpu_reduce, make_context, rel_l2  # noqa: E402
from test_oracle_golden import REF_PINGS_TOL_EXACT, ref_ping_cases  # noqa: E402


def test_plain_form_against_reference_kernel_pings(oracle):
    for name, wk, step, ref in ref_ping_cases():
        ctx = make_context(wk)
        got = gpu_reduce(ctx, wk.samples, wk.out_shape)
        assert np.isfinite(got).all(), name
        assert rel_l2(got[::step], ref) <= REF_PINGS_TOL_EXACT, name
        # the difference is the texture quantization: the exact-PSF oracle
        # matches the GPU ping at the plain form's tolerance
        assert rel_l2(got, oracle.reduce(wk.samples, wk.sensor)) <= 1e-5, name


def test_texture_psf_flag_reproduces_reference_kernel_pings(oracle):
    """RTACX_FLAG_TEXTURE_PSF evaluates the PSF on the texture unit, as the
    reference does: the pings then match the reference kernel's to float
    round-off, and the oracle's texture mode on another geometry."""
    from rtac_simulation_gb300 import _lib
    from rtac_simulation_gb300 import workloads as wl
    for name, wk, step, ref in ref_ping_cases():
        ctx = make_context(wk, flags=_lib.RTACX_FLAG_TEXTURE_PSF)
        got = gpu_reduce(ctx, wk.samples, wk.out_shape)
        assert rel_l2(got[::step], ref) <= 1e-6, (name, rel_l2(got[::step], ref))
    wk = wl.oculus_2d(n_samples=1 << 14, n_bearings=100, n_ranges=300, seed=21)
    ctx = make_context(wk, flags=_lib.RTACX_FLAG_TEXTURE_PSF)
    got = gpu_reduce(ctx, wk.samples, wk.out_shape)
    assert rel_l2(got, oracle.reduce(wk.samples, wk.sensor, mode=2)) <= 1e-6


def test_texture_psf_flag_rejected_where_unsupported():
    from rtac_simulation_gb300 import _lib
    from rtac_simulation_gb300 import workloads as wl
    wk = wl.oculus_2d(n_samples=1 << 12, n_bearings=64, n_ranges=128)
    ctx = make_context(wk, flags=_lib.RTACX_FLAG_TEXTURE_PSF)
    d = torch.from_numpy(wk.samples.reshape(-1)).cuda()
    out = torch.empty(tuple(wk.out_shape) + (2,), dtype=torch.float32, device="cuda")
    batch = _lib.Batch(0)
    with pytest.raises(_lib.RtacxError):
        batch.plan([(ctx, d, wk.n, out)])
    with pytest.raises(_lib.RtacxError):
        ctx2 = _lib.Context(0)
        ctx2.configure_2d(**wk.sensor, flags=4)


def test_full_size_ping_against_the_live_reference_kernel(tmp_path):
    """The reference's own kernel (oracle/_ref/ref_sparse2d.cubin, compiled
    from the reference's source by oracle/ref_build.sh) run live on the full
    oculus_2d ping (2^20 samples, 512 x 1024): the texture-PSF path matches it
    to float round-off, the exact plain form to the texture quantization.
    Skipped where the cubin was not built (it needs the reference tree)."""
    from oracle import ref_kernel
    from rtac_simulation_gb300 import _lib
    if not ref_kernel.CUBIN.exists():
        pytest.skip("oracle/_ref/ref_sparse2d.cubin not built here")
    exe = ref_kernel.build_harness(tmp_path)
    ref, _, wk = ref_kernel.run_case(exe, tmp_path, "oculus_2d", "oculus_2d", {})
    assert np.isfinite(ref).all()
    tex = gpu_reduce(make_context(wk, flags=_lib.RTACX_FLAG_TEXTURE_PSF), wk.samples, wk.out_shape)
    assert rel_l2(tex, ref) <= 1e-6
    exact = gpu_reduce(make_context(wk), wk.samples, wk.out_shape)
    assert rel_l2(exact, ref) <= REF_PINGS_TOL_EXACT


def test_plain_1d_against_reference_kernel_pings(oracle):
    """The 1D form against pings of the reference's own 1D kernel
    (tests/golden/ref_pings_1d.npz), with the evident-intent scaling 1 /
    (duration c) and, under RTACX_FLAG_1D_LITERAL_SCALING, the literal
    1.0f / duration * c:
      * RTACX_FLAG_TEXTURE_PSF (border) and | RTACX_FLAG_TEXTURE_CLAMP fetch
        the pulse as the reference does and reproduce its pings in either
        address mode to float round-off;
      * k_gather_1d (exact weights, zero outside the table) is twice the
        border-mode ping up to the texture weights' quantization, and meets
        the FP64 oracle at the plain form's 1e-5."""
    from rtac_simulation_gb300 import _lib
    from test_oracle_golden import REF_PINGS_TOL_EXACT_1D, ref_ping_cases_1d
    from rtac_simulation_gb300 import workloads as wl
    seen = 0
    for name, smp, sensor, literal, address, ref in ref_ping_cases_1d():
        wk = wl.Workload(name, 1, sensor, smp)
        base = _lib.RTACX_FLAG_1D_LITERAL_SCALING if literal else 0
        tex_flags = base | _lib.RTACX_FLAG_TEXTURE_PSF | (_lib.RTACX_FLAG_TEXTURE_CLAMP if address else 0)
        tex = gpu_reduce(make_context(wk, flags=tex_flags), smp, wk.out_shape)
        assert np.isfinite(tex).all(), name
        assert rel_l2(tex, ref) <= 1e-6, (name, rel_l2(tex, ref))
        if address == 0:
            got = gpu_reduce(make_context(wk, flags=base), smp, wk.out_shape)
            assert rel_l2(got, 2.0 * ref) <= REF_PINGS_TOL_EXACT_1D, (name, rel_l2(got, 2.0 * ref))
            assert rel_l2(got, oracle.reduce(smp, sensor, literal_1d=literal)) <= 1e-5, name
        seen += 1
    assert seen == 8
