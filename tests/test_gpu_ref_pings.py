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
