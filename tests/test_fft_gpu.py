"""Shared-memory FFT (hv_fft2d) against numpy's FP64 FFT. Tolerance: rel-L2 <= 1e-5 (FP32 FFT)."""

import numpy as np
import pytest

from gpu_util import call, dev, empty, host, ptr, rel_l2

SHAPES = [(64, 64), (512, 512), (768, 768), (1024, 1024), (768, 1024), (1024, 768), (256, 512), (48, 96),
          (1536, 384), (2048, 16), (16, 4096), (32, 192), (128, 128)]


@pytest.mark.gpu
@pytest.mark.parametrize("n0,n1", SHAPES)
def test_fft2d_matches_numpy(cuda, n0, n1):
    rng = np.random.default_rng(n0 * 7 + n1)
    B = 2
    x = (rng.standard_normal((B, n0, n1)) + 1j * rng.standard_normal((B, n0, n1))).astype(np.complex64)
    xd = dev(x)
    yd = empty(x.nbytes)
    call("hv_fft2d", ptr(xd), ptr(yd), n0, n1, B, 0, 1.0, None)
    y = host(yd, np.complex64, x.shape)
    ref = np.fft.fft2(x.astype(np.complex128), axes=(-2, -1))
    assert rel_l2(y, ref) <= 1e-5
    # unnormalised inverse with an explicit scale; in place
    call("hv_fft2d", ptr(yd), ptr(yd), n0, n1, B, 1, 1.0 / (n0 * n1), None)
    z = host(yd, np.complex64, x.shape)
    assert rel_l2(z, x) <= 1e-5


@pytest.mark.gpu
def test_fft_rejects_unsupported_length(cuda):
    import holovibes_gb300 as hv

    assert not hv.fft_size_supported(1000)
    x = dev(np.zeros((1, 10, 1000), np.complex64))
    st = hv.lib().hv_fft2d(ptr(x), ptr(x), 10, 1000, 1, 0, 1.0, None)
    assert st == hv.HV_ERR_UNSUPPORTED
