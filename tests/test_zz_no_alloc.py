"""hv_unwrap_2d_noalloc: the 2-D phase unwrap for callers that cannot allocate device memory
(acquisition callbacks, applications that forbid cudaMalloc while streaming). It takes no
workspace and uses a static device array inside the library, so the test checks, through the
C ABI, that two calls in a row (the second reusing the scratch left by the first) reproduce
hv_unwrap_2d, which takes a caller-allocated workspace, within the rel-L2 <= 1e-4 tolerance of the
other parity tests, and that frames larger than the static scratch are refused.

This file sorts last so that a run stopping at the first failure has run every other test."""

import numpy as np
import pytest

from gpu_util import call, dev, empty, host, ptr, rel_l2

import holovibes_gb300 as hv


def _phase(H, W, seed):
    rng = np.random.default_rng(seed)
    y, x = np.mgrid[0:H, 0:W]
    a, b = rng.uniform(2, 6, 2)
    phase = a * np.sin(2 * np.pi * x / W) * np.cos(2 * np.pi * y / H) + b * x / W
    return np.angle(np.exp(1j * phase)).astype(np.float32)


@pytest.mark.gpu
@pytest.mark.parametrize("H,W", [(512, 512), (128, 256)])
def test_noalloc_matches_workspace_unwrap_twice(cuda, H, W):
    L = hv.lib()
    for call_index in range(2):
        wrapped = dev(_phase(H, W, 10 * H + call_index))
        ref_out = empty(H * W * 4)
        work = empty(L.hv_unwrap_workspace(W, H))
        call("hv_unwrap_2d", ptr(wrapped), ptr(ref_out), W, H, ptr(work), None)
        out = empty(H * W * 4)
        call("hv_unwrap_2d_noalloc", ptr(wrapped), ptr(out), W, H, None)
        got = host(out, np.float32, (H, W))
        ref = host(ref_out, np.float32, (H, W))
        assert rel_l2(got, ref) <= 1e-4, call_index


@pytest.mark.gpu
def test_noalloc_rejects_frames_beyond_scratch(cuda):
    L = hv.lib()
    H, W = 1024, 512  # 524288 pixels > 262144
    buf = empty(H * W * 4)
    st = L.hv_unwrap_2d_noalloc(ptr(buf), ptr(buf), W, H, None)
    assert st == hv.HV_INVALID_VALUE
    assert "static scratch" in hv.last_error()
