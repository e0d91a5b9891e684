"""hv_unwrap_2d_noalloc: the 2-D phase unwrap for callers that cannot allocate device memory
(acquisition callbacks, applications that forbid cudaMalloc while streaming). It takes no
workspace and uses a static device array inside the library. The test checks, through the C ABI,
two calls in a row (the second reusing the scratch left by the first) against hv_unwrap_2d (which
takes a caller-allocated workspace) and against the oracle's unwrap, within the rel-L2 <= 1e-4
tolerance of the other parity tests; that once the first call has run on the device, a further
call leaves the device's free memory unchanged; and that frames larger than the static scratch and
empty frames are refused with their own messages.

This file sorts last so that a run stopping at the first failure has run every other test."""

import numpy as np
import pytest

import holovibes_oracle as O
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
        phase = _phase(H, W, 10 * H + call_index)
        wrapped = dev(phase)
        ref_out = empty(H * W * 4)
        work = empty(L.hv_unwrap_workspace(W, H))
        call("hv_unwrap_2d", ptr(wrapped), ptr(ref_out), W, H, ptr(work), None)
        out = empty(H * W * 4)
        call("hv_unwrap_2d_noalloc", ptr(wrapped), ptr(out), W, H, None)
        got = host(out, np.float32, (H, W))
        ref = host(ref_out, np.float32, (H, W))
        assert rel_l2(got, ref) <= 1e-4, call_index
        oracle = O.rescale_unwrap2d(O.unwrap_2d(phase.astype(np.float64)))
        assert rel_l2(got, oracle) <= 1e-4, call_index


@pytest.mark.gpu
def test_noalloc_second_call_allocates_nothing(cuda):
    """After the first call on the device (which may create the static array under lazy module
    loading), another call leaves cudaMemGetInfo's free memory where it was."""
    H, W = 256, 256
    wrapped = dev(_phase(H, W, 7))
    out = empty(H * W * 4)
    call("hv_unwrap_2d_noalloc", ptr(wrapped), ptr(out), W, H, None)
    cuda.cuda.synchronize()
    free0, _ = cuda.cuda.mem_get_info()
    call("hv_unwrap_2d_noalloc", ptr(wrapped), ptr(out), W, H, None)
    cuda.cuda.synchronize()
    free1, _ = cuda.cuda.mem_get_info()
    assert free1 == free0, (free0, free1)


@pytest.mark.gpu
def test_noalloc_rejects_frames_beyond_scratch(cuda):
    L = hv.lib()
    H, W = 1024, 512  # 524288 pixels > 262144
    buf = empty(H * W * 4)
    st = L.hv_unwrap_2d_noalloc(ptr(buf), ptr(buf), W, H, None)
    assert st == hv.HV_INVALID_VALUE
    assert "524288 pixels exceed the 262144-pixel static scratch" in hv.last_error()
    st = L.hv_unwrap_2d_noalloc(ptr(buf), ptr(buf), 0, H, None)
    assert st == hv.HV_INVALID_VALUE
    assert "must be positive" in hv.last_error()
