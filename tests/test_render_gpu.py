"""Rendering steps against the oracle: exact percentile selection, bit-exact contrast + uint16,
renormalisation, fftshift, accumulation and the 2-D unwrap (rel-L2 <= 1e-4)."""

import numpy as np
import pytest

import holovibes_oracle as O
from gpu_util import call, dev, empty, host, ptr, rel_l2, zeros

import holovibes_gb300 as hv


def _frame(H, W, seed, kind="speckle"):
    rng = np.random.default_rng(seed)
    if kind == "speckle":
        return (rng.exponential(1000.0, (H, W)) + 0.5).astype(np.float32)
    if kind == "ties":
        return rng.integers(0, 7, (H, W)).astype(np.float32)
    if kind == "signed":
        return rng.standard_normal((H, W)).astype(np.float32) * 3
    return rng.random((H, W)).astype(np.float32) * 0.5  # all below 1: clamp to 1


@pytest.mark.gpu
@pytest.mark.parametrize("H,W", [(64, 64), (512, 512), (768, 1024), (13, 7)])
@pytest.mark.parametrize("kind", ["speckle", "ties", "signed", "small"])
@pytest.mark.parametrize("lo,hi", [(0.5, 99.5), (0.02, 99.98), (0.0, 100.0)])
def test_percentile_exact(cuda, H, W, kind, lo, hi):
    f = _frame(H, W, H * W, kind)
    rng_d = empty(16)
    work = empty(hv.lib().hv_percentile_workspace(H * W))
    call("hv_percentile", ptr(dev(f)), W, H, lo, hi, 0.0, ptr(rng_d), ptr(work), None)
    got = host(rng_d, np.float32, (2,))
    ref = O.autocontrast(f, lo, hi)
    assert got[0] == np.float32(ref[0]) and got[1] == np.float32(ref[1])


@pytest.mark.gpu
@pytest.mark.parametrize("scale", [0.5, 0.2])
def test_percentile_reticle(cuda, scale):
    H, W = 96, 128
    f = _frame(H, W, 4)
    rng_d = empty(16)
    work = empty(hv.lib().hv_percentile_workspace(H * W))
    call("hv_percentile", ptr(dev(f)), W, H, 2.0, 98.0, scale, ptr(rng_d), ptr(work), None)
    got = host(rng_d, np.float32, (2,))
    ref = O.autocontrast(f, 2.0, 98.0, scale)
    assert got[0] == np.float32(ref[0]) and got[1] == np.float32(ref[1])


@pytest.mark.gpu
@pytest.mark.parametrize("invert", [0, 1])
@pytest.mark.parametrize("apply", [0, 1])
def test_contrast_ushort_bit_exact(cuda, invert, apply):
    H, W = 128, 96
    f = _frame(H, W, 7)
    f.flat[:5] = [-1.0, 0.0, 70000.0, np.inf, 65535.5]
    cr = np.array([300.0, 5000.0], np.float32)
    out = empty(H * W * 2)
    call("hv_contrast_to_ushort", ptr(dev(f)), ptr(dev(cr)), invert, apply, ptr(out), H * W, None)
    got = host(out, np.uint16, (H, W))
    c = O.apply_contrast(f, cr[0], cr[1], bool(invert)) if apply else f
    ref = O.float_to_ushort(c)
    assert np.array_equal(got, ref)


@pytest.mark.gpu
def test_renormalize(cuda):
    H, W = 64, 48
    f = _frame(H, W, 11)
    fd = dev(f)
    work = empty(hv.lib().hv_reduce_workspace(H * W))
    call("hv_renormalize", ptr(fd), H * W, 5, None, 0, ptr(work), None)
    got = host(fd, np.float32, (H, W))
    assert rel_l2(got, O.renormalize(f.astype(np.float64), 5)) <= 1e-6


@pytest.mark.gpu
def test_shift_corners(cuda):
    f = _frame(32, 64, 2)
    fd = dev(f)
    call("hv_shift_corners", ptr(fd), 64, 32, None)
    assert np.array_equal(host(fd, np.float32, (32, 64)), O.shift_corners(f))


@pytest.mark.gpu
def test_accumulation_ring(cuda):
    """Queue::enqueue + accumulate_images over 11 frames into an 4-slot ring."""
    H, W, A = 16, 16, 4
    acc = zeros(A * H * W * 4)
    model = O.Accumulator(A, (H, W))
    start, size = 0, 0
    for i in range(11):
        f = _frame(H, W, 100 + i)
        slot = (start + size) % A
        if size < A:
            size += 1
        else:
            start = (start + 1) % A
        out = empty(H * W * 4)
        call("hv_accumulate", ptr(dev(f)), ptr(acc), A, slot, start, size, ptr(out), H * W, None)
        ref = model.push(f.astype(np.float64))
        assert rel_l2(host(out, np.float32, (H, W)), ref) <= 1e-6


@pytest.mark.gpu
@pytest.mark.parametrize("H,W", [(64, 64), (128, 128), (768, 768), (64, 128)])
def test_unwrap_2d(cuda, H, W):
    y, x = np.mgrid[0:H, 0:W]
    phase = 6.0 * np.sin(2 * np.pi * x / W) * np.cos(2 * np.pi * y / H) + 0.3 * x / W
    wrapped = np.angle(np.exp(1j * phase)).astype(np.float32)
    out = empty(H * W * 4)
    work = empty(hv.lib().hv_unwrap_workspace(W, H))
    call("hv_unwrap_2d", ptr(dev(wrapped)), ptr(out), W, H, ptr(work), None)
    got = host(out, np.float32, (H, W))
    ref = O.rescale_unwrap2d(O.unwrap_2d(wrapped.astype(np.float64)))
    assert rel_l2(got, ref) <= 1e-4
