"""Fused time transform + view (hv_time_view with STFT weights) against the oracle's STFT over
the ring storage order and the reference's bin-averaged views. Tolerance: rel-L2 <= 1e-4;
the argument view is compared as wrapped angle differences (atan2 is discontinuous at +-pi)."""

import numpy as np
import pytest

import holovibes_oracle as O
from gpu_util import call, dev, empty, host, ptr, rel_l2, wrapped_diff

import holovibes_gb300 as hv


def _ring(T, H, W, seed):
    rng = np.random.default_rng(seed)
    return (rng.standard_normal((T, H, W)) + 1j * rng.standard_normal((T, H, W))).astype(np.complex64)


@pytest.mark.gpu
@pytest.mark.parametrize("T,pmin,pmax", [(16, 1, 1), (32, 0, 3), (256, 48, 80), (512, 500, 511), (8, 0, 7), (1, 0, 0)])
@pytest.mark.parametrize("img", [hv.IMG_MODULUS, hv.IMG_SQUARED_MODULUS, hv.IMG_ARGUMENT])
def test_stft_view(cuda, T, pmin, pmax, img):
    H, W = 24, 40
    ring = _ring(T, H, W, T + img)
    K = pmax - pmin + 1
    w = empty(K * T * 8)
    call("hv_stft_weights", ptr(w), T, pmin, pmax, None)
    out = empty(H * W * 4)
    npart = hv.lib().hv_time_view_partials(W, H)
    part = empty(npart * 8)
    call("hv_time_view", ptr(dev(ring)), T, W, H, ptr(w), K, img, 1.0, 0, ptr(out), ptr(part), None)
    got = host(out, np.float32, (H, W))
    planes = O.stft_bins(ring.astype(np.complex128), pmin, pmax)
    name = {0: "MODULUS", 1: "SQUARED_MODULUS", 2: "ARGUMENT"}[img]
    ref = O.view(planes, name)
    if img == hv.IMG_ARGUMENT:
        d = np.abs(got - ref)
        # a bin sitting on the branch cut may flip by 2*pi/K: allow a few such pixels
        bad = d > 1e-3
        assert bad.mean() < 2e-3
        assert np.abs(wrapped_diff(got[~bad] * K, ref[~bad] * K)).max() < 1e-3
    else:
        assert rel_l2(got, ref) <= 1e-4
    parts = host(part, np.float64, (npart,))
    assert abs(parts.sum() - got.astype(np.float64).sum()) <= 1e-9 * max(1.0, abs(got).sum())


@pytest.mark.gpu
def test_view_shift_and_scale(cuda):
    T, H, W = 16, 32, 64
    ring = _ring(T, H, W, 5)
    w = empty(T * 8)
    call("hv_stft_weights", ptr(w), T, 1, 1, None)
    out = empty(H * W * 4)
    call("hv_time_view", ptr(dev(ring)), T, W, H, ptr(w), 1, hv.IMG_MODULUS, 131071.0, 1, ptr(out), None, None)
    got = host(out, np.float32, (H, W))
    ref = O.shift_corners(O.view(O.stft_bins(ring.astype(np.complex128), 1, 1), "MODULUS") * 131071.0)
    assert rel_l2(got, ref) <= 1e-4


@pytest.mark.gpu
def test_storage_order_quirk(cuda):
    """The STFT runs over ring storage order: a rotated ring changes bin phases, not magnitudes."""
    T, H, W = 8, 8, 16
    ring = _ring(T, H, W, 9)
    rot = np.roll(ring, 3, axis=0)
    w = empty(T * 8)
    call("hv_stft_weights", ptr(w), T, 2, 2, None)
    outs = []
    for r in (ring, rot):
        out = empty(H * W * 4)
        call("hv_time_view", ptr(dev(r)), T, W, H, ptr(w), 1, hv.IMG_ARGUMENT, 1.0, 0, ptr(out), None, None)
        outs.append(host(out, np.float32, (H, W)))
    ref = [O.view(O.stft_bins(r.astype(np.complex128), 2, 2), "ARGUMENT") for r in (ring, rot)]
    for g, r in zip(outs, ref):
        assert np.abs(wrapped_diff(g, r)).max() < 1e-4
    assert np.abs(wrapped_diff(outs[0], outs[1])).max() > 0.1


def _bf16_rn(x):
    u = np.ascontiguousarray(x, np.float32).view(np.uint32)
    return ((u + (((u >> 16) & 1) + 0x7FFF)) >> 16).astype(np.uint16)


@pytest.mark.gpu
@pytest.mark.parametrize("T,K,slot0,n", [(256, 4, 64, 32), (256, 4, 240, 32), (512, 4, 0, 64), (128, 1, 0, 0),
                                         (64, 2, 63, 1), (96, 6, 40, 96), (16, 4, 8, 8)])
@pytest.mark.parametrize("img,shift", [(hv.IMG_SQUARED_MODULUS, 0), (hv.IMG_MODULUS, 1), (hv.IMG_ARGUMENT, 0)])
def test_view_from_real_planes(cuda, T, K, slot0, n, img, shift):
    """hv_time_view_planes on the real split planes of an integer ring (frames converted without a
    spatial transform), with the slots [slot0, slot0 + n) mod T read from the ring: the same view
    values as hv_time_view on the ring (bit for bit) and the same 128-pixel partial sums. Random
    complex weights (eigenvector-like); W x H a multiple of 8 but not of 128 (a partial last
    renormalisation group). K > 4 runs in chunks of 4 bins there and in one chunk on the ring:
    within 1e-6."""
    H, W = 24, 44
    rng = np.random.default_rng(T + K + slot0)
    ring = np.zeros((T, H, W), np.complex64)
    ring.real = rng.integers(0, 65536, size=(T, H, W)).astype(np.float32)
    w = ((rng.standard_normal((K, T)) + 1j * rng.standard_normal((K, T))) / np.sqrt(T)).astype(np.complex64)
    rd, wd = dev(ring), dev(w)
    # the split on the host: hi = bf16(x), lo = bf16(x - hi), round to nearest even; [2][T][HW]
    x = ring.real.reshape(T, H * W)
    hi = _bf16_rn(x)
    lo = _bf16_rn(x - (hi.astype(np.uint32) << 16).view(np.float32))
    host_planes = np.stack([hi, lo])
    planes = dev(host_planes)
    if 2 * T > 128:  # the device split (the pipe's) writes the same planes
        dp = empty(hv.lib().hv_pca_planes_bytes(T, H * W, 1))
        call("hv_pca_split_planes", ptr(rd), T, H * W, 0, T, 1, ptr(dp), None)
        assert np.array_equal(host(dp, np.uint16, host_planes.shape), host_planes)
    npart = hv.lib().hv_time_view_partials(W, H)
    outs, parts = [], []
    for fn, args in (("hv_time_view", (ptr(rd), T)), ("hv_time_view_planes", (ptr(planes), ptr(rd), slot0, n, T))):
        out, part = empty(H * W * 4), empty(npart * 8)
        call(fn, *args, W, H, ptr(wd), K, img, 131071.0, shift, ptr(out), ptr(part), None)
        outs.append(host(out, np.float32, (H, W)))
        parts.append(host(part, np.float64, (npart,)))
    assert np.isfinite(outs[0]).all()
    if K <= 4:  # both two-pixel kernels, one chunk of bins: bit for bit
        assert np.array_equal(outs[0], outs[1])
        np.testing.assert_allclose(parts[1], parts[0], rtol=1e-12, atol=0)
    else:  # chunks of 4 against one of 6: the compiler may contract the bin sums differently
        np.testing.assert_allclose(outs[1], outs[0], rtol=1e-6, atol=0)
        np.testing.assert_allclose(parts[1], parts[0], rtol=1e-6, atol=0)
