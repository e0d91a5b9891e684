"""Time transform + view on the tensor cores (hv_time_view_tc: tcgen05, split-BF16 operands, FP32
accumulation) against the oracle's STFT / PCA projection over the ring storage order and the
reference's bin-averaged views, and against the FP32 SIMT engine (hv_time_view) on the same input.

Tolerances: rel-L2 <= 1e-4 for the modulus and squared-modulus views (BF16x3 keeps about 16
mantissa bits per product); the argument view is compared as wrapped angle differences, allowing
a few pixels whose bin sits on the atan2 branch cut, and the bin-summed angle within
max(1e-3, 1e-4 K) rad at the 99.9th percentile (bins with |X_k| near 0 have a larger angle error). Per-tile partial sums add up to the frame."""

import numpy as np
import pytest

import holovibes_oracle as O
from gpu_util import call, dev, empty, host, ptr, rel_l2, wrapped_diff

import holovibes_gb300 as hv


def _ring(T, H, W, seed):
    rng = np.random.default_rng(seed)
    return (rng.standard_normal((T, H, W)) + 1j * rng.standard_normal((T, H, W))).astype(np.complex64)


def _run_tc(ring_d, T, W, H, w, K, img, scale=1.0, shift=0):
    work = empty(hv.lib().hv_time_view_tc_workspace(K, T))
    out = empty(H * W * 4)
    npart = hv.lib().hv_time_view_partials(W, H)
    part = empty(npart * 8)
    call("hv_time_view_tc", ptr(ring_d), T, W, H, ptr(w), K, img, scale, shift, ptr(out), ptr(part), ptr(work), None)
    got = host(out, np.float32, (H, W))
    assert hv.lib().hv_time_view_tc_status(ptr(work)) == hv.HV_OK
    return got, host(part, np.float64, (npart,))


def _check(got, ref, img, K):
    if img == hv.IMG_ARGUMENT:
        d = np.abs(got - ref)
        bad = d > 1e-3
        assert bad.mean() < 2e-3
        # the bin-sum of angles: each bin's angle error is the BF16x3 relative error over |X_k|, so
        # the rare bins with |X_k| near 0 form a tail; bound the 99.9th percentile and the tail size
        err = np.abs(wrapped_diff(got[~bad] * K, ref[~bad] * K))
        assert np.quantile(err, 0.999) < max(1e-3, 1e-4 * K)
        assert np.mean(err > 1e-2) < 1e-4
    else:
        assert rel_l2(got, ref) <= 1e-4


@pytest.mark.gpu
@pytest.mark.parametrize("T,pmin,pmax", [(32, 3, 13), (32, 0, 31), (64, 8, 15), (33, 0, 32), (256, 100, 132),
                                         (16, 1, 1), (128, 0, 63), (64, 8, 50), (512, 40, 103), (5, 1, 3)])
@pytest.mark.parametrize("img", [hv.IMG_MODULUS, hv.IMG_SQUARED_MODULUS, hv.IMG_ARGUMENT])
def test_stft_view_tc(cuda, T, pmin, pmax, img):
    H, W = 24, 40  # 960 pixels: 7 full 128-pixel tiles and a ragged one
    ring = _ring(T, H, W, T * 7 + img)
    K = pmax - pmin + 1
    w = empty(K * T * 8)
    call("hv_stft_weights", ptr(w), T, pmin, pmax, None)
    got, parts = _run_tc(dev(ring), T, W, H, w, K, img)
    ref = O.view(O.stft_bins(ring.astype(np.complex128), pmin, pmax), {0: "MODULUS", 1: "SQUARED_MODULUS",
                                                                       2: "ARGUMENT"}[img])
    _check(got, ref, img, K)
    assert abs(parts.sum() - got.astype(np.float64).sum()) <= 1e-9 * max(1.0, np.abs(got).sum())


@pytest.mark.gpu
@pytest.mark.parametrize("T,K", [(32, 8), (64, 33)])
def test_pca_projection_view_tc(cuda, T, K):
    """PCA weights (conjugated eigenvectors) through the same contraction."""
    H, W = 32, 64
    ring = _ring(T, H, W, 11 + T)
    rng = np.random.default_rng(T + K)
    wts = (rng.standard_normal((K, T)) + 1j * rng.standard_normal((K, T))).astype(np.complex64)
    wts /= np.linalg.norm(wts, axis=1, keepdims=True)
    got, _ = _run_tc(dev(ring), T, W, H, dev(wts), K, hv.IMG_MODULUS)
    x = np.einsum("kt,tp->kp", wts.astype(np.complex128), ring.reshape(T, -1).astype(np.complex128))
    ref = np.abs(x).mean(axis=0).reshape(H, W)
    assert rel_l2(got, ref) <= 1e-4


@pytest.mark.gpu
@pytest.mark.parametrize("img", [hv.IMG_MODULUS, hv.IMG_ARGUMENT])
def test_view_tc_matches_simt(cuda, img):
    """Both engines on one input, with fftshift placement and a scale, at a size that spans every SM."""
    T, H, W, pmin, pmax = 64, 256, 384, 5, 20
    K = pmax - pmin + 1
    ring_d = dev(_ring(T, H, W, 3))
    w = empty(K * T * 8)
    call("hv_stft_weights", ptr(w), T, pmin, pmax, None)
    got, parts = _run_tc(ring_d, T, W, H, w, K, img, scale=131071.0, shift=1)
    out = empty(H * W * 4)
    npart = hv.lib().hv_time_view_partials(W, H)
    part = empty(npart * 8)
    call("hv_time_view", ptr(ring_d), T, W, H, ptr(w), K, img, 131071.0, 1, ptr(out), ptr(part), None)
    simt = host(out, np.float32, (H, W))
    _check(got / 131071.0, simt / 131071.0, img, K)
    if img == hv.IMG_MODULUS:
        sp = host(part, np.float64, (npart,))
        assert abs(parts.sum() - sp.sum()) <= 1e-4 * abs(sp.sum())


@pytest.mark.gpu
def test_view_tc_rejects(cuda):
    assert hv.lib().hv_time_view_tc_workspace(65, 256) == 0  # K <= 64 on the tensor cores
    T, H, W = 8, 8, 8
    w = empty(129 * T * 8)
    out = empty(H * W * 4)
    work = empty(hv.lib().hv_time_view_tc_workspace(8, T))
    st = hv.lib().hv_time_view_tc(ptr(dev(_ring(T, H, W, 1))), T, W, H, ptr(w), 129, 0, 1.0, 0, ptr(out), None,
                                  ptr(work), None)
    assert st == hv.HV_ERR_UNSUPPORTED
    st = hv.lib().hv_time_view_tc(ptr(dev(_ring(T, 7, W, 1))), T, W, 7, ptr(w), 8, 0, 1.0, 1, ptr(out), None,
                                  ptr(work), None)
    assert st == hv.HV_INVALID_VALUE
    # an odd pixel count cannot be fetched with 16-byte bulk copies: rejected on the host
    st = hv.lib().hv_time_view_tc(ptr(dev(_ring(T, 7, 7, 1))), T, 7, 7, ptr(w), 8, 0, 1.0, 0, ptr(out), None,
                                  ptr(work), None)
    assert st == hv.HV_ERR_UNSUPPORTED


@pytest.mark.gpu
@pytest.mark.parametrize("T,pmin,pmax,img", [(32, 3, 13, hv.IMG_MODULUS), (256, 100, 132, hv.IMG_ARGUMENT)])
def test_prepare_then_run_matches_one_call(cuda, T, pmin, pmax, img):
    """hv_time_view_tc_prepare once + hv_time_view_tc_run per window gives exactly what
    hv_time_view_tc gives (the run reuses the prepared operand image, here for two rings)."""
    H, W = 24, 40
    K = pmax - pmin + 1
    w = empty(K * T * 8)
    call("hv_stft_weights", ptr(w), T, pmin, pmax, None)
    work = empty(hv.lib().hv_time_view_tc_workspace(K, T))
    call("hv_time_view_tc_prepare", ptr(w), K, T, ptr(work), None)
    for seed in (1, 2):
        ring_d = dev(_ring(T, H, W, seed))
        one, _ = _run_tc(ring_d, T, W, H, w, K, img)
        out = empty(H * W * 4)
        call("hv_time_view_tc_run", ptr(ring_d), T, W, H, K, img, 1.0, 0, ptr(out), None, ptr(work), None)
        assert np.array_equal(host(out, np.float32, (H, W)), one)
    assert hv.lib().hv_time_view_tc_status(ptr(work)) == hv.HV_OK
