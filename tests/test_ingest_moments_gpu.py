"""Packed 10/12-bit camera data to 16 bits (hv_unpack_*; bit-exact against the oracle's restatement
of unpack.cu:4-32) and the moment views (hv_time_moments; rel-L2 <= 1e-4 against the FP64 oracle
of fourier_transform.cc:244-338 / tools_compute.cu:38-97, including the Nyquist compensation)."""

import numpy as np
import pytest

import holovibes_oracle as O
from gpu_util import call, dev, empty, host, ptr, rel_l2

import holovibes_gb300 as hv


@pytest.mark.gpu
@pytest.mark.parametrize("bits,n", [(12, 2 * 1000), (12, 1001), (10, 4 * 777), (10, 1003), (12, 512 * 512)])
def test_unpack(cuda, bits, n):
    rng = np.random.default_rng(bits * 7 + n)
    nbytes = (n * bits + 7) // 8
    packed = rng.integers(0, 256, nbytes, dtype=np.uint8)
    out = empty(n * 2)
    call(f"hv_unpack_{bits}_to_16", ptr(dev(packed)), nbytes, ptr(out), n, None)
    got = host(out, np.uint16, (n,))
    ref = (O.unpack_12_to_16 if bits == 12 else O.unpack_10_to_16)(packed, n)
    # the last group is written only where its bytes exist (a partial trailing group)
    full = n if bits == 12 and nbytes >= ((n + 1) // 2) * 3 else None
    if bits == 12:
        valid = np.array([(3 * (i // 2) + 1 + (i % 2)) < nbytes for i in range(n)])
    else:
        valid = np.array([(5 * (i // 4) + 1 + (i % 4)) < nbytes for i in range(n)])
    assert np.array_equal(got[valid], ref[valid])
    assert full is None or valid.all()


@pytest.mark.gpu
@pytest.mark.parametrize("T,pmin,pmax", [(16, 0, 15), (16, 5, 11), (15, 2, 9), (32, 14, 20)])
@pytest.mark.parametrize("order", [0, 1, 2])
def test_moments(cuda, T, pmin, pmax, order):
    H, W = 24, 40
    rng = np.random.default_rng(T * 3 + order)
    ring = (rng.standard_normal((T, H, W)) + 1j * rng.standard_normal((T, H, W))).astype(np.complex64)
    K = pmax - pmin + 1
    w = empty(K * T * 8)
    call("hv_stft_weights", ptr(w), T, pmin, pmax, None)
    bw = empty(K * 4)
    fps = 1500.0
    call("hv_moment_bin_weights", ptr(bw), T, pmin, pmax, hv.IMG_MOMENTS_0 + order, fps, None)
    out = empty(H * W * 4)
    npart = hv.lib().hv_time_view_partials(W, H)
    part = empty(npart * 8)
    call("hv_time_moments", ptr(dev(ring)), T, W, H, ptr(w), K, ptr(bw), 0, ptr(out), ptr(part), None)
    got = host(out, np.float32, (H, W))
    ref = O.moments(O.stft_bins(ring.astype(np.complex128), pmin, pmax), pmin, T, fps, order)
    if order == 1:
        # signed sums: compare against the scale of the order-2-free magnitude
        scale = O.moments(O.stft_bins(ring.astype(np.complex128), pmin, pmax), pmin, T, fps, 0) * fps
        assert np.sqrt(np.mean((got - ref) ** 2)) <= 1e-5 * np.sqrt(np.mean(scale ** 2))
    else:
        assert rel_l2(got, ref) <= 1e-4
    parts = host(part, np.float64, (npart,))
    assert abs(parts.sum() - got.astype(np.float64).sum()) <= 1e-6 * max(1.0, np.abs(got).sum())


@pytest.mark.gpu
def test_moment_rejects_other_types(cuda):
    bw = empty(64)
    assert hv.lib().hv_moment_bin_weights(ptr(bw), 16, 0, 3, hv.IMG_MODULUS, 100.0, None) == hv.HV_WRONG_IMG_TYPE
