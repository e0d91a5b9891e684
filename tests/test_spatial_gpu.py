"""Fused convert + spatial propagation into ring slots (hv_spatial_transform) and lenses,
against the FP64 oracle. Tolerance: rel-L2 <= 1e-4 (the benchmark spec's tolerance for float views)."""

import numpy as np
import pytest

import holovibes_oracle as O
from gpu_util import call, dev, empty, host, ptr, rel_l2, zeros

import holovibes_gb300 as hv


def _lens(space, W, H, lam, z, ps, mode):
    lens = empty(W * H * 8)
    if space == hv.SPACE_FRESNELTR:
        call("hv_fresnel_lens", ptr(lens), W, H, lam, z, ps, mode, None)
        ref = O.fresnel_lens(W, H, lam, z, ps, "fp64" if mode == 0 else "ref32")
    else:
        call("hv_angular_spectrum_lens", ptr(lens), W, H, lam, z, ps, mode, None)
        ref = O.angular_spectrum_lens(W, H, lam, z, ps, "fp64" if mode == 0 else "ref32")
    return lens, ref


@pytest.mark.gpu
@pytest.mark.parametrize("space", [hv.SPACE_FRESNELTR, hv.SPACE_ANGULARSP])
@pytest.mark.parametrize("W,H", [(512, 512), (1024, 768), (768, 1024), (64, 64)])
@pytest.mark.parametrize("mode", [hv.LENS_FP64, hv.LENS_REF32])
def test_lens(cuda, space, W, H, mode):
    lens, ref = _lens(space, W, H, 852e-9, 0.30, 20.0, mode)
    got = host(lens, np.complex64, (H, W))
    # the FP64 lens is the exact phase; the ref32 lens reproduces the reference's float32 phase
    assert rel_l2(got, ref) <= 2e-6


@pytest.mark.gpu
@pytest.mark.parametrize("space", [hv.SPACE_NONE, hv.SPACE_FRESNELTR, hv.SPACE_ANGULARSP])
@pytest.mark.parametrize("dtype,max_value,big_endian", [(np.uint16, 4095, 0), (np.uint8, 255, 0), (np.float32, 1000, 0),
                                                         (np.uint16, 4095, 1)])
def test_spatial_into_ring(cuda, space, dtype, max_value, big_endian):
    W, H, B, T = 128, 64, 3, 4
    rng = np.random.default_rng(1)
    raw = (rng.random((B, H, W)) * max_value).astype(dtype)
    raw_in = O.byteswap16(raw) if big_endian else raw
    lens, ref_lens = (None, None)
    if space != hv.SPACE_NONE:
        lens, ref_lens = _lens(space, W, H, 785e-9, 0.45, 12.0, hv.LENS_FP64)
    work = empty(B * H * W * 8)
    ring = zeros(T * H * W * 8)
    slot0 = 2  # frames land in slots 2, 3, 0 (wrap)
    call("hv_spatial_transform", ptr(dev(raw_in)), np.dtype(dtype).itemsize, big_endian, W, H, B, space,
         ptr(lens) if lens is not None else None, ptr(work), ptr(ring), slot0, T, None)
    got = host(ring, np.complex64, (T, H, W))
    name = {0: "NONE", 1: "FRESNELTR", 2: "ANGULARSP"}[space]
    ref = O.spatial_transform(O.convert_frames(raw), name, ref_lens)
    for b in range(B):
        assert rel_l2(got[(slot0 + b) % T], ref[b]) <= 1e-4, b
    assert np.all(got[1] == 0)  # untouched slot


@pytest.mark.gpu
@pytest.mark.parametrize("W,H", [(512, 512), (1024, 768), (768, 768), (256, 1024)])
def test_angular_spectrum_full_frame(cuda, W, H):
    """Full-size frames with realistic interferograms (12-bit), batch of 4."""
    from holovibes_gb300.synthetic import Interferogram

    g = Interferogram(width=W, height=H, seed=3)
    raw = g.frames(0, 4)
    lens, ref_lens = _lens(hv.SPACE_ANGULARSP, W, H, 852e-9, 0.30, 20.0, hv.LENS_FP64)
    work = empty(4 * H * W * 8)
    ring = zeros(4 * H * W * 8)
    call("hv_spatial_transform", ptr(dev(raw)), 2, 0, W, H, 4, hv.SPACE_ANGULARSP, ptr(lens), ptr(work), ptr(ring), 0,
         4, None)
    got = host(ring, np.complex64, (4, H, W))
    ref = O.angular_spectrum(O.convert_frames(raw), ref_lens)
    assert rel_l2(got, ref) <= 1e-4


@pytest.mark.gpu
@pytest.mark.parametrize("W,H,n1,n2,sl,sh", [(128, 64, 4, 20, 2, 3), (64, 64, 0, 1, 0, 1), (256, 128, 10, 40, 0, 0),
                                            (96, 160, 3, 70, 5, 12)])
def test_filter2d_mask(cuda, W, H, n1, n2, sl, sh):
    """kernel_update_filter2d_circles_mask + shift_corners against the oracle's float32
    restatement (|diff| <= 2e-6: cosf / hypotf ulps), written and multiplied into a lens."""
    m = empty(W * H * 8)
    call("hv_filter2d_mask", ptr(m), W, H, n1, n2, sl, sh, 0, None)
    got = host(m, np.complex64, (H, W))
    ref = O.filter2d_mask(W, H, n1, n2, sl, sh)
    assert np.all(got.imag == 0)
    assert np.max(np.abs(got.real - ref)) <= 2e-6
    lens, ref_lens = _lens(hv.SPACE_ANGULARSP, W, H, 852e-9, 0.30, 20.0, hv.LENS_FP64)
    call("hv_filter2d_mask", ptr(lens), W, H, n1, n2, sl, sh, 1, None)
    assert rel_l2(host(lens, np.complex64, (H, W)), ref_lens * ref) <= 2e-6


@pytest.mark.gpu
@pytest.mark.parametrize("space", [hv.SPACE_NONE, hv.SPACE_FRESNELTR, hv.SPACE_ANGULARSP])
def test_spatial_filter2d_into_ring(cuda, space):
    """filter2D before / inside the propagation (fourier_transform.cc:30-72): IFFT2(FFT2(x) M)
    unnormalised for NONE and FRESNELTR, the mask folded into G for ANGULARSP; rel-L2 <= 1e-4."""
    W, H, B, T = 128, 64, 3, 4
    rng = np.random.default_rng(7)
    raw = (rng.random((B, H, W)) * 4095).astype(np.uint16)
    mask = empty(W * H * 8)
    call("hv_filter2d_mask", ptr(mask), W, H, 3, 25, 2, 4, 0, None)
    ref_mask = O.filter2d_mask(W, H, 3, 25, 2, 4).astype(np.float64)
    lens, ref_lens = (None, None)
    if space != hv.SPACE_NONE:
        lens, ref_lens = _lens(space, W, H, 785e-9, 0.45, 12.0, hv.LENS_FP64)
    if space == hv.SPACE_ANGULARSP:
        call("hv_filter2d_mask", ptr(lens), W, H, 3, 25, 2, 4, 1, None)
        ref_lens = ref_lens * ref_mask
    work, work2 = empty(B * H * W * 8), empty(B * H * W * 8)
    ring = zeros(T * H * W * 8)
    call("hv_spatial_transform_filter2d", ptr(dev(raw)), 2, 0, W, H, B, space,
         ptr(lens) if lens is not None else None, ptr(mask) if space != hv.SPACE_ANGULARSP else None, ptr(work),
         ptr(work2), ptr(ring), 1, T, None)
    got = host(ring, np.complex64, (T, H, W))
    name = {0: "NONE", 1: "FRESNELTR", 2: "ANGULARSP"}[space]
    ref = O.spatial_transform(O.convert_frames(raw), name, ref_lens,
                              ref_mask if space != hv.SPACE_ANGULARSP else None)
    for b in range(B):
        assert rel_l2(got[(1 + b) % T], ref[b]) <= 1e-4, b
    assert np.all(got[0] == 0)
