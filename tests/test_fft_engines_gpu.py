"""512-, 768- and 1024-point spatial FFT passes on both engines (hv_fft_engine_mode 0: warp engine,
1: shared-memory Stockham tiles) against numpy's FP64 FFT and against each other: the 2-D
transform, the row pass with every input encoding, the lens premultiply, inverse, scale and ring
slots, the column pass in its three modes (forward, inverse, forward * G * inverse) and frame
heights / widths that leave partial CTAs. Tolerances: rel-L2 <= 1e-5 against FP64 (FP32 FFT),
<= 2e-6 between the engines."""

import numpy as np
import pytest

import holovibes_oracle as O
from gpu_util import call, dev, empty, host, ptr, rel_l2, zeros

import holovibes_gb300 as hv


@pytest.fixture
def engine(request):
    hv.fft_engine_mode(request.param)
    yield request.param
    hv.fft_engine_mode(0)


def _c64(rng, shape):
    return (rng.standard_normal(shape) + 1j * rng.standard_normal(shape)).astype(np.complex64)


@pytest.mark.gpu
@pytest.mark.parametrize("engine", [0, 1], indirect=True)
@pytest.mark.parametrize("n0,n1", [(1024, 1024), (1024, 768), (768, 1024), (1024, 48), (16, 1024), (1024, 2048),
                                   (512, 512), (512, 768), (768, 512), (512, 48), (16, 512), (512, 1024),
                                   (768, 768), (768, 48), (16, 768), (768, 2048)])
def test_fft2d_warp_lengths(cuda, engine, n0, n1):
    rng = np.random.default_rng(n0 + 3 * n1)
    B = 2
    x = _c64(rng, (B, n0, n1))
    xd, yd = dev(x), empty(x.nbytes)
    call("hv_fft2d", ptr(xd), ptr(yd), n0, n1, B, 0, 1.0, None)
    ref = np.fft.fft2(x.astype(np.complex128), axes=(-2, -1))
    assert rel_l2(host(yd, np.complex64, x.shape), ref) <= 1e-5
    call("hv_fft2d", ptr(yd), ptr(yd), n0, n1, B, 1, 1.0 / (n0 * n1), None)
    assert rel_l2(host(yd, np.complex64, x.shape), x) <= 1e-5


def _rows(raw, in_bytes, big_endian, W, H, B, premul, inverse, scale, slot0, nslots):
    out = zeros(nslots * H * W * 8)
    call("hv_fft_rows", ptr(dev(raw)), in_bytes, big_endian, ptr(out), W, H, B,
         ptr(dev(premul)) if premul is not None else None, inverse, scale, slot0, nslots, None)
    return host(out, np.complex64, (nslots, H, W))


@pytest.mark.gpu
@pytest.mark.parametrize("dtype,big_endian", [(np.uint8, 0), (np.uint16, 0), (np.uint16, 1), (np.float32, 0),
                                              (np.complex64, 0)])
@pytest.mark.parametrize("H,use_premul,inverse", [(13, True, 0), (8, False, 1), (40, True, 1)])
@pytest.mark.parametrize("W", [512, 768, 1024])
def test_row_pass_engines(cuda, dtype, big_endian, W, H, use_premul, inverse):
    B, nslots, slot0 = 3, 4, 2
    rng = np.random.default_rng(H + int(big_endian))
    if dtype == np.complex64:
        raw = _c64(rng, (B, H, W))
        x = raw.astype(np.complex128)
    else:
        top = {np.uint8: 255, np.uint16: 4095, np.float32: 1000}[dtype]
        raw = (rng.random((B, H, W)) * top).astype(dtype)
        x = O.convert_frames(raw)
    raw_in = O.byteswap16(raw) if big_endian else raw
    premul = _c64(rng, (H, W)) if use_premul else None
    if premul is not None:
        x = x * premul.astype(np.complex128)[None]
    ref = (np.conj(np.fft.fft(np.conj(x), axis=-1)) if inverse else np.fft.fft(x, axis=-1)) * 0.5
    got = {}
    for mode in (0, 1, 2):
        hv.fft_engine_mode(mode)
        try:
            got[mode] = _rows(raw_in, np.dtype(dtype).itemsize, big_endian, W, H, B, premul, inverse, 0.5, slot0,
                              nslots)
        finally:
            hv.fft_engine_mode(0)
        for b in range(B):
            assert rel_l2(got[mode][(slot0 + b) % nslots], ref[b]) <= 1e-5, (mode, b)
        assert np.all(got[mode][1] == 0)  # untouched slot
    assert rel_l2(got[0], got[1]) <= 2e-6
    # engine 0 feeds 1024-point rows of 8-/16-bit pixels (8 | H) through the persistent TMA kernel,
    # engine 2 through the register-loading one: the same arithmetic
    assert np.array_equal(got[0], got[2])
    assert hv.lib().hv_fft_status() == hv.HV_OK


@pytest.mark.gpu
@pytest.mark.parametrize("W", [1024, 48, 96, 16])
@pytest.mark.parametrize("mode", [0, 1, 2])
@pytest.mark.parametrize("H", [512, 768, 1024])
def test_col_pass_engines(cuda, W, H, mode):
    B, nslots, slot0 = 2, 3, 1
    rng = np.random.default_rng(W + 10 * mode)
    x = _c64(rng, (B, H, W))
    G = _c64(rng, (H, W)) if mode == 2 else None
    xr = x.astype(np.complex128)
    if mode == 0:
        ref = np.fft.fft(xr, axis=-2)
    elif mode == 1:
        ref = np.conj(np.fft.fft(np.conj(xr), axis=-2))
    else:
        ref = np.conj(np.fft.fft(np.conj(np.fft.fft(xr, axis=-2) * G.astype(np.complex128)[None]), axis=-2))
    ref = ref * 0.25
    got = {}
    for eng in (0, 1, 2):
        hv.fft_engine_mode(eng)
        try:
            out = zeros(nslots * H * W * 8)
            call("hv_fft_cols", ptr(dev(x)), ptr(out), W, H, B, ptr(dev(G)) if G is not None else None, mode, 0.25,
                 slot0, nslots, None)
            got[eng] = host(out, np.complex64, (nslots, H, W))
        finally:
            hv.fft_engine_mode(0)
        for b in range(B):
            assert rel_l2(got[eng][(slot0 + b) % nslots], ref[b]) <= 1e-5, (eng, b)
    assert rel_l2(got[0], got[1]) <= 2e-6
    # the TMA-fed persistent column pass (engine 0 at H = 1024) and the register-loading one
    # (engine 2) run the same arithmetic
    assert np.array_equal(got[0], got[2])
    assert hv.lib().hv_fft_status() == hv.HV_OK


@pytest.mark.gpu
@pytest.mark.parametrize("engine", [0, 1], indirect=True)
@pytest.mark.parametrize("space", [hv.SPACE_FRESNELTR, hv.SPACE_ANGULARSP])
@pytest.mark.parametrize("W,H", [(1024, 1024), (512, 512), (1024, 512), (768, 768), (1024, 768)])
def test_spatial_engines(cuda, engine, space, W, H):
    """The fused spatial stage on u8 frames (1024 x 1024: the Fresnel + PCA workload's frames)."""
    from holovibes_gb300.synthetic import Interferogram

    B = 3
    raw = (Interferogram(width=W, height=H, seed=5).frames(0, B) >> 4).astype(np.uint8)
    lens = empty(W * H * 8)
    if space == hv.SPACE_FRESNELTR:
        call("hv_fresnel_lens", ptr(lens), W, H, 785e-9, 0.45, 12.0, 0, None)
        ref_lens = O.fresnel_lens(W, H, 785e-9, 0.45, 12.0, "fp64")
    else:
        call("hv_angular_spectrum_lens", ptr(lens), W, H, 785e-9, 0.45, 12.0, 0, None)
        ref_lens = O.angular_spectrum_lens(W, H, 785e-9, 0.45, 12.0, "fp64")
    work = empty(B * H * W * 8)
    ring = zeros(B * H * W * 8)
    call("hv_spatial_transform", ptr(dev(raw)), 1, 0, W, H, B, space, ptr(lens), ptr(work), ptr(ring), 0, B, None)
    name = {1: "FRESNELTR", 2: "ANGULARSP"}[space]
    ref = O.spatial_transform(O.convert_frames(raw), name, ref_lens)
    assert rel_l2(host(ring, np.complex64, (B, H, W)), ref) <= 1e-5


@pytest.mark.gpu
def test_spatial_sub_batches_bit_identical(cuda):
    """hv_spatial_sub_batch_mb only changes how the batch is split into launches: every frame goes
    through the same kernels, so ring contents are bit-identical with and without sub-batches."""
    W = H = 1024
    B = 5
    rng = np.random.default_rng(11)
    raw = dev((rng.random((B, H, W)) * 255).astype(np.uint8))
    lens = empty(W * H * 8)
    call("hv_fresnel_lens", ptr(lens), W, H, 785e-9, 0.45, 12.0, 0, None)
    rings = []
    for mb in (0, 16):  # 16 MB: two frames per sub-batch, the last one alone
        hv.spatial_sub_batch_mb(mb)
        try:
            work, ring = empty(B * H * W * 8), zeros(B * H * W * 8)
            call("hv_spatial_transform", ptr(raw), 1, 0, W, H, B, hv.SPACE_FRESNELTR, ptr(lens), ptr(work), ptr(ring),
                 3, B, None)
            rings.append(host(ring, np.complex64, (B, H, W)))
        finally:
            hv.spatial_sub_batch_mb(0)
    assert np.array_equal(rings[0], rings[1])
