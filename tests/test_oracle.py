"""CPU checks of the oracle itself: ring semantics of Queue::enqueue_multiple, STFT over storage
order, the float32 restatements of the percentile index / contrast / uint16 conversion, lens
symmetries and the unwrap's recovery of a smooth phase. No GPU."""

import numpy as np
import pytest

import holovibes_oracle as O


def test_ring_enqueue_multiple_wraps_and_overflows():
    r = O.Ring(4, (1,))
    r.enqueue_multiple(np.arange(3, dtype=np.complex128).reshape(3, 1))
    assert (r.start, r.size) == (0, 3)
    r.enqueue_multiple(np.arange(3, 5, dtype=np.complex128).reshape(2, 1))
    # frames 0..4: slot0 overwritten by frame 4, start advances to 1
    assert (r.start, r.size) == (1, 4)
    assert list(r.data[:, 0].real) == [4, 1, 2, 3]
    # a batch larger than the ring keeps its last T frames
    r2 = O.Ring(3, (1,))
    r2.enqueue_multiple(np.arange(7, dtype=np.complex128).reshape(7, 1))
    assert r2.size == 3
    order = [(r2.start + i) % 3 for i in range(3)]
    assert list(r2.data[order, 0].real) == [4, 5, 6]


def test_stft_bins_match_fft_over_storage():
    rng = np.random.default_rng(0)
    x = rng.standard_normal((16, 3, 5)) + 1j * rng.standard_normal((16, 3, 5))
    full = np.fft.fft(x, axis=0)
    assert np.allclose(O.stft_bins(x, 2, 6), full[2:7])


def test_p_range():
    assert O.p_range(1, 0, 16) == (1, 1)
    assert O.p_range(28, 3, 32) == (28, 31)
    assert O.p_range(30, 5, 32) == (30, 32)  # clamped to T like converts.cc:84-86


def test_percentile_index_float32():
    # 99.5 / 100 * 262144 in float32 -> 260833.28 -> 260833
    assert O.percentile_index(99.5, 262144) == 260833
    assert O.percentile_index(0.5, 262144) == 1310
    assert O.percentile_index(100.0, 10) == 9  # clamped (the reference reads past the end)


def test_float_to_ushort_edges():
    x = np.array([-1.0, 0.0, 0.5, 1.9, 65534.9, 65535.0, 65535.99, 65536.0, 1e20, np.inf, np.nan], np.float32)
    assert list(O.float_to_ushort(x)) == [0, 0, 0, 1, 65534, 65535, 65535, 65535, 65535, 65535, 0]


def test_autocontrast_clamps_to_one():
    f = np.full((4, 4), 0.25, np.float32)
    assert O.autocontrast(f, 1, 99) == (1.0, 1.0)


def test_contrast_factor_float32():
    f = np.array([[100.0, 200.0]], np.float32)
    c = O.apply_contrast(f, 100.0, 200.0)
    assert c.dtype == np.float32 and c[0, 0] == 0.0 and abs(c[0, 1] - 65535.0) < 0.1


def test_lens_modes_agree_for_small_phase():
    # with a small phase range the float32 restatement is within float rounding of the exact lens
    a = O.fresnel_lens(64, 48, 852e-9, 10.0, 5.0, "fp64")
    b = O.fresnel_lens(64, 48, 852e-9, 10.0, 5.0, "ref32")
    assert np.abs(a - b).max() < 1e-5
    g = O.angular_spectrum_lens(64, 64, 852e-9, 1e-4, 20.0, "fp64")
    g32 = O.angular_spectrum_lens(64, 64, 852e-9, 1e-4, 20.0, "ref32")
    assert np.abs(g - g32).max() < 1e-3
    # lens crops: vertical and horizontal frames are centre crops of the square lens
    sq = O.fresnel_lens(64, 64, 852e-9, 0.3, 20.0)
    assert np.allclose(O.fresnel_lens(64, 32, 852e-9, 0.3, 20.0), sq[16:48, :])
    assert np.allclose(O.fresnel_lens(32, 64, 852e-9, 0.3, 20.0), sq[:, 16:48])


def test_angular_spectrum_identity_at_tiny_z():
    rng = np.random.default_rng(1)
    x = rng.standard_normal((1, 32, 32)) + 0j
    G = O.angular_spectrum_lens(32, 32, 852e-9, 1e-12, 20.0)
    y = O.angular_spectrum(x, G)
    assert np.allclose(np.abs(y), np.abs(x), atol=1e-6)


def test_unwrap_recovers_smooth_phase():
    H = W = 64
    y, x = np.mgrid[0:H, 0:W]
    phase = 4.0 * np.sin(2 * np.pi * x / W) * np.cos(2 * np.pi * y / H)
    wrapped = np.angle(np.exp(1j * phase))
    u = O.unwrap_2d(wrapped)
    # the Fourier unwrap recovers the phase up to scale, offset and sign (the reference's
    # Im(.)/-2pi convention returns -phase for exp(+i phase)); the images correlate
    a, b = O.rescale_unwrap2d(u), O.rescale_unwrap2d(phase)
    assert abs(np.corrcoef(a.ravel(), b.ravel())[0, 1]) > 0.99


def test_oracle_pipe_stride_and_wait():
    s = O.OracleSettings(width=16, height=16, time_transformation="STFT", time_transformation_size=4, time_stride=4,
                         batch_size=2, p_start=1, contrast_enabled=False)
    p = O.OraclePipe(s)
    raw = np.random.default_rng(0).integers(0, 4096, (2, 16, 16)).astype(np.uint16)
    outs = [p.process_batch(raw) for _ in range(6)]
    # batches 1,3,5 are dropped by the stride gate; batch 2 fills half the ring; outputs from batch 4 on
    assert [o is not None for o in outs] == [False, False, False, True, False, True]


def test_pca_pipeline_dominant_components():
    rng = np.random.default_rng(3)
    T = 8
    fields = [rng.standard_normal((6, 6)) + 1j * rng.standard_normal((6, 6)) for _ in range(2)]
    t = np.arange(T)
    ring = np.exp(2j * np.pi * 0.1 * t)[:, None, None] * fields[0] * 3 + np.exp(2j * np.pi * 0.3 * t)[:, None, None] * fields[1]
    w, V = O.pca_eigh(O.pca_covariance(ring))
    assert np.all(np.diff(w) >= -1e-9)
    P = O.pca_project(ring, V, T - 2, T - 1)
    # the two dominant components carry the whole signal
    assert np.isclose((np.abs(P) ** 2).sum(), (np.abs(ring) ** 2).sum(), rtol=1e-9)


def test_unpack_known_values():
    """Packed camera formats, MSB first (unpack.cu:4-32): hand-computed groups."""
    import holovibes_oracle as O

    got12 = O.unpack_12_to_16(np.array([0xAB, 0xCD, 0xEF], np.uint8), 2)
    assert got12.tolist() == [0xABC0, 0xDEF0]
    got10 = O.unpack_10_to_16(np.array([0xFF, 0xC0, 0x3F, 0xF0, 0x0F], np.uint8), 4)
    # 10-bit values 0x3FF, 0x000, 0x3FF, 0x00F... left-aligned
    assert got10.tolist() == [0xFFC0, 0x0000 | ((0x3F & 0xF0) << 2), ((0x3F & 0x0F) << 12) | ((0xF0 & 0xFC) << 4),
                              ((0xF0 & 0x03) << 14) | (0x0F << 6)]


def test_moment_frequencies():
    """fft_freqs (icompute.cc:26-69): even windows keep the Nyquist bin negative."""
    import holovibes_oracle as O

    assert O.fft_freqs(8, 1000.0).tolist() == [0, 125, 250, 375, -500, -375, -250, -125]
    assert O.fft_freqs(5, 1000.0).tolist() == [0, 200, 400, -400, -200]
    X = np.ones((8, 1, 1), complex)
    assert O.moments(X, 0, 8, 1000.0, 0)[0, 0] == 9.0  # Nyquist bin counted twice
    assert O.moments(X, 0, 8, 1000.0, 1)[0, 0] == 0.0
    assert O.moments(X, 0, 8, 1000.0, 2)[0, 0] == 937500.0


def test_ssa_all_columns_is_stft():
    """SSA_STFT with q width 0 keeps every eigenvector: V V^H = I, so the bins are the STFT's."""
    import holovibes_oracle as O

    rng = np.random.default_rng(3)
    ring = rng.standard_normal((12, 5, 7)) + 1j * rng.standard_normal((12, 5, 7))
    _, V = O.pca_eigh(O.pca_covariance(ring))
    got = O.ssa_stft_bins(ring, V, 4, 0, 2, 6)
    assert np.allclose(got, O.stft_bins(ring, 2, 6), rtol=1e-10, atol=1e-10)
    # a kept range of columns projects onto that eigenspace before the STFT
    P = O.ssa_stft_bins(ring, V, 9, 3, 0, 11)
    Vq = V[:, 9:12]
    proj = (ring.reshape(12, -1).T @ Vq @ Vq.conj().T).T.reshape(ring.shape)
    assert np.allclose(P, np.fft.fft(proj, axis=0), rtol=1e-10, atol=1e-10)


def test_phase_increase_history_and_rescale():
    """phase_increase (tools_unwrap.cu:210-267) with a one-frame history: out_n = d_n + d_{n-1},
    the first increment 0; rescale_float's min / max over the first 16384 pixels only."""
    import holovibes_oracle as O

    pi = O.PhaseIncrease()
    X0 = np.exp(1j * np.array([0.1, 1.0, -2.0]))
    X1 = X0 * np.exp(1j * np.array([0.2, 0.5, -1.5]))
    X2 = X1 * np.exp(1j * np.array([0.3, 0.25, 3.0]))
    assert np.allclose(pi.push(X0), 0.0)
    assert np.allclose(pi.push(X1), [0.2, 0.5, -1.5])
    d2 = np.angle(np.exp(1j * np.array([0.3, 0.25, 3.0])))
    assert np.allclose(pi.push(X2), d2 + np.array([0.2, 0.5, -1.5]))
    img = np.zeros(20000, np.float32)
    img[:16384] = np.linspace(-1.0, 2.0, 16384)
    img[17000] = 50.0  # past the prefix: not part of the range
    r = O.rescale_float(img)
    assert r[0] == 0.0 and np.isclose(r[16383], 65535.0 * 3.0 / 3.0)
    assert r[17000] > 65535.0


def test_filter2d_mask_shape():
    """filter2D band-pass (filter2D.cu:52-88): 0 inside n1, 1 between n1 and n2 (no smoothing),
    0 outside, centred on (W/2, H/2) before the quadrant swap."""
    import holovibes_oracle as O

    m = O.shift_corners(O.filter2d_mask(16, 16, 2, 5, 0, 0))  # back to centred layout
    assert m[8, 8] == 0.0 and m[8, 10] == 1.0 and m[8, 11] == 1.0 and m[8, 13] == 0.0
    s = O.shift_corners(O.filter2d_mask(32, 32, 2, 5, 0, 4))
    # roll-off between 5 and 9 pixels: cos((r - 5) / 4 * pi / 2)
    assert np.isclose(s[16, 16 + 7], np.cos(2 / 4 * np.pi / 2), atol=1e-6) and s[16, 16 + 9] == 0.0
    # the AS path folds the mask into G; a filtered frame keeps only the band's frequencies
    rng = np.random.default_rng(0)
    x = rng.standard_normal((1, 32, 32))
    y = O.filter2d(x, O.filter2d_mask(32, 32, 2, 5, 0, 0))
    spec = np.abs(np.fft.fftshift(np.fft.fft2(y[0])))
    assert spec[16, 16] < 1e-9 and spec[16, 16 + 12] < 1e-9
