"""The seeded interferogram generator: deterministic, in range, with the requested Doppler tone."""

import numpy as np

from holovibes_gb300.synthetic import CONFIGS, Interferogram, generator


def test_deterministic_and_ranged():
    g1 = Interferogram(width=64, height=32, seed=5)
    g2 = Interferogram(width=64, height=32, seed=5)
    a, b = g1.frames(3, 4), g2.frames(3, 4)
    assert a.dtype == np.uint16 and a.shape == (4, 32, 64)
    assert np.array_equal(a, b)
    assert a.max() <= 4095 and a.mean() > 100
    u8 = Interferogram(width=32, height=32, dtype=np.uint8, max_value=255).frames(0, 2)
    assert u8.dtype == np.uint8 and u8.max() <= 255


def test_doppler_tone_visible_in_time():
    g = Interferogram(width=32, height=32, seed=1, doppler=0.25)
    f = g.frames(0, 32).astype(np.float64)
    spec = np.abs(np.fft.fft(f - f.mean(axis=0), axis=0)).sum(axis=(1, 2))
    assert np.argmax(spec[1:16]) + 1 == 8  # 0.25 cycles/frame over 32 frames


def test_configs_construct():
    for name in CONFIGS:
        g = generator(name, width=16, height=16)
        assert g.frames(0, 1).shape == (1, 16, 16)
