"""Seeded synthetic off-axis interferograms for the benchmark configurations.

There is no public dataset for this path; every input is generated here from a seed:
I_t = |R + O_t|^2 with R a unit plane wave tilted in x and O_t a random-phase speckle object
(amplitude ``object_amp``, complex Gaussian speckle smoothed with a Gaussian of ``speckle_sigma``
pixels), propagated by ``z`` with an FP64 angular spectrum and modulated in time (Doppler tone,
optional linear sweep, optional extra sinusoids or a sum of seeded temporal modes). Poisson noise
is added and the intensity scaled to ``max_value`` (4095 for 12-bit data in uint16, 255 for uint8).
"""

from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np


def _gaussian_smooth(a: np.ndarray, sigma: float) -> np.ndarray:
    """Periodic Gaussian blur through the FFT (FP64)."""
    H, W = a.shape
    fy = np.fft.fftfreq(H)[:, None]
    fx = np.fft.fftfreq(W)[None, :]
    g = np.exp(-2.0 * (math.pi * sigma) ** 2 * (fx * fx + fy * fy))
    return np.fft.ifft2(np.fft.fft2(a) * g)


def _propagate(field: np.ndarray, z: float, lam: float, pitch: float) -> np.ndarray:
    H, W = field.shape
    fy = np.fft.fftfreq(H, d=pitch)[:, None]
    fx = np.fft.fftfreq(W, d=pitch)[None, :]
    arg = 1.0 - (lam * fx) ** 2 - (lam * fy) ** 2
    kz = 2.0 * math.pi / lam * np.sqrt(np.maximum(arg, 0.0))
    return np.fft.ifft2(np.fft.fft2(field) * np.exp(1j * np.mod(kz * z, 2 * math.pi)))


@dataclass
class Interferogram:
    width: int
    height: int
    dtype: type = np.uint16
    max_value: int = 4095
    z: float = 0.30
    lam: float = 852e-9
    pitch_um: float = 20.0
    tilt_deg: float = 2.0
    object_amp: float = 0.3
    speckle_sigma: float = 3.0
    doppler: float = 0.2  # cycles per frame (fraction of the frame rate)
    doppler_end: float | None = None  # linear sweep across `sweep_frames`
    sweep_frames: int = 256
    sinusoids: tuple = ()  # ((freq_per_frame, amplitude), ...)
    modes: int = 0  # > 0: sum of seeded temporal modes, amplitude ~ 1/m (eigenvalues ~ m^-2)
    seed: int = 0
    _obj: np.ndarray | None = field(default=None, repr=False)
    _ref: np.ndarray | None = field(default=None, repr=False)
    _mode_fields: list | None = field(default=None, repr=False)
    _mode_freqs: np.ndarray | None = field(default=None, repr=False)

    def _object(self, rng) -> np.ndarray:
        H, W = self.height, self.width
        speck = _gaussian_smooth(rng.standard_normal((H, W)) + 1j * rng.standard_normal((H, W)), self.speckle_sigma)
        amp = np.abs(speck)
        amp = self.object_amp * amp / max(amp.mean(), 1e-30)
        phase = rng.uniform(0.0, 2.0 * math.pi, (H, W))
        return _propagate(amp * np.exp(1j * phase), self.z, self.lam, self.pitch_um * 1e-6)

    def _setup(self):
        if self._obj is not None:
            return
        rng = np.random.default_rng(self.seed)
        H, W = self.height, self.width
        x = np.arange(W)[None, :] * self.pitch_um * 1e-6
        k = 2.0 * math.pi * math.sin(math.radians(self.tilt_deg)) / self.lam
        self._ref = np.broadcast_to(np.exp(1j * np.mod(k * x, 2 * math.pi)), (H, W))
        self._obj = self._object(rng)
        if self.modes > 0:
            self._mode_fields = [self._object(rng) / (m + 1) for m in range(self.modes)]
            self._mode_freqs = rng.uniform(0.02, 0.48, self.modes)

    def field_at(self, t: int) -> np.ndarray:
        self._setup()
        if self.modes > 0:
            O = sum(f * np.exp(2j * math.pi * fr * t) for f, fr in zip(self._mode_fields, self._mode_freqs))
        else:
            if self.doppler_end is None:
                ph = 2.0 * math.pi * self.doppler * t
            else:  # linear sweep: instantaneous frequency from doppler to doppler_end
                tt = t % self.sweep_frames
                slope = (self.doppler_end - self.doppler) / self.sweep_frames
                ph = 2.0 * math.pi * (self.doppler * tt + 0.5 * slope * tt * tt)
            amp = 1.0 + sum(a * math.sin(2.0 * math.pi * f * t) for f, a in self.sinusoids)
            O = self._obj * amp * np.exp(1j * ph)
        return self._ref + O

    def frames(self, start: int, count: int) -> np.ndarray:
        """Frames start .. start+count-1 (seeded per frame index)."""
        out = np.empty((count, self.height, self.width), dtype=self.dtype)
        for i in range(count):
            t = start + i
            I = np.abs(self.field_at(t)) ** 2
            scale = 0.5 * self.max_value / max(I.mean(), 1e-30)
            rng = np.random.default_rng((self.seed, t))
            noisy = rng.poisson(I * scale)
            out[i] = np.clip(noisy, 0, self.max_value).astype(self.dtype)
        return out


# ---------------------------------------------------------------------------------- configurations
# The five workloads of the benchmark (sizes, transforms and generator parameters). `settings`
# uses the field names of holovibes_gb300.Settings; `gen` the Interferogram fields.

CONFIGS = {
    "cfg0": dict(
        desc="512x512 u16 12-bit, angular spectrum + STFT, B=S=T=16, modulus, p=1, pacc=0",
        width=512, height=512, depth=2,
        settings=dict(space_transformation=2, time_transformation=1, time_transformation_size=16, time_stride=16,
                      batch_size=16, lambda_=852e-9, z_distance=0.30, pixel_size=20.0, image_type=0, p_start=1,
                      p_width=0, fft_shift=1, renorm=0, accumulation=0, contrast_enabled=1, contrast_auto_refresh=1,
                      contrast_lower=0.5, contrast_upper=99.5),
        gen=dict(dtype=np.uint16, max_value=4095, z=0.30, lam=852e-9, pitch_um=20.0, doppler=0.2),
    ),
    "cfg1": dict(
        desc="1024x1024 u8, Fresnel + PCA, B=S=T=32, squared modulus, 4 dominant components (p=28, pacc=3)",
        width=1024, height=1024, depth=1,
        settings=dict(space_transformation=1, time_transformation=2, time_transformation_size=32, time_stride=32,
                      batch_size=32, lambda_=785e-9, z_distance=0.45, pixel_size=12.0, image_type=1, p_start=28,
                      p_width=3, fft_shift=0, renorm=1, accumulation=0, contrast_enabled=1, contrast_auto_refresh=1,
                      contrast_lower=0.5, contrast_upper=99.5),
        gen=dict(dtype=np.uint8, max_value=255, z=0.45, lam=785e-9, pitch_um=12.0, doppler=0.2,
                 sinusoids=((0.05, 1.0), (0.15, 0.5), (0.30, 0.2))),
    ),
    "cfg2": dict(
        desc="768x768 u16, angular spectrum + STFT, B=S=64, T=256, K=33 bins, accumulation 8, argument",
        width=768, height=768, depth=2,
        settings=dict(space_transformation=2, time_transformation=1, time_transformation_size=256, time_stride=64,
                      batch_size=64, lambda_=852e-9, z_distance=0.30, pixel_size=20.0, image_type=2, p_start=48,
                      p_width=32, fft_shift=1, renorm=0, accumulation=8, contrast_enabled=1, contrast_auto_refresh=1,
                      contrast_lower=0.5, contrast_upper=99.5),
        gen=dict(dtype=np.uint16, max_value=4095, z=0.30, lam=852e-9, pitch_um=20.0, doppler=0.2, doppler_end=0.3,
                 sweep_frames=256),
    ),
    "cfg3": dict(
        desc="512x512 u16, PCA T=512, B=S=64, 16 seeded modes with k^-2 eigenvalue decay",
        width=512, height=512, depth=2,
        settings=dict(space_transformation=0, time_transformation=2, time_transformation_size=512, time_stride=64,
                      batch_size=64, lambda_=852e-9, z_distance=0.30, pixel_size=20.0, image_type=0, p_start=508,
                      p_width=3, fft_shift=0, renorm=1, accumulation=0, contrast_enabled=1, contrast_auto_refresh=1,
                      contrast_lower=0.5, contrast_upper=99.5),
        gen=dict(dtype=np.uint16, max_value=4095, z=0.30, lam=852e-9, pitch_um=20.0, modes=16),
    ),
}


def generator(name: str, seed: int = 0, width: int | None = None, height: int | None = None) -> Interferogram:
    c = CONFIGS[name]
    return Interferogram(width=width or c["width"], height=height or c["height"], seed=seed, **c["gen"])


def settings_for(name: str, **overrides):
    from . import Settings

    s = Settings.defaults()
    s.update(**CONFIGS[name]["settings"])
    s.update(**overrides)
    return s
