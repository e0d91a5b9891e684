"""Helpers for the GPU parity tests: device buffers through torch, C-ABI calls, error metrics."""

from __future__ import annotations

import numpy as np
import torch

import holovibes_gb300 as hv


_KEEP: list = []  # device copies stay alive until the end of the test (pointers outlive temporaries)


def release() -> None:
    if _KEEP:
        torch.cuda.synchronize()
        _KEEP.clear()


def dev(a: np.ndarray) -> torch.Tensor:
    t = _dev(a)
    _KEEP.append(t)
    return t


def _dev(a: np.ndarray) -> torch.Tensor:
    a = np.ascontiguousarray(a)
    if a.dtype == np.complex64:
        t = torch.from_numpy(a.view(np.float32).copy())
    elif a.dtype == np.complex128:
        t = torch.from_numpy(a.view(np.float64).copy())
    elif a.dtype == np.uint16:
        t = torch.from_numpy(a.view(np.int16).copy())
    else:
        t = torch.from_numpy(a.copy())
    return t.cuda()


def empty(nbytes: int) -> torch.Tensor:
    return torch.empty(max(int(nbytes), 16), dtype=torch.uint8, device="cuda")


def zeros(nbytes: int) -> torch.Tensor:
    return torch.zeros(max(int(nbytes), 16), dtype=torch.uint8, device="cuda")


def host(t: torch.Tensor, dtype, shape) -> np.ndarray:
    torch.cuda.synchronize()
    raw = t.detach().cpu().contiguous().numpy().view(np.uint8)
    n = int(np.prod(shape)) * np.dtype(dtype).itemsize
    return raw[:n].view(dtype).reshape(shape)


def ptr(t: torch.Tensor) -> int:
    return t.data_ptr()


def call(name: str, *args) -> None:
    st = getattr(hv.lib(), name)(*args)
    hv.check(st, name)


def rel_l2(a, b) -> float:
    a = np.asarray(a, dtype=np.complex128 if np.iscomplexobj(a) or np.iscomplexobj(b) else np.float64)
    b = np.asarray(b, dtype=a.dtype)
    den = np.linalg.norm(b.ravel())
    return float(np.linalg.norm((a - b).ravel()) / (den if den > 0 else 1.0))


def wrapped_diff(a, b) -> np.ndarray:
    """Angle difference in (-pi, pi]."""
    d = np.asarray(a, np.float64) - np.asarray(b, np.float64)
    return (d + np.pi) % (2 * np.pi) - np.pi


IMG = {0: "MODULUS", 1: "SQUARED_MODULUS", 2: "ARGUMENT", 3: "PHASE_INCREASE", 5: "MOMENTS_0", 6: "MOMENTS_1",
       7: "MOMENTS_2"}
SPACE = {0: "NONE", 1: "FRESNELTR", 2: "ANGULARSP"}
TIME = {0: "NONE", 1: "STFT", 2: "PCA", 3: "SSA_STFT"}


def oracle_settings(fd, s):
    """The oracle's settings record for a validated hv.Settings on frames of `fd`."""
    import holovibes_oracle as O

    return O.OracleSettings(
        width=fd.width, height=fd.height, depth=fd.depth, space_transformation=SPACE[s.space_transformation],
        time_transformation=TIME[s.time_transformation], time_transformation_size=s.time_transformation_size,
        time_stride=s.time_stride, batch_size=s.batch_size, lam=s.lambda_, z=s.z_distance, pixel_size=s.pixel_size,
        image_type=IMG[s.image_type], p_start=s.p_start, p_width=s.p_width, fft_shift=bool(s.fft_shift),
        renorm=bool(s.renorm), renorm_constant=s.renorm_constant, accumulation=s.accumulation,
        log_enabled=bool(s.log_enabled), contrast_enabled=bool(s.contrast_enabled),
        contrast_auto_refresh=bool(s.contrast_auto_refresh), contrast_invert=bool(s.contrast_invert),
        contrast_min=s.contrast_min, contrast_max=s.contrast_max, contrast_lower=s.contrast_lower,
        contrast_upper=s.contrast_upper, reticle_display=bool(s.reticle_display), reticle_scale=s.reticle_scale,
        unwrap_2d=bool(s.unwrap_2d), lens_mode="fp64" if s.lens_mode == 0 else "ref32", camera_fps=s.camera_fps,
        q_start=s.q_start, q_width=s.q_width, filter2d_enabled=bool(s.filter2d_enabled), filter2d_n1=s.filter2d_n1,
        filter2d_n2=s.filter2d_n2, filter2d_smooth_low=s.filter2d_smooth_low,
        filter2d_smooth_high=s.filter2d_smooth_high, cuts_enabled=bool(s.cuts_enabled), x_start=s.x_start,
        x_width=s.x_width, y_start=s.y_start, y_width=s.y_width, xz_accumulation=s.xz_accumulation,
        yz_accumulation=s.yz_accumulation, xz_log_enabled=bool(s.xz_log_enabled),
        yz_log_enabled=bool(s.yz_log_enabled), xz_contrast_enabled=bool(s.xz_contrast_enabled),
        xz_contrast_auto_refresh=bool(s.xz_contrast_auto_refresh), xz_contrast_invert=bool(s.xz_contrast_invert),
        xz_contrast_min=s.xz_contrast_min, xz_contrast_max=s.xz_contrast_max,
        yz_contrast_enabled=bool(s.yz_contrast_enabled), yz_contrast_auto_refresh=bool(s.yz_contrast_auto_refresh),
        yz_contrast_invert=bool(s.yz_contrast_invert), yz_contrast_min=s.yz_contrast_min,
        yz_contrast_max=s.yz_contrast_max, cuts_contrast_offset=s.cuts_contrast_offset,
        filter2d_view_enabled=bool(s.filter2d_view_enabled), filter2d_log_enabled=bool(s.filter2d_log_enabled),
        filter2d_contrast_enabled=bool(s.filter2d_contrast_enabled),
        filter2d_contrast_auto_refresh=bool(s.filter2d_contrast_auto_refresh),
        filter2d_contrast_invert=bool(s.filter2d_contrast_invert), filter2d_contrast_min=s.filter2d_contrast_min,
        filter2d_contrast_max=s.filter2d_contrast_max)
