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
