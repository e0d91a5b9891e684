"""ctypes wrapper of the reference's own GPU build (oracle/_ref/libhvref.so). TEST INFRASTRUCTURE ONLY.

``RefPipe`` runs one Pipe cycle per batch through the reference's unmodified cuFFT / cuBLAS /
cuSOLVER / thrust code (driven by ``oracle/ref_pipe.cu``). Only ``tests/`` and ``bench.py`` use it,
as a comparator; the product never loads it.
"""

from __future__ import annotations

import ctypes as C
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE))
import ref_build  # noqa: E402

SPACE = {"NONE": 0, "FRESNELTR": 1, "ANGULARSP": 2}
TIME = {"NONE": 0, "STFT": 1, "PCA": 2}
IMG = {"MODULUS": 0, "SQUARED_MODULUS": 1, "ARGUMENT": 2}


class Config(C.Structure):
    _fields_ = [(n, C.c_int) for n in ("width", "height", "depth", "space", "time", "time_transformation_size",
                                       "time_stride", "batch_size")] + \
               [(n, C.c_float) for n in ("lam", "z", "pixel_size")] + \
               [(n, C.c_int) for n in ("img_type", "p_start", "p_width", "fft_shift", "renorm", "renorm_constant",
                                       "accumulation", "log_enabled", "contrast_enabled", "contrast_invert")] + \
               [(n, C.c_float) for n in ("contrast_lower", "contrast_upper")] + \
               [(n, C.c_int) for n in ("unwrap_2d", "keep_float_frame")]


_LIB = None


def available() -> bool:
    return ref_build.LIB.exists() or ref_build.staged()


def lib():
    """Loads the reference build, compiling it first when only the staged sources are present."""
    global _LIB
    if _LIB is None:
        path = ref_build.build() if ref_build.staged() else ref_build.LIB
        L = C.CDLL(str(path))
        L.hvref_create.restype = C.c_void_p
        L.hvref_create.argtypes = [C.POINTER(Config)]
        L.hvref_destroy.argtypes = [C.c_void_p]
        L.hvref_push.argtypes = [C.c_void_p, C.c_void_p, C.c_int]
        L.hvref_run_device_batches.restype = C.c_double
        L.hvref_run_device_batches.argtypes = [C.c_void_p, C.POINTER(C.c_void_p), C.c_int, C.c_int]
        L.hvref_outputs.argtypes = [C.c_void_p]
        L.hvref_output.argtypes = [C.c_void_p, C.c_void_p]
        L.hvref_float_frame.argtypes = [C.c_void_p, C.c_void_p]
        L.hvref_contrast_range.argtypes = [C.c_void_p, C.c_void_p]
        L.hvref_ring.argtypes = [C.c_void_p, C.c_void_p, C.POINTER(C.c_int), C.POINTER(C.c_int)]
        L.hvref_eigenvalues.argtypes = [C.c_void_p, C.c_void_p]
        L.hvref_lens.restype = C.c_longlong
        L.hvref_lens.argtypes = [C.c_void_p, C.c_void_p]
        L.hvref_last_error.restype = C.c_char_p
        _LIB = L
    return _LIB


def _check(rc: int, what: str) -> int:
    if rc < 0:
        raise RuntimeError(f"{what}: {lib().hvref_last_error().decode()}")
    return rc


class RefPipe:
    """One Pipe of the reference build. Settings use the oracle's names and units."""

    def __init__(self, width, height, depth, space="NONE", time="NONE", time_transformation_size=1, time_stride=1,
                 batch_size=1, lam=852e-9, z=0.0, pixel_size=12.0, image_type="MODULUS", p_start=0, p_width=0,
                 fft_shift=False, renorm=True, renorm_constant=5, accumulation=0, log_enabled=False,
                 contrast_enabled=True, contrast_invert=False, contrast_lower=0.02, contrast_upper=99.98,
                 unwrap_2d=False, keep_float_frame=True):
        self.cfg = Config(width, height, depth, SPACE[space], TIME[time], time_transformation_size, time_stride,
                          batch_size, lam, z, pixel_size, IMG[image_type], p_start, p_width, int(fft_shift),
                          int(renorm), renorm_constant, accumulation, int(log_enabled), int(contrast_enabled),
                          int(contrast_invert), contrast_lower, contrast_upper, int(unwrap_2d), int(keep_float_frame))
        self.h = lib().hvref_create(C.byref(self.cfg))
        if not self.h:
            raise RuntimeError(f"hvref_create: {lib().hvref_last_error().decode()}")
        self.W, self.H = width, height

    @classmethod
    def from_oracle_settings(cls, s, keep_float_frame=True):
        return cls(s.width, s.height, s.depth, s.space_transformation, s.time_transformation,
                   s.time_transformation_size, s.time_stride, s.batch_size, s.lam, s.z, s.pixel_size, s.image_type,
                   s.p_start, s.p_width, s.fft_shift, s.renorm, s.renorm_constant, s.accumulation, s.log_enabled,
                   s.contrast_enabled, s.contrast_invert, s.contrast_lower, s.contrast_upper, s.unwrap_2d,
                   keep_float_frame)

    def close(self):
        if self.h:
            lib().hvref_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def push(self, batch: np.ndarray) -> bool:
        """One host batch through one cycle; True when a hologram was produced."""
        a = np.ascontiguousarray(batch)
        return bool(_check(lib().hvref_push(self.h, a.ctypes.data, 0), "hvref_push"))

    def push_device(self, ptr: int) -> bool:
        return bool(_check(lib().hvref_push(self.h, ptr, 1), "hvref_push"))

    def run_device_batches(self, ptrs: list[int], count: int) -> float:
        arr = (C.c_void_p * len(ptrs))(*ptrs)
        ms = lib().hvref_run_device_batches(self.h, arr, len(ptrs), count)
        if ms < 0:
            raise RuntimeError(f"hvref_run_device_batches: {lib().hvref_last_error().decode()}")
        return ms

    def output(self) -> np.ndarray:
        out = np.empty((self.H, self.W), np.uint16)
        _check(lib().hvref_output(self.h, out.ctypes.data), "hvref_output")
        return out

    def float_frame(self) -> np.ndarray:
        out = np.empty((self.H, self.W), np.float32)
        _check(lib().hvref_float_frame(self.h, out.ctypes.data), "hvref_float_frame")
        return out

    def contrast_range(self) -> tuple[float, float]:
        r = np.empty(2, np.float32)
        lib().hvref_contrast_range(self.h, r.ctypes.data)
        return float(r[0]), float(r[1])

    def ring(self):
        T = self.cfg.time_transformation_size
        out = np.empty((T, self.H, self.W), np.complex64)
        st, sz = C.c_int(), C.c_int()
        _check(lib().hvref_ring(self.h, out.ctypes.data, C.byref(st), C.byref(sz)), "hvref_ring")
        return out, st.value, sz.value

    def eigenvalues(self) -> np.ndarray:
        out = np.empty(self.cfg.time_transformation_size, np.float32)
        _check(lib().hvref_eigenvalues(self.h, out.ctypes.data), "hvref_eigenvalues")
        return out

    def lens(self) -> np.ndarray | None:
        n = lib().hvref_lens(self.h, None)
        if n <= 0:
            return None
        out = np.empty((self.H, self.W), np.complex64)
        _check(int(lib().hvref_lens(self.h, out.ctypes.data)), "hvref_lens")
        return out
