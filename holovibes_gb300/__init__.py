"""holovibes_gb300: GB300-native Holovibes hologram pipeline (sm_103a CUDA behind a C ABI).

Python mirror of the reference's Pipe / compute-step interface over ctypes. The compute runs
in ``lib/libholovibes_gb300.so``; there is no CPU fallback: every entry point raises when the
library is missing or a CUDA call fails.

    fd = FrameDescriptor(width=512, height=512, depth=2)
    s = Settings.defaults(); s.space_transformation = SPACE_ANGULARSP; ...
    pipe = Pipe(fd, s)
    pipe.enqueue(frames_uint16)        # BatchInputQueue::enqueue
    img = pipe.pull()                  # output Queue dequeue (uint16 H x W)
"""

from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

import numpy as np

from . import _build

# ---------------------------------------------------------------------------------- constants
HV_OK = 0
HV_NO_CHANGE = 1
HV_INVALID_VALUE = 2
HV_NO_IN_DATA = 3
HV_NOT_STARTED = 4
HV_WRONG_COMP_MODE = 5
HV_WRONG_IMG_TYPE = 6
HV_FAILURE = 7
HV_ERR_CUDA = 8
HV_ERR_OOM = 9
HV_ERR_TIMEOUT = 10
HV_ERR_ADMISSION = 11
HV_ERR_UNSUPPORTED = 12
STATUS_NAMES = {
    0: "OK", 1: "NO_CHANGE", 2: "INVALID_VALUE", 3: "NO_IN_DATA", 4: "NOT_STARTED", 5: "WRONG_COMP_MODE",
    6: "WRONG_IMG_TYPE", 7: "FAILURE", 8: "ERR_CUDA", 9: "ERR_OOM", 10: "ERR_TIMEOUT", 11: "ERR_ADMISSION",
    12: "ERR_UNSUPPORTED",
}

SPACE_NONE, SPACE_FRESNELTR, SPACE_ANGULARSP = 0, 1, 2
TIME_NONE, TIME_STFT, TIME_PCA, TIME_SSA_STFT = 0, 1, 2, 3
IMG_MODULUS, IMG_SQUARED_MODULUS, IMG_ARGUMENT, IMG_PHASE_INCREASE = 0, 1, 2, 3
IMG_MOMENTS_0, IMG_MOMENTS_1, IMG_MOMENTS_2 = 5, 6, 7
LENS_FP64, LENS_REF32 = 0, 1
EIG_FP32, EIG_FP64 = 0, 1
MEM_HOST, MEM_DEVICE = 0, 1
VIEW_XZ, VIEW_YZ, VIEW_FILTER2D = 0, 1, 2

SPACE_NAMES = {"NONE": 0, "None": 0, "FRESNELTR": 1, "FFT1": 1, "1FFT": 1, "Fresnel Tr.": 1,
               "ANGULARSP": 2, "FFT2": 2, "2FFT": 2, "Angular SP.": 2}
TIME_NAMES = {"NONE": 0, "None": 0, "STFT": 1, "PCA": 2, "SSA_STFT": 3}
IMG_NAMES = {"MODULUS": 0, "SQUARED_MODULUS": 1, "ARGUMENT": 2}


class HoloError(RuntimeError):
    """A non-OK hv_status from the library (the reference's ApiCode / CUDA failures)."""

    def __init__(self, status: int, what: str):
        self.status = status
        super().__init__(f"{what}: {STATUS_NAMES.get(status, status)}: {last_error()}")


# ---------------------------------------------------------------------------------- structs
class FrameDescriptor(C.Structure):
    """camera::FrameDescriptor (Camera/include/frame_desc.hh:13-48)."""

    _fields_ = [("width", C.c_uint16), ("height", C.c_uint16), ("depth", C.c_uint32), ("byte_endian", C.c_uint32)]

    def __init__(self, width=0, height=0, depth=2, byte_endian=0):
        super().__init__(width, height, depth, byte_endian)

    @property
    def frame_res(self) -> int:
        return int(self.width) * int(self.height)

    @property
    def frame_size(self) -> int:
        return self.frame_res * int(self.depth)


class Settings(C.Structure):
    """Flat record of the compute settings this path reads (include/holovibes_gb300.h hv_settings)."""

    _fields_ = [
        ("space_transformation", C.c_int32), ("time_transformation", C.c_int32),
        ("time_transformation_size", C.c_int32), ("time_stride", C.c_int32), ("batch_size", C.c_int32),
        ("lambda_", C.c_float), ("z_distance", C.c_float), ("pixel_size", C.c_float), ("image_type", C.c_int32),
        ("p_start", C.c_int32), ("p_width", C.c_int32), ("fft_shift", C.c_int32), ("renorm", C.c_int32),
        ("renorm_constant", C.c_int32), ("accumulation", C.c_int32), ("log_enabled", C.c_int32),
        ("contrast_enabled", C.c_int32), ("contrast_auto_refresh", C.c_int32), ("contrast_invert", C.c_int32),
        ("contrast_min", C.c_float), ("contrast_max", C.c_float), ("contrast_lower", C.c_float),
        ("contrast_upper", C.c_float), ("reticle_display", C.c_int32), ("reticle_scale", C.c_float),
        ("unwrap_2d", C.c_int32), ("lens_mode", C.c_int32), ("output_buffer_size", C.c_int32),
        ("input_buffer_size", C.c_int32),
        ("camera_fps", C.c_int32),
        ("q_start", C.c_int32),
        ("q_width", C.c_int32),
        ("filter2d_enabled", C.c_int32),
        ("filter2d_n1", C.c_int32),
        ("filter2d_n2", C.c_int32),
        ("filter2d_smooth_low", C.c_int32),
        ("filter2d_smooth_high", C.c_int32),
        ("cuts_enabled", C.c_int32),
        ("x_start", C.c_int32),
        ("x_width", C.c_int32),
        ("y_start", C.c_int32),
        ("y_width", C.c_int32),
        ("xz_accumulation", C.c_int32),
        ("yz_accumulation", C.c_int32),
        ("xz_log_enabled", C.c_int32),
        ("yz_log_enabled", C.c_int32),
        ("xz_contrast_enabled", C.c_int32),
        ("xz_contrast_auto_refresh", C.c_int32),
        ("xz_contrast_invert", C.c_int32),
        ("xz_contrast_min", C.c_float),
        ("xz_contrast_max", C.c_float),
        ("yz_contrast_enabled", C.c_int32),
        ("yz_contrast_auto_refresh", C.c_int32),
        ("yz_contrast_invert", C.c_int32),
        ("yz_contrast_min", C.c_float),
        ("yz_contrast_max", C.c_float),
        ("cuts_contrast_offset", C.c_int32),
        ("cuts_buffer_size", C.c_int32),
        ("filter2d_view_enabled", C.c_int32),
        ("filter2d_log_enabled", C.c_int32),
        ("filter2d_contrast_enabled", C.c_int32),
        ("filter2d_contrast_auto_refresh", C.c_int32),
        ("filter2d_contrast_invert", C.c_int32),
        ("filter2d_contrast_min", C.c_float),
        ("filter2d_contrast_max", C.c_float),
    ]

    @classmethod
    def defaults(cls) -> "Settings":
        s = cls()
        lib().hv_settings_default(C.byref(s))
        return s

    @classmethod
    def from_json(cls, text: str, base: "Settings | None" = None) -> "Settings":
        """ComputeSettingsApi::load_compute_settings (compute_settings.cc:66-99): partial merge."""
        s = cls() if base is None else base.copy()
        if base is None:
            lib().hv_settings_default(C.byref(s))
        check(lib().hv_settings_from_json(text.encode(), C.byref(s)), "hv_settings_from_json")
        return s

    def copy(self) -> "Settings":
        s = Settings()
        C.memmove(C.byref(s), C.byref(self), C.sizeof(Settings))
        return s

    def validate(self, fd: FrameDescriptor | None = None) -> "Settings":
        s = self.copy()
        check(lib().hv_settings_validate(C.byref(s), C.byref(fd) if fd is not None else None), "hv_settings_validate")
        return s

    def as_dict(self) -> dict:
        return {name: getattr(self, name) for name, _ in self._fields_}

    def update(self, **kw) -> "Settings":
        for k, v in kw.items():
            if k == "lambda":
                k = "lambda_"
            if not hasattr(self, k):
                raise AttributeError(k)
            setattr(self, k, v)
        return self


# ---------------------------------------------------------------------------------- library
_LIB = None


def lib_path() -> Path:
    return _build.lib_path()


def lib() -> C.CDLL:
    """Loads the in-tree shared library (building it first if it is absent)."""
    global _LIB
    if _LIB is not None:
        return _LIB
    path = lib_path()
    if not path.exists():
        if os.environ.get("HV_NO_BUILD"):
            raise RuntimeError(f"{path} is missing; run __graft_entry__.build()")
        _build.build_library()
    L = C.CDLL(str(path))
    _declare(L)
    _LIB = L
    return L


def _declare(L: C.CDLL) -> None:
    vp, sz, i32, f32, i64, u64, u32 = C.c_void_p, C.c_size_t, C.c_int, C.c_float, C.c_int64, C.c_uint64, C.c_uint
    st = C.c_int
    sig = {
        "hv_version": (C.c_char_p, []),
        "hv_last_error": (C.c_char_p, []),
        "hv_kernel_launches": (u64, []),
        "hv_settings_default": (None, [C.POINTER(Settings)]),
        "hv_settings_from_json": (st, [C.c_char_p, C.POINTER(Settings)]),
        "hv_settings_validate": (st, [C.POINTER(Settings), C.POINTER(FrameDescriptor)]),
        "hv_pipe_create": (vp, [C.POINTER(FrameDescriptor), C.POINTER(Settings), vp, C.POINTER(C.c_int)]),
        "hv_pipe_destroy": (None, [vp]),
        "hv_pipe_footprint": (sz, [C.POINTER(FrameDescriptor), C.POINTER(Settings)]),
        "hv_pipe_push_frames": (st, [vp, vp, sz, i32]),
        "hv_pipe_output_count": (sz, [vp]),
        "hv_pipe_pull_output": (st, [vp, vp, i32, i64]),
        "hv_pipe_update_settings": (st, [vp, C.POINTER(Settings)]),
        "hv_pipe_request_autocontrast": (st, [vp]),
        "hv_pipe_sync": (st, [vp]),
        "hv_pipe_join": (st, [vp]),
        "hv_pipe_get_contrast_range": (st, [vp, C.POINTER(C.c_float), C.POINTER(C.c_float)]),
        "hv_pipe_get_float_frame": (st, [vp, vp]),
        "hv_pipe_view_output_count": (sz, [vp, i32]),
        "hv_pipe_pull_view": (st, [vp, i32, vp, i32, i64]),
        "hv_pipe_get_view_float_frame": (st, [vp, i32, vp, vp]),
        "hv_time_cuts": (st, [vp, i32, i32, i32, vp, i32, i32, i32, i32, i32, vp, vp, vp, vp]),
        "hv_time_cuts_workspace": (sz, [i32, i32, i32, i32, i32, i32, i32]),
        "hv_pipe_get_ring": (st, [vp, vp, C.POINTER(C.c_int32), C.POINTER(C.c_int32)]),
        "hv_pipe_kernel_launches": (u64, [vp]),
        "hv_pipe_stream": (vp, [vp]),
        "hv_fft_size_supported": (i32, [i32]),
        "hv_fft_engine_mode": (None, [i32]),
        "hv_fft_status": (st, []),
        "hv_spatial_sub_batch_mb": (None, [i32]),
        "hv_fresnel_lens": (st, [vp, i32, i32, f32, f32, f32, i32, vp]),
        "hv_angular_spectrum_lens": (st, [vp, i32, i32, f32, f32, f32, i32, vp]),
        "hv_spatial_transform": (st, [vp, i32, i32, i32, i32, i32, i32, vp, vp, vp, i32, i32, vp]),
        "hv_filter2d_mask": (st, [vp, i32, i32, i32, i32, i32, i32, i32, vp]),
        "hv_spatial_transform_filter2d": (st, [vp, i32, i32, i32, i32, i32, i32, vp, vp, vp, vp, vp, i32, i32, vp]),
        "hv_fft2d": (st, [vp, vp, i32, i32, i32, i32, f32, vp]),
        "hv_fft_rows": (st, [vp, i32, i32, vp, i32, i32, i32, vp, i32, f32, i32, i32, vp]),
        "hv_fft_cols": (st, [vp, vp, i32, i32, i32, vp, i32, f32, i32, i32, vp]),
        "hv_time_view": (st, [vp, i32, i32, i32, vp, i32, i32, f32, i32, vp, vp, vp]),
        "hv_time_view_partials": (i32, [i32, i32]),
        "hv_time_view_planes": (st, [vp, vp, i32, i32, i32, i32, i32, vp, i32, i32, f32, i32, vp, vp, vp]),
        "hv_time_view_tc": (st, [vp, i32, i32, i32, vp, i32, i32, f32, i32, vp, vp, vp, vp]),
        "hv_time_view_tc_prepare": (st, [vp, i32, i32, vp, vp]),
        "hv_time_view_tc_run": (st, [vp, i32, i32, i32, i32, i32, f32, i32, vp, vp, vp, vp]),
        "hv_time_view_tc_workspace": (sz, [i32, i32]),
        "hv_time_view_tc_status": (st, [vp]),
        "hv_time_view_mode": (None, [i32]),
        "hv_unpack_12_to_16": (st, [vp, sz, vp, sz, vp]),
        "hv_unpack_10_to_16": (st, [vp, sz, vp, sz, vp]),
        "hv_moment_bin_weights": (st, [vp, i32, i32, i32, i32, f32, vp]),
        "hv_time_moments": (st, [vp, i32, i32, i32, vp, i32, vp, i32, vp, vp, vp]),
        "hv_stft_weights": (st, [vp, i32, i32, i32, vp]),
        "hv_ssa_weights": (st, [vp, i32, i32, i32, i32, i32, vp, vp]),
        "hv_phase_increase": (st, [vp, i32, i32, i32, vp, vp, vp, i32, i32, vp, vp, vp]),
        "hv_phase_increase_workspace": (sz, [sz]),
        "hv_rescale_float": (st, [vp, sz, vp, f32, vp, vp]),
        "hv_pca_covariance": (st, [vp, i32, sz, vp, vp, vp]),
        "hv_pca_cov_workspace": (sz, [i32, sz]),
        "hv_pca_covariance_mode": (None, [i32]),
        "hv_pca_cov_incremental": (None, [i32]),
        "hv_pca_planes_bytes": (sz, [i32, sz, i32]),
        "hv_pca_split_planes": (st, [vp, i32, sz, i32, i32, i32, vp, vp]),
        "hv_pca_covariance_planes": (st, [vp, i32, sz, i32, u32, vp, vp, vp]),
        "hv_pca_covariance_status": (st, [vp]),
        "hv_pca_eigh": (st, [vp, i32, vp, vp, i32, i32, vp, vp, vp]),
        "hv_pca_eigh_workspace": (sz, [i32]),
        "hv_pca_eig_precision": (None, [i32]),
        "hv_pca_eig_cholqr": (None, [i32]),
        "hv_unwrap_2d": (st, [vp, vp, i32, i32, vp, vp]),
        "hv_unwrap_workspace": (sz, [i32, i32]),
        "hv_unwrap_2d_noalloc": (st, [vp, vp, i32, i32, vp]),
        "hv_renormalize": (st, [vp, sz, i32, vp, i32, vp, vp]),
        "hv_reduce_workspace": (sz, [sz]),
        "hv_shift_corners": (st, [vp, i32, i32, vp]),
        "hv_accumulate": (st, [vp, vp, i32, i32, i32, i32, vp, sz, vp]),
        "hv_log10": (st, [vp, sz, vp]),
        "hv_percentile": (st, [vp, i32, i32, f32, f32, f32, vp, vp, vp]),
        "hv_percentile_workspace": (sz, [sz]),
        "hv_contrast_to_ushort": (st, [vp, vp, i32, i32, vp, sz, vp]),
        "hv_server_create": (vp, [sz, i32, C.POINTER(C.c_int)]),
        "hv_server_destroy": (None, [vp]),
        "hv_server_stream_footprint": (sz, [C.POINTER(FrameDescriptor), C.POINTER(Settings)]),
        "hv_server_open_stream": (st, [vp, C.POINTER(FrameDescriptor), C.POINTER(Settings), i64,
                                       C.POINTER(C.c_int32)]),
        "hv_server_close_stream": (st, [vp, C.c_int32]),
        "hv_server_push": (st, [vp, C.c_int32, vp, sz, i32]),
        "hv_server_output_count": (sz, [vp, C.c_int32]),
        "hv_server_pull": (st, [vp, C.c_int32, vp, i32, i64]),
        "hv_server_get_float_frame": (st, [vp, C.c_int32, vp]),
        "hv_server_sync": (st, [vp, i64]),
        "hv_server_get_stats": (st, [vp, C.POINTER(ServerStats)]),
        "hv_server_reset_stats": (st, [vp]),
        "hv_server_set_batch_window": (st, [vp, i64]),
        "hv_holo_open": (st, [C.c_char_p, C.POINTER(vp)]),
        "hv_holo_close": (None, [vp]),
        "hv_holo_get_header": (st, [vp, C.POINTER(HoloHeader), C.POINTER(FrameDescriptor)]),
        "hv_holo_read_frames": (st, [vp, u64, u64, vp]),
        "hv_holo_get_footer": (st, [vp, C.c_char_p, sz, C.POINTER(sz)]),
        "hv_holo_get_settings": (st, [vp, C.POINTER(Settings)]),
        "hv_holo_create": (st, [C.c_char_p, C.POINTER(FrameDescriptor), i32, C.POINTER(vp)]),
        "hv_holo_write_frames": (st, [vp, vp, u64]),
        "hv_holo_finish": (st, [vp, C.c_char_p]),
        "hv_holo_make_footer": (st, [C.POINTER(Settings), i32, i32, C.c_char_p, sz, C.POINTER(sz)]),
        "hv_holo_convert_footer": (st, [C.c_char_p, i32, C.c_char_p, sz, C.POINTER(sz)]),
        "hv_settings_to_json": (st, [C.POINTER(Settings), C.c_char_p, sz, C.POINTER(sz)]),
        "hv_settings_convert_json": (st, [C.c_char_p, C.c_char_p, sz, C.POINTER(sz)]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args


def last_error() -> str:
    if _LIB is None:
        return ""
    msg = _LIB.hv_last_error()
    return msg.decode() if msg else ""


def check(status: int, what: str) -> int:
    if status not in (HV_OK, HV_NO_CHANGE):
        raise HoloError(status, what)
    return status


def version() -> str:
    return lib().hv_version().decode()


def kernel_launches() -> int:
    return int(lib().hv_kernel_launches())


def fft_size_supported(n: int) -> bool:
    return bool(lib().hv_fft_size_supported(n))


def fft_engine_mode(mode: int) -> None:
    """Engine of the 512/768/1024-point spatial FFT passes: 0 automatic (warp engine, TMA-fed
    1024-point passes), 1 tile engine, 2 warp engine with register-loading passes only."""
    lib().hv_fft_engine_mode(int(mode))


def spatial_sub_batch_mb(mb: int) -> None:
    """Spatial-stage batching: 0 one launch per pass (default), n > 0 sub-batches of <= n MB."""
    lib().hv_spatial_sub_batch_mb(int(mb))


# ---------------------------------------------------------------------------------- Pipe
class Pipe:
    """Drop-in for the reference's Pipe (Backend/includes/core/pipe.hh:70-125): raw frames in,
    uint16 holograms out, settings applied at cycle boundaries."""

    def __init__(self, fd: FrameDescriptor, settings: Settings, stream: int | None = None):
        self.fd = fd
        self.settings = settings.copy()
        status = C.c_int(0)
        self._p = lib().hv_pipe_create(C.byref(fd), C.byref(self.settings), stream, C.byref(status))
        if not self._p:
            raise HoloError(status.value, "hv_pipe_create")

    def close(self) -> None:
        if getattr(self, "_p", None):
            lib().hv_pipe_destroy(self._p)
            self._p = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    @staticmethod
    def footprint(fd: FrameDescriptor, settings: Settings) -> int:
        return int(lib().hv_pipe_footprint(C.byref(fd), C.byref(settings)))

    @property
    def stream(self) -> int:
        return lib().hv_pipe_stream(self._p)

    def enqueue(self, frames) -> None:
        """BatchInputQueue::enqueue: numpy array (host) of n frames, or an object with
        ``data_ptr()`` and ``is_cuda`` (device memory, consumed in place)."""
        if hasattr(frames, "data_ptr") and getattr(frames, "is_cuda", False):
            n = frames.numel() * frames.element_size() // self.fd.frame_size
            check(lib().hv_pipe_push_frames(self._p, frames.data_ptr(), n, MEM_DEVICE), "hv_pipe_push_frames")
            return
        arr = np.ascontiguousarray(frames)
        n = arr.nbytes // self.fd.frame_size
        check(lib().hv_pipe_push_frames(self._p, arr.ctypes.data, n, MEM_HOST), "hv_pipe_push_frames")

    def enqueue_ptr(self, ptr: int, n: int, mem: int) -> None:
        check(lib().hv_pipe_push_frames(self._p, ptr, n, mem), "hv_pipe_push_frames")

    def output_count(self) -> int:
        return int(lib().hv_pipe_output_count(self._p))

    def pull(self, timeout_us: int = 10_000_000) -> np.ndarray:
        out = np.empty((self.fd.height, self.fd.width), dtype=np.uint16)
        check(lib().hv_pipe_pull_output(self._p, out.ctypes.data, MEM_HOST, timeout_us), "hv_pipe_pull_output")
        return out

    def pull_into(self, ptr: int, mem: int, timeout_us: int = 10_000_000) -> None:
        check(lib().hv_pipe_pull_output(self._p, ptr, mem, timeout_us), "hv_pipe_pull_output")

    def pull_all(self) -> list[np.ndarray]:
        out = []
        while self.output_count() > 0:
            out.append(self.pull())
        return out

    def update_settings(self, settings: Settings) -> int:
        st = lib().hv_pipe_update_settings(self._p, C.byref(settings))
        check(st, "hv_pipe_update_settings")
        if st == HV_OK:
            self.settings = settings.copy()
        return st

    def request_autocontrast(self) -> None:
        check(lib().hv_pipe_request_autocontrast(self._p), "hv_pipe_request_autocontrast")

    def sync(self) -> None:
        check(lib().hv_pipe_sync(self._p), "hv_pipe_sync")

    def join(self) -> None:
        """Make the pipe's stream wait on the device for all rendering enqueued so far."""
        check(lib().hv_pipe_join(self._p), "hv_pipe_join")

    def contrast_range(self) -> tuple[float, float]:
        lo, hi = C.c_float(), C.c_float()
        check(lib().hv_pipe_get_contrast_range(self._p, C.byref(lo), C.byref(hi)), "hv_pipe_get_contrast_range")
        return lo.value, hi.value

    def float_frame(self) -> np.ndarray:
        out = np.empty((self.fd.height, self.fd.width), dtype=np.float32)
        check(lib().hv_pipe_get_float_frame(self._p, out.ctypes.data), "hv_pipe_get_float_frame")
        return out

    def _view_shape(self, which: int) -> tuple[int, int]:
        T = self.settings.time_transformation_size
        if which == VIEW_XZ:
            return T, self.fd.width
        if which == VIEW_YZ:
            return self.fd.height, T
        return self.fd.height, self.fd.width

    def view_output_count(self, which: int) -> int:
        return int(lib().hv_pipe_view_output_count(self._p, which))

    def pull_view(self, which: int, timeout_us: int = 10_000_000) -> np.ndarray:
        """Oldest uint16 output of a secondary view: XZ (T x W), YZ (H x T) or filter2D (H x W)."""
        out = np.empty(self._view_shape(which), dtype=np.uint16)
        check(lib().hv_pipe_pull_view(self._p, which, out.ctypes.data, MEM_HOST, timeout_us), "hv_pipe_pull_view")
        return out

    def view_float_frame(self, which: int) -> tuple[np.ndarray, tuple[float, float]]:
        out = np.empty(self._view_shape(which), dtype=np.float32)
        rng = (C.c_float * 2)()
        check(lib().hv_pipe_get_view_float_frame(self._p, which, out.ctypes.data, rng),
              "hv_pipe_get_view_float_frame")
        return out, (rng[0], rng[1])

    def ring(self) -> tuple[np.ndarray, int, int]:
        T = self.settings.time_transformation_size
        out = np.empty((T, self.fd.height, self.fd.width), dtype=np.complex64)
        a, b = C.c_int32(), C.c_int32()
        check(lib().hv_pipe_get_ring(self._p, out.ctypes.data, C.byref(a), C.byref(b)), "hv_pipe_get_ring")
        return out, a.value, b.value

    def kernel_launches(self) -> int:
        return int(lib().hv_pipe_kernel_launches(self._p))


SERVER_NO_GRAPHS = 1
SERVER_STREAM_GRAPHS = 2
HOLO_RAW, HOLO_PROCESSED, HOLO_MOMENTS = 0, 1, 2


class HoloHeader(C.Structure):
    _fields_ = [("magic", C.c_char * 4), ("version", C.c_uint16), ("bits_per_pixel", C.c_uint16),
                ("width", C.c_uint32), ("height", C.c_uint32), ("img_nb", C.c_uint32),
                ("total_data_size", C.c_uint64), ("endianness", C.c_uint8), ("data_type", C.c_uint8)]


def _string_call(name: str, *args) -> str:
    """Calls an entry point that returns a string into a caller buffer (query, then fill)."""
    n = C.c_size_t(0)
    check(getattr(lib(), name)(*args, None, 0, C.byref(n)), name)
    buf = C.create_string_buffer(n.value + 1)
    check(getattr(lib(), name)(*args, buf, n.value + 1, C.byref(n)), name)
    return buf.value.decode()


class HoloFile:
    """A .holo recording (Backend/includes/io/holo_file.hh), footer converted to the current version."""

    def __init__(self, path: str):
        h = C.c_void_p()
        check(lib().hv_holo_open(str(path).encode(), C.byref(h)), "hv_holo_open")
        self._h = h
        self.header = HoloHeader()
        self.fd = FrameDescriptor()
        check(lib().hv_holo_get_header(self._h, C.byref(self.header), C.byref(self.fd)), "hv_holo_get_header")

    @property
    def nb_frames(self) -> int:
        return int(self.header.img_nb)

    def read(self, first: int = 0, n: int | None = None) -> np.ndarray:
        n = self.nb_frames - first if n is None else n
        dt = {1: np.uint8, 2: np.uint16, 4: np.float32}.get(self.fd.depth, np.uint8)
        out = np.empty((n, self.fd.height, self.fd.width * self.fd.depth // np.dtype(dt).itemsize), dtype=dt)
        check(lib().hv_holo_read_frames(self._h, first, n, out.ctypes.data), "hv_holo_read_frames")
        return out

    def footer(self) -> dict:
        import json as _json
        return _json.loads(_string_call("hv_holo_get_footer", self._h))

    def settings(self, base: "Settings | None" = None) -> "Settings":
        s = (base or Settings.defaults()).copy()
        check(lib().hv_holo_get_settings(self._h, C.byref(s)), "hv_holo_get_settings")
        return s

    def close(self) -> None:
        if getattr(self, "_h", None):
            lib().hv_holo_close(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def write_holo(path: str, fd: FrameDescriptor, frames, settings: "Settings | None" = None, input_fps: int = 0,
               camera_fps: int = 0, data_type: int = HOLO_RAW, footer: str | None = None) -> None:
    """Writes frames (numpy, n x H x W of fd.depth bytes per pixel) with the reference's footer."""
    w = C.c_void_p()
    check(lib().hv_holo_create(str(path).encode(), C.byref(fd), data_type, C.byref(w)), "hv_holo_create")
    arr = np.ascontiguousarray(frames)
    n = arr.nbytes // fd.frame_size
    st = lib().hv_holo_write_frames(w, arr.ctypes.data, n)
    if footer is None and settings is not None:
        footer = _string_call("hv_holo_make_footer", C.byref(settings), input_fps, camera_fps)
    st2 = lib().hv_holo_finish(w, footer.encode() if footer else None)
    check(st, "hv_holo_write_frames")
    check(st2, "hv_holo_finish")


def convert_holo_footer(footer_json: str, version: int) -> str:
    return _string_call("hv_holo_convert_footer", footer_json.encode(), version)


def settings_to_json(settings: "Settings") -> str:
    return _string_call("hv_settings_to_json", C.byref(settings))


def convert_settings_json(text: str) -> str:
    return _string_call("hv_settings_convert_json", text.encode())



class ServerStats(C.Structure):
    _fields_ = [("batches", C.c_uint64), ("outputs", C.c_uint64), ("graph_launches", C.c_uint64),
                ("graph_kernels", C.c_uint64), ("eager_cycles", C.c_uint64), ("captures", C.c_uint64),
                ("latency_samples", C.c_uint64), ("latency_p50_us", C.c_double), ("latency_p99_us", C.c_double),
                ("streams", C.c_int32), ("buckets", C.c_int32), ("hbm_used", C.c_size_t), ("hbm_budget", C.c_size_t)]

    def as_dict(self) -> dict:
        return {k: getattr(self, k) for k, _ in self._fields_}


class ServedStream:
    """One frame stream of a Server: same settings, kernels and outputs as a Pipe."""

    def __init__(self, server: "Server", sid: int, fd: FrameDescriptor, settings: Settings):
        self.server, self.id, self.fd, self.settings = server, sid, fd, settings

    def enqueue(self, frames) -> None:
        if hasattr(frames, "data_ptr"):
            mem = MEM_DEVICE if getattr(frames, "is_cuda", False) else MEM_HOST
            n = frames.numel() * frames.element_size() // self.fd.frame_size
            check(lib().hv_server_push(self.server._s, self.id, frames.data_ptr(), n, mem), "hv_server_push")
            return
        arr = np.ascontiguousarray(frames)
        n = arr.nbytes // self.fd.frame_size
        check(lib().hv_server_push(self.server._s, self.id, arr.ctypes.data, n, MEM_HOST), "hv_server_push")

    def enqueue_ptr(self, ptr: int, n: int, mem: int) -> None:
        check(lib().hv_server_push(self.server._s, self.id, ptr, n, mem), "hv_server_push")

    def output_count(self) -> int:
        return int(lib().hv_server_output_count(self.server._s, self.id))

    def pull(self, timeout_us: int = 10_000_000) -> np.ndarray:
        out = np.empty((self.fd.height, self.fd.width), dtype=np.uint16)
        check(lib().hv_server_pull(self.server._s, self.id, out.ctypes.data, MEM_HOST, timeout_us), "hv_server_pull")
        return out

    def pull_into(self, ptr: int, mem: int, timeout_us: int = 10_000_000) -> None:
        check(lib().hv_server_pull(self.server._s, self.id, ptr, mem, timeout_us), "hv_server_pull")

    def float_frame(self) -> np.ndarray:
        out = np.empty((self.fd.height, self.fd.width), dtype=np.float32)
        check(lib().hv_server_get_float_frame(self.server._s, self.id, out.ctypes.data), "hv_server_get_float_frame")
        return out

    def close(self) -> None:
        if self.id is not None:
            check(lib().hv_server_close_stream(self.server._s, self.id), "hv_server_close_stream")
            self.id = None


class Server:
    """Serving engine: streams admitted by HBM footprint, grouped in shape buckets, cycles launched
    by one engine thread (one CUDA graph launch per bucket for the steady streams)."""

    def __init__(self, hbm_budget: int = 0, flags: int = 0):
        status = C.c_int(0)
        self._s = lib().hv_server_create(hbm_budget, flags, C.byref(status))
        if not self._s:
            raise HoloError(status.value, "hv_server_create")

    @staticmethod
    def footprint(fd: FrameDescriptor, settings: Settings) -> int:
        return int(lib().hv_server_stream_footprint(C.byref(fd), C.byref(settings)))

    def open_stream(self, fd: FrameDescriptor, settings: Settings, admit_timeout_us: int = 0) -> ServedStream:
        sid = C.c_int32(0)
        st = settings.copy()
        check(lib().hv_server_open_stream(self._s, C.byref(fd), C.byref(st), admit_timeout_us, C.byref(sid)),
              "hv_server_open_stream")
        return ServedStream(self, sid.value, fd, st)

    def sync(self, timeout_us: int = 30_000_000) -> None:
        check(lib().hv_server_sync(self._s, timeout_us), "hv_server_sync")

    def stats(self) -> dict:
        out = ServerStats()
        check(lib().hv_server_get_stats(self._s, C.byref(out)), "hv_server_get_stats")
        return out.as_dict()

    def reset_stats(self) -> None:
        check(lib().hv_server_reset_stats(self._s), "hv_server_reset_stats")

    def set_batch_window(self, window_us: int) -> None:
        check(lib().hv_server_set_batch_window(self._s, window_us), "hv_server_set_batch_window")

    def close(self) -> None:
        if getattr(self, "_s", None):
            lib().hv_server_destroy(self._s)
            self._s = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


__all__ = [n for n in dir() if not n.startswith("_")]
