"""FP64 CPU oracle of the Holovibes hologram path. TEST INFRASTRUCTURE ONLY.

This module is the checker: only ``tests/``, ``__graft_entry__.smoke()`` and the
``cpu_baseline`` / ``--impl reference`` legs of ``bench.py`` import it. The product
(``holovibes_gb300``) never imports it and has no CPU fallback.

It restates, in numpy complex128 / float64, the equations of the reference's hot path
(raw frames -> complex -> spatial propagation -> time ring -> STFT bins / PCA -> view ->
unwrap -> renorm -> fftshift -> accumulation -> percentile contrast -> uint16). Every
function cites the reference file:line it follows (paths relative to the Holovibes tree).

Parity status: pinned against the reference's own GPU build. The reference's test data are
Git-LFS pointers with no committed ``R_ref.holo`` outputs, so there are no golden vectors; instead
``oracle/ref_build.py`` compiles the reference's hot-path translation units unmodified (cuFFT,
cuBLAS Cgemm3m, cuSOLVER Cheevd, thrust) with ``oracle/ref_pipe.cu`` replaying one Pipe cycle, and
``tests/test_reference_build_gpu.py`` runs it on the same seeded interferograms as this module at
the benchmark sizes: the float frame fed to the contrast stage agrees within rel-L2 ~1e-6 (7e-6
for the T = 512 PCA), the ring within ~2e-7, and this module's contrast / percentile / uint16
stages applied to the reference's own float frame reproduce its contrast range and uint16 frame
exactly. ``tests/test_library_anchor_gpu.py`` also replays the reference's library call
sequences through torch's cuFFT / cuBLAS / cuSOLVER and a device sort.

Stages that the reference computes in float32 on the host/GPU with integer or float
truncation (percentile index, contrast factor, float->ushort) are restated here in
float32 with the same operation order, so that uint16 output can be compared bit for
bit when the float input frame is identical.
"""

from __future__ import annotations

import math
import os
from dataclasses import dataclass, field

import numpy as np

try:  # multi-threaded pocketfft when scipy is present (FFTW is not available on these hosts)
    import scipy.fft as _sfft
except ImportError:  # pragma: no cover
    _sfft = None

F32 = np.float32
FFT_WORKERS = int(os.environ.get("HV_ORACLE_FFT_WORKERS", "0")) or (os.cpu_count() or 1)


def fft2(a: np.ndarray, axes=(-2, -1)) -> np.ndarray:
    if _sfft is not None:
        return _sfft.fft2(a, axes=axes, workers=FFT_WORKERS)
    return np.fft.fft2(a, axes=axes)


def ifft2(a: np.ndarray, axes=(-2, -1)) -> np.ndarray:
    """Normalised inverse (1/N), like numpy.fft.ifft2."""
    if _sfft is not None:
        return _sfft.ifft2(a, axes=axes, workers=FFT_WORKERS)
    return np.fft.ifft2(a, axes=axes)

# ----------------------------------------------------------------------------------------
# a1: raw -> complex  (Backend/cuda_sources/tools_conversion.cu:107-171)
# ----------------------------------------------------------------------------------------


def convert_frames(raw: np.ndarray) -> np.ndarray:
    """u8 -> x*257, u16 -> x, f32 -> x; imaginary part 0 (tools_conversion.cu:134-145)."""
    if raw.dtype == np.uint8:
        return raw.astype(np.float64) * 257.0 + 0j
    if raw.dtype == np.uint16:
        return raw.astype(np.float64) + 0j
    if raw.dtype == np.float32:
        return raw.astype(np.float64) + 0j
    raise TypeError(f"unsupported raw dtype {raw.dtype}")


def unpack_12_to_16(packed: np.ndarray, n: int) -> np.ndarray:
    """unpack_12_to_16bit (unpack.cu:4-16): 12-bit pairs in 3 bytes, MSB first, left-aligned in 16 bits."""
    b = np.zeros(((n + 1) // 2) * 3, np.uint32)
    b[:min(len(packed), len(b))] = packed[:len(b)]
    b0, b1, b2 = b[0::3], b[1::3], b[2::3]
    out = np.empty(((n + 1) // 2) * 2, np.uint32)
    out[0::2] = (b0 << 8) | (b1 & 0xF0)
    out[1::2] = ((b1 & 0x0F) << 12) | (b2 << 4)
    return (out[:n] & 0xFFFF).astype(np.uint16)


def unpack_10_to_16(packed: np.ndarray, n: int) -> np.ndarray:
    """unpack_10_to_16bit (unpack.cu:18-32): 10-bit quadruples in 5 bytes, MSB first, left-aligned."""
    g = (n + 3) // 4
    b = np.zeros(g * 5, np.uint32)
    b[:min(len(packed), len(b))] = packed[:len(b)]
    b0, b1, b2, b3, b4 = (b[i::5] for i in range(5))
    out = np.empty(g * 4, np.uint32)
    out[0::4] = (b0 << 8) | (b1 & 0xC0)
    out[1::4] = ((b1 & 0x3F) << 10) | ((b2 & 0xF0) << 2)
    out[2::4] = ((b2 & 0x0F) << 12) | ((b3 & 0xFC) << 4)
    out[3::4] = ((b3 & 0x03) << 14) | (b4 << 6)
    return (out[:n] & 0xFFFF).astype(np.uint16)


def byteswap16(raw: np.ndarray) -> np.ndarray:
    """Big-endian 16-bit input (Backend/sources/data_struct/queue.cc:191-202, tools_conversion.cu endianness_conversion)."""
    return ((raw.astype(np.uint16) << 8) | (raw.astype(np.uint16) >> 8)).astype(np.uint16)


# ----------------------------------------------------------------------------------------
# a2: Fresnel quadratic lens (Backend/cuda_sources/masks.cu:7-29, fresnel_transform.cu:14-63)
# ----------------------------------------------------------------------------------------


def fma32(a, b, c) -> np.ndarray:
    """fmaf(a, b, c) on float32 arrays: the exact a*b + c rounded once to float32 (the product of
    two float32 values is exact in the extended format, and the sum is rounded once more there
    before the final rounding, which can differ from a single rounding only on exact ties)."""
    ld = np.longdouble
    r = np.asarray(a, F32).astype(ld) * np.asarray(b, F32).astype(ld) + np.asarray(c, F32).astype(ld)
    return np.asarray(r.astype(F32))


def _crop_square(square: np.ndarray, W: int, H: int) -> np.ndarray:
    """Centre crop of the max(W,H) square lens (fresnel_transform.cu:37-62)."""
    S = square.shape[0]
    if W == H:
        return square
    if W > H:  # contiguous rows starting at row (S-H)/2
        r0 = (S - H) // 2
        return square[r0:r0 + H, :W]
    c0 = (S - W) // 2  # H > W: row-by-row copy with a column offset
    return square[:H, c0:c0 + W]


def fresnel_lens(W: int, H: int, lam: float, z: float, pixel_size_um: float, mode: str = "fp64") -> np.ndarray:
    """L[j,i] = exp(i*pi/(lam*z)*(x^2+y^2)), x=(i-S/2)*dx, dx = pixel_size*1e-6 on the S=max(W,H) square.

    mode "fp64": the exact phase in float64. mode "ref32": the reference's float32 expression
    (masks.cu:10-27: c = (float)(M_PI/(lam*z)), x = (i - (float)(S>>1))*dx, csquare = c*(x*x+y*y)).
    """
    S = max(W, H)
    idx = np.arange(S)
    # the reference holds lambda, z and the pixel pitch as float32 settings
    lam, z, pixel_size_um = float(F32(lam)), float(F32(z)), float(F32(pixel_size_um))
    if mode == "fp64":
        dx = pixel_size_um * 1e-6
        x = (idx - (S >> 1)) * dx
        c = math.pi / (lam * z)
        ph = c * (x[None, :] ** 2 + x[:, None] ** 2)
        lens = np.exp(1j * ph)
    elif mode == "ref32":
        lam32, z32, ps32 = F32(lam), F32(z), F32(pixel_size_um)
        c = F32(math.pi / float(F32(lam32 * z32)))
        dx = F32(ps32 * F32(1.0e-6))
        x = (idx.astype(F32) - F32(S >> 1)) * dx
        xx = (x * x).astype(F32)
        # x * x + y * y as one fused multiply-add (the reference's compiled form)
        cs = (c * fma32(x[None, :], x[None, :], xx[:, None])).astype(F32)
        lens = np.cos(cs.astype(np.float64)) + 1j * np.sin(cs.astype(np.float64))
    else:
        raise ValueError(mode)
    return _crop_square(lens, W, H)


# ----------------------------------------------------------------------------------------
# a4: angular-spectrum transfer function (masks.cu:31-59, angular_spectrum.cu:14-31,
#     fourier_transform.cc:121-137 (+ shift_corners))
# ----------------------------------------------------------------------------------------


def shift_corners(img: np.ndarray) -> np.ndarray:
    """Quadrant swap of shift_corners.cu:8-44 for even W,H (= fftshift = ifftshift)."""
    H, W = img.shape[-2:]
    if H % 2 or W % 2:
        raise ValueError("shift_corners is a quadrant swap only for even dimensions")
    return np.roll(np.roll(img, H // 2, axis=-2), W // 2, axis=-1)


def angular_spectrum_lens(W: int, H: int, lam: float, z: float, pixel_size_um: float, mode: str = "fp64") -> np.ndarray:
    """G[y,x] = exp(i*2*pi*z/lam*sqrt(max(0, 1-lam^2(u^2+v^2)))), u=(x-W/2)/(W*dx), v=(y-H/2)/(H*dy),
    then quadrant-swapped into FFT layout (fourier_transform.cc:134).

    mode "ref32" follows the float32 expression of masks.cu:43-55: u_step = 1.0f/(Nx*x_step),
    u = (x-(Nx>>1))*u_step, tmp = 1.0f - lam*lam*(u*u+v*v) in float32 with the two fused
    multiply-adds the reference's compiler forms (fmaf(u, u, v*v), then fmaf(-lam^2, s, 1); the
    reference's own build matches this bit for bit), and the phase 2.0f*M_PI*z/lam*sqrtf(tmp)
    evaluated in double (M_PI is a double) then rounded to float32.
    """
    xs = np.arange(W)
    ys = np.arange(H)
    lam, z, pixel_size_um = float(F32(lam)), float(F32(z)), float(F32(pixel_size_um))
    if mode == "fp64":
        step = pixel_size_um * 1e-6
        u = (xs - (W >> 1)) / (W * step)
        v = (ys - (H >> 1)) / (H * step)
        tmp = 1.0 - lam * lam * (u[None, :] ** 2 + v[:, None] ** 2)
        tmp = np.maximum(tmp, 0.0)
        ph = 2.0 * math.pi * z / lam * np.sqrt(tmp)
        # reduce the large phase modulo 2*pi before exponentiation (pure float64 identity)
        G = np.exp(1j * np.mod(ph, 2.0 * math.pi))
    elif mode == "ref32":
        lam32, z32 = F32(lam), F32(z)
        step = F32(F32(pixel_size_um) * F32(1e-6))
        u_step = F32(F32(1.0) / F32(F32(W) * step))
        v_step = F32(F32(1.0) / F32(F32(H) * step))
        u = (xs - (W >> 1)).astype(F32) * u_step
        v = (ys - (H >> 1)).astype(F32) * v_step
        vv = (v * v).astype(F32)
        s = fma32(u[None, :], u[None, :], vv[:, None])
        ll = F32(lam32 * lam32)
        tmp = fma32(-ll, s, F32(1.0))
        tmp = np.maximum(tmp, F32(0.0))
        sq = np.sqrt(tmp).astype(F32).astype(np.float64)
        ph = ((2.0 * math.pi * float(z32)) / float(lam32)) * sq
        ph32 = ph.astype(F32).astype(np.float64)
        G = np.cos(ph32) + 1j * np.sin(ph32)
    else:
        raise ValueError(mode)
    return shift_corners(G)


# ----------------------------------------------------------------------------------------
# a3/a5/a6: spatial transforms (fresnel_transform.cu:65-83, angular_spectrum.cu:33-63,
#            apply_mask.cu:7-34)
# ----------------------------------------------------------------------------------------


def fresnel_transform(frames: np.ndarray, lens: np.ndarray) -> np.ndarray:
    """x <- FFT2(x * L), forward, unnormalised, no shift (fresnel_transform.cu:74-79)."""
    return fft2(frames * lens[None], axes=(-2, -1))


def angular_spectrum(frames: np.ndarray, lens: np.ndarray) -> np.ndarray:
    """x <- IFFT2(FFT2(x) * G) / (H*W): cuFFT's unnormalised inverse then kernel_complex_divide
    (angular_spectrum.cu:47-61). numpy's ifft2 carries the same 1/(H*W)."""
    return ifft2(fft2(frames, axes=(-2, -1)) * lens[None], axes=(-2, -1))


def filter2d_mask(W: int, H: int, n1: int, n2: int, smooth_low: int, smooth_high: int) -> np.ndarray:
    """kernel_update_filter2d_circles_mask (filter2D.cu:52-88) in its float32 arithmetic, then
    shift_corners (filter2D.cu:113): r = hypotf(x - W/2, y - H/2); A = 1 for r < n2, else
    cos((r - n2) / smooth_high * pi/2) for r < n2 + smooth_high (the product in double, rounded to
    float for cosf), else 0; B the same with n1 / smooth_low; mask = A * (1 - B)."""
    x = np.arange(W, dtype=F32) - F32(W // 2)
    y = np.arange(H, dtype=F32) - F32(H // 2)
    r = np.hypot(x[None, :], y[:, None]).astype(F32)

    def disc(radius, smooth):
        out = np.zeros((H, W), F32)
        out[r < F32(radius)] = 1.0
        band = (r >= F32(radius)) & (r < F32(radius + smooth))
        if smooth > 0:
            q = ((r[band] - F32(radius)) / F32(smooth)).astype(F32)
            out[band] = np.cos((q.astype(np.float64) * (math.pi / 2)).astype(F32))
        return out

    a = disc(n2, smooth_high)
    b = disc(n1, smooth_low)
    return shift_corners((a * (F32(1.0) - b)).astype(F32))


def filter2d(frames: np.ndarray, mask: np.ndarray) -> np.ndarray:
    """filter2D (filter2D.cu:28-46): forward FFT2, * mask, cuFFT's unnormalised inverse."""
    H, W = frames.shape[-2:]
    return ifft2(fft2(frames, axes=(-2, -1)) * mask[None], axes=(-2, -1)) * (H * W)


def spatial_transform(frames: np.ndarray, kind: str, lens: np.ndarray | None,
                      f2d_mask: np.ndarray | None = None) -> np.ndarray:
    """Dispatch of FourierTransform::insert_fft (fourier_transform.cc:30-72). With filter2D, the
    frames are filtered first for FRESNELTR and NONE; for ANGULARSP the mask is already part of
    the transfer function (`lens`)."""
    if f2d_mask is not None and kind != "ANGULARSP":
        frames = filter2d(frames, f2d_mask)
    if kind == "NONE":
        return frames
    if kind == "FRESNELTR":
        return fresnel_transform(frames, lens)
    if kind == "ANGULARSP":
        return angular_spectrum(frames, lens)
    raise ValueError(kind)


# ----------------------------------------------------------------------------------------
# a7: time-transformation ring (Backend/sources/data_struct/queue.cc:332-380)
# ----------------------------------------------------------------------------------------


class Ring:
    """Circular queue of T frames with the reference's start/size bookkeeping.

    enqueue_multiple follows queue.cc:332-380: frames land at (start+size) % T with wrap;
    a batch larger than T keeps only its last T frames; when the queue overflows, start
    advances. ``data`` is the raw STORAGE (slot order), which is what the time transforms
    read (fourier_transform.cc:238-240, get_data()).
    """

    def __init__(self, T: int, shape: tuple, dtype=np.complex128):
        self.T = T
        self.data = np.zeros((T,) + tuple(shape), dtype=dtype)
        self.start = 0
        self.size = 0

    def enqueue_multiple(self, elts: np.ndarray) -> None:
        nb = elts.shape[0]
        T = self.T
        if nb > T:
            elts = elts[nb - T:]
            self.start = (self.start + nb - T) % T
            nb = T
        begin = (self.start + self.size) % T
        for j in range(nb):
            self.data[(begin + j) % T] = elts[j]
        self.size += nb
        if self.size > T:
            self.start = (self.start + self.size - T) % T
            self.size = T

    def enqueue(self, elt: np.ndarray) -> None:
        """Single enqueue (queue.cc:149-189)."""
        end = (self.start + self.size) % self.T
        self.data[end] = elt
        if self.size < self.T:
            self.size += 1
        else:
            self.start = (self.start + 1) % self.T

    def is_full(self) -> bool:
        return self.size == self.T

    def clear(self) -> None:
        self.start = 0
        self.size = 0


# ----------------------------------------------------------------------------------------
# a8: STFT over ring storage order (stft.cu:9-15, icompute.cc:109-115)
# a12: p range (converts.cc:76-92)
# ----------------------------------------------------------------------------------------


def p_range(p_start: int, p_width: int, T: int) -> tuple[int, int]:
    """pmin = p.start; pmax = max(0, min(pmin + width, T)) if width else pmin (converts.cc:81-88)."""
    pmin = p_start
    pmax = max(0, min(pmin + p_width, T)) if p_width != 0 else pmin
    return pmin, pmax


def stft_bins(storage: np.ndarray, pmin: int, pmax: int) -> np.ndarray:
    """X[k] = sum_t storage[t] * exp(-2*pi*i*k*t/T) for k in [pmin, pmax]: cuFFT forward along time
    (planMany batch=HW, stride=HW) restricted to the bins the view reads."""
    T = storage.shape[0]
    t = np.arange(T)
    ks = np.arange(pmin, pmax + 1)
    W = np.exp(-2j * np.pi * np.outer(ks, t) / T).astype(np.result_type(storage.dtype, np.complex64))  # [K, T]
    flat = storage.reshape(T, -1)
    return (W @ flat).reshape((len(ks),) + storage.shape[1:])


# ----------------------------------------------------------------------------------------
# a9-a11: PCA (matrix_operations.cc:9-103, fourier_transform.cc:340-377)
# ----------------------------------------------------------------------------------------


def pca_covariance(storage: np.ndarray) -> np.ndarray:
    """cov = H^H H with H the column-major HW x T view of the ring storage (matrix_operations.cc:9-26).
    cov[i, j] = sum_pix conj(H[pix, i]) * H[pix, j]."""
    T = storage.shape[0]
    Hm = storage.reshape(T, -1).T  # [HW, T]
    return Hm.conj().T @ Hm


def pca_eigh(cov: np.ndarray) -> tuple[np.ndarray, np.ndarray]:
    """Ascending eigenvalues, eigenvectors as columns, from the LOWER triangle (cusolverDnCheevd,
    matrix_operations.cc:44-65). numpy.linalg.eigh(UPLO='L') has the same contract."""
    w, V = np.linalg.eigh(cov, UPLO="L")
    return w, V


def pca_project(storage: np.ndarray, V: np.ndarray, pmin: int, pmax: int) -> np.ndarray:
    """p_acc[:, j] = H @ V[:, j] (matrix_multiply_complex, matrix_operations.cc:77-103), for j in [pmin, pmax]."""
    T = storage.shape[0]
    Hm = storage.reshape(T, -1).T
    P = Hm @ V[:, pmin:pmax + 1].astype(np.result_type(storage.dtype, np.complex64))  # [HW, K]
    return P.T.reshape((pmax - pmin + 1,) + storage.shape[1:])


# ----------------------------------------------------------------------------------------
# SSA_STFT (fourier_transform.cc:379-444)
# ----------------------------------------------------------------------------------------


def ssa_q_range(q_start: int, q_width: int, T: int) -> tuple[int, int]:
    """Eigenvector columns kept (fourier_transform.cc:409-412): [q, q + q_acc), every column
    when the width is 0."""
    return (q_start, q_width) if q_width != 0 else (0, T)


def ssa_stft_bins(storage: np.ndarray, V: np.ndarray, q_start: int, q_width: int, pmin: int, pmax: int) -> np.ndarray:
    """V's columns outside [q, q + q_acc) zeroed (cudaMemsetAsync :413-415), tmp = V V^H
    (matrix_multiply_complex OP_N / OP_C), P = H tmp, then the STFT of P along time (stft plan
    over the p_acc buffer); bins pmin..pmax."""
    T = storage.shape[0]
    q, qn = ssa_q_range(q_start, q_width, T)
    Vq = np.zeros_like(V)
    Vq[:, q:q + qn] = V[:, q:q + qn]
    tmp = Vq @ Vq.conj().T
    Hm = storage.reshape(T, -1).T  # [HW, T] column-major H
    P = Hm @ tmp
    return stft_bins(P.T.reshape(storage.shape), pmin, pmax)


# ----------------------------------------------------------------------------------------
# phase increase (tools_unwrap.cu:210-267, converts.cc:251-300, tools_conversion.cu:245-313)
# ----------------------------------------------------------------------------------------


class PhaseIncrease:
    """phase_increase with UnwrappingResources of capacity 1 (converts.cc:257-259): the newest
    increment d = atan2 of cur * conj(pred) (kernel_compute_angle_mult), corrected by the one
    stored increment (kernel_correct_angles), then stored; pred <- cur. The first call takes
    pred = cur (the function's first_time copy), so its increment is 0 (exactly 0 here; the
    reference takes atan2 of the rounding residue of cur * conj(cur))."""

    def __init__(self):
        self.pred = None
        self.hist = None

    def push(self, cur: np.ndarray) -> np.ndarray:
        if self.pred is None:
            d = np.zeros(cur.shape)
        else:
            cp = cur * np.conj(self.pred)
            d = np.arctan2(cp.imag, cp.real)
        out = d + self.hist if self.hist is not None else d.copy()
        self.hist = d
        self.pred = cur.copy()
        return out


def rescale_float(img: np.ndarray) -> np.ndarray:
    """rescale_float (tools_conversion.cu:275-313): (x + |min|) * 65535 / (|max| + |min|) in
    float32, min / max taken from the first 128 block results of 128 pixels each, i.e. over the
    first min(N, 16384) pixels (the whole frame below that: the reference reads past its results)."""
    f = img.astype(F32)
    n = min(f.size, 16384)
    head = f.reshape(-1)[:n]
    amin = np.abs(head.min())
    amax = np.abs(head.max())
    if amax + amin == 0:
        return np.zeros_like(f)  # an all-zero prefix (first window): 0 instead of 0 / 0
    return ((f + amin) * F32(65535.0)) / (amax + amin)


# ----------------------------------------------------------------------------------------
# time-transformation cuts (stft.cu:17-115, fourier_transform.cc:462-503)
# ----------------------------------------------------------------------------------------


def cut_view(X: np.ndarray, img_type: str) -> np.ndarray:
    """fill_32bit_slices' per-element view: hypotf for MODULUS / PHASE_INCREASE / COMPOSITE, its
    square for SQUARED_MODULUS, atanf(Im / Re) + pi/2 for ARGUMENT (float32 quotient and atan,
    the pi/2 added in double), 0 for the others."""
    if img_type in ("MODULUS", "PHASE_INCREASE", "COMPOSITE"):
        return np.abs(X)
    if img_type == "SQUARED_MODULUS":
        return np.abs(X) ** 2
    if img_type == "ARGUMENT":
        with np.errstate(divide="ignore", invalid="ignore"):
            q = (X.imag.astype(F32) / X.real.astype(F32)).astype(F32)
        return (np.arctan(q).astype(F32).astype(np.float64) + math.pi / 2).astype(F32).astype(np.float64)
    return np.zeros(X.shape)


def time_cuts(p_acc: np.ndarray, xmin: int, xmax: int, ymin: int, ymax: int, img_type: str):
    """XZ[t][x] = mean over y in [ymin, ymax] of view(p_acc[t][y][x]) (T x W) and
    YZ[y][t] = mean over x in [xmin, xmax] (H x T), p_acc holding all T bins / components."""
    v_xz = cut_view(p_acc[:, ymin:ymax + 1, :], img_type)  # [T, ny, W]
    v_yz = cut_view(p_acc[:, :, xmin:xmax + 1], img_type)  # [T, H, nx]
    return v_xz.mean(axis=1), v_yz.mean(axis=2).T


def all_bins(storage: np.ndarray, time_transformation: str, V: np.ndarray | None = None, q_start: int = 0,
             q_width: int = 0) -> np.ndarray:
    """The reference's gpu_p_acc_buffer with every bin / component: the STFT (stft.cu:9-15), H V
    (PCA), FFT_t(H V_Q V_Q^H) (SSA_STFT), the ring itself (NONE, fourier_transform.cc:213-224)."""
    T = storage.shape[0]
    if time_transformation == "STFT":
        return stft_bins(storage, 0, T - 1)
    if time_transformation == "PCA":
        return pca_project(storage, V, 0, T - 1)
    if time_transformation == "SSA_STFT":
        return ssa_stft_bins(storage, V, q_start, q_width, 0, T - 1)
    return storage.copy()


# ----------------------------------------------------------------------------------------
# a13-a16: views (tools_conversion.cu:11-103,199-218; converts.cc:50-62)
# ----------------------------------------------------------------------------------------

PCA_SCALE = float((2 << 16) - 1)  # 131071, converts.cc:58


def view(planes: np.ndarray, img_type: str) -> np.ndarray:
    """Mean over the selected planes of |X|, |X|^2 or atan2(Im, Re)."""
    if img_type == "MODULUS":
        v = np.abs(planes)
    elif img_type == "SQUARED_MODULUS":
        v = np.abs(planes) ** 2
    elif img_type == "ARGUMENT":
        v = np.arctan2(planes.imag, planes.real)
    else:
        raise ValueError(img_type)
    return v.mean(axis=0)


# ----------------------------------------------------------------------------------------
# Moments 0/1/2 (fourier_transform.cc:244-338, icompute.cc:26-69 fft_freqs,
# tools_compute.cu:38-97, converts.cc:112-125, pipe.cc:429-454)
# ----------------------------------------------------------------------------------------


def fft_freqs(T: int, camera_fps: float) -> np.ndarray:
    """f1 of ICompute::fft_freqs: [0, 1, ..., n/2-1, -n/2, ..., -1] * fs/n for even n (the Nyquist
    bin kept negative), [0, ..., (n-1)/2, -(n-1)/2, ..., -1] * fs/n for odd n; d in float32."""
    d = float(F32(camera_fps) / F32(T))
    k = np.arange(T, dtype=np.float64)
    if T % 2 == 0:
        f1 = np.where(k < T // 2, k, -(T - k))
    else:
        f1 = np.where(k < (T + 1) // 2, k, k - T)
    return f1 * d


def moments(planes: np.ndarray, pmin: int, T: int, camera_fps: float, order: int) -> np.ndarray:
    """Moment of order 0, 1 or 2 of the selected bins pmin.. (planes[k] = X_{pmin+k}):
    sum_k |X_k|^2 f1[k]^order, with the Nyquist bin (even T) counted twice for orders 0 and 2 and
    not at all for order 1 (tensor_multiply_vector_nyquist_compensation)."""
    f1 = fft_freqs(T, camera_fps)
    f = {0: np.ones(T), 1: f1, 2: f1 * f1}[order]
    p2 = np.abs(planes) ** 2
    idx = pmin + np.arange(planes.shape[0])
    w = f[idx].copy()
    if T % 2 == 0:
        ny = (idx == T // 2)
        w[ny] = 0.0 if order == 1 else 2.0 * w[ny]
    return np.tensordot(w, p2, axes=(0, 0))


# ----------------------------------------------------------------------------------------
# a17: 2-D phase unwrap (tools_unwrap.cu:79-95,269-369; tools.cu:50-68) + rescale
#      (tools_conversion.cu:315-335)
# ----------------------------------------------------------------------------------------

M_2PI_F = float(F32(6.28318530717959))  # common.cuh:29


def unwrap_2d(phase: np.ndarray) -> np.ndarray:
    """Fourier-domain unwrap of an H x W phase image.

    The reference plans its unwrap FFT as plan(width, height) (icompute.hh:140), i.e. it
    transforms the row-major buffer as ``width`` rows of ``height`` samples; this restatement
    does the same by viewing the buffer as a (W, H) array. Frequency indices come from the
    circ-shifted fx/fy grids (tools_unwrap.cu:79-95, 269-296). cuFFT transforms are unnormalised.
    """
    H, W = phase.shape
    flat = phase.reshape(-1)
    j, i = np.divmod(np.arange(H * W), W)
    fx = (i - (W >> 1)).astype(np.float64)
    fy = (j - (H >> 1)).astype(np.float64)
    # circ_shift(out, in, W, H, -W/2, -H/2): out[(y-H/2)%H][(x-W/2)%W] = in[y][x]
    def circ(a):
        a2 = a.reshape(H, W)
        return np.roll(np.roll(a2, -(H >> 1), axis=0), -(W >> 1), axis=1).reshape(-1)
    sfx, sfy = circ(fx), circ(fy)
    z = np.exp(1j * flat)
    n0, n1 = W, H  # plan(width, height): slowest dimension = width

    def fft(a):
        return fft2(a.reshape(n0, n1)).reshape(-1)

    def ifft(a):  # unnormalised inverse
        return ifft2(a.reshape(n0, n1)).reshape(-1) * (n0 * n1)

    Z = fft(z)
    gx = ifft(Z * sfx) * (1j * M_2PI_F)
    gy = ifft(Z * sfy) * (1j * M_2PI_F)
    zc = np.conj(z * 1j)
    gx = fft(gx * zc)
    gy = fft(gy * zc)
    norm = sfx * sfx + sfy * sfy
    with np.errstate(divide="ignore", invalid="ignore"):
        cx = np.where(norm != 0, sfx / np.where(norm != 0, norm, 1), 0.0)
        cy = np.where(norm != 0, sfy / np.where(norm != 0, norm, 1), 0.0)
    acc = ifft(gx * cx + gy * cy)
    return (acc.imag / -M_2PI_F).reshape(H, W)


def rescale_unwrap2d(img: np.ndarray) -> np.ndarray:
    """(in+|min|)/(|min|+max)*65535 if min<0 else (in-min)/(max-min)*65535 (tools_conversion.cu:315-335)."""
    mn, mx = img.min(), img.max()
    if mx == mn:
        return np.zeros_like(img)  # a constant frame: 0 instead of 0 / 0
    if mn < 0:
        return (img + abs(mn)) / (abs(mn) + mx) * 65535.0
    return (img - mn) / (mx - mn) * 65535.0


# ----------------------------------------------------------------------------------------
# a18: renormalisation (tools_compute.cu:99-123, postprocessing.cc:135-155)
# ----------------------------------------------------------------------------------------


def renormalize(img: np.ndarray, renorm_constant: int) -> np.ndarray:
    """x <- x * 2^c * N / sum(x); a zero-sum frame becomes 0 (the reference's N / 0 gives NaN)."""
    total = img.sum(dtype=np.float64)
    if total == 0:
        return np.zeros_like(img)
    return img * float(1 << renorm_constant) * (img.size / total)


# ----------------------------------------------------------------------------------------
# a20: image accumulation (tools_conversion.cu:418-441, image_accumulation.cc:136-157)
# ----------------------------------------------------------------------------------------


class Accumulator:
    """Rolling mean over the last A frames; a frame is enqueued, then the mean of the current size."""

    def __init__(self, A: int, shape: tuple):
        self.ring = Ring(A, shape, dtype=np.float64)

    def push(self, img: np.ndarray) -> np.ndarray:
        self.ring.enqueue(img)
        r = self.ring
        idx = [(r.start + i) % r.T for i in range(r.size)]
        return r.data[idx].mean(axis=0)


# ----------------------------------------------------------------------------------------
# a21-a23: percentile contrast and uint16 (percentile.cu:75-94,139-222; contrast_api.cc:137-146;
#          contrast_correction.cu:5-17; tools_conversion.cu:350-359,382-387). float32 math.
# ----------------------------------------------------------------------------------------


def percentile_index(pct: float, n: int) -> int:
    """(uint)(h_percent / 100 * frame_res) evaluated in float32 (percentile.cu:85), clamped to n-1."""
    idx = int(np.floor(F32(F32(pct) / F32(100)) * F32(n)))
    return min(max(idx, 0), n - 1)


def reticle_values(img32: np.ndarray, scale: float) -> np.ndarray:
    """Pixels inside the contrast reticle circle (percentile.cu:15-43,159-181)."""
    H, W = img32.shape
    radius = int(F32(scale) * F32(min(W, H)) / F32(2))
    cx, cy = W // 2, H // 2
    y, x = np.mgrid[0:H, 0:W]
    m = (x - cx) ** 2 + (y - cy) ** 2 <= radius * radius
    return img32[m]


def autocontrast(img32: np.ndarray, lower: float, upper: float, reticle_scale: float | None = None) -> tuple[float, float]:
    """Sorted-copy percentiles, then update_contrast's clamp of both ends to >= 1.0."""
    vals = img32.reshape(-1) if reticle_scale is None else reticle_values(img32, reticle_scale)
    s = np.sort(vals.astype(F32))
    n = s.size
    lo = F32(s[percentile_index(lower, n)])
    hi = F32(s[percentile_index(upper, n)])
    lo = lo if lo > F32(1.0) else F32(1.0)
    hi = hi if hi > F32(1.0) else F32(1.0)
    return float(lo), float(hi)


def apply_contrast(img32: np.ndarray, cmin: float, cmax: float, invert: bool = False) -> np.ndarray:
    """factor = 65535 / (max - min + FLT_EPSILON); x <- factor * (x - min), in float32."""
    mn, mx = (F32(cmax), F32(cmin)) if invert else (F32(cmin), F32(cmax))
    eps = F32(np.finfo(np.float32).eps)
    factor = F32(F32(65535.0) / F32(F32(mx - mn) + eps))
    return (factor * (img32.astype(F32) - mn).astype(F32)).astype(F32)


def float_to_ushort(img32: np.ndarray) -> np.ndarray:
    """x<=0 -> 0; (uint)x > 65535 -> 65535; else truncation (tools_conversion.cu:350-359). NaN -> 0."""
    x = img32.astype(F32)
    out = np.zeros(x.shape, dtype=np.uint16)
    with np.errstate(invalid="ignore"):
        pos = x > 0
        big = x >= F32(65536.0)
        mid = pos & ~big
    out[big & pos] = 65535
    out[mid] = np.trunc(x[mid]).astype(np.uint16)
    return out


def log10_view(img: np.ndarray) -> np.ndarray:
    """map_log10 (rendering.cc:127-138)."""
    return np.log10(img)


# ----------------------------------------------------------------------------------------
# Pipe model (Backend/sources/core/pipe.cc:255-387, 389-467; rendering.cc:239-299)
# ----------------------------------------------------------------------------------------


@dataclass
class OracleSettings:
    width: int
    height: int
    depth: int = 2  # bytes per pixel: 1, 2 or 4 (float)
    space_transformation: str = "NONE"  # NONE / FRESNELTR / ANGULARSP
    time_transformation: str = "NONE"  # NONE / STFT / PCA
    time_transformation_size: int = 1
    time_stride: int = 1
    batch_size: int = 1
    lam: float = 852e-9
    z: float = 0.0
    pixel_size: float = 12.0
    image_type: str = "MODULUS"
    p_start: int = 0
    p_width: int = 0
    fft_shift: bool = False
    renorm: bool = True
    renorm_constant: int = 5
    accumulation: int = 0
    log_enabled: bool = False
    contrast_enabled: bool = True
    contrast_auto_refresh: bool = True
    contrast_invert: bool = False
    contrast_min: float = 1.0
    contrast_max: float = 65535.0
    contrast_lower: float = 0.02
    contrast_upper: float = 99.98
    reticle_display: bool = False
    reticle_scale: float = 0.5
    unwrap_2d: bool = False
    lens_mode: str = "fp64"
    camera_fps: float = 0.0  # moments: frequencies in units of camera_fps / T
    q_start: int = 0  # SSA_STFT eigenvector range (view.z2)
    q_width: int = 0
    filter2d_enabled: bool = False
    filter2d_n1: int = 0
    filter2d_n2: int = 1
    filter2d_smooth_low: int = 0
    filter2d_smooth_high: int = 1
    cuts_enabled: bool = False
    x_start: int = 0
    x_width: int = 0
    y_start: int = 0
    y_width: int = 0
    xz_accumulation: int = 1
    yz_accumulation: int = 1
    xz_log_enabled: bool = False
    yz_log_enabled: bool = False
    xz_contrast_enabled: bool = False
    xz_contrast_auto_refresh: bool = True
    xz_contrast_invert: bool = False
    xz_contrast_min: float = 1.0
    xz_contrast_max: float = 65535.0
    yz_contrast_enabled: bool = False
    yz_contrast_auto_refresh: bool = True
    yz_contrast_invert: bool = False
    yz_contrast_min: float = 1.0
    yz_contrast_max: float = 65535.0
    cuts_contrast_offset: int = 2
    filter2d_view_enabled: bool = False
    filter2d_log_enabled: bool = False
    filter2d_contrast_enabled: bool = False
    filter2d_contrast_auto_refresh: bool = True
    filter2d_contrast_invert: bool = False
    filter2d_contrast_min: float = 1.0
    filter2d_contrast_max: float = 65535.0
    # "fp64" (the oracle), or "fp32": the same equations in complex64 / float32 (the FP32 CPU
    # baseline; FFTs in single precision, covariance and eigensolve in complex64)
    precision: str = "fp64"


@dataclass
class OracleOutput:
    float_frame: np.ndarray  # the frame fed to the contrast stage (float64)
    contrast: tuple
    ushort: np.ndarray
    autocontrast_applied: bool = False
    cuts: list | None = None  # [XZ, YZ] CutOutput when the cuts are enabled
    filter2d_view: "CutOutput | None" = None  # the filter2D view when enabled


@dataclass
class CutOutput:
    float_frame: np.ndarray  # XZ: T x W, YZ: H x T, fed to the view's contrast stage
    contrast: tuple
    ushort: np.ndarray
    autocontrast_applied: bool = False


def float_to_ushort_normalized(img32: np.ndarray) -> np.ndarray:
    """float_to_ushort_normalized (tools_conversion.cu:389-393): x * 65535 in float32 converted to
    ushort, i.e. truncated and saturated to [0, 65535] (NaN -> 0)."""
    w = (np.asarray(img32, F32) * F32(65535.0)).astype(F32)
    out = np.zeros(w.shape, np.uint16)
    with np.errstate(invalid="ignore"):
        pos = w > 0
        out[pos] = np.minimum(np.trunc(w[pos]), 65535).astype(np.uint16)
    return out


def filter2d_view_frame(frame0: np.ndarray, mult: np.ndarray) -> np.ndarray:
    """The filter2D view (pipe.cc:526-546): the stored spectrum of the batch's first frame
    (FFT2(x0) times the mask, or the masked transfer function for AS: filter2D.cu:36-44,
    angular_spectrum.cu:50-55), shift_corners, complex_to_modulus over one bin."""
    return np.abs(shift_corners(fft2(frame0) * mult))


def cut_autocontrast(img32: np.ndarray, which: int, s: "OracleSettings") -> tuple[float, float]:
    """autocontrast_caller for XZ / YZ (rendering.cc:305-340, percentile.cu:139-250): the bins
    offset .. T-1-offset (rows of XZ, columns of YZ; the whole window when that range is empty),
    or for XZ the reticle disc of the whole T x W image when the reticle is displayed."""
    T = s.time_transformation_size
    off = s.cuts_contrast_offset if 2 * s.cuts_contrast_offset < T else 0
    if which == 0 and s.reticle_display:
        return autocontrast(img32, s.contrast_lower, s.contrast_upper, s.reticle_scale)
    if which == 0:
        return autocontrast(img32[off:T - off], s.contrast_lower, s.contrast_upper)
    return autocontrast(img32[:, off:T - off], s.contrast_lower, s.contrast_upper)


class CutModel:
    """One cut window's post-processing (image_accumulation.cc:159-257, rendering.cc:75-340,
    percentile.cu:139-250, converts.cc:321-350): accumulation, log10, autocontrast gated like the
    XY view on its own queue (bins offset .. T-1-offset; XZ over the reticle disc when the
    reticle is displayed), contrast and uint16."""

    def __init__(self, s: "OracleSettings", which: int):
        self.which = which
        p = "xz" if which == 0 else "yz"
        self.A = getattr(s, p + "_accumulation")
        self.log = getattr(s, p + "_log_enabled")
        self.enabled = getattr(s, p + "_contrast_enabled")
        self.invert = getattr(s, p + "_contrast_invert")
        self.pending = self.enabled and getattr(s, p + "_contrast_auto_refresh")
        self.crange = (getattr(s, p + "_contrast_min"), getattr(s, p + "_contrast_max"))
        T = s.time_transformation_size
        shape = (T, s.width) if which == 0 else (s.height, T)
        self.acc = Accumulator(self.A, shape) if self.A > 1 else None
        self.s = s
        self.img = np.zeros(shape)

    def push(self, img: np.ndarray | None) -> CutOutput:
        s = self.s
        if img is not None:
            self.img = img
        img = self.img
        if self.acc is not None:
            img = self.acc.push(img)
        if self.log:
            img = log10_view(img)
        img32 = img.astype(F32)
        applied = False
        if self.enabled and self.pending:
            r = self.acc.ring if self.acc is not None else None
            if r is None or r.is_full() or r.size == 1:
                applied = True
                self.crange = cut_autocontrast(img32, self.which, s)
                if r is None or r.is_full():
                    self.pending = False
        c = apply_contrast(img32, self.crange[0], self.crange[1], self.invert) if self.enabled else img32
        return CutOutput(float_frame=img, contrast=self.crange, ushort=float_to_ushort(c), autocontrast_applied=applied)


class OraclePipe:
    """Cycle-level model of Pipe::exec/refresh: stride gate, ring, wait-T, time transform,
    view, unwrap, renorm, fftshift, accumulation, autocontrast and uint16."""

    def __init__(self, s: OracleSettings):
        self.s = s
        H, W = s.height, s.width
        self.cdtype = np.complex64 if s.precision == "fp32" else np.complex128
        self.ring = Ring(s.time_transformation_size, (H, W), dtype=self.cdtype)
        self.batch_index = 0
        self.lens = None
        if s.space_transformation == "FRESNELTR":
            self.lens = fresnel_lens(W, H, s.lam, s.z, s.pixel_size, s.lens_mode).astype(self.cdtype)
        elif s.space_transformation == "ANGULARSP":
            self.lens = angular_spectrum_lens(W, H, s.lam, s.z, s.pixel_size, s.lens_mode).astype(self.cdtype)
        self.f2d_mask = None
        if s.filter2d_enabled:
            m = filter2d_mask(W, H, s.filter2d_n1, s.filter2d_n2, s.filter2d_smooth_low, s.filter2d_smooth_high)
            if s.space_transformation == "ANGULARSP":
                self.lens = self.lens * m  # apply_mask on the shifted lens (fourier_transform.cc:136-137)
            else:
                self.f2d_mask = m.astype(np.float64)
        self.acc = Accumulator(s.accumulation, (H, W)) if s.accumulation > 1 else None
        self.autocontrast_pending = s.contrast_enabled and s.contrast_auto_refresh
        self.crange = (s.contrast_min, s.contrast_max)
        self.last_V = None
        self.phase_increase = PhaseIncrease() if s.image_type == "PHASE_INCREASE" else None
        self.cut_models = [CutModel(s, 0), CutModel(s, 1)] if s.cuts_enabled else None
        self.f2d_view = s.filter2d_enabled and s.filter2d_view_enabled
        self.f2d_pending = s.filter2d_contrast_enabled and s.filter2d_contrast_auto_refresh
        self.f2d_range = (s.filter2d_contrast_min, s.filter2d_contrast_max)
        self.frame0 = None

    def process_batch(self, raw: np.ndarray, convert_f32=True) -> OracleOutput | None:
        s = self.s
        # wait_time_stride (pipe.cc:400-416)
        self.batch_index += s.batch_size
        if self.batch_index != s.time_stride:
            return None
        self.batch_index = 0
        frames = convert_frames(raw).astype(self.cdtype, copy=False)
        self.frame0 = frames[0]
        frames = spatial_transform(frames, s.space_transformation, self.lens, self.f2d_mask)
        self.ring.enqueue_multiple(frames)
        if self.ring.size < s.time_transformation_size:
            return None
        return self._render()

    def _render(self) -> OracleOutput:
        s = self.s
        T = s.time_transformation_size
        pmin, pmax = p_range(s.p_start, s.p_width, T)
        if s.time_transformation == "STFT":
            planes = stft_bins(self.ring.data, pmin, pmax)
        elif s.time_transformation == "PCA":
            cov = pca_covariance(self.ring.data)
            _, V = pca_eigh(cov)
            self.last_V = V
            planes = pca_project(self.ring.data, V, pmin, pmax)
        elif s.time_transformation == "SSA_STFT":
            cov = pca_covariance(self.ring.data)
            _, V = pca_eigh(cov)
            self.last_V = V
            planes = ssa_stft_bins(self.ring.data, V, s.q_start, s.q_width, pmin, pmax)
        else:
            planes = self.ring.data[pmin:pmax + 1]
        if s.image_type.startswith("MOMENTS_"):
            # the moment replaces the post-processing frame after the PCA scaling (pipe.cc:346)
            img = moments(planes, pmin, T, s.camera_fps, int(s.image_type[-1]))
        elif s.image_type == "PHASE_INCREASE":
            # the stored p plane (fourier_transform.cc:446-460): bin / component p_start
            first = self.phase_increase.pred is None
            d = self.phase_increase.push(planes[0])
            if s.unwrap_2d:
                # the first window's increments are all 0: the zero frame, not an unwrap of residues
                img = np.zeros(d.shape) if first else rescale_unwrap2d(unwrap_2d(d))
            else:
                img = rescale_float(d).astype(np.float64)
        else:
            img = view(planes, s.image_type)
        if s.image_type == "ARGUMENT" and s.unwrap_2d:
            img = rescale_unwrap2d(unwrap_2d(img))
        if s.time_transformation == "PCA" and not s.image_type.startswith("MOMENTS_"):
            img = img * PCA_SCALE
        if s.renorm:
            img = renormalize(img, s.renorm_constant)
        if s.fft_shift:
            img = shift_corners(img)
        if self.acc is not None:
            img = self.acc.push(img)
        if s.log_enabled:
            img = log10_view(img)
        img32 = img.astype(F32)
        applied = False
        if s.contrast_enabled:
            if self.autocontrast_pending and self._should_autocontrast():
                applied = True
                self.crange = autocontrast(img32, s.contrast_lower, s.contrast_upper,
                                           s.reticle_scale if s.reticle_display else None)
                if self.acc is None or self.acc.ring.is_full():
                    self.autocontrast_pending = False
            c = apply_contrast(img32, self.crange[0], self.crange[1], s.contrast_invert)
        else:
            c = img32
        cuts = None
        if self.cut_models is not None:
            slices = (None, None)
            if s.x_start < s.width and s.y_start < s.height:
                p_acc = all_bins(self.ring.data, s.time_transformation, self.last_V, s.q_start, s.q_width)
                slices = time_cuts(p_acc, s.x_start, s.x_start + s.x_width, s.y_start, s.y_start + s.y_width,
                                   s.image_type)
            cuts = [m.push(sl) for m, sl in zip(self.cut_models, slices)]
        f2d = None
        if self.f2d_view:
            mult = self.lens if s.space_transformation == "ANGULARSP" else self.f2d_mask
            fimg = filter2d_view_frame(self.frame0, mult)
            if s.filter2d_log_enabled:
                fimg = log10_view(fimg)
            f32 = fimg.astype(F32)
            f_applied = False
            if s.filter2d_contrast_enabled and self.f2d_pending:
                self.f2d_range = autocontrast(f32, s.contrast_lower, s.contrast_upper)
                self.f2d_pending = False
                f_applied = True
            fc = (apply_contrast(f32, self.f2d_range[0], self.f2d_range[1], s.filter2d_contrast_invert)
                  if s.filter2d_contrast_enabled else f32)
            f2d = CutOutput(float_frame=fimg, contrast=self.f2d_range, ushort=float_to_ushort_normalized(fc),
                            autocontrast_applied=f_applied)
        return OracleOutput(float_frame=img, contrast=self.crange, ushort=float_to_ushort(c),
                            autocontrast_applied=applied, cuts=cuts, filter2d_view=f2d)

    def _should_autocontrast(self) -> bool:
        """should_apply_contrast (rendering.hh:168-181)."""
        if self.acc is None:
            return True
        r = self.acc.ring
        return r.is_full() or r.size == 1
