"""Library anchors for the oracle: the reference's call sequences replayed on the GPU through the
same NVIDIA libraries it calls (cuFFT for the spatial and time transforms, cuBLAS for the
covariance and projection, cuSOLVER for the Hermitian eigensolve, a device sort for the
percentile), here reached through torch, and compared with the FP64 oracle. They pin the oracle's
conventions (FFT signs, normalisations, storage order along time, lower-triangle eigensolve with
ascending eigenvalues, percentile index) to what those libraries do. The product path is not
involved. Bars: rel-L2 <= 1e-5 against the FP64 oracle for FP32 library results (complex64
transforms of 12-bit frames), eigenvalues within 1e-5 of the largest, exact percentile values."""

import numpy as np
import pytest

import holovibes_oracle as O
from gpu_util import rel_l2
from holovibes_gb300.synthetic import Interferogram


def _frames(W, H, n, seed):
    return Interferogram(width=W, height=H, seed=seed).frames(0, n)


@pytest.mark.gpu
@pytest.mark.parametrize("W,H", [(256, 256), (384, 256)])
def test_fresnel_matches_cufft_sequence(cuda, W, H):
    """fresnel_transform.cu:65-83: apply_mask(x, L) then cufftExecC2C(FORWARD), no 1/N."""
    import torch

    x = O.convert_frames(_frames(W, H, 3, 1))
    L = O.fresnel_lens(W, H, 785e-9, 0.45, 12.0)
    got = torch.fft.fft2(torch.from_numpy((x * L[None]).astype(np.complex64)).cuda()).cpu().numpy()
    assert rel_l2(got, O.fresnel_transform(x, L)) <= 1e-5


@pytest.mark.gpu
@pytest.mark.parametrize("W,H", [(256, 256), (512, 384)])
def test_angular_spectrum_matches_cufft_sequence(cuda, W, H):
    """angular_spectrum.cu:33-63: forward cuFFT, x shifted G, inverse cuFFT (unnormalised),
    kernel_complex_divide by W*H."""
    import torch

    x = O.convert_frames(_frames(W, H, 2, 2))
    G = O.angular_spectrum_lens(W, H, 852e-9, 0.30, 20.0)
    xd = torch.from_numpy(x.astype(np.complex64)).cuda()
    Gd = torch.from_numpy(G.astype(np.complex64)).cuda()
    y = torch.fft.ifft2(torch.fft.fft2(xd) * Gd[None], norm="forward") / (W * H)
    assert rel_l2(y.cpu().numpy(), O.angular_spectrum(x, G)) <= 1e-5


@pytest.mark.gpu
@pytest.mark.parametrize("T,pmin,pmax", [(16, 1, 1), (32, 5, 12), (33, 0, 32)])
def test_stft_matches_batched_cufft_over_storage(cuda, T, pmin, pmax):
    """stft.cu:9-15 with the plan of icompute.cc:109-115: a forward 1-D cuFFT along time, batch =
    pixels, stride = frame size, over the ring's storage order."""
    import torch

    rng = np.random.default_rng(T)
    ring = (rng.standard_normal((T, 24, 40)) + 1j * rng.standard_normal((T, 24, 40))).astype(np.complex64)
    got = torch.fft.fft(torch.from_numpy(ring).cuda(), dim=0)[pmin:pmax + 1].cpu().numpy()
    assert rel_l2(got, O.stft_bins(ring.astype(np.complex128), pmin, pmax)) <= 1e-5


@pytest.mark.gpu
@pytest.mark.parametrize("T", [16, 32])
def test_pca_matches_cublas_cusolver_sequence(cuda, T):
    """matrix_operations.cc:9-103: cov = H^H H (Cgemm, H column-major HW x T), Cheevd on the lower
    triangle (ascending), p_acc = H V; compared on the eigenvalues and on |H v| of separated
    components (eigenvector phases are arbitrary)."""
    import torch

    rng = np.random.default_rng(T + 1)
    t = np.arange(T)
    ring = np.zeros((T, 2048), np.complex128)
    for m in range(4):
        ring += np.exp(2j * np.pi * (0.05 + 0.11 * m) * t)[:, None] * (rng.standard_normal(2048) / (m + 1))[None]
    ring += 0.01 * rng.standard_normal((T, 2048))
    ring = ring.astype(np.complex64)
    H = torch.from_numpy(ring).cuda().T  # HW x T
    cov = H.conj().T @ H
    w, V = torch.linalg.eigh(cov, UPLO="L")
    ref_cov = O.pca_covariance(ring.astype(np.complex128))
    assert rel_l2(cov.cpu().numpy(), ref_cov) <= 1e-5
    wr, Vr = O.pca_eigh(ref_cov)
    assert np.abs(w.cpu().numpy() - wr).max() <= 1e-5 * np.abs(wr).max()
    P = (H @ V).cpu().numpy()
    Pr = O.pca_project(ring.astype(np.complex128), Vr, 0, T - 1).reshape(T, -1).T
    for j in range(T - 3, T):  # the separated dominant components
        assert rel_l2(np.abs(P[:, j]), np.abs(Pr[:, j])) <= 1e-4


@pytest.mark.gpu
@pytest.mark.parametrize("n", [1000, 4096, 262144])
def test_percentile_matches_device_sort(cuda, n):
    """percentile.cu:75-94: thrust::sort of a copy, element (uint)(pct / 100 * n) in float32."""
    import torch

    rng = np.random.default_rng(n)
    v = (rng.gamma(2.0, 300.0, n)).astype(np.float32)
    s = torch.sort(torch.from_numpy(v).cuda()).values.cpu().numpy()
    for lower, upper in [(0.5, 99.5), (0.02, 99.98), (0.0, 100.0)]:
        i, j = O.percentile_index(lower, n), O.percentile_index(upper, n)
        lo, hi = O.autocontrast(v, lower, upper)
        assert lo == max(float(s[i]), 1.0) and hi == max(float(s[j]), 1.0)
