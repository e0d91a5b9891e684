"""The two covariance engines (FP32 SIMT and tcgen05 split-BF16 tensor cores: one tile for T <= 64,
128 x 128 tiles of the Gram matrix above) and the two Jacobi
paths (shared-memory for T <= 64, global-memory beyond) against the FP64 oracle.
Tolerances: SIMT covariance rel-L2 <= 1e-6, tensor-core (BF16x3, FP32 accumulation) <= 2e-5;
eigenvalues within 1e-6 of the largest (FP64 Jacobi on the FP64-summed covariance)."""

import numpy as np
import pytest

import holovibes_oracle as O
from gpu_util import call, dev, empty, host, ptr, rel_l2

import holovibes_gb300 as hv


def _ring(T, npix, seed):
    rng = np.random.default_rng(seed)
    t = np.arange(T)
    ring = np.zeros((T, npix), np.complex128)
    for m in range(min(T, 8)):
        f = rng.uniform(0.02, 0.48)
        ring += np.exp(2j * np.pi * f * t)[:, None] * ((rng.standard_normal(npix) + 1j * rng.standard_normal(npix)) / (m + 1))[None]
    ring += 0.05 * (rng.standard_normal((T, npix)) + 1j * rng.standard_normal((T, npix)))
    return (ring * 1000).astype(np.complex64)


@pytest.mark.gpu
@pytest.mark.parametrize("mode,tol", [(1, 1e-6), (2, 2e-5)])
@pytest.mark.parametrize("T,npix", [(32, 65536), (64, 4096), (17, 1000), (1, 64), (32, 64 * 1024 + 8),
                                    # tiled tensor-core kernel (T > 64): 128 x 128 tiles of G, split K
                                    (65, 1000), (96, 8192), (128, 65536), (200, 4104), (512, 16384)])
def test_covariance_engine(cuda, mode, tol, T, npix):
    ring = _ring(T, npix, T * 3 + mode)
    rd = dev(ring)
    cov = empty(T * T * 16)
    work = empty(hv.lib().hv_pca_cov_workspace(T, npix))
    hv.lib().hv_pca_covariance_mode(mode)
    try:
        call("hv_pca_covariance", ptr(rd), T, npix, ptr(cov), ptr(work), None)
        cuda.cuda.synchronize()
        assert hv.lib().hv_pca_covariance_status(ptr(work)) == hv.HV_OK
    finally:
        hv.lib().hv_pca_covariance_mode(0)
    got = host(cov, np.complex128, (T, T))
    ref = O.pca_covariance(ring.astype(np.complex128).reshape(T, npix, 1))
    assert rel_l2(got, ref) <= tol
    assert np.abs(got - got.conj().T).max() <= 1e-9 * np.abs(got).max()


@pytest.mark.gpu
@pytest.mark.parametrize("real", [0, 1])
@pytest.mark.parametrize("T,npix", [(65, 1000), (128, 65536), (200, 4104), (512, 16384)])
def test_covariance_planes_bit_identical(cuda, T, npix, real):
    """The tiled tensor-core covariance from split-BF16 planes the caller keeps (hv_pca_split_planes,
    then hv_pca_covariance_planes: tensor copies straight into the MMA operand layout). Complex
    planes: bit-identical to hv_pca_covariance on the ring (which splits it into its workspace). Real
    planes (a ring with zero imaginary parts, as without a spatial transform): within rel-L2 2e-5 of
    FP64 and exactly real. Either way, after a wrapping range of ring slots is rewritten and only
    those slots re-split, the update of the rows and columns of their slot blocks (64 frames complex,
    128 real) equals the full recomputation from the planes bit for bit."""
    L = hv.lib()
    ring = _ring(T, npix, T + 7)
    if real:
        ring = ring.real.astype(np.complex64)
    rd = dev(ring)
    work = empty(L.hv_pca_cov_workspace(T, npix))
    planes = empty(L.hv_pca_planes_bytes(T, npix, real))
    assert L.hv_pca_planes_bytes(T, npix, real) == (4 if real else 8) * T * npix
    cov_ring, cov_pl = empty(T * T * 16), empty(T * T * 16)
    L.hv_pca_covariance_mode(2)
    try:
        call("hv_pca_covariance", ptr(rd), T, npix, ptr(cov_ring), ptr(work), None)
        call("hv_pca_split_planes", ptr(rd), T, npix, 0, T, real, ptr(planes), None)
        call("hv_pca_covariance_planes", ptr(planes), T, npix, real, 0xFFFFFFFF, ptr(cov_pl), ptr(work), None)
        cuda.cuda.synchronize()
        assert L.hv_pca_covariance_status(ptr(work)) == hv.HV_OK
        a, b = host(cov_ring, np.complex128, (T, T)), host(cov_pl, np.complex128, (T, T))
        if real:
            assert not np.any(b.imag)
            assert rel_l2(b, a) <= 2e-5
        else:
            assert np.array_equal(a, b), float(np.abs(a - b).max() / np.abs(a).max())
        assert rel_l2(b, O.pca_covariance(ring.astype(np.complex128).reshape(T, npix, 1))) <= 2e-5
        # rewrite slots T - 20 .. T + 29 (mod T)
        slot0, n = T - 20, min(50, T)
        slots = [(slot0 + f) % T for f in range(n)]
        ring2 = ring.copy()
        new = _ring(T, npix, T + 8)
        ring2[slots] = (new.real.astype(np.complex64) if real else new)[slots]
        rd2 = dev(ring2)
        fb = 128 if real else 64
        blocks = 0
        for sl in slots:
            blocks |= 1 << (sl // fb)
        call("hv_pca_split_planes", ptr(rd2), T, npix, slot0, n, real, ptr(planes), None)
        call("hv_pca_covariance_planes", ptr(planes), T, npix, real, blocks, ptr(cov_pl), ptr(work), None)
        # the full recomputation from freshly split planes
        planes2 = empty(L.hv_pca_planes_bytes(T, npix, real))
        cov_full = empty(T * T * 16)
        call("hv_pca_split_planes", ptr(rd2), T, npix, 0, T, real, ptr(planes2), None)
        call("hv_pca_covariance_planes", ptr(planes2), T, npix, real, 0xFFFFFFFF, ptr(cov_full), ptr(work), None)
        if not real:
            call("hv_pca_covariance", ptr(rd2), T, npix, ptr(cov_ring), ptr(work), None)
        cuda.cuda.synchronize()
        assert L.hv_pca_covariance_status(ptr(work)) == hv.HV_OK
    finally:
        L.hv_pca_covariance_mode(0)
    a, b = host(cov_full, np.complex128, (T, T)), host(cov_pl, np.complex128, (T, T))
    assert np.array_equal(a, b), float(np.abs(a - b).max() / np.abs(a).max())
    if not real:
        assert np.array_equal(host(cov_ring, np.complex128, (T, T)), b)
    # the SIMT mode has no planes path
    L.hv_pca_covariance_mode(1)
    try:
        assert L.hv_pca_covariance_planes(ptr(planes), T, npix, real, 0xFFFFFFFF, ptr(cov_pl), ptr(work), None) == \
            hv.HV_ERR_UNSUPPORTED
    finally:
        L.hv_pca_covariance_mode(0)


@pytest.mark.gpu
@pytest.mark.parametrize("precision", [0, 1])
@pytest.mark.parametrize("T", [2, 31, 64, 96, 129, 256, 512])
def test_jacobi_paths(cuda, T, precision):
    """T <= 64: one CTA, A and V in shared memory; 64 < T <= 512: FP32 sweeps over a cooperative
    grid (precision 0) or one CTA in FP64 (precision 1, run here up to T = 129); both followed by
    the FP64 Rayleigh finish."""
    if precision == 1 and T > 129:
        pytest.skip("the single-CTA FP64 sweeps are only run at small T")
    rng = np.random.default_rng(T)
    X = rng.standard_normal((T, T)) + 1j * rng.standard_normal((T, T))
    A = X @ X.conj().T + np.diag(np.arange(T) * 3.0)
    covd = dev(A.astype(np.complex128))
    evals = empty(T * 8)
    evecs = empty(T * T * 16)
    work = empty(hv.lib().hv_pca_eigh_workspace(T))
    hv.lib().hv_pca_eig_precision(precision)
    try:
        call("hv_pca_eigh", ptr(covd), T, ptr(evals), ptr(evecs), 0, 0, None, ptr(work), None)
    finally:
        hv.lib().hv_pca_eig_precision(0)
    ev = host(evals, np.float64, (T,))
    V = host(evecs, np.complex128, (T, T)).T
    w = np.linalg.eigvalsh(A)
    fp64 = precision == 1
    # FP32 sweeps: eigenvectors to ~1e-6 (a few times more at T = 512), eigenvalues (Rayleigh
    # quotients in FP64) to second order; the column of rank pmin..pmax (here 0) is then refined in
    # FP64, so it is checked apart: its residual at the FP64 level (the FP32 columns are
    # orthonormal among themselves; the refined one is more accurate than they are)
    big = max(1.0, T / 64.0)
    tol_v, tol_w = (1e-10, 1e-9) if fp64 else (2e-5 * big, 1e-7 * big)
    assert np.abs(ev - w).max() <= tol_w * np.abs(w).max()
    rest = slice(1, T)
    Vr = V[:, rest]
    assert np.abs(Vr.conj().T @ Vr - np.eye(Vr.shape[1])).max() < tol_v
    assert np.abs(A @ Vr - Vr * ev[None, rest]).max() <= (1e-9 if fp64 else 3e-5 * big) * np.abs(w).max()
    v0 = V[:, 0]
    assert abs(np.linalg.norm(v0) - 1.0) < 1e-12
    assert np.linalg.norm(A @ v0 - ev[0] * v0) <= 1e-9 * np.abs(w).max()
