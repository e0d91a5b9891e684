"""PCA time transform: covariance H^H H (FP32 accumulation), FP64 Jacobi eigensolve and the fused
projection + view, against the oracle (numpy FP64 eigh). Tolerances: covariance rel-L2 <= 1e-5,
eigenvalues rel <= 1e-6 of the largest, views of |projection| rel-L2 <= 1e-4 (eigenvector phases
are arbitrary, so only |.| and |.|^2 views are comparable)."""

import numpy as np
import pytest

import holovibes_oracle as O
from gpu_util import call, dev, empty, host, ptr, rel_l2

import holovibes_gb300 as hv


def _modal_ring(T, H, W, modes, seed):
    rng = np.random.default_rng(seed)
    t = np.arange(T)
    ring = np.zeros((T, H, W), np.complex128)
    for m in range(modes):
        f = rng.uniform(0.02, 0.48)
        field = (rng.standard_normal((H, W)) + 1j * rng.standard_normal((H, W))) / (m + 1)
        ring += np.exp(2j * np.pi * f * t)[:, None, None] * field[None]
    ring += 0.01 * (rng.standard_normal((T, H, W)) + 1j * rng.standard_normal((T, H, W)))
    return ring.astype(np.complex64)


@pytest.mark.gpu
@pytest.mark.parametrize("T,H,W", [(32, 64, 64), (16, 40, 24), (64, 32, 32), (33, 16, 16), (8, 128, 128)])
def test_covariance_and_eigh(cuda, T, H, W):
    ring = _modal_ring(T, H, W, min(T, 6), T)
    npix = H * W
    cov = empty(T * T * 16)
    work = empty(hv.lib().hv_pca_cov_workspace(T, npix))
    rd = dev(ring)
    call("hv_pca_covariance", ptr(rd), T, npix, ptr(cov), ptr(work), None)
    got = host(cov, np.complex128, (T, T))
    ref = O.pca_covariance(ring.astype(np.complex128))
    assert rel_l2(got, ref) <= 1e-5
    evals = empty(T * 8)
    evecs = empty(T * T * 16)
    pmin, pmax = T - 4 if T >= 4 else 0, T - 1
    K = pmax - pmin + 1
    wts = empty(K * T * 8)
    ework = empty(hv.lib().hv_pca_eigh_workspace(T))
    call("hv_pca_eigh", ptr(cov), T, ptr(evals), ptr(evecs), pmin, pmax, ptr(wts), ptr(ework), None)
    ev = host(evals, np.float64, (T,))
    w_ref, V_ref = O.pca_eigh(ref)
    assert np.all(np.diff(ev) >= -1e-9 * abs(ev).max())
    assert np.abs(ev - w_ref).max() <= 1e-6 * np.abs(w_ref).max()
    V = host(evecs, np.complex128, (T, T)).T  # stored column-major: V[:, j] = evecs[j]
    # orthonormal and A V = V diag(w): FP32 sweeps (the default for T <= 64) give eigenvectors to
    # ~1e-6; each column is normalised in FP64
    assert np.abs(np.abs(np.diag(V.conj().T @ V)) - 1.0).max() < 1e-12
    assert np.abs(V.conj().T @ V - np.eye(T)).max() < 2e-6
    assert np.abs(ref @ V - V * ev[None, :]).max() <= 3e-5 * np.abs(w_ref).max()
    # fused projection + squared-modulus view on the selected components
    out = empty(npix * 4)
    call("hv_time_view", ptr(rd), T, W, H, ptr(wts), K, hv.IMG_SQUARED_MODULUS, 131071.0, 0, ptr(out), None, None)
    got_view = host(out, np.float32, (H, W))
    ref_view = O.view(O.pca_project(ring.astype(np.complex128), V_ref, pmin, pmax), "SQUARED_MODULUS") * O.PCA_SCALE
    assert rel_l2(got_view, ref_view) <= 1e-4
