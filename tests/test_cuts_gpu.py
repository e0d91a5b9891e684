"""XZ / YZ time-transformation cuts (hv_time_cuts) against the oracle's restatement of
fill_32bit_slices (stft.cu:17-115): rel-L2 <= 1e-5 for modulus / squared modulus; argument
(atanf(Im/Re) + pi/2, which jumps by pi where Re changes sign) elementwise within 1e-4 on all but
1% of the elements; other image types give 0."""

import numpy as np
import pytest

import holovibes_oracle as O
from gpu_util import call, dev, empty, host, ptr, rel_l2

import holovibes_gb300 as hv

IMG = {0: "MODULUS", 1: "SQUARED_MODULUS", 2: "ARGUMENT", 3: "PHASE_INCREASE", 6: "MOMENTS_1"}


@pytest.mark.gpu
@pytest.mark.parametrize("W,H,T,band", [(64, 48, 16, (10, 12, 20, 23)), (40, 24, 7, (0, 0, 23, 23)),
                                        (96, 64, 32, (95, 95, 0, 63)), (32, 32, 128, (5, 9, 3, 3))])
@pytest.mark.parametrize("img", [0, 1, 2, 3, 6])
def test_time_cuts_stft(cuda, W, H, T, band, img):
    xmin, xmax, ymin, ymax = band
    rng = np.random.default_rng(W + T + img)
    ring = (rng.standard_normal((T, H, W)) + 1j * rng.standard_normal((T, H, W))).astype(np.complex64)
    w = empty(T * T * 8)
    call("hv_stft_weights", ptr(w), T, 0, T - 1, None)
    xz, yz = empty(T * W * 4), empty(H * T * 4)
    work = empty(hv.lib().hv_time_cuts_workspace(W, H, T, xmin, xmax, ymin, ymax))
    call("hv_time_cuts", ptr(dev(ring)), T, W, H, ptr(w), xmin, xmax, ymin, ymax, img, ptr(xz), ptr(yz), ptr(work),
         None)
    got = (host(xz, np.float32, (T, W)), host(yz, np.float32, (H, T)))
    p_acc = O.all_bins(ring.astype(np.complex128), "STFT")
    ref = O.time_cuts(p_acc, xmin, xmax, ymin, ymax, IMG[img])
    for g, r in zip(got, ref):
        if img == 6:
            assert np.all(g == 0)
        elif img == 2:
            assert np.mean(np.abs(g - r) > 1e-4) < 1e-2
        else:
            assert rel_l2(g, r) <= 1e-5


@pytest.mark.gpu
def test_time_cuts_pca_components(cuda):
    """With the eigenvector columns as weights the cuts show every PCA component (H V)."""
    W, H, T = 48, 32, 12
    rng = np.random.default_rng(11)
    ring = (rng.standard_normal((T, H, W)) + 1j * rng.standard_normal((T, H, W))).astype(np.complex64)
    _, V = O.pca_eigh(O.pca_covariance(ring.astype(np.complex128)))
    w = dev(np.ascontiguousarray(V.T).astype(np.complex64))  # row j = column j of V
    xz, yz = empty(T * W * 4), empty(H * T * 4)
    work = empty(hv.lib().hv_time_cuts_workspace(W, H, T, 3, 4, 30, 31))
    call("hv_time_cuts", ptr(dev(ring)), T, W, H, ptr(w), 3, 4, 30, 31, 1, ptr(xz), ptr(yz), ptr(work), None)
    ref = O.time_cuts(O.all_bins(ring.astype(np.complex128), "PCA", V), 3, 4, 30, 31, "SQUARED_MODULUS")
    assert rel_l2(host(xz, np.float32, (T, W)), ref[0]) <= 1e-5
    assert rel_l2(host(yz, np.float32, (H, T)), ref[1]) <= 1e-5


@pytest.mark.gpu
def test_time_cuts_rejects(cuda):
    lib = hv.lib()
    w, out, work = empty(64), empty(64), empty(64)
    ring = empty(64)
    # band outside the frame, window above the shared-memory bound
    assert lib.hv_time_cuts(ptr(ring), 4, 8, 8, ptr(w), 7, 8, 0, 0, 0, ptr(out), ptr(out), ptr(work), None) == \
        hv.HV_INVALID_VALUE
    assert lib.hv_time_cuts(ptr(ring), 513, 8, 8, ptr(w), 0, 0, 0, 0, 0, ptr(out), ptr(out), ptr(work), None) == \
        hv.HV_ERR_UNSUPPORTED
