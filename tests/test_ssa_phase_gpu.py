"""SSA_STFT weights (hv_ssa_weights against the oracle's V_Q V_Q^H then STFT, rel-L2 <= 1e-6: FP64
arithmetic rounded to complex64) and the phase increase kernels (hv_phase_increase over three
windows with its history, then hv_rescale_float; increments compared as wrapped angles within
2e-6 rad on all but branch-cut pixels, the rescale bit-exact on the kernel's own increments)."""

import numpy as np
import pytest

import holovibes_oracle as O
from gpu_util import call, dev, empty, host, ptr, rel_l2, wrapped_diff, zeros

import holovibes_gb300 as hv


@pytest.mark.gpu
@pytest.mark.parametrize("T,q_start,q_width,pmin,pmax", [(16, 13, 2, 1, 3), (32, 4, 9, 0, 31), (12, 0, 0, 2, 7),
                                                         (64, 40, 20, 5, 20)])
def test_ssa_weights(cuda, T, q_start, q_width, pmin, pmax):
    rng = np.random.default_rng(T + q_start)
    A = rng.standard_normal((T, T)) + 1j * rng.standard_normal((T, T))
    _, V = np.linalg.eigh(A @ A.conj().T)
    K = pmax - pmin + 1
    w = empty(K * T * 8)
    call("hv_ssa_weights", ptr(dev(np.ascontiguousarray(V.T))), T, q_start, q_width, pmin, pmax, ptr(w), None)
    got = host(w, np.complex64, (K, T))
    q, qn = O.ssa_q_range(q_start, q_width, T)
    tmp = V[:, q:q + qn] @ V[:, q:q + qn].conj().T
    t = np.arange(T)
    F = np.exp(-2j * np.pi * np.outer(np.arange(pmin, pmax + 1), t) / T)  # [K, T]
    ref = (tmp @ F.T).T  # w[k][s] = sum_t tmp[s, t] F[k, t]
    assert rel_l2(got, ref) <= 1e-6
    # the weights reproduce the oracle's SSA bins on a ring
    ring = (rng.standard_normal((T, 3, 5)) + 1j * rng.standard_normal((T, 3, 5)))
    bins = np.tensordot(got.astype(np.complex128), ring, axes=(1, 0))
    assert rel_l2(bins, O.ssa_stft_bins(ring, V, q_start, q_width, pmin, pmax)) <= 1e-6


@pytest.mark.gpu
def test_ssa_weights_rejects_bad_ranges(cuda):
    w = empty(64 * 8)
    ev = zeros(16 * 16 * 16)
    lib = hv.lib()
    assert lib.hv_ssa_weights(ptr(ev), 16, 10, 7, 0, 1, ptr(w), None) == hv.HV_INVALID_VALUE  # q past T
    assert lib.hv_ssa_weights(ptr(ev), 16, 0, 2, 3, 16, ptr(w), None) == hv.HV_INVALID_VALUE  # p past T


@pytest.mark.gpu
@pytest.mark.parametrize("W,H,T", [(160, 128, 8), (40, 24, 5)])
def test_phase_increase_windows(cuda, W, H, T):
    HW = W * H
    rng = np.random.default_rng(W + T)
    wrow = np.exp(-2j * np.pi * 1 * np.arange(T) / T).astype(np.complex64)
    pred, hist = empty(HW * 8), empty(HW * 4)
    out, res = empty(HW * 4), empty(HW * 4)
    mm = empty(hv.lib().hv_phase_increase_workspace(HW))
    pi = O.PhaseIncrease()
    base = rng.standard_normal((T, H, W)) + 1j * rng.standard_normal((T, H, W))
    for n in range(3):
        ring = (base * np.exp(1j * 0.7 * n * rng.standard_normal((1, H, W)))).astype(np.complex64)
        call("hv_phase_increase", ptr(dev(ring)), T, W, H, ptr(dev(wrow)), ptr(pred), ptr(hist), int(n == 0),
             int(n > 0), ptr(out), ptr(mm), None)
        call("hv_rescale_float", ptr(out), HW, ptr(mm), 1.0, ptr(res), None)
        got = host(out, np.float32, (H, W))
        X = np.tensordot(wrow.astype(np.complex128), ring.astype(np.complex128), axes=(0, 0))
        ref = pi.push(X)
        d = np.abs(wrapped_diff(got, ref))
        assert np.mean(d > 1e-4) < 2e-3
        assert np.median(d) < 2e-6
        # the rescale of the kernel's own increments: bit-exact float32 arithmetic
        assert np.array_equal(host(res, np.float32, (H, W)), O.rescale_float(got).astype(np.float32))
