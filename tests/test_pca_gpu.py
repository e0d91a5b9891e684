"""PCA time transform: covariance H^H H (FP32 accumulation), the Jacobi eigensolve (FP32 sweeps, FP64
Rayleigh quotients, FP64 refinement of the kept eigenvectors) and the fused projection + view,
against the oracle (numpy FP64 eigh). Tolerances: covariance rel-L2 <= 1e-5, eigenvalues within
1e-5 of the largest (kept ones 1e-6, the covariance's FP32 accumulation), views of |projection| rel-L2 <= 1e-4 (eigenvector phases are
arbitrary, so only |.| and |.|^2 views are comparable). A second window of the same ring through
a Pipe exercises the warm start from the previous window's eigenvectors."""

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
    wmax = np.abs(w_ref).max()
    assert np.all(np.diff(ev) >= -1e-9 * abs(ev).max())
    V = host(evecs, np.complex128, (T, T)).T  # stored column-major: V[:, j] = evecs[j]
    # FP32 sweeps (the default for T <= 64, stopping at the round-off level of the matrix) give
    # eigenvectors orthonormal to ~1e-6 and eigenvalues (FP64 Rayleigh quotients) to ~1e-5 of the
    # largest; the kept columns pmin..pmax are then refined in FP64 against the GPU's covariance
    # (their residual and eigenvalue are then limited by that covariance). Every column is
    # normalised in FP64.
    kept = np.arange(pmin, pmax + 1)
    rest = np.setdiff1d(np.arange(T), kept)
    assert np.abs(ev - w_ref).max() <= 1e-5 * wmax
    # (against the exact covariance: the FP32-accumulated covariance bounds these)
    assert np.abs(ev[kept] - w_ref[kept]).max() <= 1e-6 * wmax
    assert np.abs(np.abs(np.diag(V.conj().T @ V)) - 1.0).max() < 1e-12
    Vr = V[:, rest]
    assert np.abs(Vr.conj().T @ Vr - np.eye(len(rest))).max() < 2e-6
    assert np.abs(ref @ V - V * ev[None, :]).max() <= 3e-5 * wmax
    assert np.abs(ref @ V[:, kept] - V[:, kept] * ev[None, kept]).max() <= 1e-6 * wmax
    # fused projection + squared-modulus view on the selected components
    out = empty(npix * 4)
    call("hv_time_view", ptr(rd), T, W, H, ptr(wts), K, hv.IMG_SQUARED_MODULUS, 131071.0, 0, ptr(out), None, None)
    got_view = host(out, np.float32, (H, W))
    ref_view = O.view(O.pca_project(ring.astype(np.complex128), V_ref, pmin, pmax), "SQUARED_MODULUS") * O.PCA_SCALE
    assert rel_l2(got_view, ref_view) <= 1e-4


@pytest.mark.gpu
@pytest.mark.parametrize("T,img,cholqr", [(32, 0, 1), (64, 1, 1), (16, 0, 1), (128, 0, 1), (256, 1, 1), (128, 0, 0),
                                         (256, 1, 0)])
def test_pipe_pca_windows_warm_start(cuda, T, img, cholqr):
    """Consecutive PCA windows of one Pipe: from the second window on, the eigensolve starts from
    the previous window's eigenvectors (T <= 64: the FP32 Jacobi sweeps; T > 64 with the dominant
    components kept: the subspace iteration from the previous Ritz vectors, orthonormalised by
    Cholesky-QR, or by Gram-Schmidt with cholqr = 0). Every window's float frame within rel-L2 1e-4
    of the oracle (modulus views depend on each kept eigenvector, not only on the kept subspace)."""
    from gpu_util import oracle_settings

    from holovibes_gb300.synthetic import Interferogram

    W = H = 64
    fd = hv.FrameDescriptor(W, H, 2)
    s = hv.Settings.defaults().update(space_transformation=1, time_transformation=2, time_transformation_size=T,
                                      time_stride=T // 2, batch_size=T // 2, z_distance=0.3, pixel_size=20.0,
                                      image_type=img, p_start=T - 4, p_width=3, renorm=1,
                                      contrast_enabled=0).validate(fd)
    raw = Interferogram(width=W, height=H, seed=T + img, modes=8).frames(0, 6 * T // 2)
    oracle = O.OraclePipe(oracle_settings(fd, s))
    hv.lib().hv_pca_eig_cholqr(cholqr)
    try:
        pipe = hv.Pipe(fd, s)
        errs = []
        for b in range(6):
            batch = raw[b * (T // 2):(b + 1) * (T // 2)]
            ref = oracle.process_batch(batch)
            pipe.enqueue(batch)
            if ref is None:
                continue
            pipe.pull()
            errs.append(rel_l2(pipe.float_frame(), ref.float_frame))
        pipe.close()
    finally:
        hv.lib().hv_pca_eig_cholqr(1)
    assert len(errs) == 5
    assert max(errs) <= 1e-4, errs


@pytest.mark.gpu
@pytest.mark.parametrize("T,B,p_start,modes,space,depth", [(128, 24, 124, 8, 1, 2), (192, 40, 175, 24, 1, 2),
                                                             (256, 64, 252, 8, 1, 2), (128, 32, 124, 8, 0, 2),
                                                             (192, 64, 188, 8, 0, 1)])
def test_pipe_incremental_covariance_bit_identical(cuda, T, B, p_start, modes, space, depth):
    """Sliding windows (stride B < T): between two renders only the ring slots of one stride are
    rewritten, and the Pipe recomputes only the covariance rows and columns of the 64-frame slot
    blocks holding them (batches not aligned to the blocks and wrapping around the ring here; the
    subspace iteration for the dominant components, the block Jacobi for ranks 175-178 of T = 192 with
    24 seeded modes: two pairs of close eigenvalues with gaps of 25% and 18% to the ranks outside, and
    the squared-modulus view, invariant to rotations inside the kept subspace, so that the oracle
    comparison is well conditioned; without a spatial transform the windows run on the three-stream
    pipeline with real planes). Every output (float frame and uint16) is bit-identical to the same Pipe recomputing the whole covariance at
    every window, and within rel-L2 1e-4 of the oracle."""
    from gpu_util import oracle_settings

    from holovibes_gb300.synthetic import Interferogram

    W = H = 64
    fd = hv.FrameDescriptor(W, H, depth)
    s = hv.Settings.defaults().update(space_transformation=space, time_transformation=2, time_transformation_size=T,
                                      time_stride=B, batch_size=B, z_distance=0.3, pixel_size=20.0, image_type=1,
                                      p_start=p_start, p_width=3, renorm=1, contrast_enabled=1).validate(fd)
    nb = -(-T // B) + 8
    raw = Interferogram(width=W, height=H, seed=T + B, modes=modes, dtype=np.uint8 if depth == 1 else np.uint16,
                        max_value=255 if depth == 1 else 4095).frames(0, nb * B)
    outs = {}
    for inc in (1, 0):
        hv.lib().hv_pca_cov_incremental(inc)
        try:
            pipe = hv.Pipe(fd, s)
            frames = []
            for b in range(nb):
                pipe.enqueue(raw[b * B:(b + 1) * B])
                if pipe.output_count():
                    u16 = pipe.pull()
                    frames.append((pipe.float_frame().copy(), np.array(u16, copy=True)))
            pipe.close()
        finally:
            hv.lib().hv_pca_cov_incremental(1)
        outs[inc] = frames
    assert len(outs[1]) == len(outs[0]) >= 8
    for k, ((f1, u1), (f0, u0)) in enumerate(zip(outs[1], outs[0])):
        assert np.array_equal(f1, f0), (k, float(np.abs(f1 - f0).max()))
        assert np.array_equal(u1, u0), k
    oracle = O.OraclePipe(oracle_settings(fd, s))
    errs = []
    for b in range(nb):
        ref = oracle.process_batch(raw[b * B:(b + 1) * B])
        if ref is not None:
            errs.append(rel_l2(outs[1][len(errs)][0], ref.float_frame))
    assert len(errs) == len(outs[1])
    assert max(errs) <= 1e-4, errs


@pytest.mark.gpu
def test_pipe_pca_pipeline_unaligned_device_batches(cuda):
    """PCA windows on the three-stream pipeline fed with device batches off 16-byte alignment (the
    conversion then writes the ring on the pipe stream and splits it): every output equals the same
    windows fed from aligned host batches, and is within rel-L2 1e-4 of the oracle."""
    import torch
    from gpu_util import oracle_settings

    from holovibes_gb300.synthetic import Interferogram

    T, B, W, H = 128, 32, 64, 64
    fd = hv.FrameDescriptor(W, H, 2)
    s = hv.Settings.defaults().update(space_transformation=0, time_transformation=2, time_transformation_size=T,
                                      time_stride=B, batch_size=B, image_type=1, p_start=T - 4, p_width=3, renorm=1,
                                      contrast_enabled=1).validate(fd)
    nb = T // B + 6
    raw = Interferogram(width=W, height=H, seed=7, modes=8).frames(0, nb * B)
    outs = []
    for unaligned in (0, 1):
        pipe = hv.Pipe(fd, s)
        frames = []
        buf = torch.empty(raw[:B].nbytes + 16, dtype=torch.uint8, device="cuda")
        for b in range(nb):
            batch = np.ascontiguousarray(raw[b * B:(b + 1) * B])
            if unaligned:
                src = torch.from_numpy(batch.view(np.uint8).reshape(-1).copy()).cuda()
                buf[2:2 + src.numel()].copy_(src)
                torch.cuda.synchronize()
                pipe.enqueue_ptr(buf.data_ptr() + 2, B, hv.MEM_DEVICE)
                pipe.sync()
            else:
                pipe.enqueue(batch)
            if pipe.output_count():
                pipe.pull()
                frames.append(pipe.float_frame().copy())
        pipe.close()
        outs.append(frames)
    assert len(outs[0]) == len(outs[1]) == nb - T // B + 1
    for a, b2 in zip(*outs):
        assert np.array_equal(a, b2)
    oracle = O.OraclePipe(oracle_settings(fd, s))
    k = 0
    for b in range(nb):
        ref = oracle.process_batch(raw[b * B:(b + 1) * B])
        if ref is not None:
            assert rel_l2(outs[0][k], ref.float_frame) <= 1e-4
            k += 1
