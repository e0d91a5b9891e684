"""Serving engine (hv_server_*): every served stream produces exactly the holograms of a plain Pipe
fed the same frames (uint16 outputs and float frames bit-identical), alone and in a mix of
streams of different shapes, time transforms and settings sharing buckets and graphs; with and
without CUDA graphs; admission by HBM footprint (immediate refusal and bounded wait); latency
statistics. Bar: bit-exact (same kernels, same inputs, deterministic reductions)."""

import threading
import time

import numpy as np
import pytest

import holovibes_gb300 as hv
from holovibes_gb300.synthetic import Interferogram

# name: (W, H, depth, settings, batches)
STREAMS = {
    "as_stft_mod": (64, 64, 2, dict(space_transformation=2, time_transformation=1, time_transformation_size=8,
                                    time_stride=4, batch_size=4, z_distance=0.3, pixel_size=20.0, p_start=1,
                                    fft_shift=1, renorm=0, contrast_enabled=1, contrast_lower=0.5,
                                    contrast_upper=99.5), 8),
    # same bucket as as_stft_mod (same shape key), other physical and view parameters
    "as_stft_acc": (64, 64, 2, dict(space_transformation=2, time_transformation=1, time_transformation_size=8,
                                    time_stride=4, batch_size=4, z_distance=0.45, pixel_size=12.0, p_start=2,
                                    p_width=1, renorm=1, accumulation=3, contrast_enabled=1, contrast_lower=1.0,
                                    contrast_upper=99.0), 9),
    "fresnel_tc_arg": (96, 64, 1, dict(space_transformation=1, time_transformation=1, time_transformation_size=32,
                                       time_stride=8, batch_size=8, lambda_=785e-9, z_distance=0.45, pixel_size=12.0,
                                       image_type=2, p_start=3, p_width=10, renorm=1, contrast_enabled=1), 7),
    "fresnel_pca": (64, 64, 1, dict(space_transformation=1, time_transformation=2, time_transformation_size=16,
                                    time_stride=8, batch_size=8, lambda_=785e-9, z_distance=0.45, pixel_size=12.0,
                                    image_type=1, p_start=12, p_width=3, renorm=1, contrast_enabled=1), 5),
    "as_unwrap": (64, 64, 2, dict(space_transformation=2, time_transformation=1, time_transformation_size=8,
                                  time_stride=8, batch_size=8, z_distance=0.3, pixel_size=20.0, image_type=2,
                                  p_start=1, unwrap_2d=1, renorm=1, contrast_enabled=1), 4),
    "stride_drop": (32, 32, 2, dict(space_transformation=0, time_transformation=1, time_transformation_size=4,
                                    time_stride=4, batch_size=2, p_start=1, renorm=1, contrast_enabled=0), 12),
    # same bucket as as_stft_mod, but its history keeps every cycle eager (never in a graph)
    "as_phase_inc": (64, 64, 2, dict(space_transformation=2, time_transformation=1, time_transformation_size=8,
                                     time_stride=4, batch_size=4, z_distance=0.35, pixel_size=20.0, image_type=3,
                                     p_start=1, renorm=1, contrast_enabled=1), 8),
    "as_ssa": (64, 64, 2, dict(space_transformation=2, time_transformation=3, time_transformation_size=16,
                               time_stride=8, batch_size=8, z_distance=0.3, pixel_size=20.0, q_start=13, q_width=2,
                               p_start=1, p_width=2, renorm=1, contrast_enabled=1), 5),
}


def _bucket_count(names):
    keys = set()
    for n in names:
        W, H, depth, over, _ = STREAMS[n]
        keys.add((W, H, depth, over["space_transformation"], over["time_transformation"],
                  over["time_transformation_size"], over["batch_size"]))
    return len(keys)


def _setup(name):
    W, H, depth, over, nb = STREAMS[name]
    fd = hv.FrameDescriptor(W, H, depth, 0)
    s = hv.Settings.defaults().update(**over).validate(fd)
    dt = {1: np.uint8, 2: np.uint16}[depth]
    g = Interferogram(width=W, height=H, seed=len(name) * 7 + 1, dtype=dt, max_value=255 if depth == 1 else 4095,
                      modes=6)
    frames = g.frames(0, s.batch_size * nb)
    return fd, s, frames


def _plain(name):
    fd, s, frames = _setup(name)
    B = s.batch_size
    pipe = hv.Pipe(fd, s)
    outs, floats = [], []
    for b in range(len(frames) // B):
        pipe.enqueue(frames[b * B:(b + 1) * B])
        while pipe.output_count():
            outs.append(pipe.pull())
            floats.append(pipe.float_frame())
    pipe.close()
    return outs, floats


def _served(names, flags=0):
    """Pushes every stream's batches round-robin into one server; returns outputs per stream."""
    setups = {n: _setup(n) for n in names}
    srv = hv.Server(flags=flags)
    streams = {n: srv.open_stream(fd, s) for n, (fd, s, _) in setups.items()}
    outs = {n: [] for n in names}
    last_float = {}
    nmax = max(len(f) // s.batch_size for (_, s, f) in setups.values())
    for b in range(nmax):
        for n in names:
            fd, s, frames = setups[n]
            B = s.batch_size
            if (b + 1) * B <= len(frames):
                streams[n].enqueue(frames[b * B:(b + 1) * B])
        # pull as we go (the output queues stay short), in any order
        for n in names:
            while streams[n].output_count():
                outs[n].append(streams[n].pull())
    srv.sync()
    for n in names:
        while streams[n].output_count():
            outs[n].append(streams[n].pull())
        if outs[n]:
            last_float[n] = streams[n].float_frame()
    stats = srv.stats()
    srv.close()
    return outs, last_float, stats


@pytest.mark.gpu
def test_served_mix_matches_plain(cuda):
    names = sorted(STREAMS)
    outs, last_float, stats = _served(names)
    total = 0
    for n in names:
        ref, ref_f = _plain(n)
        assert len(outs[n]) == len(ref) and len(ref) > 0, n
        for a, b in zip(outs[n], ref):
            assert np.array_equal(a, b), n
        assert np.array_equal(last_float[n], ref_f[-1]), n
        total += len(ref)
    assert stats["outputs"] == total
    assert stats["graph_launches"] > 0 and stats["captures"] > 0
    assert stats["eager_cycles"] > 0  # PCA / unwrap streams and warm-up cycles
    assert stats["latency_samples"] == total
    assert 0 < stats["latency_p50_us"] <= stats["latency_p99_us"]
    assert stats["streams"] == len(names) and stats["buckets"] == _bucket_count(names) < len(names)


@pytest.mark.gpu
def test_same_alone_and_in_the_mix(cuda):
    alone, alone_f, _ = _served(["fresnel_tc_arg"])
    mix, mix_f, _ = _served(["fresnel_tc_arg", "as_stft_mod", "as_stft_acc", "fresnel_pca"])
    assert len(alone["fresnel_tc_arg"]) == len(mix["fresnel_tc_arg"]) > 0
    for a, b in zip(alone["fresnel_tc_arg"], mix["fresnel_tc_arg"]):
        assert np.array_equal(a, b)
    assert np.array_equal(alone_f["fresnel_tc_arg"], mix_f["fresnel_tc_arg"])


@pytest.mark.gpu
def test_graphs_and_direct_launches_agree(cuda):
    names = ["as_stft_mod", "as_stft_acc", "stride_drop"]
    g_out, _, g_stats = _served(names)
    e_out, _, e_stats = _served(names, flags=hv.SERVER_NO_GRAPHS)
    s_out, _, s_stats = _served(names, flags=hv.SERVER_STREAM_GRAPHS)
    assert g_stats["graph_launches"] > 0 and e_stats["graph_launches"] == 0 and s_stats["graph_launches"] > 0
    for n in names:
        assert len(g_out[n]) == len(e_out[n]) == len(s_out[n]) > 0
        for a, b, c in zip(g_out[n], e_out[n], s_out[n]):
            assert np.array_equal(a, b), n
            assert np.array_equal(a, c), n


@pytest.mark.gpu
def test_stream_graph_mode_mix_matches_plain(cuda):
    names = sorted(STREAMS)
    outs, last_float, stats = _served(names, flags=hv.SERVER_STREAM_GRAPHS)
    for n in names:
        ref, ref_f = _plain(n)
        assert len(outs[n]) == len(ref) > 0, n
        for a, b in zip(outs[n], ref):
            assert np.array_equal(a, b), n
        assert np.array_equal(last_float[n], ref_f[-1]), n
    assert stats["graph_launches"] > 0


@pytest.mark.gpu
def test_device_push(cuda):
    import torch

    fd, s, frames = _setup("as_stft_mod")
    ref, _ = _plain("as_stft_mod")
    srv = hv.Server()
    st = srv.open_stream(fd, s)
    dev = torch.from_numpy(frames.view(np.int16).copy()).cuda()
    B = s.batch_size
    got = []
    for b in range(len(frames) // B):
        st.enqueue(dev[b * B:(b + 1) * B])
        srv.sync()
        while st.output_count():
            got.append(st.pull())
    srv.close()
    assert len(got) == len(ref)
    for a, b in zip(got, ref):
        assert np.array_equal(a, b)


@pytest.mark.gpu
def test_admission_by_footprint(cuda):
    fd, s, frames = _setup("as_stft_mod")
    fp = hv.Server.footprint(fd, s)
    assert fp > 0
    srv = hv.Server(hbm_budget=fp + fp // 2)
    a = srv.open_stream(fd, s)
    with pytest.raises(hv.HoloError) as e:
        srv.open_stream(fd, s)
    assert e.value.status == hv.HV_ERR_ADMISSION
    assert srv.stats()["hbm_used"] == fp
    # a waiting open is admitted once the first stream closes
    got = {}

    def opener():
        got["s"] = srv.open_stream(fd, s, admit_timeout_us=5_000_000)

    t = threading.Thread(target=opener)
    t.start()
    time.sleep(0.2)
    assert "s" not in got
    a.close()
    t.join(10)
    assert "s" in got
    b = got["s"]
    B = s.batch_size
    for k in range(len(frames) // B):
        b.enqueue(frames[k * B:(k + 1) * B])
    srv.sync()
    assert b.output_count() > 0
    srv.close()
    # a stream larger than the whole budget is refused outright
    small = hv.Server(hbm_budget=fp // 2)
    with pytest.raises(hv.HoloError) as e:
        small.open_stream(fd, s, admit_timeout_us=1_000_000)
    assert e.value.status == hv.HV_ERR_ADMISSION
    small.close()


@pytest.mark.gpu
def test_served_rejects_batch_larger_than_window(cuda):
    fd = hv.FrameDescriptor(32, 48, 2, 0)
    s = hv.Settings.defaults().update(space_transformation=0, time_transformation=1, time_transformation_size=3,
                                      time_stride=5, batch_size=5, p_start=1).validate(fd)
    srv = hv.Server()
    with pytest.raises(hv.HoloError) as e:
        srv.open_stream(fd, s)
    assert e.value.status == hv.HV_INVALID_VALUE
    assert srv.stats()["hbm_used"] == 0
    srv.close()
