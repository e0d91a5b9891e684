"""The CLI flow of the reference (cli.cc:100-162) through this build: a raw .holo recording with
its compute-settings footer -> Pipe -> a processed .holo of the uint16 holograms, read back
identical to the pipe's outputs, with the same settings in both footers."""

import numpy as np
import pytest

import holovibes_gb300 as hv
from holovibes_gb300.synthetic import Interferogram


@pytest.mark.gpu
def test_holo_in_pipe_holo_out(cuda, tmp_path):
    fd = hv.FrameDescriptor(64, 64, 2, 0)
    s = hv.Settings.defaults().update(space_transformation=2, time_transformation=1, time_transformation_size=8,
                                      time_stride=4, batch_size=4, z_distance=0.3, pixel_size=20.0, p_start=1,
                                      fft_shift=1, renorm=1, contrast_enabled=1, contrast_lower=0.5,
                                      contrast_upper=99.5).validate(fd)
    frames = Interferogram(width=64, height=64, seed=3).frames(0, 24)
    raw_path, out_path = tmp_path / "raw.holo", tmp_path / "out.holo"
    hv.write_holo(raw_path, fd, frames, s, input_fps=1000, data_type=hv.HOLO_RAW)

    with hv.HoloFile(raw_path) as f:
        fs = f.settings().validate(f.fd)
        pipe = hv.Pipe(f.fd, fs)
        B = fs.batch_size
        outs = []
        for b in range(f.nb_frames // B):
            pipe.enqueue(f.read(b * B, B))
            outs.extend(pipe.pull_all())
        pipe.close()
    assert len(outs) > 0
    ofd = hv.FrameDescriptor(64, 64, 2, 0)
    hv.write_holo(out_path, ofd, np.stack(outs), fs, input_fps=1000, data_type=hv.HOLO_PROCESSED)

    # the same holograms as a plain pipe fed the in-memory frames
    ref_pipe = hv.Pipe(fd, s)
    ref = []
    for b in range(len(frames) // 4):
        ref_pipe.enqueue(frames[b * 4:(b + 1) * 4])
        ref.extend(ref_pipe.pull_all())
    ref_pipe.close()
    with hv.HoloFile(out_path) as g:
        assert g.header.data_type == hv.HOLO_PROCESSED and g.nb_frames == len(ref)
        got = g.read()
        assert np.array_equal(got, np.stack(ref))
        gs = g.settings()
    for k in ("space_transformation", "time_transformation_size", "batch_size", "p_start", "fft_shift",
              "contrast_lower", "contrast_upper"):
        assert np.float32(getattr(gs, k)) == np.float32(getattr(s, k)), k
    assert gs.pixel_size == 20.0 and np.float32(gs.z_distance) == np.float32(0.3)
