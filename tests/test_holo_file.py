""".holo files (hv_holo_*, host only): the 64-byte header layout of the reference's format
(Backend/includes/io/holo_file.hh), frames and footer round trips, the reader's checks, and the
conversion of older footers (versions 2..6) and compute-settings documents (v0) to the current
version. The old-version documents below are written from the layouts those versions used."""

import json
import struct

import numpy as np
import pytest

import holovibes_gb300 as hv


def _settings():
    return hv.Settings.defaults().update(
        space_transformation=2, time_transformation=1, time_transformation_size=16, time_stride=8, batch_size=4,
        lambda_=785e-9, z_distance=0.45, pixel_size=12.0, image_type=1, p_start=3, p_width=2, fft_shift=1, renorm=1,
        renorm_constant=6, accumulation=3, log_enabled=0, contrast_enabled=1, contrast_auto_refresh=1,
        contrast_invert=1, contrast_min=3.0, contrast_max=4000.0, contrast_lower=0.5, contrast_upper=99.5,
        reticle_display=1, reticle_scale=0.4, output_buffer_size=64, input_buffer_size=128, q_start=3, q_width=4)


FIELDS = ["space_transformation", "time_transformation", "time_transformation_size", "time_stride", "batch_size",
          "lambda_", "z_distance", "pixel_size", "image_type", "p_start", "p_width", "fft_shift", "renorm",
          "renorm_constant", "accumulation", "log_enabled", "contrast_enabled", "contrast_auto_refresh",
          "contrast_invert", "contrast_min", "contrast_max", "contrast_lower", "contrast_upper", "reticle_display",
          "reticle_scale", "output_buffer_size", "input_buffer_size", "q_start", "q_width"]


def test_header_layout_and_round_trip(tmp_path):
    fd = hv.FrameDescriptor(40, 24, 2, 0)
    frames = (np.arange(7 * 24 * 40) % 4096).astype(np.uint16).reshape(7, 24, 40)
    s = _settings()
    path = tmp_path / "a.holo"
    hv.write_holo(path, fd, frames, s, input_fps=2000, camera_fps=2500, data_type=hv.HOLO_RAW)
    raw = path.read_bytes()
    magic, ver, bits, w, h, n, size, endian, dtype = struct.unpack_from("<4sHHIIIQBB", raw, 0)
    assert (magic, ver, bits, w, h, n, size, endian, dtype) == (b"HOLO", 7, 16, 40, 24, 7, 7 * 24 * 40 * 2, 0, 0)
    assert raw[30:64] == bytes(34)  # padding up to 64 bytes
    footer = json.loads(raw[64 + size:])
    assert set(footer) == {"compute_settings", "info"}
    assert footer["info"]["pixel_pitch"] == {"x": 12, "y": 12}
    assert footer["info"]["input_fps"] == 2000 and footer["info"]["camera_fps"] == 2500
    cs = footer["compute_settings"]
    assert cs["version"] == "v1"
    assert cs["image_rendering"]["space_transformation"] == "ANGULARSP"
    assert cs["view"]["image_type"] == "SQUARED_MODULUS"
    assert cs["view"]["z"] == {"width": 2, "start": 3}
    assert cs["view"]["z2"] == {"width": 4, "start": 3}
    with hv.HoloFile(path) as f:
        assert f.nb_frames == 7 and (f.fd.width, f.fd.height, f.fd.depth, f.fd.byte_endian) == (40, 24, 2, 0)
        assert np.array_equal(f.read(), frames)
        assert np.array_equal(f.read(3, 2), frames[3:5])
        got = f.settings()
    for k in FIELDS:
        assert np.float32(getattr(got, k)) == np.float32(getattr(s, k)), k


def test_reader_checks(tmp_path):
    fd = hv.FrameDescriptor(8, 8, 1, 0)
    frames = np.zeros((3, 8, 8), np.uint8)
    p = tmp_path / "b.holo"
    hv.write_holo(p, fd, frames)  # no footer
    with hv.HoloFile(p) as f:
        assert f.footer() == {}
        with pytest.raises(hv.HoloError) as e:
            f.settings()
        assert e.value.status == hv.HV_NO_IN_DATA
        with pytest.raises(hv.HoloError):
            f.read(2, 2)  # past the end
    raw = bytearray(p.read_bytes())
    bad = tmp_path / "c.holo"
    bad.write_bytes(b"HOLA" + bytes(raw[4:]))
    with pytest.raises(hv.HoloError):
        hv.HoloFile(bad)
    # total data size inconsistent with the frame description
    raw2 = bytearray(raw)
    struct.pack_into("<Q", raw2, 20, 3 * 64 + 1)
    bad.write_bytes(bytes(raw2))
    with pytest.raises(hv.HoloError):
        hv.HoloFile(bad)
    # a newer version than this build
    raw3 = bytearray(raw)
    raw3 += b'{"compute_settings": {"version": "v1"}, "info": {}}'
    struct.pack_into("<H", raw3, 4, 9)
    bad.write_bytes(bytes(raw3))
    with pytest.raises(hv.HoloError) as e:
        hv.HoloFile(bad)
    assert e.value.status == hv.HV_ERR_UNSUPPORTED
    # an unreadable footer is skipped like the reference does
    raw4 = bytearray(raw) + b"{not json"
    bad.write_bytes(bytes(raw4))
    with hv.HoloFile(bad) as f:
        assert f.footer() == {}


def test_big_endian_and_processed_output(tmp_path):
    fd = hv.FrameDescriptor(16, 16, 2, 1)
    frames = np.arange(2 * 256, dtype=np.uint16).reshape(2, 16, 16)
    p = tmp_path / "d.holo"
    hv.write_holo(p, fd, frames, _settings(), input_fps=100, data_type=hv.HOLO_PROCESSED)
    with hv.HoloFile(p) as f:
        assert f.fd.byte_endian == 1 and f.header.data_type == hv.HOLO_PROCESSED


V4_FOOTER = {
    "compute settings": {
        "image rendering": {"space transformation": "FRESNELTR", "time transformation": "PCA",
                            "time transformation size": 32, "time transformation stride": 32, "batch size": 32,
                            "lambda": 7.85e-07, "z distance": 0.45, "image mode": "HOLOGRAM",
                            "filter2d": {"enabled": False, "n1": 0, "n2": 1}},
        "view": {"type": "SQUAREDMODULUS", "fft shift": True, "renorm": True,
                 "p": {"index": 28, "accu level": 3}, "q": {"index": 0, "accu level": 0},
                 "window": {"xy": {"img accu level": 2, "log enabled": False, "flip": False, "rot": 0.0,
                                   "contrast": {"enabled": True, "auto refresh": True, "invert": False,
                                                "min": 1.0, "max": 65535.0}}}},
        "advanced": {"renorm constant": 7, "buffer size": {"input": 256, "output": 512},
                     "contrast": {"lower": 0.5, "upper": 99.5, "cuts p offset": 2}},
    },
    "info": {"input fps": 500, "contiguous": 1, "pixel size": {"x": 12.0, "y": 12.0}, "raw bitshift": 0},
}


def test_v4_footer_conversion(tmp_path):
    out = json.loads(hv.convert_holo_footer(json.dumps(V4_FOOTER), 4))
    cs = out["compute_settings"]
    assert cs["version"] == "v1"
    assert cs["image_rendering"]["propagation_distance"] == 0.45
    assert cs["image_rendering"]["filter2d"] == {"enabled": False, "inner_radius": 0, "outer_radius": 1}
    assert cs["view"]["image_type"] == "SQUARED_MODULUS"
    assert cs["view"]["z"] == {"start": 28, "width": 3}
    assert cs["view"]["window"]["xy"]["output_image_accumulation"] == 2
    assert cs["view"]["window"]["xy"]["horizontal_flip"] is False
    assert cs["advanced"]["contrast"]["frame_index_offset"] == 2 and cs["advanced"]["raw_bitshift"] == 0
    assert out["info"]["pixel_pitch"] == {"x": 12, "y": 12} and out["info"]["input_fps"] == 500
    # through a file of version 4: the settings come out of the converted footer
    fd = hv.FrameDescriptor(32, 32, 1, 0)
    p = tmp_path / "v4.holo"
    hv.write_holo(p, fd, np.zeros((2, 32, 32), np.uint8), footer=json.dumps(V4_FOOTER))
    raw = bytearray(p.read_bytes())
    struct.pack_into("<H", raw, 4, 4)
    p.write_bytes(bytes(raw))
    with hv.HoloFile(p) as f:
        s = f.settings()
        assert f.header.data_type == 0  # no data type before version 7
    assert (s.space_transformation, s.time_transformation, s.time_transformation_size) == (1, 2, 32)
    assert (s.image_type, s.p_start, s.p_width, s.accumulation, s.renorm_constant) == (1, 28, 3, 2, 7)
    assert np.float32(s.z_distance) == np.float32(0.45) and s.pixel_size == 12.0 and s.fft_shift == 1
    assert (s.input_buffer_size, s.output_buffer_size) == (256, 512)


def test_v3_flat_footer_conversion():
    flat = {"#img": 16, "algorithm": 2, "mode": 2, "time_filter": 1, "lambda": 8.52e-07, "z": 0.3,
            "contrast_max": 1000.0, "contrast_min": 10.0, "fft_shift_enabled": True, "img_acc_slice_xy_level": 4,
            "log_scale": False, "p": 1, "p_acc_level": 0, "renorm_enabled": False, "pixel_size": 20.0}
    for version in (2, 3):
        out = json.loads(hv.convert_holo_footer(json.dumps(flat), version))
        cs = out["compute_settings"]
        ir, view = cs["image_rendering"], cs["view"]
        assert ir["space_transformation"] == "ANGULARSP" and ir["time_transformation"] == "STFT"
        assert ir["image_mode"] == "HOLOGRAM" and ir["time_transformation_size"] == 16
        assert ir["propagation_distance"] == 0.3 and view["fft_shift"] is True and view["renorm"] is False
        assert view["z"] == {"start": 1, "width": 0}
        assert view["window"]["xy"]["contrast"] == {"max": 1000, "min": 10}
        assert view["window"]["xy"]["output_image_accumulation"] == 4
        assert out["info"]["pixel_pitch"] == {"x": 20, "y": 20}


def test_current_footers_unchanged_and_settings_v0():
    s = _settings()
    fd_json = hv.settings_to_json(s)
    doc = json.loads(fd_json)
    for v in (5, 6, 7):
        footer = {"compute_settings": doc, "info": {"pixel_pitch": {"x": 12, "y": 12}, "input_fps": 10}}
        assert json.loads(hv.convert_holo_footer(json.dumps(footer), v)) == footer
    # a compute-settings document without a version is v0 (ComputeSettingsConverter)
    v0 = json.loads(fd_json)
    del v0["version"]
    v0["image_rendering"]["convolution"]["enabled"] = False
    v0["image_rendering"]["input_filter"]["enabled"] = False
    v0["advanced"]["record_mode"] = "RAW"
    del v0["view"]["registration"]
    v1 = json.loads(hv.convert_settings_json(json.dumps(v0)))
    assert v1["version"] == "v1" and v1["view"]["registration"] == {"registration_enabled": False,
                                                                   "registration_zone": 0.7}
    assert "enabled" not in v1["image_rendering"]["convolution"] and "record_mode" not in v1["advanced"]
    assert hv.Settings.from_json(json.dumps(v1)).p_start == 3
    with pytest.raises(hv.HoloError):
        hv.convert_settings_json(json.dumps({"version": "v9"}))


def test_settings_json_round_trip():
    s = _settings()
    back = hv.Settings.from_json(hv.settings_to_json(s))
    for k in FIELDS:
        if k == "pixel_size":  # not part of the compute settings (the .holo footer's info)
            continue
        assert np.float32(getattr(back, k)) == np.float32(getattr(s, k)), k
