"""Compute-settings JSON through the C ABI (host logic only, no GPU): full documents in the
reference's ComputeSettings layout, partial merges, enum aliases and unknown-key rejection
(merge_json, Backend/sources/core/compute_settings.cc:24-36)."""

import json
from pathlib import Path

import pytest

import holovibes_gb300 as hv

GOLDEN = Path(__file__).resolve().parent / "golden"


def test_full_document():
    s = hv.Settings.from_json((GOLDEN / "compute_settings_2fft_stft.json").read_text())
    assert s.space_transformation == hv.SPACE_ANGULARSP and s.time_transformation == hv.TIME_STFT
    assert s.time_transformation_size == 32 and s.batch_size == 1
    assert s.lambda_ == pytest.approx(852e-9, rel=1e-6) and s.z_distance == pytest.approx(0.385, rel=1e-6)
    assert s.contrast_enabled == 1 and s.contrast_lower == pytest.approx(0.5) and s.contrast_upper == pytest.approx(99.5)
    assert s.renorm == 0 and s.fft_shift == 0 and s.accumulation == 0
    assert s.output_buffer_size == 64 and s.input_buffer_size == 256


@pytest.mark.parametrize("alias,val", [("FFT1", 1), ("1FFT", 1), ("Fresnel Tr.", 1), ("FFT2", 2), ("2FFT", 2),
                                       ("Angular SP.", 2), ("None", 0), ("NONE", 0)])
def test_space_aliases(alias, val):
    s = hv.Settings.from_json(json.dumps({"image_rendering": {"space_transformation": alias}}))
    assert s.space_transformation == val


def test_partial_merge_keeps_base():
    base = hv.Settings.defaults().update(batch_size=8, time_stride=8)
    s = hv.Settings.from_json('{"view": {"image_type": "SQUARED_MODULUS", "z": {"start": 3}}}', base)
    assert s.image_type == hv.IMG_SQUARED_MODULUS and s.p_start == 3 and s.batch_size == 8


def test_unknown_key_rejected():
    with pytest.raises(hv.HoloError) as e:
        hv.Settings.from_json('{"view": {"not_a_setting": 1}}')
    assert e.value.status == hv.HV_FAILURE
    with pytest.raises(hv.HoloError) as e:
        hv.Settings.from_json('{"view": {"image_type": "MODULUS"')
    assert e.value.status == hv.HV_FAILURE
    with pytest.raises(hv.HoloError) as e:
        hv.Settings.from_json('{}')
    assert e.value.status == hv.HV_NO_IN_DATA
    with pytest.raises(hv.HoloError):
        hv.Settings.from_json('{"image_rendering": {"time_transformation": "WAVELET"}}')
