"""The C ABI surface on CPU: the library loads without a GPU, exports every function that
include/holovibes_gb300.h declares, and its host-side logic (settings defaults, JSON merge,
validation, footprint) works. No kernel is launched here."""

import ctypes as C
import re
from pathlib import Path

import pytest

import holovibes_gb300 as hv

HEADER = Path(__file__).resolve().parents[1] / "include" / "holovibes_gb300.h"


def declared_functions():
    text = re.sub(r"/\*.*?\*/", "", HEADER.read_text(), flags=re.S)
    return sorted(set(re.findall(r"\b(hv_[a-z0-9_]+)\s*\(", text)))


def test_library_exports_every_declared_symbol():
    L = hv.lib()
    names = declared_functions()
    assert len(names) > 30
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing, missing


def test_every_declared_function_has_a_python_signature():
    """The ctypes binding sets restype / argtypes for every function of the header (an untyped
    call would pass 64-bit pointers and sizes as C ints); the argument count matches the
    declaration's."""
    L = hv.lib()
    text = re.sub(r"/\*.*?\*/", "", HEADER.read_text(), flags=re.S)
    untyped, wrong_count = [], []
    for name in declared_functions():
        fn = getattr(L, name)
        if fn.argtypes is None:
            untyped.append(name)
            continue
        m = re.search(r"\b" + name + r"\s*\(([^)]*)\)", text)
        params = [a for a in m.group(1).split(",") if a.strip() and a.strip() != "void"]
        if len(params) != len(fn.argtypes):
            wrong_count.append((name, len(params), len(fn.argtypes)))
    assert not untyped, untyped
    assert not wrong_count, wrong_count


def test_version_and_defaults():
    assert "sm_103a" in hv.version()
    s = hv.Settings.defaults()
    # Backend/includes/core/holovibes.hh:370-450 defaults
    assert s.batch_size == 1 and s.time_stride == 1 and s.time_transformation_size == 1
    assert abs(s.lambda_ - 852e-9) < 1e-13 and s.pixel_size == 12.0
    assert s.renorm == 1 and s.renorm_constant == 5
    assert abs(s.contrast_lower - 0.02) < 1e-6 and abs(s.contrast_upper - 99.98) < 1e-4


def test_validate_rules():
    fd = hv.FrameDescriptor(512, 512, 2)
    s = hv.Settings.defaults().update(batch_size=16, time_stride=20, time_transformation_size=8, p_start=9,
                                      p_width=3, z_distance=0.0, space_transformation=2)
    v = s.validate(fd)
    assert v.time_stride == 16  # lowered to a multiple of the batch (transform_api.cc:62-67)
    assert v.p_width == 3 and v.p_start == 4  # check_p_limits: start <= T-1-width
    assert v.z_distance == pytest.approx(1e-6)
    s2 = hv.Settings.defaults().update(batch_size=16, time_stride=4)
    assert s2.validate(fd).time_stride == 16
    with pytest.raises(hv.HoloError) as e:
        hv.Settings.defaults().update(space_transformation=2).validate(hv.FrameDescriptor(1000, 512, 2))
    assert e.value.status == hv.HV_ERR_UNSUPPORTED
    with pytest.raises(hv.HoloError) as e:
        hv.Settings.defaults().update(image_type=4).validate(fd)  # COMPOSITE is outside the path
    assert e.value.status == hv.HV_WRONG_IMG_TYPE
    # check_q_limits (transform_api.cc:208-225): width <= T-1, start <= T-1-width
    q = hv.Settings.defaults().update(time_transformation=3, time_transformation_size=16, q_start=15,
                                      q_width=20).validate(fd)
    assert (q.q_width, q.q_start) == (15, 0)
    q = hv.Settings.defaults().update(time_transformation=3, time_transformation_size=16, q_start=14,
                                      q_width=2).validate(fd)
    assert (q.q_width, q.q_start) == (2, 13)


def test_footprint_scales_with_ring():
    fd = hv.FrameDescriptor(512, 512, 2)
    a = hv.Pipe.footprint(fd, hv.Settings.defaults().update(time_transformation_size=16, time_transformation=1))
    b = hv.Pipe.footprint(fd, hv.Settings.defaults().update(time_transformation_size=32, time_transformation=1))
    assert b - a >= 16 * 512 * 512 * 8
