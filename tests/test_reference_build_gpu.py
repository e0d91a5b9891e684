"""The reference's own GPU build (its unmodified cuFFT / cuBLAS / cuSOLVER / thrust translation units,
driven in Pipe::refresh order by oracle/ref_pipe.cu) against the oracle and the product on the same
seeded interferograms. This pins the oracle to outputs of the reference's code.

* Lenses: the product's HV_LENS_REF32 lens against the lens the reference's kernels computed, bit
  for bit (the angular-spectrum phase is ~2e6 rad, rounded to float: one ulp is 0.25 rad, so only
  bit-identical lenses give comparable holograms), and the oracle's float32 restatement of it. The
  reference's compiler contracts u*u + v*v and 1 - lam^2 s into fused multiply-adds; the table of
  float32 variants printed for the angular spectrum shows which contraction its lens has.
* Whole cycles at the benchmark sizes (cfg0..cfg3): float frame fed to the contrast stage and the
  time ring of the reference build against the FP64 oracle (float32 lens restatement, as the
  reference computes its lens) and against the product (lens mode HV_LENS_REF32).
* Contrast stage: the oracle's percentile / contrast / float->ushort restatement run on the
  reference build's own float frame gives the reference's contrast range and uint16 frame exactly.

Skipped when the reference build is not available (its sources are staged from the reference tree
by oracle/ref_build.py; the staged copy travels with the working tree)."""

import sys
from pathlib import Path

import numpy as np
import pytest

import holovibes_oracle as O
from gpu_util import call, empty, host, oracle_settings, ptr, rel_l2, wrapped_diff

import holovibes_gb300 as hv
from holovibes_gb300.synthetic import CONFIGS, generator, settings_for

sys.path.insert(0, str(Path(__file__).resolve().parents[1] / "oracle"))
import ref_pipe  # noqa: E402

pytestmark = pytest.mark.skipif(not ref_pipe.available(), reason="reference build sources are not staged")

# float frame bars, reference build against the FP64 oracle and against the product; the 2-D
# unwrap spreads branch-cut flips of the argument over the frame (the reference's own build is
# 2.9e-4 from the FP64 oracle on the cfg2 frames)
BARS = {"STFT": 1e-4, "PCA": 1e-4, "UNWRAP": 2e-3}


def _f32_fma(a, b, c):
    """fmaf(a, b, c) for float32 arrays: the exact a*b + c rounded once (extended precision sum)."""
    ld = np.longdouble
    return (np.asarray(a, np.float32).astype(ld) * np.asarray(b, np.float32).astype(ld)
            + np.asarray(c, np.float32).astype(ld)).astype(np.float32)


def _as_lens_variants(W, H, lam, z, pixel_size_um):
    """The float32 angular-spectrum lens (masks.cu:31-59) with and without fused multiply-adds in
    tmp = 1 - lam^2 (u^2 + v^2), as the reference's compiler may contract them; quadrant-swapped."""
    F = np.float32
    lam32, z32 = F(lam), F(z)
    step = F(F(pixel_size_um) * F(1e-6))
    u = (np.arange(W) - (W >> 1)).astype(F) * F(F(1.0) / F(F(W) * step))
    v = (np.arange(H) - (H >> 1)).astype(F) * F(F(1.0) / F(F(H) * step))
    U, V = np.meshgrid(u, v)
    ll = F(lam32 * lam32)
    sums = {"u*u+v*v": (U * U).astype(F) + (V * V).astype(F), "fma(u,u,v*v)": _f32_fma(U, U, (V * V).astype(F)),
            "fma(v,v,u*u)": _f32_fma(V, V, (U * U).astype(F))}
    out = {}
    for sname, s in sums.items():
        s = s.astype(F)
        for tname, tmp in (("1-ll*s", (F(1.0) - (ll * s).astype(F)).astype(F)),
                           ("fma(-ll,s,1)", _f32_fma(-ll, s, np.ones_like(s)))):
            tmp = np.maximum(tmp, F(0.0))
            ph = ((2.0 * np.pi * float(z32)) / float(lam32) * np.sqrt(tmp).astype(F).astype(np.float64)).astype(F)
            out[f"{sname}, {tname}"] = O.shift_corners(ph.astype(np.float64))
    return out


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["cfg0", "cfg1", "cfg2"])
def test_lens_bits(cuda, name):
    c = CONFIGS[name]
    st = c["settings"]
    W, H = c["width"], c["height"]
    ref = ref_pipe.RefPipe(W, H, c["depth"], space=["NONE", "FRESNELTR", "ANGULARSP"][st["space_transformation"]],
                           time="STFT", time_transformation_size=st["time_transformation_size"],
                           time_stride=st["batch_size"], batch_size=st["batch_size"], lam=st["lambda_"],
                           z=st["z_distance"], pixel_size=st["pixel_size"])
    ref_lens = ref.lens()
    ref.close()
    fd = hv.FrameDescriptor(W, H, c["depth"])
    s = settings_for(name).validate(fd)
    lens = empty(W * H * 8)
    fn = "hv_fresnel_lens" if st["space_transformation"] == 1 else "hv_angular_spectrum_lens"
    call(fn, ptr(lens), W, H, s.lambda_, s.z_distance, s.pixel_size, hv.LENS_REF32, None)
    got = host(lens, np.complex64, (H, W))
    mism = int(np.count_nonzero(got != ref_lens))
    report = {"product REF32 mismatching elements": mism}
    if st["space_transformation"] == 2:
        ref_phase = np.angle(ref_lens.astype(np.complex128))
        for k, ph in _as_lens_variants(W, H, s.lambda_, s.z_distance, s.pixel_size).items():
            d = np.abs(wrapped_diff(np.angle(np.exp(1j * ph)), ref_phase))
            report[f"float32 phase {k}: pixels off by > 1e-3 rad"] = int(np.count_nonzero(d > 1e-3))
        oracle_phase = np.angle(O.angular_spectrum_lens(W, H, s.lambda_, s.z_distance, s.pixel_size, "ref32"))
    else:
        oracle_phase = np.angle(O.fresnel_lens(W, H, s.lambda_, s.z_distance, s.pixel_size, "ref32"))
    # the oracle's float32 restatement: the same phases (cosf / sinf against numpy's cos / sin aside)
    d = np.abs(wrapped_diff(oracle_phase, np.angle(ref_lens.astype(np.complex128))))
    report["oracle ref32 max phase diff (rad)"] = float(d.max())
    print(f"\n{name} lens vs the reference build: {report}")
    assert mism == 0, report
    assert report["oracle ref32 max phase diff (rad)"] <= 1e-5, report


def _reference_cycle_compare(name, nbatches, **over):
    c = CONFIGS[name]
    fd = hv.FrameDescriptor(c["width"], c["height"], c["depth"])
    s = settings_for(name, lens_mode=hv.LENS_REF32, **over).validate(fd)
    os_ = oracle_settings(fd, s)
    oracle = O.OraclePipe(os_)
    ref = ref_pipe.RefPipe.from_oracle_settings(os_)
    pipe = hv.Pipe(fd, s)
    gen = generator(name, seed=1234)
    B = s.batch_size
    argument = s.image_type == hv.IMG_ARGUMENT and not s.unwrap_2d
    bar = BARS["UNWRAP" if s.unwrap_2d else "PCA" if s.time_transformation == hv.TIME_PCA else "STFT"]
    rows = []
    for b in range(nbatches):
        raw = gen.frames(b * B, B)
        o = oracle.process_batch(raw)
        r = ref.push(raw)
        pipe.enqueue(raw)
        assert r == (o is not None) == (pipe.output_count() == 1), (name, b)
        if o is None:
            continue
        rf = ref.float_frame()
        ru16 = ref.output()
        pipe.pull()
        pf = pipe.float_frame()
        row = {"batch": b}
        for label, x, y in (("ref_vs_oracle", rf, o.float_frame), ("product_vs_ref", pf, rf)):
            if argument:
                wd = wrapped_diff(x, y)
                cut = np.abs(wd) > 1e-3
                row[label] = float(np.linalg.norm(wd[~cut]) / np.linalg.norm(np.asarray(y)[~cut]))
                row[label + "_branch_cut_fraction"] = float(np.mean(cut))
            else:
                row[label] = rel_l2(x, y)
        # the oracle's contrast stage on the reference's own float frame reproduces its output
        lo, hi = ref.contrast_range()
        if o.autocontrast_applied:
            olo, ohi = O.autocontrast(rf, s.contrast_lower, s.contrast_upper)
            row["contrast_range_equal"] = (np.float32(olo), np.float32(ohi)) == (np.float32(lo), np.float32(hi))
        u16 = O.float_to_ushort(O.apply_contrast(rf, lo, hi, bool(s.contrast_invert)))
        row["u16_mismatch_oracle_stage_on_ref_frame"] = int(np.count_nonzero(u16 != ru16))
        rows.append(row)
    rring, rstart, rsize = ref.ring()
    ref.close()
    pipe.close()
    assert (rstart, rsize) == (oracle.ring.start, oracle.ring.size), name
    ring_err = rel_l2(rring, oracle.ring.data)
    print(f"\n{name} {over or ''} reference build: ring vs oracle rel-L2 {ring_err:.2e}; {rows}")
    assert ring_err <= 1e-5, (name, ring_err)
    assert rows, name
    for row in rows:
        assert row.get("contrast_range_equal", True), (name, row)
        for label in ("ref_vs_oracle", "product_vs_ref"):
            assert row.get(label + "_branch_cut_fraction", 0.0) < 5e-3, (name, label, row)
        assert row["u16_mismatch_oracle_stage_on_ref_frame"] == 0, (name, row)
        assert row["ref_vs_oracle"] <= bar, (name, row)
        assert row["product_vs_ref"] <= bar, (name, row)


@pytest.mark.gpu
def test_reference_cycle_cfg0(cuda):
    _reference_cycle_compare("cfg0", 2)


@pytest.mark.gpu
def test_reference_cycle_cfg1(cuda):
    _reference_cycle_compare("cfg1", 2)


@pytest.mark.gpu
@pytest.mark.parametrize("unwrap", [0, 1])
def test_reference_cycle_cfg2(cuda, unwrap):
    _reference_cycle_compare("cfg2", 5, unwrap_2d=unwrap)


@pytest.mark.gpu
def test_reference_cycle_cfg3(cuda):
    _reference_cycle_compare("cfg3", 8)
